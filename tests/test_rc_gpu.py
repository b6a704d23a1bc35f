"""Radiance cache on the GPU: the fused BF16 tensor-core encode+MLP forward
and backward against the FP64 oracle (oracle/rc_oracle.py), training
behaviour, and what the trained cache gains over the path tracer without it.

Tolerances: the kernels round the network input, every activation and the
backward deltas to BF16 (8-bit mantissa) and read FP16 table values; the
oracle applies the same roundings (emulate_params, bf16=True) and computes
everything else in FP64, so the remaining differences are FP32 accumulation
order and values that land on the other side of a BF16 rounding boundary:
predictions are compared at 1 % and gradient vectors at 3 % relative L2
error with cosine similarity above 0.999.  Against the unrounded FP64
network the errors stay below 3 % (forward) and 25 % (gradients: BF16
deltas through six layers).
"""
import numpy as np
import pytest

import atlas_rt
import rc_oracle
from atlas_rt import ptscene, scenes

pytestmark = pytest.mark.gpu

LO, HI = (0.0, -2.0, 0.0), (100.0, 62.0, 100.0)


def random_records(n, seed):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 16), np.float32)
    rec[:, 0:3] = rng.uniform(LO, HI, (n, 3))
    rec[:, 3] = rng.uniform(0.05, 1.0, n)
    d = rng.normal(size=(n, 3))
    rec[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3))
    rec[:, 8:11] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    rec[:, 12:15] = rng.uniform(0.0, 0.5, (n, 3))
    rec[:, 11] = rng.integers(0, 3, n)
    rec[:, 15] = 1.0
    return rec


@pytest.fixture(scope="module")
def cache():
    ctx = atlas_rt.Context(device=0)
    rc = atlas_rt.RadianceCache(ctx, LO, HI, log2_table=14, seed=3)
    yield ctx, rc
    rc.close()
    ctx.close()


def scaled_params(rc, seed):
    """Parameters large enough that every part of the input matters."""
    rng = np.random.default_rng(seed)
    mlp, grid = rc.get_params()
    mlp = mlp * 1.5
    grid = rng.uniform(-0.5, 0.5, grid.shape).astype(np.float32)
    return mlp.astype(np.float32), grid


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def cosine(a, b):
    return float(np.dot(a, b) / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30))


def test_forward_matches_fp64_oracle(cache):
    import torch
    ctx, rc = cache
    mlp, grid = scaled_params(rc, 1)
    rc.set_params(mlp, grid)
    rec = random_records(1000, 2)
    q = torch.from_numpy(rec).cuda()
    out = torch.zeros((len(rec), 4), dtype=torch.float32, device="cuda")
    rc.predict(q, out)
    ctx.synchronize()
    got = out.cpu().numpy()[:, :3]
    orc = rc_oracle.Cache(2 ** 14, LO, HI)
    m64, g64 = rc_oracle.emulate_params(mlp, grid)
    _, P = orc.forward(m64, g64.reshape(16, -1, 2), rec, bf16=True)
    assert rel(got, P[:, :3]) < 0.01, rel(got, P[:, :3])
    _, P64 = orc.forward(m64, g64.reshape(16, -1, 2), rec)
    assert rel(got, P64[:, :3]) < 0.03, rel(got, P64[:, :3])


def test_tensor_memory_wait_times_out_cleanly():
    """Failure detection without a fault: the inference kernel run with no
    MMA issued waits on an mbarrier that nothing completes; the bounded wait
    gives up (~200 ms), the kernel frees its tensor memory and returns, and
    the host reads AE_RT_TIMEOUT.  The context then still predicts correctly."""
    import torch
    ctx = atlas_rt.Context(device=0)
    rc = atlas_rt.RadianceCache(ctx, LO, HI, log2_table=14, seed=3)
    try:
        assert rc.selftest_wait_timeout()
        mlp, grid = scaled_params(rc, 1)
        rc.set_params(mlp, grid)
        rec = random_records(300, 4)
        out = torch.zeros((len(rec), 4), dtype=torch.float32, device="cuda")
        rc.predict(torch.from_numpy(rec).cuda(), out)
        ctx.synchronize()
        m64, g64 = rc_oracle.emulate_params(mlp, grid)
        _, P = rc_oracle.Cache(2 ** 14, LO, HI).forward(m64, g64.reshape(16, -1, 2), rec, bf16=True)
        assert rel(out.cpu().numpy()[:, :3], P[:, :3]) < 0.01
    finally:
        rc.close()
        ctx.close()


def test_gradients_match_fp64_oracle(cache):
    import torch
    ctx, rc = cache
    mlp, grid = scaled_params(rc, 4)
    rc.set_params(mlp, grid)
    rec = random_records(512, 5)
    q = torch.from_numpy(rec).cuda()
    gm = np.zeros(rc.n_mlp, np.float32)
    gg = np.zeros(rc.n_grid, np.float32)
    loss = rc.gradients(q, gm, gg)
    orc = rc_oracle.Cache(2 ** 14, LO, HI)
    m64, g64 = rc_oracle.emulate_params(mlp, grid)
    l_ref, gm_ref, gg_ref, _ = orc.loss_and_grads(m64, g64.reshape(16, -1, 2), rec, bf16=True)
    assert abs(loss - l_ref) / l_ref < 0.01, (loss, l_ref)
    assert rel(gm, gm_ref) < 0.03 and cosine(gm, gm_ref) > 0.999, (rel(gm, gm_ref), cosine(gm, gm_ref))
    assert rel(gg, gg_ref) < 0.03 and cosine(gg, gg_ref) > 0.999, (rel(gg, gg_ref), cosine(gg, gg_ref))
    _, gm64, gg64, _ = orc.loss_and_grads(m64, g64.reshape(16, -1, 2), rec)
    assert rel(gm, gm64) < 0.25 and rel(gg, gg64) < 0.25, (rel(gm, gm64), rel(gg, gg64))
    # per-layer check of the weight gradients
    for l in range(6):
        a = l * 4096
        b = a + (4096 if l < 5 else 16 * 64)
        assert cosine(gm[a:b], gm_ref[a:b]) > 0.998, l


@pytest.mark.parametrize("n", [512, 58_445])
def test_tensor_memory_training_equals_warp_mma(n):
    """The default training kernel (tcgen05, weight gradients accumulated in
    tensor memory over every tile of a CTA and added to the global sums once)
    and the warp-level mma.sync kernel give the same loss and gradients up to
    the order of FP32 additions (and the BF16 roundings that order can
    flip).  58,445 records give each CTA several tiles and a ragged last
    one."""
    import torch
    ctx = atlas_rt.Context(device=0)
    rcs = [atlas_rt.RadianceCache(ctx, LO, HI, log2_table=14, seed=3, warp_mma_training=w) for w in (False, True)]
    try:
        mlp, grid = scaled_params(rcs[0], 4)
        rec = random_records(n, 6)
        q = torch.from_numpy(rec).cuda()
        res = []
        for rc in rcs:
            rc.set_params(mlp, grid)
            gm = np.zeros(rc.n_mlp, np.float32)
            gg = np.zeros(rc.n_grid, np.float32)
            loss = rc.gradients(q, gm, gg)
            res.append((loss, gm, gg))
        (l0, gm0, gg0), (l1, gm1, gg1) = res
        assert abs(l0 - l1) / l1 < 1e-3, (l0, l1)
        assert rel(gm0, gm1) < 0.01 and cosine(gm0, gm1) > 0.9999, (rel(gm0, gm1), cosine(gm0, gm1))
        assert rel(gg0, gg1) < 0.01 and cosine(gg0, gg1) > 0.9999, (rel(gg0, gg1), cosine(gg0, gg1))
        for l in range(6):
            a = l * 4096
            b = a + (4096 if l < 5 else 16 * 64)
            assert rel(gm0[a:b], gm1[a:b]) < 0.02, l
    finally:
        for rc in rcs:
            rc.close()
        ctx.close()


def test_training_fits_a_smooth_field(cache):
    """Adam on a fixed batch drives the relative L2 loss down by 20x."""
    import torch
    ctx, rc = cache
    rc2 = atlas_rt.RadianceCache(ctx, LO, HI, log2_table=16, seed=9)
    try:
        rec = random_records(16384, 7)
        p = rec[:, 0:3] / 100.0
        rec[:, 12] = 0.2 + 0.1 * np.sin(6 * p[:, 0])
        rec[:, 13] = 0.15 + 0.1 * np.cos(4 * p[:, 2])
        rec[:, 14] = 0.1 + 0.05 * p[:, 1]
        q = torch.from_numpy(rec).cuda()
        losses = [rc2.train_batch(q) for _ in range(300)]
        assert losses[-1] < losses[0] / 20, (losses[0], losses[-1])
        mlp, grid = rc2.get_params()
        assert np.isfinite(mlp).all() and np.isfinite(grid).all()
    finally:
        rc2.close()


def test_params_roundtrip_and_checkpoint(cache):
    """get/set restore the cache exactly (checkpoint and resume)."""
    import torch
    ctx, rc = cache
    mlp, grid = scaled_params(rc, 11)
    rc.set_params(mlp, grid)
    m2, g2 = rc.get_params()
    assert np.array_equal(m2, mlp) and np.array_equal(g2, grid)
    rec = random_records(300, 12)
    q = torch.from_numpy(rec).cuda()
    o1 = torch.zeros((300, 4), dtype=torch.float32, device="cuda")
    o2 = torch.zeros((300, 4), dtype=torch.float32, device="cuda")
    rc.predict(q, o1)
    rc.train_batch(q)
    rc.set_params(mlp, grid)
    rc.predict(q, o2)
    ctx.synchronize()
    assert torch.equal(o1, o2)


def test_cache_gains_over_plain_path_tracer():
    """Online use (every frame trains the cache on 65,536 paths and renders
    one sample per pixel with paths ending in it, ae_rc_frame): after 16 training frames,
    4 rendered frames are at least twice as close (rel-MSE) to the converged
    image as the plain path tracer at 4 samples per pixel.  (960 x 540: at
    lower resolutions the variance of pixel-footprint sampling, which both
    share, dominates.)  Speed at equal error is the bench's measurement."""
    import torch
    w, h = 960, 540
    ctx = atlas_rt.Context(device=0)
    try:
        sc = ptscene.build()
        ptscene.upload(ctx, sc)
        cam = atlas_rt.make_camera(scenes.pinhole_camera(w, h))
        n = w * h
        ref = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        ref64 = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        for k in range(8):
            ctx.pathtrace(cam, ref, ref64, spp=512, sample_offset=100000 + 512 * k, seed=7)
        ctx.synchronize()
        refimg = (ref64 / 4096).cpu().numpy().reshape(h, w, 3)
        pt = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        ctx.pathtrace(cam, pt, spp=4, seed=3)
        ctx.synchronize()
        pt_err = ptscene.rel_mse((pt[:, :3] / 4).cpu().numpy().reshape(h, w, 3), refimg)
        ctx.pathtrace(cam, pt, spp=12, sample_offset=4, seed=3)
        ctx.synchronize()
        pt16_err = ptscene.rel_mse((pt[:, :3] / 16).cpu().numpy().reshape(h, w, 3), refimg)
        scale = 1.0 / float(ref[:, :3].mean() / 4096)
        bounds_lo, bounds_hi = atlas_rt.mesh_bounds(sc["bvh"])
        rc = atlas_rt.RadianceCache(ctx, bounds_lo - 0.5, bounds_hi + 0.5, seed=5, radiance_scale=scale)
        try:
            acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
            for f in range(20):
                if f < 16:
                    rc.train_frame(cam, f, n_paths=65536, steps=2)
                else:
                    rc.frame(cam, f, acc, n_paths=65536, steps=2)     # render beside training, then train
            ctx.synchronize()
            rc_img = (acc[:, :3] / 4).cpu().numpy().reshape(h, w, 3)
            rc_err = ptscene.rel_mse(rc_img, refimg)
        finally:
            rc.close()
        assert np.isfinite(rc_img).all()
        assert rc_err < pt_err / 2, (rc_err, pt_err, pt16_err)
    finally:
        ctx.close()
