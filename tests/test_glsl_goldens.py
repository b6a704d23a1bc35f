"""The engine's shading math pinned to the reference's own code.

tests/golden/glsl_shading.npz holds golden vectors written by the reference's
GLSL helpers -- UpdateSurface, EvaluateDiffuseBRDF / EvaluateSpecularBRDF,
SampleDiffuseBRDF / SampleSpecularBRDF (GGX VNDF), SampleTriangleLight,
IntersectTriangle / IntersectAABB and the engine's random() -- compiled
unmodified on the host by oracle/glsl/make_ref.py.  Here the oracle's
restatement (CPU) and the path tracer's and traversal's own device functions
(GPU, through ae_rt_selftest_shading) are held to them: the intersections bit
for bit, the BRDF from the reference's own surface terms to a few ulps, and
everything from raw vectors within the rounding of normalize / sqrt / pow
(shading_util.check states the tolerance and why).
"""
import numpy as np
import pytest

import shading_util as S


def test_fixture_is_what_the_reference_writes():
    """Where the reference tree is present, rebuilding the goldens from its
    GLSL gives the committed fixture bit for bit."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import gen_glsl_goldens as G
    lib = G.reference_lib()
    if lib is None:
        pytest.skip("reference tree not present")
    g = S.golden()
    ins = G.inputs()
    for k, v in ins.items():
        assert np.array_equal(v.view(np.uint32), g[k].view(np.uint32)), k
    for k, v in G.evaluate(lib, ins).items():
        assert np.array_equal(v.view(np.uint32), g[k].view(np.uint32)), k


def test_reference_random_is_the_documented_hash():
    """random(x, seed) of common/random.hsh: Jenkins' one-at-a-time hash of the
    bits of vec2(x, seed), its low 23 bits as a float in [0, 1); the engine's
    draws, restated in numpy, equal the compiled GLSL's (the library's own
    RNG is a PCG hash instead, a documented deviation)."""
    g = S.golden()

    def h(x):
        x = np.uint64(x)
        M = np.uint64(0xFFFFFFFF)
        x = (x + (x << np.uint64(10))) & M
        x ^= x >> np.uint64(6)
        x = (x + (x << np.uint64(3))) & M
        x ^= x >> np.uint64(11)
        x = (x + (x << np.uint64(15))) & M
        return x
    out = np.zeros_like(g["random_out"])
    for i, x in enumerate(g["random_x"]):
        seed = np.float32(1.0)
        for k in range(8):
            bx, bs = np.float32(x).view(np.uint32), np.float32(seed).view(np.uint32)
            m = (int(bx) ^ int(h(int(bs)))) & 0xFFFFFFFF
            m = int(h(m)) & 0x007FFFFF | 0x3F800000
            out[i, k] = np.uint32(m).view(np.float32) - np.float32(1.0)
            seed = np.float32(seed + np.float32(1.0))
    assert np.array_equal(out.view(np.uint32), g["random_out"].view(np.uint32))


@pytest.mark.parametrize("name", sorted(S.SETS))
def test_oracle_matches_reference_glsl(name):
    g = S.golden()
    ik, ok, w, fn, extra, _ = S.SETS[name]
    got = S.run_oracle(fn, g[ik], w, *extra)
    S.check(name, got, g[ok], exact=name in ("triangle", "aabb", "triangle_light"))


def test_oracle_brdf_from_reference_terms():
    """The restated BRDF formulas, fed the reference's own surface terms, give
    its values to a few ulps (x^5 as products where the GLSL calls pow)."""
    g = S.golden()
    rows, ref = S.terms_rows(g)
    got = S.run_oracle("aeo_shade_eval_terms", rows, 6)
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-30)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(S.SETS))
def test_gpu_device_functions_match_reference_glsl(name):
    import atlas_rt
    g = S.golden()
    ik, ok, w, _, _, kind = S.SETS[name]
    ctx = atlas_rt.Context(device=0)
    try:
        got = S.run_gpu(ctx, kind, g[ik], w)
    finally:
        ctx.close()
    S.check(name, got, g[ok], exact=name in ("triangle", "aabb"))


@pytest.mark.gpu
def test_gpu_brdf_from_reference_terms():
    """The path tracer's BRDF device functions, fed the reference's own surface
    terms, give its values to a few ulps."""
    import atlas_rt
    g = S.golden()
    rows, ref = S.terms_rows(g)
    ctx = atlas_rt.Context(device=0)
    try:
        got = S.run_gpu(ctx, 4, rows, 6)
    finally:
        ctx.close()
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-30)
