"""Golden vectors of the engine's shading math (tests/golden/glsl_shading.npz,
written by tests/golden/gen_glsl_goldens.py from the reference's own GLSL
compiled on the host) and the runners of the oracle's restatement and of the
GPU's device functions over them, with the tolerances both must meet."""
import ctypes as C
from pathlib import Path

import numpy as np

F32 = np.float32
GOLDEN = Path(__file__).resolve().parent / "golden" / "glsl_shading.npz"

# set -> (input key, output key, output width, oracle function, oracle extra args, GPU kind)
SETS = {
    "eval": ("eval_in", "eval_out", 16, "aeo_shade_eval", (), 0),
    "sample_diffuse": ("sample_in", "sample_diffuse_out", 8, "aeo_shade_sample", (0,), 1),
    "sample_specular": ("sample_in", "sample_specular_out", 8, "aeo_shade_sample", (1,), 2),
    "triangle_light": ("light_in", "light_out", 7, "aeo_shade_triangle_light", (), 3),
    "triangle": ("tri_in", "tri_out", 4, "aeo_shade_intersect_triangle", (), 5),
    "aabb": ("box_in", "box_out", 2, "aeo_shade_intersect_aabb", (), 6),
}


def golden():
    return dict(np.load(GOLDEN))


def terms_rows(g):
    """EVAL_TERMS rows from the reference's own surface terms: NdotL NdotV NdotH
    LdotH F0 F90 (its eval outputs 6..13) with the row's material."""
    e_in, e_out = g["eval_in"], g["eval_out"]
    return np.concatenate([e_out[:, 6:14], e_in[:, 9:14]], 1).astype(F32), e_out[:, 0:6]


def run_oracle(fn_name, x, width, *extra):
    import pyoracle
    L = pyoracle.port()
    x = np.ascontiguousarray(x, F32)
    out = np.zeros((len(x), width), F32)
    getattr(L, fn_name)(x.ctypes.data_as(C.c_void_p), C.c_int(len(x)), *[C.c_int(e) for e in extra],
                        out.ctypes.data_as(C.c_void_p))
    return out


def run_gpu(ctx, kind, x, width):
    from atlas_rt import _native
    x = np.ascontiguousarray(x, F32)
    out = np.zeros((len(x), width), F32)
    st = _native.lib().ae_rt_selftest_shading(ctx.handle, kind, x.ctypes.data, len(x), out.ctypes.data)
    assert st == 0, st
    return out


def check(name, got, ref, exact=False):
    """The tolerance each quantity is held to.  The intersections are
    bit-exact.  Everything else goes through normalize / sqrt / pow, which the
    reference's GLSL (compiled on the host: x / length(x), powf) and the
    restatements (x * rsqrt, x^5 as products) round differently by an ulp or
    two; cascaded normalizations and the reflection L = 2 (V.M) M - V leave
    absolute errors of unit-vector components below 5e-5, and the GGX term
    at roughness 0.05 (alpha^2 ~ 5e-6, where 1 - NdotH^2 cancels) turns
    last-place differences of NdotH into relative 2e-4."""
    if exact:
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), name
        return
    assert not np.any(np.isnan(got) != np.isnan(ref)), name
    np.testing.assert_allclose(got, ref, rtol=5e-4, atol=5e-5, err_msg=name)
