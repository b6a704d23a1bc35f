"""The C-ABI boundary without a GPU: the library loads, exports every symbol
that include/atlas_rt.h declares, its structs have the engine's sizes, and
argument errors come back as status codes."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from atlas_rt import _native

REPO = Path(__file__).resolve().parent.parent
HEADER = REPO / "include" / "atlas_rt.h"


def declared_functions(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ae_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native):
    names = declared_functions(HEADER)
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, f"not exported: {missing}"
    # and the Python binding declares exactly those
    assert sorted(_native.EXPORTED) == names


def test_struct_sizes_match_engine_layouts(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include "atlas_rt.h"\n'
        '_Static_assert(sizeof(ae_aabb) == 24, "GPUAABB");\n'
        '_Static_assert(sizeof(ae_bvh_node) == 64, "GPUBVHNode");\n'
        '_Static_assert(sizeof(ae_bvh_triangle) == 48, "GPUBVHTriangle");\n'
        '_Static_assert(sizeof(ae_triangle) == 96, "GPUTriangle");\n'
        '_Static_assert(sizeof(ae_bvh_instance) == 64, "GPUBVHInstance");\n'
        '_Static_assert(sizeof(ae_material) == 92, "GPUMaterial");\n'
        '_Static_assert(sizeof(ae_light) == 64, "GPULight");\n'
        '_Static_assert(sizeof(ae_packed_ray) == 48, "PackedRay");\n'
        '_Static_assert(sizeof(ae_hit) == 32, "hit record");\n'
        'int main(void) { return 0; }\n')
    r = subprocess.run(["gcc", "-std=c11", "-fsyntax-only", f"-I{REPO / 'include'}", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_builder_argument_errors(native):
    h = C.c_void_p()
    assert native.ae_bvh_build_triangles(None, None, 5, 0, C.byref(h)) == 1
    assert native.ae_bvh_build_triangles(None, None, 0, 0, None) == 1
    assert native.ae_bvh_build_aabbs(None, 3, 0, C.byref(h)) == 1
    assert native.ae_bvh_get_nodes(None, None) == 1
    assert native.ae_bvh_node_count(None) == 0


def test_context_calls_reject_null(native):
    assert native.ae_rt_ctx_create(None, None) == 1
    assert native.ae_rt_trace_closest(None, 0, None, 0, 0.0, 1.0, None, None) == 1
    assert native.ae_rt_synchronize(None, None) == 1
    assert native.ae_rt_last_error(None) == b"null context"


def test_no_device_status_without_gpu(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert native.ae_rt_ctx_create(None, C.byref(h)) == 8  # AE_RT_NO_DEVICE
