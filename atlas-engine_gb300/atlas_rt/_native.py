"""ctypes declarations of libatlas_rt.so (include/atlas_rt.h).

The library is loaded from this directory only; if it is missing, importing
fails loudly -- there is no Python or CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libatlas_rt.so"

P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int32
F32 = C.c_float

STATUS_NAMES = {
    0: "AE_RT_OK", 1: "AE_RT_INVALID_ARG", 2: "AE_RT_BAD_BVH", 3: "AE_RT_OUT_OF_MEMORY",
    4: "AE_RT_CUDA_ERROR", 5: "AE_RT_TIMEOUT", 6: "AE_RT_STACK_OVERFLOW",
    7: "AE_RT_ITERATION_LIMIT", 8: "AE_RT_NO_DEVICE", 9: "AE_RT_NOT_BUILT",
}


class AeRtError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class Config(C.Structure):
    _fields_ = [("device", I32), ("blocks_per_sm", U32), ("threads_per_block", U32),
                ("max_steps", U32), ("flags", U32), ("refill_steps", U32), ("stack_entries_smem", U32),
                ("refill_below", U32), ("leaf_wait", U32)]


class BatchDesc(C.Structure):
    _fields_ = [("mesh_id", I32), ("any", U32), ("rays", P), ("out", P), ("n_rays", U32),
                ("tmin", F32), ("tmax", F32), ("reserved", U32)]


class Camera(C.Structure):
    _fields_ = [("location", F32 * 4), ("origin", F32 * 4), ("right", F32 * 4), ("bottom", F32 * 4),
                ("width", U32), ("height", U32), ("jitter", F32 * 2)]


class BounceParams(C.Structure):
    _fields_ = [("light_dir", F32 * 4), ("epsilon", F32), ("seed", U32), ("reserved", U32 * 2)]


class CastOutputs(C.Structure):
    _fields_ = [("primary_hits", P), ("secondary_rays", P), ("secondary_hits", P),
                ("shadow_rays", P), ("shadow_occluded", P), ("counts", U32 * 3)]


class MeshAssetInfo(C.Structure):
    _fields_ = [("vertex_count", U32), ("index_count", U32), ("triangle_count", U32), ("sub_count", U32),
                ("material_count", U32), ("tex_coord_count", U32), ("normal_count", U32), ("tangent_count", U32),
                ("color_count", U32), ("cull_back_faces", I32), ("invert_uvs", I32), ("cast_shadow", I32),
                ("primitive_type", I32), ("mobility", I32), ("usage", I32), ("radius", F32), ("aabb", F32 * 6)]


class MeshSub(C.Structure):
    _fields_ = [("indices_offset", U32), ("indices_count", U32), ("material_idx", I32), ("aabb", F32 * 6)]


class PtRealtime(C.Structure):
    _fields_ = [("depth", P), ("material_idx", P), ("normal", P), ("velocity", P), ("view", F32 * 16),
                ("proj", F32 * 16), ("pv_last", F32 * 16), ("last_matrices", P), ("n_last_matrices", U32)]


class PtParams(C.Structure):
    _fields_ = [("spp", U32), ("max_bounces", U32), ("sample_offset", U32), ("seed", U32),
                ("epsilon", F32), ("flags", U32), ("reserved", U32 * 2)]


class RcConfig(C.Structure):
    _fields_ = [("log2_table", U32), ("base_resolution", U32), ("max_resolution", U32),
                ("learning_rate", F32), ("beta1", F32), ("beta2", F32), ("epsilon", F32), ("seed", U32),
                ("aabb_min", F32 * 3), ("aabb_max", F32 * 3), ("radiance_scale", F32), ("rough_cut", F32),
                ("glossy_split", U32), ("flags", U32)]


class GBuffer(C.Structure):
    _fields_ = [("depth", P), ("normal", P), ("offset", P), ("roughness", P), ("samples", P), ("width", U32),
                ("height", U32), ("half_res", U32), ("reserved", U32), ("ip_matrix", F32 * 16),
                ("iv_matrix", F32 * 16), ("scrambling_ranking", P), ("sobol_sequence", P)]


class PassParams(C.Structure):
    _fields_ = [("radius", F32), ("bias", F32), ("roughness_cutoff", F32), ("radiance_limit", F32),
                ("environment", F32 * 3), ("flags", U32), ("frame_seed", U32), ("seed", U32),
                ("texture_level", U32), ("reserved", U32)]


class DdgiProbes(C.Structure):
    _fields_ = [("probes", P), ("ray_dirs", P), ("ray_dirs_inactive", P), ("rotation", F32 * 16),
                ("n_probes", U32), ("ray_count", U32), ("inactive_ray_count", U32), ("reserved", U32)]


# (name, restype, argtypes)
_SIGNATURES = [
    ("ae_bvh_build_triangles", C.c_int, [P, P, U32, C.c_int, C.POINTER(P)]),
    ("ae_bvh_build_aabbs", C.c_int, [P, U32, C.c_int, C.POINTER(P)]),
    ("ae_bvh_destroy", None, [P]),
    ("ae_bvh_node_count", U32, [P]),
    ("ae_bvh_primitive_count", U32, [P]),
    ("ae_bvh_get_nodes", C.c_int, [P, P]),
    ("ae_bvh_get_order", C.c_int, [P, P, P]),
    ("ae_bvh_pack_triangles", C.c_int, [P, P, P, P, P]),
    ("ae_bvh_pack_shading", C.c_int, [P, P, P, P, P, P]),
    ("ae_bvh_pack_uvs", C.c_int, [P, P, P]),
    ("ae_bvh_pack_attributes", C.c_int, [P, P, P, P, P, P]),
    ("ae_asset_last_error", C.c_char_p, []),
    ("ae_rt_scene_set_environment", C.c_int, [P, P]),
    ("ae_lights_from_mesh", C.c_int, [P, U32, P, P, U32, P, U32, C.POINTER(U32)]),
    ("ae_lights_instance", C.c_int, [P, U32, P, I32, P]),
    ("ae_light_directional", C.c_int, [P, F32, P, U32, P]),
    ("ae_lights_normalize", C.c_int, [P, U32]),
    ("ae_lights_select", C.c_int, [P, U32, U32, P, P, C.POINTER(U32)]),
    ("ae_mesh_asset_load", C.c_int, [P, C.c_size_t, C.POINTER(P)]),
    ("ae_mesh_asset_load_file", C.c_int, [C.c_char_p, C.POINTER(P)]),
    ("ae_mesh_asset_destroy", None, [P]),
    ("ae_mesh_asset_get_info", C.c_int, [P, C.POINTER(MeshAssetInfo)]),
    ("ae_mesh_asset_name", C.c_char_p, [P]),
    ("ae_mesh_asset_material_path", C.c_char_p, [P, U32]),
    ("ae_mesh_asset_get_sub", C.c_int, [P, U32, C.POINTER(MeshSub)]),
    ("ae_mesh_asset_get_arrays", C.c_int, [P, P, P, P, P, P, P]),
    ("ae_mesh_asset_triangles", C.c_int, [P, P, U32, P, P, P, P, P, P]),
    ("ae_material_asset_load", C.c_int, [P, C.c_size_t, C.POINTER(P)]),
    ("ae_material_asset_load_file", C.c_int, [C.c_char_p, C.POINTER(P)]),
    ("ae_material_asset_destroy", None, [P]),
    ("ae_material_asset_name", C.c_char_p, [P]),
    ("ae_material_asset_map_path", C.c_char_p, [P, U32]),
    ("ae_material_asset_get_emissive", C.c_int, [P, P, P]),
    ("ae_material_asset_to_gpu", C.c_int, [P, P, P, I32, P]),
    ("ae_rt_ctx_create", C.c_int, [C.POINTER(Config), C.POINTER(P)]),
    ("ae_rt_ctx_destroy", None, [P]),
    ("ae_rt_last_error", C.c_char_p, [P]),
    ("ae_rt_mesh_upload", C.c_int, [P, P, U32, P, P, U32, C.POINTER(I32)]),
    ("ae_rt_trace_closest", C.c_int, [P, I32, P, U32, F32, F32, P, P]),
    ("ae_rt_retest_near_ties", C.c_int, [P, I32, P, P, U32, F32, F32, P, C.POINTER(U32), P]),
    ("ae_rt_mesh_build", C.c_int, [P, P, U32, P, P, C.POINTER(I32), P, P]),
    ("ae_rc_frame", C.c_int, [P, P, U32, U32, U32, U32, U32, P, P, P]),
    ("ae_rt_mesh_get_bvh", C.c_int, [P, I32, P, P, C.POINTER(U32), C.POINTER(U32)]),
    ("ae_rt_trace_any", C.c_int, [P, I32, P, U32, F32, F32, P, P]),
    ("ae_rt_scene_set", C.c_int, [P, P, U32, P, U32]),
    ("ae_rt_scene_build", C.c_int, [P, P, P, U32, P, P]),
    ("ae_rt_trace_scene_closest", C.c_int, [P, P, U32, F32, F32, U32, P, P]),
    ("ae_rt_trace_scene_any", C.c_int, [P, P, U32, F32, F32, U32, P, P]),
    ("ae_rt_trace_scene_closest_transparency", C.c_int, [P, P, U32, F32, F32, U32, P, P]),
    ("ae_rt_trace_scene_any_transparency", C.c_int, [P, P, U32, F32, F32, U32, P, P]),
    ("ae_rt_trace_scene_closest_queue", C.c_int, [P, P, P, U32, F32, F32, U32, P, P]),
    ("ae_rt_trace_scene_any_queue", C.c_int, [P, P, P, U32, F32, F32, U32, P, P]),
    ("ae_rt_trace_batched", C.c_int, [P, P, U32, P]),
    ("ae_rt_batch_plan_create", C.c_int, [P, P, U32, C.POINTER(P)]),
    ("ae_rt_batch_plan_launch", C.c_int, [P, P]),
    ("ae_rt_batch_plan_destroy", None, [P]),
    ("ae_rt_scene_set_materials", C.c_int, [P, P, U32]),
    ("ae_rt_scene_set_textures", C.c_int, [P, P, U32]),
    ("ae_rt_scene_set_lights", C.c_int, [P, P, U32]),
    ("ae_rt_pathtrace", C.c_int, [P, C.POINTER(Camera), C.POINTER(PtParams), P, P, P]),
    ("ae_rt_pt_tonemap_tile", C.c_int, [P, P, U32, U32, U32, U32, U32, U32, U32, F32, F32, P, P]),
    ("ae_rt_pathtrace_tile", C.c_int, [P, C.POINTER(Camera), C.POINTER(PtParams), U32, U32, U32, U32, P, P, P]),
    ("ae_rt_pathtrace_realtime", C.c_int, [P, C.POINTER(Camera), C.POINTER(PtParams), P, P, F32, P]),
    ("ae_rt_pt_tonemap", C.c_int, [P, P, U32, U32, U32, F32, F32, P, P]),
    ("ae_rt_rtao", C.c_int, [P, C.POINTER(GBuffer), C.POINTER(PassParams), P, P]),
    ("ae_rt_reflections", C.c_int, [P, C.POINTER(GBuffer), C.POINTER(PassParams), P, P]),
    ("ae_rt_rtgi", C.c_int, [P, C.POINTER(GBuffer), C.POINTER(PassParams), P, P]),
    ("ae_rt_ddgi_trace", C.c_int, [P, C.POINTER(DdgiProbes), C.POINTER(PassParams), P, P]),
    ("ae_rc_create", C.c_int, [P, C.POINTER(RcConfig), C.POINTER(P)]),
    ("ae_rc_destroy", None, [P]),
    ("ae_rc_param_counts", C.c_int, [P, C.POINTER(U32), C.POINTER(C.c_uint64)]),
    ("ae_rc_get_params", C.c_int, [P, P, P]),
    ("ae_rc_set_params", C.c_int, [P, P, P]),
    ("ae_rc_predict", C.c_int, [P, P, U32, P, P]),
    ("ae_rc_selftest_wait_timeout", C.c_int, [P, C.POINTER(U32)]),
    ("ae_rc_gradients", C.c_int, [P, P, U32, P, P, C.POINTER(F32), P]),
    ("ae_rc_train_batch", C.c_int, [P, P, U32, C.POINTER(F32), P]),
    ("ae_rc_train_frame", C.c_int, [P, C.POINTER(Camera), U32, U32, U32, U32, C.POINTER(F32), P]),
    ("ae_rc_render", C.c_int, [P, C.POINTER(Camera), U32, U32, P, P]),
    ("ae_rt_trace_closest_noalloc", C.c_int, [P, U32, P, U32, P, U32, F32, F32, P, P]),
    ("ae_rt_raygen", C.c_int, [P, C.POINTER(Camera), P, P]),
    ("ae_rt_trace_closest_queue", C.c_int, [P, I32, P, P, U32, F32, F32, P, P]),
    ("ae_rt_trace_any_queue", C.c_int, [P, I32, P, P, U32, F32, F32, P, P]),
    ("ae_rt_spawn_bounce", C.c_int, [P, I32, P, P, P, U32, C.POINTER(BounceParams), P, P, P, P]),
    ("ae_rt_trace_camera_closest", C.c_int, [P, I32, C.POINTER(Camera), F32, F32, P, P]),
    ("ae_rt_spawn_bounce_camera", C.c_int, [P, I32, C.POINTER(Camera), P, C.POINTER(BounceParams), P, P, P, P]),
    ("ae_rt_cast_pass", C.c_int, [P, I32, C.POINTER(Camera), C.POINTER(BounceParams), C.POINTER(CastOutputs), P]),
    ("ae_rt_synchronize", C.c_int, [P, P]),
    ("ae_rt_selftest_division", C.c_int, [P, C.c_uint64, U32, C.POINTER(C.c_uint64)]),
    ("ae_rt_selftest_shading", C.c_int, [P, U32, P, U32, P]),
    ("ae_rt_get_fetch_counts", C.c_int, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
]

EXPORTED = [s[0] for s in _SIGNATURES]

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() "
                              "(the CUDA library is required, there is no fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in _SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib
