"""ctypes binding of librdn.so (include/rdn.h).

The library is built in-tree by ``rendiation_gb300.build_native.build()``.
Loading fails loudly when it is missing: there is no CPU fallback for any
query in this package.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librdn.so")

RDN_OK = 0
STATUS_NAMES = {
    0: "RDN_OK", -1: "RDN_ERR_INVALID_ARG", -2: "RDN_ERR_INVALID_HANDLE", -3: "RDN_ERR_OOM", -4: "RDN_ERR_CUDA",
    -5: "RDN_ERR_QUEUE_OVERFLOW", -6: "RDN_ERR_TIMEOUT", -7: "RDN_ERR_NOT_BUILT", -8: "RDN_ERR_UNSUPPORTED",
}

# every symbol include/rdn.h declares; tests check the library exports each one
EXPORTED_SYMBOLS = [
    "rdn_api_version", "rdn_create", "rdn_destroy", "rdn_last_error", "rdn_blas_create", "rdn_blas_delete",
    "rdn_tlas_create", "rdn_tlas_delete", "rdn_bind_tlas", "rdn_build", "rdn_get_build_stats", "rdn_get_built_array",
    "rdn_trace", "rdn_trace_counted", "rdn_wavefront_scratch_size", "rdn_wavefront_shadow_bounce",
    "rdn_wavefront_shadow_bounce_static", "rdn_paths_scratch_size", "rdn_trace_paths", "rdn_trace_paths_graph",
    "rdn_graph_launch", "rdn_graph_destroy", "rdn_attr_loss_forward", "rdn_attr_loss_adjoint",
    "rdn_hit_diff_forward", "rdn_hit_diff_adjoint",
    "rdn_scan_scratch_size", "rdn_scan_u32", "rdn_compact_scratch_size", "rdn_compact_u32",
    "rdn_radix_sort_scratch_size", "rdn_radix_sort_u32", "rdn_attr_paths_forward", "rdn_attr_paths_adjoint",
    "rdn_attr_paths_graph", "rdn_check_errors", "rdn_set_iteration_limit", "rdn_task_graph_create",
    "rdn_task_graph_destroy", "rdn_task_graph_dispatch_init", "rdn_task_graph_execute", "rdn_task_graph_states",
    "rdn_task_graph_debug", "rdn_task_graph_check_errors", "rdn_ao_pipeline_create", "rdn_ao_render_graph",
    "rdn_ao_render", "rdn_ao_capture", "rdn_task_graph_capture", "rdn_task_graph_set_poll", "rdn_trace_params",
    "rdn_path_tracing_render", "rdn_pt_scratch_size", "rdn_pt_capture",
]


# device error-word bits (rdn_check_errors)
ERROR_STACK_OVERFLOW, ERROR_BAD_TLAS_INDEX, ERROR_ITERATION_LIMIT = 0x1, 0x2, 0x4


class RdnError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Geometry(C.Structure):
    _fields_ = [("type", C.c_uint32), ("flags", C.c_uint32), ("positions", C.c_void_p), ("vertex_count", C.c_uint32),
                ("index_count", C.c_uint32), ("indices", C.c_void_p)]


class Instance(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("custom_index", C.c_uint32), ("mask", C.c_uint32),
                ("sbt_offset", C.c_uint32), ("flags", C.c_uint32), ("blas_handle", C.c_uint32)]


class BuildOpts(C.Structure):
    _fields_ = [("blas_bin_size", C.c_uint32), ("blas_max_depth", C.c_uint32), ("tlas_bin_size", C.c_uint32),
                ("tlas_max_depth", C.c_uint32), ("host_threads", C.c_uint32), ("device_build", C.c_uint32),
                ("reserved", C.c_uint32 * 2)]


class BuildStats(C.Structure):
    _fields_ = [("device_bytes", C.c_uint64), ("triangles", C.c_uint64), ("nodes", C.c_uint64),
                ("sah_splits", C.c_uint64), ("median_fallbacks", C.c_uint64), ("max_blas_depth", C.c_uint32),
                ("device_built", C.c_uint32), ("build_seconds", C.c_double), ("upload_seconds", C.c_double),
                ("device_seconds", C.c_double)]


class TraceDesc(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("hits", C.c_void_p), ("hits_ext", C.c_void_p), ("tlas_idx", C.c_void_p),
                ("count", C.c_uint32), ("tlas_uniform", C.c_uint32), ("ray_flags", C.c_uint32),
                ("cull_mask", C.c_uint32), ("traversal", C.c_uint32), ("anyhit_mode", C.c_uint32),
                ("block_size", C.c_uint32), ("local_stack", C.c_uint32), ("anyhit_mask", C.c_void_p)]


class Counters(C.Structure):
    _fields_ = [("node_visits", C.c_uint64), ("tri_tests", C.c_uint64), ("tri_hits", C.c_uint64),
                ("bad_tlas_rays", C.c_uint64)]


class Camera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("forward", C.c_float * 3), ("right", C.c_float * 3),
                ("up", C.c_float * 3), ("tan_half", C.c_float), ("aspect", C.c_float), ("width", C.c_uint32),
                ("height", C.c_uint32)]


class WavefrontDesc(C.Structure):
    _fields_ = [("camera", Camera), ("light", C.c_float * 3), ("sample_index", C.c_uint32),
                ("tlas_uniform", C.c_uint32), ("traversal", C.c_uint32), ("block_size", C.c_uint32),
                ("out", C.c_void_p), ("scratch", C.c_void_p), ("scratch_bytes", C.c_size_t),
                ("ray_counts", C.c_void_p), ("phases", C.c_uint32), ("refill", C.c_uint32),
                ("local_stack", C.c_uint32), ("register_tier", C.c_uint32), ("speculation", C.c_uint32),
                ("row_offset", C.c_uint32), ("frame_height", C.c_uint32)]


class PathDesc(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("tlas_idx", C.c_void_p), ("count", C.c_uint32), ("tlas_uniform", C.c_uint32),
                ("max_bounces", C.c_uint32), ("rr_start", C.c_uint32), ("albedo", C.c_float),
                ("rr_survive", C.c_float), ("seed", C.c_uint32), ("traversal", C.c_uint32),
                ("block_size", C.c_uint32), ("sort_key", C.c_uint32), ("out", C.c_void_p), ("scratch", C.c_void_p),
                ("scratch_bytes", C.c_size_t), ("segment_counts", C.c_void_p), ("refill", C.c_uint32),
                ("local_stack", C.c_uint32), ("speculation", C.c_uint32)]


class AttrLossDesc(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("count", C.c_uint32), ("tlas_uniform", C.c_uint32),
                ("attributes", C.c_void_p), ("targets", C.c_void_p), ("ray_value", C.c_void_p),
                ("ray_loss", C.c_void_p), ("loss_sum", C.c_void_p), ("grad_vertices", C.c_void_p),
                ("grad_ray_origin", C.c_void_p), ("grad_ray_direction", C.c_void_p), ("grad_scale", C.c_float),
                ("traversal", C.c_uint32), ("block_size", C.c_uint32), ("from_record", C.c_uint32),
                ("hit_tri", C.c_void_p), ("hit_inst", C.c_void_p), ("local_stack", C.c_uint32),
                ("speculation", C.c_uint32)]


class HitDiffDesc(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("count", C.c_uint32), ("tlas_uniform", C.c_uint32),
                ("attributes", C.c_void_p), ("hit", C.c_void_p), ("hit_tri", C.c_void_p), ("hit_inst", C.c_void_p),
                ("grad_hit", C.c_void_p), ("grad_vertices", C.c_void_p), ("grad_ray_origin", C.c_void_p),
                ("grad_ray_direction", C.c_void_p), ("traversal", C.c_uint32), ("block_size", C.c_uint32),
                ("from_record", C.c_uint32), ("local_stack", C.c_uint32), ("speculation", C.c_uint32)]


class AttrPathDesc(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("tlas_idx", C.c_void_p), ("count", C.c_uint32), ("tlas_uniform", C.c_uint32),
                ("segments", C.c_uint32), ("seed", C.c_uint32), ("attributes", C.c_void_p), ("targets", C.c_void_p),
                ("values", C.c_void_p), ("loss_sum", C.c_void_p), ("grad_vertices", C.c_void_p),
                ("seg_tri", C.c_void_p), ("seg_rays", C.c_void_p), ("grad_scale", C.c_float),
                ("traversal", C.c_uint32), ("block_size", C.c_uint32), ("from_record", C.c_uint32),
                ("seg_inst", C.c_void_p), ("local_stack", C.c_uint32), ("speculation", C.c_uint32)]


class TaskGroupDesc(C.Structure):
    _fields_ = [("program", C.c_uint32), ("max_in_flight", C.c_uint32), ("payload_words", C.c_uint32),
                ("n_spawn", C.c_uint32), ("spawn_type", C.c_uint32 * 4), ("spawn_op", C.c_uint32 * 4),
                ("map_op", C.c_uint32)]


class AoDesc(C.Structure):
    _fields_ = [("view_projection_inv", C.c_float * 16), ("camera_position", C.c_float * 3), ("width", C.c_uint32),
                ("height", C.c_uint32), ("sample_count", C.c_uint32), ("tlas_uniform", C.c_uint32),
                ("traversal", C.c_uint32), ("normals", C.c_void_p), ("image", C.c_void_p),
                ("sbt_closest", C.c_uint32 * 2), ("sbt_miss", C.c_uint32), ("block_size", C.c_uint32),
                ("ray_counts", C.c_void_p), ("sample_counter", C.c_void_p), ("speculation", C.c_uint32)]


class PtDesc(C.Structure):
    _fields_ = [("view_projection_inv", C.c_float * 16), ("camera_position", C.c_float * 3), ("width", C.c_uint32),
                ("height", C.c_uint32), ("sample_count", C.c_uint32), ("max_path_depth", C.c_uint32),
                ("tlas_uniform", C.c_uint32), ("traversal", C.c_uint32), ("tone_map", C.c_uint32),
                ("exposure", C.c_float), ("background", C.c_uint32), ("background_color", C.c_float * 3),
                ("lights", C.c_void_p), ("light_count", C.c_uint32), ("material_count", C.c_uint32),
                ("materials", C.c_void_p), ("sm_to_material", C.c_void_p), ("sm_count", C.c_uint32),
                ("block_size", C.c_uint32), ("normals", C.c_void_p), ("image", C.c_void_p), ("radiance", C.c_void_p),
                ("ray_counts", C.c_void_p), ("schedule", C.c_uint32), ("register_tier", C.c_uint32),
                ("scratch", C.c_void_p), ("scratch_bytes", C.c_size_t), ("env_cube", C.c_void_p),
                ("env_size", C.c_uint32), ("env_transform", C.c_float * 16), ("env_intensity", C.c_float),
                ("sample_counter", C.c_void_p), ("speculation", C.c_uint32)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with rendiation_gb300.build_native.build() (nvcc, sm_103a)")
    L = C.CDLL(LIB_PATH)
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int32
    L.rdn_api_version.restype = u32
    L.rdn_create.argtypes = [C.POINTER(vp), C.c_int]
    L.rdn_create.restype = i32
    L.rdn_destroy.argtypes = [vp]
    L.rdn_destroy.restype = i32
    L.rdn_last_error.argtypes = [vp]
    L.rdn_last_error.restype = C.c_char_p
    L.rdn_blas_create.argtypes = [vp, vp, u32, C.POINTER(u32)]
    L.rdn_blas_create.restype = i32
    L.rdn_blas_delete.argtypes = [vp, u32]
    L.rdn_blas_delete.restype = i32
    L.rdn_tlas_create.argtypes = [vp, vp, u32, C.POINTER(u32)]
    L.rdn_tlas_create.restype = i32
    L.rdn_tlas_delete.argtypes = [vp, u32]
    L.rdn_tlas_delete.restype = i32
    L.rdn_bind_tlas.argtypes = [vp, vp, u32]
    L.rdn_bind_tlas.restype = i32
    L.rdn_build.argtypes = [vp, vp]
    L.rdn_build.restype = i32
    L.rdn_get_build_stats.argtypes = [vp, C.POINTER(BuildStats)]
    L.rdn_get_build_stats.restype = i32
    L.rdn_get_built_array.argtypes = [vp, u32, vp, C.c_size_t, C.POINTER(C.c_size_t)]
    L.rdn_get_built_array.restype = i32
    L.rdn_trace.argtypes = [vp, C.POINTER(TraceDesc), vp]
    L.rdn_trace.restype = i32
    L.rdn_trace_counted.argtypes = [vp, C.POINTER(TraceDesc), vp, C.POINTER(Counters)]
    L.rdn_trace_counted.restype = i32
    L.rdn_check_errors.argtypes = [vp, vp, C.POINTER(u32)]
    L.rdn_check_errors.restype = i32
    L.rdn_set_iteration_limit.argtypes = [vp, u32]
    L.rdn_set_iteration_limit.restype = i32
    L.rdn_wavefront_scratch_size.argtypes = [u32, u32, C.POINTER(C.c_size_t)]
    L.rdn_wavefront_scratch_size.restype = i32
    L.rdn_wavefront_shadow_bounce.argtypes = [vp, C.POINTER(WavefrontDesc), vp]
    L.rdn_wavefront_shadow_bounce.restype = i32
    L.rdn_wavefront_shadow_bounce_static.argtypes = [vp, C.POINTER(WavefrontDesc), vp]
    L.rdn_wavefront_shadow_bounce_static.restype = i32
    L.rdn_paths_scratch_size.argtypes = [u32, u32, u32, C.POINTER(C.c_size_t)]
    L.rdn_paths_scratch_size.restype = i32
    L.rdn_trace_paths.argtypes = [vp, C.POINTER(PathDesc), vp]
    L.rdn_trace_paths.restype = i32
    L.rdn_trace_paths_graph.argtypes = [vp, C.POINTER(PathDesc), C.POINTER(vp)]
    L.rdn_trace_paths_graph.restype = i32
    L.rdn_graph_launch.argtypes = [vp, vp]
    L.rdn_graph_launch.restype = i32
    L.rdn_graph_destroy.argtypes = [vp]
    L.rdn_graph_destroy.restype = i32
    L.rdn_hit_diff_forward.argtypes = [vp, C.POINTER(HitDiffDesc), vp]
    L.rdn_hit_diff_forward.restype = i32
    L.rdn_hit_diff_adjoint.argtypes = [vp, C.POINTER(HitDiffDesc), vp]
    L.rdn_hit_diff_adjoint.restype = i32
    L.rdn_attr_loss_forward.argtypes = [vp, C.POINTER(AttrLossDesc), vp]
    L.rdn_attr_loss_forward.restype = i32
    L.rdn_attr_loss_adjoint.argtypes = [vp, C.POINTER(AttrLossDesc), vp]
    L.rdn_attr_loss_adjoint.restype = i32
    for name in ("rdn_scan_scratch_size", "rdn_compact_scratch_size", "rdn_radix_sort_scratch_size"):
        getattr(L, name).argtypes = [u32, C.POINTER(C.c_size_t)]
        getattr(L, name).restype = i32
    L.rdn_scan_u32.argtypes = [vp, vp, u32, C.c_int, u32, vp, C.c_size_t, vp]
    L.rdn_scan_u32.restype = i32
    L.rdn_compact_u32.argtypes = [vp, vp, vp, vp, u32, vp, C.c_size_t, vp]
    L.rdn_compact_u32.restype = i32
    L.rdn_radix_sort_u32.argtypes = [vp, vp, u32, u32, vp, C.c_size_t, vp]
    L.rdn_radix_sort_u32.restype = i32
    for name in ("rdn_attr_paths_forward", "rdn_attr_paths_adjoint"):
        getattr(L, name).argtypes = [vp, C.POINTER(AttrPathDesc), vp]
        getattr(L, name).restype = i32
    L.rdn_attr_paths_graph.argtypes = [vp, C.POINTER(AttrPathDesc), C.c_uint64, C.POINTER(vp)]
    L.rdn_attr_paths_graph.restype = i32
    L.rdn_task_graph_create.argtypes = [vp, C.POINTER(TaskGroupDesc), u32, u32, vp, C.POINTER(vp)]
    L.rdn_task_graph_create.restype = i32
    L.rdn_task_graph_destroy.argtypes = [vp]
    L.rdn_task_graph_destroy.restype = i32
    L.rdn_task_graph_dispatch_init.argtypes = [vp, u32, u32, u32, vp]
    L.rdn_task_graph_dispatch_init.restype = i32
    L.rdn_task_graph_execute.argtypes = [vp, u32, C.POINTER(AoDesc), vp]
    L.rdn_task_graph_execute.restype = i32
    L.rdn_task_graph_states.argtypes = [vp, vp, vp, vp, vp]
    L.rdn_task_graph_states.restype = i32
    L.rdn_task_graph_debug.argtypes = [vp, u32, vp, C.POINTER(u32), vp, C.POINTER(u32), vp, vp]
    L.rdn_task_graph_debug.restype = i32
    L.rdn_task_graph_check_errors.argtypes = [vp, vp, C.POINTER(u32)]
    L.rdn_task_graph_check_errors.restype = i32
    L.rdn_ao_pipeline_create.argtypes = [vp, u32, u32, vp, C.POINTER(vp)]
    L.rdn_ao_pipeline_create.restype = i32
    L.rdn_ao_render_graph.argtypes = [vp, C.POINTER(AoDesc), vp]
    L.rdn_ao_render_graph.restype = i32
    L.rdn_ao_render.argtypes = [vp, C.POINTER(AoDesc), vp]
    L.rdn_ao_render.restype = i32
    L.rdn_ao_capture.argtypes = [vp, vp, C.POINTER(AoDesc), C.POINTER(vp)]
    L.rdn_ao_capture.restype = i32
    L.rdn_task_graph_capture.argtypes = [vp, u32, u32, u32, u32, C.POINTER(AoDesc), C.POINTER(vp)]
    L.rdn_task_graph_capture.restype = i32
    L.rdn_task_graph_set_poll.argtypes = [vp, u32, vp, vp]
    L.rdn_task_graph_set_poll.restype = i32
    L.rdn_trace_params.argtypes = [vp, u32, vp, C.POINTER(C.c_size_t)]
    L.rdn_trace_params.restype = i32
    L.rdn_path_tracing_render.argtypes = [vp, C.POINTER(PtDesc), vp]
    L.rdn_path_tracing_render.restype = i32
    L.rdn_pt_scratch_size.argtypes = [u32, u32, C.POINTER(C.c_size_t)]
    L.rdn_pt_scratch_size.restype = i32
    L.rdn_pt_capture.argtypes = [vp, C.POINTER(PtDesc), C.POINTER(vp)]
    L.rdn_pt_capture.restype = i32
    _lib = L
    return L
