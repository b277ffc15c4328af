"""ctypes binding of the path_gb300 C ABI (include/path_gb300.h).

The structures here mirror the header field for field.  The library is the
in-tree build path_gb300/_lib/libpath_gb300.so; loading fails loudly when it
is missing -- there is no Python or CPU fallback for the render path.
"""

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpath_gb300.so")

c_u32 = ctypes.c_uint32
c_f32 = ctypes.c_float


class PathMaterial(ctypes.Structure):
    _fields_ = [("type", c_u32), ("diffuse", c_f32 * 3), ("specular", c_f32 * 3),
                ("shininess", c_f32), ("ior", c_f32), ("diffuse_weight", c_f32),
                ("glossy_weight", c_f32), ("roughness", c_f32), ("emission", c_f32 * 3),
                ("pad", c_f32)]


class WorkDivisionSettings(ctypes.Structure):
    _fields_ = [("block_size", c_u32), ("target_x_block_size", c_u32),
                ("force_target_samples", c_u32), ("forced_target_samples_per_thread", c_u32),
                ("base_num_threads", c_u32), ("samples_per_thread_scaling_power", c_f32),
                ("max_samples_per_thread", c_u32)]


class PathSettings(ctypes.Structure):
    _fields_ = [("kernel_approach", c_u32), ("max_blocks_per_launch_gpu", c_u32),
                ("max_blocks_per_launch_cpu", c_u32),
                ("render_work_division", WorkDivisionSettings),
                ("reduce_work_division", WorkDivisionSettings),
                ("overlap_threshold", c_f32), ("use_spatial_splits", c_u32),
                ("traversal_per_intersect_cost", c_f32), ("target_objects", c_u32),
                ("light_sampler", c_u32), ("binary_search_threshold", c_u32),
                ("dir_sampler", c_u32), ("term_prob", c_u32), ("term_prob_prob", c_f32),
                ("term_prob_iters", c_u32), ("term_prob_exp", c_f32),
                ("term_prob_min_prob", c_f32), ("rng", c_u32), ("max_sample_size", c_u32),
                ("back_cull_emission", c_u32), ("traversal", c_u32),
                ("persistent_ctas_per_sm", c_u32), ("count_work", c_u32),
                ("upload_scene_every_render", c_u32), ("trace_min_blocks", c_u32),
                ("time_kernels", c_u32), ("gpu_build", c_u32), ("wavefront_slots_log2", c_u32),
                ("trace_staged_nodes", c_u32)]


class SampleSpec(ctypes.Structure):
    _fields_ = [("type", c_u32), ("x_dim", c_u32), ("y_dim", c_u32),
                ("film_to_world", c_f32 * 12), ("rays", ctypes.POINTER(c_f32)),
                ("n_rays", c_u32), ("idxs", ctypes.POINTER(c_u32)), ("row_start", c_u32),
                ("row_end", c_u32), ("sample_offset", c_u32)]


class Output(ctypes.Structure):
    _fields_ = [("type", c_u32), ("data", ctypes.c_void_p), ("on_device", c_u32),
                ("n_steps", c_u32)]


class BatchItem(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("x_dim", c_u32), ("y_dim", c_u32),
                ("film_to_world", c_f32 * 12), ("samples_per", c_u32), ("output", Output),
                ("sample_offset", c_u32)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("slots_log2", c_u32), ("trace_min_blocks", c_u32),
                ("shade_ctas_per_sm", c_u32), ("iterations_per_graph", c_u32)]


class RenderStats(ctypes.Structure):
    _fields_ = [("seconds", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("bvh_build_seconds", ctypes.c_double), ("rays_traced", ctypes.c_uint64),
                ("nodes_visited", ctypes.c_uint64), ("triangles_tested", ctypes.c_uint64),
                ("gpu_launches", c_u32), ("device_status", c_u32),
                ("num_bvh_nodes", c_u32), ("num_wide_nodes", c_u32),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("trace_ms", ctypes.c_double), ("trace_launches", c_u32)]


# enums
PATH_OK = 0
STATUS_NAMES = {0: "PATH_OK", 1: "PATH_ERR_ARGUMENT", 2: "PATH_ERR_SCENE_PARSE",
                3: "PATH_ERR_OOM", 4: "PATH_ERR_DEVICE_TIMEOUT", 5: "PATH_ERR_UNSUPPORTED",
                6: "PATH_ERR_CUDA", 7: "PATH_ERR_IO"}
EXEC_CPU, EXEC_GPU = 0, 1
BSDF = {"Diffuse": 0, "Glossy": 1, "DiffuseGlossy": 2, "DiffuseMirror": 3, "Mirror": 4,
        "DielectricRefractive": 5, "GGX": 6}
SAMPLE_SQUARE_IMAGE, SAMPLE_INITIAL_RAYS, SAMPLE_INITIAL_IDX_AND_DIR = 0, 1, 2
OUTPUT_BGRA, OUTPUT_FLOAT_RGB, OUTPUT_PER_STEP = 0, 1, 2
MAX_OUTPUT_STEPS = 64
TRAVERSAL_BINARY, TRAVERSAL_WIDE8 = 0, 1
TERM = {"Constant": 0, "NIters": 1, "MultiplierFunc": 2, "Normalize": 3}

# every symbol the header declares, with (restype, argtypes)
_P = ctypes.c_void_p
_PF = ctypes.POINTER(c_f32)
_PU = ctypes.POINTER(c_u32)
_PI = ctypes.POINTER(ctypes.c_int32)
SIGNATURES = {
    "path_last_error": (ctypes.c_char_p, []),
    "path_version": (ctypes.c_char_p, []),
    "path_settings_default": (ctypes.c_int, [ctypes.POINTER(PathSettings)]),
    "path_settings_load_yaml": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(PathSettings)]),
    "path_scene_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "path_scene_destroy": (None, [_P]),
    "path_scene_add_material": (ctypes.c_int, [_P, ctypes.POINTER(PathMaterial), _PU]),
    "path_scene_add_mesh": (ctypes.c_int, [_P, _PF, _PF, _PU, c_u32, _PF]),
    "path_scene_load_xml": (ctypes.c_int, [ctypes.c_char_p, c_f32, ctypes.POINTER(_P), _PF]),
    "path_camera_transform": (ctypes.c_int, [_PF, _PF, _PF, c_f32, c_f32, _PF]),
    "path_scene_sizes": (ctypes.c_int, [_P, _PU]),
    "path_scene_export": (ctypes.c_int, [_P, _PF, _PF, _PU, _PU, _PU, _PF, _PU, _PU,
                                         ctypes.POINTER(PathMaterial)]),
    "path_renderer_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "path_renderer_destroy": (None, [_P]),
    "path_render": (ctypes.c_int, [_P, c_u32, ctypes.POINTER(SampleSpec), ctypes.POINTER(Output),
                                   _P, c_u32, ctypes.POINTER(PathSettings), c_u32,
                                   ctypes.POINTER(ctypes.c_double)]),
    "path_renderer_stats": (ctypes.c_int, [_P, ctypes.POINTER(RenderStats)]),
    "path_sbvh_build": (ctypes.c_int, [_PF, c_u32, ctypes.POINTER(PathSettings), _PU, _PU, _PF,
                                       _PU, _PU]),
    "path_wide_build": (ctypes.c_int, [_PF, c_u32, ctypes.POINTER(PathSettings), _PU, _P, _PU,
                                       _PU]),
    "path_intersect": (ctypes.c_int, [_P, _PF, c_u32, _PF, c_u32, ctypes.POINTER(PathSettings),
                                      _PI, _PF]),
    "path_sobol_table": (ctypes.c_int, [c_u32, c_u32, _PF]),
    "path_sobol_table_curand": (ctypes.c_int, [c_u32, c_u32, _PF]),
    "path_debug_pmath": (ctypes.c_int, [c_u32, _PF, _PF, _PF, c_u32]),
    "path_debug_bsdf": (ctypes.c_int, [ctypes.POINTER(PathMaterial), c_u32, _PF, c_u32, _PF]),
    "path_debug_set_device_alloc_cap": (None, [ctypes.c_uint64]),
    "path_debug_sobol_draws": (ctypes.c_int, [c_u32, c_u32, c_u32, c_u32, _PF, _PU]),
    "path_cache_frame_queries": (ctypes.c_int, [_P, c_u32, c_u32, _PF, _PF, _PU]),
    "path_work_division": (ctypes.c_int, [ctypes.POINTER(WorkDivisionSettings), c_u32, c_u32,
                                          c_u32, _PU]),
    "path_cache_create": (ctypes.c_int, [c_u32, c_f32, ctypes.POINTER(_P)]),
    "path_cache_destroy": (None, [_P]),
    "path_cache_set_bounds": (ctypes.c_int, [_P, _PF, _PF]),
    "path_cache_use_batch_cells": (ctypes.c_int, [_P]),
    "path_cache_set_ema": (ctypes.c_int, [_P, c_f32]),
    "path_cache_query": (ctypes.c_int, [_P, _PF, c_u32, _PF]),
    "path_cache_train": (ctypes.c_int, [_P, _PF, c_u32, c_u32, _PF]),
    "path_cache_access": (ctypes.c_int, [_P, _PF, _PF, _PF, _PF, c_u32]),
    "path_render_cached": (ctypes.c_int, [_P, _P, ctypes.POINTER(SampleSpec),
                                          ctypes.POINTER(Output), _P, c_u32,
                                          ctypes.POINTER(PathSettings), c_u32, c_u32, c_u32,
                                          ctypes.POINTER(ctypes.c_double)]),
    "path_debug_tc_wait_timeout": (ctypes.c_int, [c_u32]),
    "path_debug_tc_gemm": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint16),
                                          ctypes.POINTER(ctypes.c_uint16), c_u32, c_u32, _PF]),
    "path_render_adjoint": (ctypes.c_int, [_P, ctypes.POINTER(SampleSpec), _P, c_u32,
                                           ctypes.POINTER(PathSettings), _PF, c_u32,
                                           ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]),
    "path_scene_set_material": (ctypes.c_int, [_P, c_u32, ctypes.POINTER(PathMaterial)]),
    "path_render_batch": (ctypes.c_int, [_P, ctypes.POINTER(BatchItem), c_u32,
                                         ctypes.POINTER(PathSettings),
                                         ctypes.POINTER(BatchTuning),
                                         ctypes.POINTER(ctypes.c_double)]),
    "path_render_batch_cached": (ctypes.c_int, [_P, _P, ctypes.POINTER(BatchItem), c_u32,
                                                ctypes.POINTER(PathSettings),
                                                ctypes.POINTER(BatchTuning), c_u32, c_u32,
                                                c_u32, ctypes.POINTER(ctypes.c_double)]),
    "path_batch_autotune": (ctypes.c_int, [_P, ctypes.POINTER(BatchItem), c_u32,
                                           ctypes.POINTER(PathSettings), ctypes.c_uint64,
                                           ctypes.POINTER(BatchTuning)]),
    "path_render_noalloc": (ctypes.c_int, [_P, ctypes.POINTER(SampleSpec), ctypes.POINTER(Output),
                                           _P, c_u32, ctypes.POINTER(PathSettings),
                                           ctypes.POINTER(ctypes.c_double)]),
}

_lib = None


class PathError(RuntimeError):
    """A C-ABI call returned a status other than PATH_OK."""

    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(build_if_missing=True):
    """Load the in-tree library, building it first if it does not exist."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"path_gb300 native library missing: {LIB_PATH}")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != PATH_OK:
        msg = load().path_last_error().decode(errors="replace")
        raise PathError(status, msg)
