"""Build and load the CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (oracle.cpp) is a CPU restatement of the reference's render hot
path used to check the CUDA kernels; see oracle.h.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
The reference itself cannot be built here (it needs clang-CUDA, Eigen,
Boost.Hana, Qt5, yaml-cpp and other absent libraries), so no oracle/_ref is
produced.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")
# the same oracle with the C library's sinf / cosf / asinf / acosf / powf in
# place of the shared polynomials (the reference calls std:: functions)
LIB_LIBM = os.path.join(BUILD_DIR, "liboracle_libm.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

c_u32 = ctypes.c_uint32
c_f32 = ctypes.c_float
_PF = ctypes.POINTER(c_f32)
_PU = ctypes.POINTER(c_u32)
_PI = ctypes.POINTER(ctypes.c_int32)


class OracleMaterial(ctypes.Structure):
    _fields_ = [("type", c_u32), ("diffuse", c_f32 * 3), ("specular", c_f32 * 3),
                ("shininess", c_f32), ("ior", c_f32), ("diffuse_weight", c_f32),
                ("glossy_weight", c_f32), ("roughness", c_f32), ("emission", c_f32 * 3),
                ("pad", c_f32)]


class OracleScene(ctypes.Structure):
    _fields_ = [("triangles", _PF), ("normals", _PF), ("tri_material", _PU),
                ("n_triangles", c_u32), ("mesh_ends", _PU), ("cluster_ends_per_mesh", _PU),
                ("n_meshes", c_u32), ("instance_xforms", _PF), ("instance_mesh", _PU),
                ("n_instances", c_u32), ("clusters", _PU), ("n_clusters", c_u32),
                ("materials", ctypes.POINTER(OracleMaterial)), ("n_materials", c_u32)]


class WD(ctypes.Structure):
    _fields_ = [("block_size", c_u32), ("target_x_block_size", c_u32),
                ("force_target_samples", c_u32), ("forced_target_samples_per_thread", c_u32),
                ("base_num_threads", c_u32), ("samples_per_thread_scaling_power", c_f32),
                ("max_samples_per_thread", c_u32)]


class OracleSettings(ctypes.Structure):
    _fields_ = [("render_wd", WD), ("reduce_wd", WD), ("max_blocks_per_launch", c_u32),
                ("overlap_threshold", c_f32), ("use_spatial_splits", c_u32),
                ("traversal_per_intersect_cost", c_f32), ("target_objects", c_u32),
                ("light_sampler", c_u32), ("dir_sampler", c_u32), ("term_prob", c_u32),
                ("term_prob_prob", c_f32), ("term_prob_iters", c_u32), ("term_prob_exp", c_f32),
                ("term_prob_min_prob", c_f32), ("max_sample_size", c_u32),
                ("back_cull_emission", c_u32), ("reduce_order", c_u32), ("n_threads", c_u32),
                ("rng", c_u32), ("tie_rule", c_u32)]


class RenderOptions(ctypes.Structure):
    _fields_ = [("row_start", c_u32), ("row_end", c_u32), ("row_stride", c_u32),
                ("sample_offset", c_u32), ("mode", c_u32)]


class WorkDivision(ctypes.Structure):
    _fields_ = [(n, c_u32) for n in ["block_size", "base_samples_per_thread",
                                     "n_threads_per_unit_extra", "sample_block_size",
                                     "x_block_size", "y_block_size", "num_sample_blocks",
                                     "num_x_blocks", "num_y_blocks", "x_dim", "y_dim"]]


def _build_one(lib_path, defines, force):
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(HERE, "oracle.h"),
            os.path.join(ROOT, "path_gb300", "csrc", "pmath.h"),
            os.path.join(ROOT, "path_gb300", "csrc", "pmath_coeffs.h")]
    if not force and os.path.exists(lib_path) and all(
            os.path.getmtime(d) <= os.path.getmtime(lib_path) for d in deps):
        return None
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = lib_path + ".tmp"
    cmd = ["g++", "-O2", "-std=gnu++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           *defines, "-I" + os.path.join(CUDA_HOME, "include"), src, "-o", tmp,
           "-L" + os.path.join(CUDA_HOME, "lib64"), "-lcurand",
           "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")]
    return subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), \
        tmp, lib_path


def build(force=False):
    """Compiles liboracle.so and liboracle_libm.so (in parallel) when stale."""
    jobs = [j for j in (_build_one(LIB, [], force), _build_one(LIB_LIBM, ["-DORACLE_LIBM"], force))
            if j is not None]
    for proc, tmp, lib_path in jobs:
        out, _ = proc.communicate()
        if proc.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + out)
        os.replace(tmp, lib_path)
    return LIB


_libs = {}
_lib = None


def load(libm=False):
    """The oracle library; libm=True loads the build that calls the C
    library's transcendental functions."""
    global _lib
    key = bool(libm)
    if key not in _libs:
        build()
        lib = ctypes.CDLL(LIB_LIBM if key else LIB)
        lib.oracle_sbvh_build.restype = ctypes.c_void_p
        lib.oracle_sbvh_build.argtypes = [_PF, c_u32, c_f32, c_u32, c_f32, c_u32]
        for name in ["oracle_sbvh_free", "oracle_sbvh_sizes", "oracle_sbvh_export",
                     "oracle_bvh_intersect", "oracle_sah_cost"]:
            getattr(lib, name).argtypes = None
        lib.oracle_sbvh_free.argtypes = [ctypes.c_void_p]
        lib.oracle_sbvh_sizes.argtypes = [ctypes.c_void_p, _PU]
        lib.oracle_sbvh_export.argtypes = [ctypes.c_void_p, _PU, _PF, _PU, _PU]
        lib.oracle_bvh_intersect.argtypes = [ctypes.c_void_p, _PF, ctypes.c_size_t, _PI, _PF]
        lib.oracle_sah_cost.argtypes = [ctypes.c_void_p, c_f32]
        lib.oracle_sah_cost.restype = c_f32
        lib.oracle_render.argtypes = [ctypes.POINTER(OracleScene),
                                      ctypes.POINTER(OracleSettings), c_u32, c_u32, c_u32, _PF,
                                      c_u32, c_u32, _PF, ctypes.POINTER(ctypes.c_double)]
        lib.oracle_render_rays.argtypes = [ctypes.POINTER(OracleScene),
                                           ctypes.POINTER(OracleSettings), c_u32, _PF, _PU,
                                           c_u32, c_u32, _PF]
        lib.oracle_render_steps.argtypes = [ctypes.POINTER(OracleScene),
                                            ctypes.POINTER(OracleSettings), c_u32, c_u32, c_u32,
                                            _PF, c_u32, _PF]
        lib.oracle_render_bgra.argtypes = [ctypes.POINTER(OracleScene),
                                           ctypes.POINTER(OracleSettings), c_u32, c_u32, c_u32,
                                           _PF, ctypes.POINTER(ctypes.c_uint8)]
        lib.oracle_render_samples.argtypes = [ctypes.POINTER(OracleScene),
                                              ctypes.POINTER(OracleSettings), c_u32, c_u32,
                                              c_u32, _PF, c_u32, c_u32, _PF]
        lib.oracle_work_division_make.argtypes = [ctypes.POINTER(WD), c_u32, c_u32, c_u32,
                                                  ctypes.POINTER(WorkDivision)]
        lib.oracle_work_division_thread_info.argtypes = [ctypes.POINTER(WorkDivision), c_u32,
                                                         c_u32, _PU]
        lib.oracle_sub_block_reduce.argtypes = [_PF, c_u32, c_u32, c_u32, c_u32, _PF]
        lib.oracle_sobol_table.argtypes = [c_u32, c_u32, _PF]
        lib.oracle_pmath.argtypes = [ctypes.c_int, _PF, _PF, _PF, ctypes.c_size_t]
        lib.oracle_triangle_intersect.argtypes = [_PF, _PF, ctypes.c_size_t, _PF, _PI]
        lib.oracle_loop_all.argtypes = [_PF, c_u32, _PF, ctypes.c_size_t, _PI, _PF]
        lib.oracle_clipped_new_bounds.argtypes = [_PF, _PF, c_f32, c_f32, c_u32, _PF]
        lib.oracle_rotate_to.argtypes = [_PF, _PF, _PF]
        lib.oracle_find_relative_vec.argtypes = [_PF, c_f32, c_f32, _PF]
        lib.oracle_camera_transform.argtypes = [_PF, _PF, _PF, c_f32, c_f32, _PF]
        lib.oracle_debug_bsdf.argtypes = [ctypes.POINTER(OracleMaterial), c_u32, _PF, c_u32, _PF]
        lib.oracle_prepare.restype = ctypes.c_void_p
        lib.oracle_prepare.argtypes = [ctypes.POINTER(OracleScene), ctypes.POINTER(OracleSettings)]
        lib.oracle_prepared_free.argtypes = [ctypes.c_void_p]
        lib.oracle_render_prepared.argtypes = [ctypes.c_void_p, ctypes.POINTER(OracleSettings),
                                               c_u32, c_u32, c_u32, _PF,
                                               ctypes.POINTER(RenderOptions), _PF,
                                               ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(ctypes.c_double)]
        _libs[key] = lib
        if not key:
            _lib = lib
    return _libs[key]


def _f(a):
    return a.ctypes.data_as(_PF)


def _u(a):
    return a.ctypes.data_as(_PU)


def _i(a):
    return a.ctypes.data_as(_PI)


def pmath(fn, x, y=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(x) if y is None else np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(x)
    load().oracle_pmath(fn, _f(x), _f(y), _f(out), x.size)
    return out


def triangle_intersect(tris, rays):
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    t = np.zeros(len(tris), np.float32)
    back = np.zeros(len(tris), np.int32)
    load().oracle_triangle_intersect(_f(tris), _f(rays), len(tris), _f(t), _i(back))
    return t, back


def loop_all(tris, rays):
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    idx = np.zeros(len(rays), np.int32)
    t = np.zeros(len(rays), np.float32)
    load().oracle_loop_all(_f(tris), len(tris), _f(rays), len(rays), _i(idx), _f(t))
    return idx, t


class SBVH:
    """The oracle's SBVH (generator.cu restated) over world-space triangles."""

    def __init__(self, tris, overlap_threshold=1e-5, use_spatial_splits=False,
                 traversal_cost=0.5, target_objects=4):
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        self._h = load().oracle_sbvh_build(_f(tris), len(tris), overlap_threshold,
                                           int(use_spatial_splits), traversal_cost,
                                           target_objects)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.oracle_sbvh_free(self._h)
            self._h = None

    def export(self):
        sizes = np.zeros(3, np.uint32)
        load().oracle_sbvh_sizes(self._h, _u(sizes))
        words = np.zeros((sizes[0], 2), np.uint32)
        boxes = np.zeros((sizes[0], 6), np.float32)
        extra = np.zeros(max(int(sizes[1]), 1), np.uint32)
        perm = np.zeros(max(int(sizes[2]), 1), np.uint32)
        load().oracle_sbvh_export(self._h, _u(words), _f(boxes), _u(extra), _u(perm))
        return {"node_words": words, "node_aabbs": boxes, "extra_idxs": extra[:sizes[1]],
                "permutation": perm[:sizes[2]]}

    def intersect(self, rays):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        idx = np.zeros(len(rays), np.int32)
        t = np.zeros(len(rays), np.float32)
        load().oracle_bvh_intersect(self._h, _f(rays), len(rays), _i(idx), _f(t))
        return idx, t

    def sah_cost(self, traversal_cost=0.0):
        return load().oracle_sah_cost(self._h, traversal_cost)


def camera_transform(look, up, pos, height_angle_deg, width_height_ratio):
    """get_camera_transform (camera.cpp:4-27) restated: 3x4 film_to_world."""
    arr = [np.ascontiguousarray(v, np.float32) for v in (look, up, pos)]
    out = np.zeros(12, np.float32)
    load().oracle_camera_transform(_f(arr[0]), _f(arr[1]), _f(arr[2]), height_angle_deg,
                                   width_height_ratio, _f(out))
    return out


def debug_bsdf(material, op, records):
    """The oracle's BSDF code (oracle_debug_bsdf), same ops and layout as
    path_gb300.api.debug_bsdf; material = any ctypes structure with the
    path_material layout."""
    rec = np.ascontiguousarray(records, np.float32).reshape(-1, 9)
    width = {0: 3, 1: 6, 2: 1}[op]
    out = np.zeros((len(rec), width), np.float32)
    m = OracleMaterial()
    ctypes.memmove(ctypes.byref(m), ctypes.byref(material), ctypes.sizeof(OracleMaterial))
    if load().oracle_debug_bsdf(ctypes.byref(m), op, _f(rec), len(rec), _f(out)) != 0:
        raise ValueError("bad BSDF probe arguments")
    return out[:, 0] if op == 2 else out


def clipped_new_bounds(tri, bounds, left, right, axis):
    tri = np.ascontiguousarray(tri, np.float32).reshape(9)
    bounds = np.ascontiguousarray(bounds, np.float32).reshape(6)
    out = np.zeros(6, np.float32)
    load().oracle_clipped_new_bounds(_f(tri), _f(bounds), left, right, axis, _f(out))
    return out


def rotate_to(inp, target):
    a = np.ascontiguousarray(inp, np.float32)
    b = np.ascontiguousarray(target, np.float32)
    out = np.zeros(3, np.float32)
    load().oracle_rotate_to(_f(a), _f(b), _f(out))
    return out


def find_relative_vec(vec, phi, theta):
    a = np.ascontiguousarray(vec, np.float32)
    out = np.zeros(3, np.float32)
    load().oracle_find_relative_vec(_f(a), phi, theta, _f(out))
    return out


def wd_settings(block_size=256, target_x_block_size=32, force_target_samples=False,
                forced_target_samples_per_thread=8, base_num_threads=16384,
                samples_per_thread_scaling_power=0.5, max_samples_per_thread=32):
    return WD(block_size, target_x_block_size, int(force_target_samples),
              forced_target_samples_per_thread, base_num_threads,
              samples_per_thread_scaling_power, max_samples_per_thread)


def work_division(settings, samples_per, x_dim, y_dim):
    out = WorkDivision()
    if load().oracle_work_division_make(ctypes.byref(settings), samples_per, x_dim, y_dim,
                                        ctypes.byref(out)) != 0:
        raise ValueError("invalid work division settings")
    return out


def thread_info(wd, block_idx, thread_idx):
    out = np.zeros(5, np.uint32)
    load().oracle_work_division_thread_info(ctypes.byref(wd), block_idx, thread_idx, _u(out))
    return tuple(int(v) for v in out)


def sub_block_reduce(vals, n_blocks, block_size, sub_block_size, order):
    vals = np.ascontiguousarray(vals, np.float32)
    out = np.zeros(n_blocks * block_size // sub_block_size, np.float32)
    load().oracle_sub_block_reduce(_f(vals), n_blocks, block_size, sub_block_size, order, _f(out))
    return out


def sobol_table(dimension_bound, count):
    out = np.zeros(dimension_bound * count, np.float32)
    if load().oracle_sobol_table(dimension_bound, count, _f(out)) != 0:
        raise RuntimeError("cuRAND direction vectors unavailable")
    return out.reshape(count, dimension_bound)


def settings_from(s, reduce_order=1, n_threads=0, tie_rule=0):
    """Oracle settings from a path_gb300 api.Settings (same field meaning);
    tie_rule 1 takes the 8-wide traversal's closest hit at equal distance
    (smallest BVH-order index) instead of the reference's."""
    r = s.raw
    w = lambda x: WD(x.block_size, x.target_x_block_size, x.force_target_samples,  # noqa: E731
                     x.forced_target_samples_per_thread, x.base_num_threads,
                     x.samples_per_thread_scaling_power, x.max_samples_per_thread)
    return OracleSettings(w(r.render_work_division), w(r.reduce_work_division),
                          r.max_blocks_per_launch_cpu, r.overlap_threshold, r.use_spatial_splits,
                          r.traversal_per_intersect_cost, r.target_objects, r.light_sampler,
                          r.dir_sampler, r.term_prob, r.term_prob_prob, r.term_prob_iters,
                          r.term_prob_exp, r.term_prob_min_prob, r.max_sample_size,
                          r.back_cull_emission, reduce_order, n_threads, r.rng, tie_rule)


def workload_settings(max_depth, reduce_order=0, n_threads=0, tie_rule=0):
    """Oracle settings for 'max depth D, no Russian roulette, Sobol' without
    the library: render::Settings{} defaults (include/render/settings.h
    :27-45 -- WorkDivision {256, 32, no forcing, 8, 16384, 0.5, 32}, reducer
    x-block 256, 128 CPU blocks per launch, SBVH overlap 1e-5 without
    spatial splits, traversal cost 0.5, 4 target objects, RandomTriangle,
    BSDF sampler) with NIters{D - 1}, 256 Sobol dimensions and back-face
    culled emission."""
    return OracleSettings(WD(256, 32, 0, 8, 16384, 0.5, 32), WD(256, 256, 0, 8, 16384, 0.5, 32),
                          128, 1e-5, 0, 0.5, 4, 0, 0, 1, 0.5, max_depth - 1, 50.0, 0.1, 256, 1,
                          reduce_order, n_threads, 0, tie_rule)


class SceneArrays:
    """Keeps numpy arrays alive for an OracleScene view."""

    def __init__(self, exported):
        self.a = exported
        mats = exported["materials"]
        n_m = exported["n_materials"]
        self.mats = (OracleMaterial * max(n_m, 1))()
        ctypes.memmove(self.mats, mats, ctypes.sizeof(OracleMaterial) * n_m)
        e = exported
        self.c = OracleScene(_f(e["triangles"]), _f(e["normals"]), _u(e["tri_material"]),
                             len(e["tri_material"]), _u(e["mesh_ends"]),
                             _u(e["cluster_ends_per_mesh"]), len(e["mesh_ends"]),
                             _f(e["instance_xforms"]), _u(e["instance_mesh"]),
                             len(e["instance_mesh"]), _u(e["clusters"]), len(e["clusters"]),
                             self.mats, n_m)


def render(scene_arrays, settings, samples_per, x_dim, y_dim, film_to_world, rows=None):
    """FloatRGB image [y_dim, x_dim, 3]; rows=(start, end) renders a band."""
    out = np.zeros((y_dim, x_dim, 3), np.float32)
    f2w = np.ascontiguousarray(film_to_world, np.float32).reshape(12)
    r0, r1 = (0, y_dim) if rows is None else rows
    secs = ctypes.c_double()
    rc = load().oracle_render(ctypes.byref(scene_arrays.c), ctypes.byref(settings), samples_per,
                              x_dim, y_dim, _f(f2w), r0, r1, _f(out), ctypes.byref(secs))
    if rc != 0:
        raise RuntimeError("oracle render failed")
    return out, secs.value


def render_bgra(scene_arrays, settings, samples_per, x_dim, y_dim, film_to_world):
    out = np.zeros((y_dim, x_dim, 4), np.uint8)
    f2w = np.ascontiguousarray(film_to_world, np.float32).reshape(12)
    rc = load().oracle_render_bgra(ctypes.byref(scene_arrays.c), ctypes.byref(settings),
                                   samples_per, x_dim, y_dim, _f(f2w),
                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    if rc != 0:
        raise RuntimeError("oracle render failed")
    return out


def render_samples(scene_arrays, settings, samples_per, x_dim, y_dim, film_to_world, x, y):
    out = np.zeros((samples_per, 3), np.float32)
    f2w = np.ascontiguousarray(film_to_world, np.float32).reshape(12)
    rc = load().oracle_render_samples(ctypes.byref(scene_arrays.c), ctypes.byref(settings),
                                      samples_per, x_dim, y_dim, _f(f2w), x, y, _f(out))
    if rc != 0:
        raise RuntimeError("oracle render failed")
    return out


def render_rays(scene_arrays, settings, samples_per, rays, idxs=None, n_steps=0):
    """InitialRays (idxs None) / InitialIdxAndDir radiance: [n_rays, 3], or
    [n_steps, n_rays, 3] with OutputPerStep."""
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    shape = (n_steps, len(rays), 3) if n_steps else (len(rays), 3)
    out = np.zeros(shape, np.float32)
    ip = None
    if idxs is not None:
        idxs = np.ascontiguousarray(idxs, np.uint32).reshape(-1)
        ip = _u(idxs)
    rc = load().oracle_render_rays(ctypes.byref(scene_arrays.c), ctypes.byref(settings),
                                   samples_per, _f(rays), ip, len(rays), n_steps, _f(out))
    if rc != 0:
        raise RuntimeError("oracle render failed")
    return out


def render_steps(scene_arrays, settings, samples_per, x_dim, y_dim, film_to_world, n_steps):
    """OutputPerStep of a square image: [n_steps, y_dim, x_dim, 3]."""
    f2w = np.ascontiguousarray(film_to_world, np.float32).reshape(12)
    out = np.zeros((n_steps, y_dim, x_dim, 3), np.float32)
    rc = load().oracle_render_steps(ctypes.byref(scene_arrays.c), ctypes.byref(settings),
                                    samples_per, x_dim, y_dim, _f(f2w), n_steps, _f(out))
    if rc != 0:
        raise RuntimeError("oracle render failed")
    return out


class Prepared:
    """A scene flattened and its SBVH built once (oracle_prepare), for
    several renders with the same accel settings and light sampler.
    libm=True uses the build with the C library's transcendental functions."""

    def __init__(self, scene_arrays, settings, libm=False):
        self._arrays = scene_arrays
        self._lib = load(libm)
        self._h = self._lib.oracle_prepare(ctypes.byref(scene_arrays.c), ctypes.byref(settings))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.oracle_prepared_free(h)
            self._h = None

    def _run(self, settings, spp, x_dim, y_dim, f2w, rows, stride, sample_offset, mode, out,
             out64):
        r0, r1 = (0, y_dim) if rows is None else rows
        opt = RenderOptions(r0, r1, max(1, stride), sample_offset, mode)
        f2w = np.ascontiguousarray(f2w, np.float32).reshape(12)
        secs = ctypes.c_double()
        rc = self._lib.oracle_render_prepared(
            self._h, ctypes.byref(settings), spp, x_dim, y_dim, _f(f2w), ctypes.byref(opt),
            None if out is None else _f(out),
            None if out64 is None else out64.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            ctypes.byref(secs))
        if rc == 2:
            raise ValueError("settings differ from the ones the scene was prepared with")
        if rc != 0:
            raise RuntimeError("oracle render failed")
        return secs.value

    def render(self, settings, spp, x_dim, y_dim, f2w, rows=None, stride=1, sample_offset=0):
        """FP32 image through WorkDivision and the reducer (the reference's
        CPU path): ([y_dim, x_dim, 3] with the selected rows written,
        seconds)."""
        out = np.zeros((y_dim, x_dim, 3), np.float32)
        secs = self._run(settings, spp, x_dim, y_dim, f2w, rows, stride, sample_offset, 0, out,
                         None)
        return out, secs

    def render_f64(self, settings, spp, x_dim, y_dim, f2w, rows=None, stride=1, sample_offset=0):
        """Mean radiance with every sample summed in double: ([y_dim, x_dim,
        3] float64 with the selected rows written, seconds)."""
        out = np.zeros((y_dim, x_dim, 3), np.float64)
        secs = self._run(settings, spp, x_dim, y_dim, f2w, rows, stride, sample_offset, 1, None,
                         out)
        return out, secs

    def sample_values(self, settings, spp, x_dim, y_dim, f2w, rows=None, stride=1,
                      sample_offset=0):
        """Per-sample radiance [selected rows, x_dim, spp, 3]."""
        r0, r1 = (0, y_dim) if rows is None else rows
        n_rows = len(range(r0, min(r1, y_dim), max(1, stride)))
        out = np.zeros((n_rows, x_dim, spp, 3), np.float32)
        self._run(settings, spp, x_dim, y_dim, f2w, rows, stride, sample_offset, 2, out, None)
        return out
