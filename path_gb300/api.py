"""Python mirror of the reference's render API, on top of the C ABI.

Names follow the reference: ``Renderer.render`` (include/render/renderer.h:
43-70), ``RendererFromFiles`` (include/render/renderer_from_files.h:22-43),
``Settings`` (include/render/settings.h), ``TriangleConstructor``-style scene
building (include/scene/triangle_constructor.h) and ``ExecutionModel``.
Errors are raised as ``capi.PathError`` carrying the C status code.
"""

import ctypes
import enum

import numpy as np

from . import capi


class ExecutionModel(enum.IntEnum):
    CPU = capi.EXEC_CPU
    GPU = capi.EXEC_GPU


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _uptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


class Settings:
    """render::Settings as a flat C struct with attribute access."""

    def __init__(self, raw=None):
        self.raw = capi.PathSettings()
        if raw is not None:
            ctypes.memmove(ctypes.byref(self.raw), ctypes.byref(raw), ctypes.sizeof(raw))
        else:
            capi.check(capi.load().path_settings_default(ctypes.byref(self.raw)))

    @classmethod
    def from_yaml(cls, path):
        s = cls()
        capi.check(capi.load().path_settings_load_yaml(str(path).encode(), ctypes.byref(s.raw)))
        return s

    def copy(self):
        return Settings(self.raw)

    def __getattr__(self, name):
        if name == "raw":
            raise AttributeError(name)
        return getattr(self.raw, name)

    def __setattr__(self, name, value):
        if name == "raw":
            object.__setattr__(self, name, value)
        else:
            setattr(self.raw, name, value)

    def set_term_prob(self, kind, **kw):
        self.raw.term_prob = capi.TERM[kind]
        for k, v in kw.items():
            setattr(self.raw, {"prob": "term_prob_prob", "iters": "term_prob_iters",
                               "exp": "term_prob_exp", "min_prob": "term_prob_min_prob"}[k], v)
        return self


def material(kind, diffuse=(0, 0, 0), specular=(0, 0, 0), emission=(0, 0, 0), shininess=0.0,
             ior=1.0, diffuse_weight=0.0, glossy_weight=0.0, roughness=0.0):
    m = capi.PathMaterial()
    m.type = capi.BSDF[kind]
    m.diffuse[:] = [float(x) for x in diffuse]
    m.specular[:] = [float(x) for x in specular]
    m.emission[:] = [float(x) for x in emission]
    m.shininess = shininess
    m.ior = ior
    m.diffuse_weight = diffuse_weight
    m.glossy_weight = glossy_weight
    m.roughness = roughness
    return m


class Scene:
    """scene::Scene built like scene::TriangleConstructor, or loaded from XML."""

    def __init__(self, handle=None):
        lib = capi.load()
        if handle is None:
            handle = ctypes.c_void_p()
            capi.check(lib.path_scene_create(ctypes.byref(handle)))
        self._h = handle

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and capi._lib is not None:
            capi._lib.path_scene_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def add_material(self, m):
        idx = ctypes.c_uint32()
        capi.check(capi.load().path_scene_add_material(self._h, ctypes.byref(m), ctypes.byref(idx)))
        return idx.value

    def add_mesh(self, triangles, material_idx, normals=None, object_to_world=None):
        tris = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, 9)
        mats = np.ascontiguousarray(material_idx, dtype=np.uint32).reshape(-1)
        if mats.size == 1 and tris.shape[0] > 1:
            mats = np.full(tris.shape[0], mats[0], dtype=np.uint32)
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 9)
        xf = None if object_to_world is None else np.ascontiguousarray(object_to_world, dtype=np.float32).reshape(12)
        capi.check(capi.load().path_scene_add_mesh(
            self._h, _fptr(tris), None if nrm is None else _fptr(nrm), _uptr(mats),
            tris.shape[0], None if xf is None else _fptr(xf)))

    def set_material(self, idx, m):
        """Replace material idx in place (no BVH rebuild on the next render)."""
        capi.check(capi.load().path_scene_set_material(self._h, int(idx), ctypes.byref(m)))

    def sizes(self):
        s = (ctypes.c_uint32 * 5)()
        capi.check(capi.load().path_scene_sizes(self._h, s))
        return dict(zip(["triangles", "meshes", "instances", "clusters", "materials"], list(s)))

    def export(self):
        """Arrays in the reference's scene::Scene layout (for the oracle)."""
        z = self.sizes()
        n, m, k, c, nm = (z["triangles"], z["meshes"], z["instances"], z["clusters"],
                          z["materials"])
        out = {
            "triangles": np.zeros((n, 9), np.float32), "normals": np.zeros((n, 9), np.float32),
            "tri_material": np.zeros(n, np.uint32), "mesh_ends": np.zeros(m, np.uint32),
            "cluster_ends_per_mesh": np.zeros(m, np.uint32),
            "instance_xforms": np.zeros((k, 12), np.float32),
            "instance_mesh": np.zeros(k, np.uint32), "clusters": np.zeros((c, 3), np.uint32),
            "materials": (capi.PathMaterial * max(nm, 1))(),
        }
        capi.check(capi.load().path_scene_export(
            self._h, _fptr(out["triangles"]), _fptr(out["normals"]), _uptr(out["tri_material"]),
            _uptr(out["mesh_ends"]), _uptr(out["cluster_ends_per_mesh"]),
            _fptr(out["instance_xforms"]), _uptr(out["instance_mesh"]), _uptr(out["clusters"]),
            out["materials"]))
        out["n_materials"] = nm
        return out

    @classmethod
    def load_xml(cls, path, width_height_ratio):
        h = ctypes.c_void_p()
        f2w = np.zeros(12, np.float32)
        capi.check(capi.load().path_scene_load_xml(str(path).encode(), width_height_ratio,
                                                   ctypes.byref(h), _fptr(f2w)))
        return cls(h), f2w


def camera_transform(look, up, pos, height_angle_deg, width_height_ratio):
    """scene::get_camera_transform (src/scene/camera.cpp:4-27): 3x4 film_to_world."""
    out = np.zeros(12, np.float32)
    arr = [np.asarray(v, np.float32) for v in (look, up, pos)]
    capi.check(capi.load().path_camera_transform(_fptr(arr[0]), _fptr(arr[1]), _fptr(arr[2]),
                                                 height_angle_deg, width_height_ratio, _fptr(out)))
    return out


class SquareImage:
    """render::SquareImageSpec; ``rows=(start, end)`` renders only that band
    of rows (bit-identical to the same rows of the whole render)."""

    def __init__(self, x_dim, y_dim, film_to_world, rows=None, sample_offset=0):
        self.x_dim = int(x_dim)
        self.y_dim = int(y_dim)
        self.film_to_world = np.asarray(film_to_world, np.float32).reshape(12)
        self.rows = rows
        self.sample_offset = int(sample_offset)

    def to_c(self):
        s = capi.SampleSpec()
        s.type = capi.SAMPLE_SQUARE_IMAGE
        s.x_dim = self.x_dim
        s.y_dim = self.y_dim
        s.film_to_world[:] = [float(v) for v in self.film_to_world]
        if self.rows is not None:
            s.row_start, s.row_end = int(self.rows[0]), int(self.rows[1])
        s.sample_offset = self.sample_offset
        return s


class InitialRays:
    """render::SampleSpec InitialRays: one output value per caller ray
    (origin xyz, unit direction xyz); the camera draws no random numbers."""

    def __init__(self, rays):
        self.rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)

    def to_c(self):
        s = capi.SampleSpec()
        s.type = capi.SAMPLE_INITIAL_RAYS
        s.rays = self.rays.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        s.n_rays = self.rays.shape[0]
        return s


class InitialIdxAndDir:
    """render::InitialIdxAndDirSpec list (include/render/renderer.h:31-35):
    each path starts at triangle idxs[i] (scene order) hit at distance 1
    along rays[i] (origin xyz, unit direction xyz), front side."""

    def __init__(self, idxs, rays):
        self.idxs = np.ascontiguousarray(idxs, np.uint32).reshape(-1)
        self.rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        if self.idxs.shape[0] != self.rays.shape[0]:
            raise ValueError("one triangle index per ray")

    def to_c(self):
        s = capi.SampleSpec()
        s.type = capi.SAMPLE_INITIAL_IDX_AND_DIR
        s.rays = self.rays.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        s.idxs = _uptr(self.idxs)
        s.n_rays = self.rays.shape[0]
        return s


class OutputPerStep:
    """OutputType::OutputPerStep: float32 array [n_steps, ..., 3] (numpy, or a
    torch tensor on the host or the GPU) receiving each path step's radiance."""

    def __init__(self, array):
        self.array = array
        self.n_steps = int(array.shape[0])


class Renderer:
    """render::Renderer: caches the scene's accel and device buffers."""

    def __init__(self):
        h = ctypes.c_void_p()
        capi.check(capi.load().path_renderer_create(ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and capi._lib is not None:
            capi._lib.path_renderer_destroy(h)
            self._h = None

    def render(self, execution_model, sample_spec, output, scene, samples_per, settings,
               show_progress=False):
        """Render into ``output``; returns the reference's timed seconds.

        output: numpy float32 [H, W, 3] (FloatRGB) or uint8 [H, W, 4] (BGRA) in
        host memory, or a torch CUDA tensor of the same shape (device output);
        or an ``OutputPerStep`` wrapping [n_steps, H, W, 3] float32.
        """
        o = capi.Output()
        if isinstance(output, OutputPerStep):
            o.n_steps = output.n_steps
            output = output.array
            per_step = True
        else:
            per_step = False
        dtype = getattr(output, "dtype", None)
        is_torch = hasattr(output, "data_ptr")
        if is_torch:
            import torch
            if not output.is_contiguous():
                raise ValueError("output tensor must be contiguous")
            o.type = capi.OUTPUT_BGRA if output.dtype == torch.uint8 else capi.OUTPUT_FLOAT_RGB
            o.data = output.data_ptr()
            o.on_device = 1 if output.is_cuda else 0
        else:
            if not output.flags["C_CONTIGUOUS"]:
                raise ValueError("output array must be C contiguous")
            o.type = capi.OUTPUT_BGRA if dtype == np.uint8 else capi.OUTPUT_FLOAT_RGB
            o.data = output.ctypes.data
            o.on_device = 0
        if per_step:
            o.type = capi.OUTPUT_PER_STEP
        spec = sample_spec.to_c()
        secs = ctypes.c_double()
        capi.check(capi.load().path_render(self._h, int(execution_model), ctypes.byref(spec),
                                           ctypes.byref(o), scene.handle, int(samples_per),
                                           ctypes.byref(settings.raw), int(show_progress),
                                           ctypes.byref(secs)))
        return secs.value

    def render_adjoint(self, sample_spec, scene, samples_per, settings, d_image):
        """path_render_adjoint: dLoss/d(material parameters) as float64
        [materials, 7] (reflectance rgb, roughness, emission rgb) for
        dLoss/d(image) = d_image ([H, W, 3] float32, numpy or torch)."""
        n_mat = scene.sizes()["materials"]
        out = np.zeros((max(n_mat, 1), 7), np.float64)
        spec = sample_spec.to_c()
        secs = ctypes.c_double()
        if hasattr(d_image, "data_ptr"):
            d_image = d_image.contiguous()
            ptr = ctypes.cast(d_image.data_ptr(), ctypes.POINTER(ctypes.c_float))
            on_dev = 1 if d_image.is_cuda else 0
            keep = d_image
        else:
            keep = np.ascontiguousarray(d_image, np.float32)
            ptr = _fptr(keep)
            on_dev = 0
        capi.check(capi.load().path_render_adjoint(
            self._h, ctypes.byref(spec), scene.handle, int(samples_per),
            ctypes.byref(settings.raw), ptr, on_dev,
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(secs)))
        del keep
        return out[:n_mat]

    def render_cached(self, cache, sample_spec, output, scene, samples_per, settings,
                      cache_depth=2, train_paths=1 << 16, train_steps=4):
        """One frame with the radiance cache (path_render_cached)."""
        o = self._output_c(output)
        spec = sample_spec.to_c()
        secs = ctypes.c_double()
        capi.check(capi.load().path_render_cached(
            self._h, cache.handle, ctypes.byref(spec), ctypes.byref(o), scene.handle,
            int(samples_per), ctypes.byref(settings.raw), int(cache_depth), int(train_paths),
            int(train_steps), ctypes.byref(secs)))
        return secs.value

    def cached_frame_queries(self, max_n=1 << 16, stride=1):
        """path_cache_frame_queries: (queries [n, 12], throughput [n, 3]) of
        the last cached frame's samples whose paths ended into the cache."""
        q = np.zeros((max_n, 12), np.float32)
        b = np.zeros((max_n, 3), np.float32)
        n = ctypes.c_uint32()
        capi.check(capi.load().path_cache_frame_queries(self._h, int(max_n), int(stride),
                                                        _fptr(q), _fptr(b), ctypes.byref(n)))
        return q[:n.value], b[:n.value]

    @staticmethod
    def _output_c(output):
        """(capi.Output, array) for a numpy or torch FloatRGB / BGRA image."""
        o = capi.Output()
        if hasattr(output, "data_ptr"):
            import torch
            if not output.is_contiguous():
                raise ValueError("output tensor must be contiguous")
            o.type = capi.OUTPUT_BGRA if output.dtype == torch.uint8 else capi.OUTPUT_FLOAT_RGB
            o.data = output.data_ptr()
            o.on_device = 1 if output.is_cuda else 0
        else:
            if not output.flags["C_CONTIGUOUS"]:
                raise ValueError("output array must be C contiguous")
            o.type = capi.OUTPUT_BGRA if output.dtype == np.uint8 else capi.OUTPUT_FLOAT_RGB
            o.data = output.ctypes.data
            o.on_device = 0
        return o

    @staticmethod
    def _batch_c(items):
        """items: sequence of (scene, SquareImage, output, samples_per)."""
        arr = (capi.BatchItem * len(items))()
        for k, (scene, spec, output, spp) in enumerate(items):
            arr[k].scene = scene.handle
            arr[k].x_dim = spec.x_dim
            arr[k].y_dim = spec.y_dim
            arr[k].film_to_world[:] = [float(v) for v in spec.film_to_world]
            arr[k].samples_per = int(spp)
            arr[k].output = Renderer._output_c(output)
            arr[k].sample_offset = int(getattr(spec, "sample_offset", 0))
        return arr

    def render_batch(self, items, settings, tuning=None):
        """Batched render (path_render_batch): items are (scene, SquareImage,
        output, samples_per); tuning a dict of path_batch_tuning fields or
        None.  Returns seconds."""
        arr = self._batch_c(items)
        t = None
        if tuning is not None:
            t = capi.BatchTuning()
            for k, v in tuning.items():
                setattr(t, k, int(v))
        secs = ctypes.c_double()
        capi.check(capi.load().path_render_batch(self._h, arr, len(items),
                                                 ctypes.byref(settings.raw),
                                                 None if t is None else ctypes.byref(t),
                                                 ctypes.byref(secs)))
        return secs.value

    def render_batch_cached(self, cache, items, settings, tuning=None, cache_depth=2,
                            train_paths=1 << 16, train_steps=4):
        """One frame of a batch with one radiance cache for all its items
        (path_render_batch_cached); items as for render_batch.  Returns
        seconds."""
        arr = self._batch_c(items)
        t = None
        if tuning is not None:
            t = capi.BatchTuning()
            for k, v in tuning.items():
                setattr(t, k, int(v))
        secs = ctypes.c_double()
        capi.check(capi.load().path_render_batch_cached(
            self._h, cache.handle, arr, len(items), ctypes.byref(settings.raw),
            None if t is None else ctypes.byref(t), int(cache_depth), int(train_paths),
            int(train_steps), ctypes.byref(secs)))
        return secs.value

    def autotune_batch(self, items, settings, sample_budget=0):
        """Fastest launch shape for the batch (path_batch_autotune), as a dict."""
        arr = self._batch_c(items)
        t = capi.BatchTuning()
        capi.check(capi.load().path_batch_autotune(self._h, arr, len(items),
                                                   ctypes.byref(settings.raw),
                                                   int(sample_budget), ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in capi.BatchTuning._fields_}

    def stats(self):
        s = capi.RenderStats()
        capi.check(capi.load().path_renderer_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in capi.RenderStats._fields_}

    def intersect(self, triangles, rays, settings):
        """Closest hit on the GPU: (idx int32, t float32); idx -1 = miss."""
        tris = np.ascontiguousarray(triangles, np.float32).reshape(-1, 9)
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        idx = np.zeros(r.shape[0], np.int32)
        t = np.zeros(r.shape[0], np.float32)
        capi.check(capi.load().path_intersect(
            self._h, _fptr(tris), tris.shape[0], _fptr(r), r.shape[0], ctypes.byref(settings.raw),
            idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _fptr(t)))
        return idx, t


class RendererFromFiles:
    """render::RendererFromFiles: scene file + YAML config + render."""

    def __init__(self):
        self.renderer = Renderer()
        self.settings = Settings()
        self.scene = None
        self.film_to_world = None

    def load_scene(self, path, width_height_ratio, quiet=True):
        self.scene, self.film_to_world = Scene.load_xml(path, width_height_ratio)

    def load_config(self, path):
        self.settings = Settings.from_yaml(path)

    def render(self, execution_model, x_dim, y_dim, output, samples_per, show_progress=False):
        return self.renderer.render(execution_model, SquareImage(x_dim, y_dim, self.film_to_world),
                                    output, self.scene, samples_per, self.settings, show_progress)


def sbvh_build(triangles, settings):
    """Binary SBVH of a triangle soup: dict of node words, boxes, extra idxs, permutation."""
    tris = np.ascontiguousarray(triangles, np.float32).reshape(-1, 9)
    n = tris.shape[0]
    sizes = (ctypes.c_uint32 * 2)()
    lib = capi.load()
    capi.check(lib.path_sbvh_build(_fptr(tris), n, ctypes.byref(settings.raw), sizes, None, None,
                                   None, None))
    words = np.zeros((sizes[0], 2), np.uint32)
    boxes = np.zeros((sizes[0], 6), np.float32)
    extra = np.zeros(max(sizes[1], 1), np.uint32)
    perm = np.zeros(max(n, 1), np.uint32)
    capi.check(lib.path_sbvh_build(_fptr(tris), n, ctypes.byref(settings.raw), sizes,
                                   _uptr(words), _fptr(boxes), _uptr(extra), _uptr(perm)))
    return {"node_words": words, "node_aabbs": boxes, "extra_idxs": extra[:sizes[1]],
            "permutation": perm[:n]}


WIDE_NODE_DTYPE = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"),
                            ("child_base", "<u4"), ("tri_base", "<u4"), ("meta", "u1", 8),
                            ("qlo", "u1", (3, 8)), ("qhi", "u1", (3, 8))])


def wide_build(triangles, settings):
    """The 8-wide BVH the GPU traverses: dict of nodes (WIDE_NODE_DTYPE
    records), leaf_refs (BVH-order triangle per wide-leaf entry), permutation
    (BVH order -> input order) and depth."""
    tris = np.ascontiguousarray(triangles, np.float32).reshape(-1, 9)
    n = tris.shape[0]
    sizes = (ctypes.c_uint32 * 3)()
    lib = capi.load()
    capi.check(lib.path_wide_build(_fptr(tris), n, ctypes.byref(settings.raw), sizes, None, None,
                                   None))
    nodes = np.zeros(sizes[0], WIDE_NODE_DTYPE)
    refs = np.zeros(max(sizes[1], 1), np.uint32)
    perm = np.zeros(max(n, 1), np.uint32)
    capi.check(lib.path_wide_build(_fptr(tris), n, ctypes.byref(settings.raw), sizes,
                                   nodes.ctypes.data, _uptr(refs), _uptr(perm)))
    return {"nodes": nodes, "leaf_refs": refs[:sizes[1]], "permutation": perm[:n],
            "depth": sizes[2]}


def sobol_table(dimension_bound, count, use_curand=False):
    out = np.zeros(dimension_bound * count, np.float32)
    fn = capi.load().path_sobol_table_curand if use_curand else capi.load().path_sobol_table
    capi.check(fn(dimension_bound, count, _fptr(out)))
    return out.reshape(count, dimension_bound)


def debug_pmath(fn, x, y=None):
    x = np.ascontiguousarray(x, np.float32)
    yy = None if y is None else np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(x)
    capi.check(capi.load().path_debug_pmath(fn, _fptr(x), None if yy is None else _fptr(yy),
                                            _fptr(out), x.size))
    return out


def debug_bsdf(material, op, records):
    """The kernels' BSDF code on the GPU (path_debug_bsdf): op 0 eval
    (records [n, 9] = in dir, out dir, normal) -> [n, 3]; op 1 sample
    (records = in dir, normal, u0, u1, u2) -> [n, 6] (dir, multiplier); op 2
    GGX D (records [:, 0] = n.h, [:, 1] = alpha) -> [n]."""
    rec = np.ascontiguousarray(records, np.float32).reshape(-1, 9)
    width = {0: 3, 1: 6, 2: 1}[op]
    out = np.zeros((len(rec), width), np.float32)
    capi.check(capi.load().path_debug_bsdf(ctypes.byref(material), op, _fptr(rec), len(rec),
                                           _fptr(out)))
    return out[:, 0] if op == 2 else out


def debug_sobol_draws(mode, n_paths, spp, draws):
    """path_debug_sobol_draws: (ms per launch, checksum) of n_paths paths of
    `draws` Sobol draws, read from the table (mode 0) or formed from the
    direction vectors in registers (1: vectors through L1, 2: in shared
    memory)."""
    ms = np.zeros(1, np.float32)
    cs = np.zeros(1, np.uint32)
    capi.check(capi.load().path_debug_sobol_draws(int(mode), int(n_paths), int(spp), int(draws),
                                                  _fptr(ms), _uptr(cs)))
    return float(ms[0]), int(cs[0])


def work_division(wd_settings, samples_per, x_dim, y_dim):
    out = (ctypes.c_uint32 * 11)()
    capi.check(capi.load().path_work_division(ctypes.byref(wd_settings), samples_per, x_dim,
                                              y_dim, out))
    names = ["block_size", "base_samples_per_thread", "n_threads_per_unit_extra",
             "sample_block_size", "x_block_size", "y_block_size", "num_sample_blocks",
             "num_x_blocks", "num_y_blocks", "x_dim", "y_dim"]
    return dict(zip(names, list(out)))


def bf16_bits(x):
    """float32 array -> BF16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16_value(bits):
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def debug_tc_gemm(a, b):
    """One tcgen05 tile: a [128][k], b [n][k] (rounded to BF16) -> a . b^T in
    FP32, and the BF16-rounded operands."""
    ab = bf16_bits(a)
    bb = bf16_bits(b)
    k, n = ab.shape[1], bb.shape[0]
    d = np.zeros((128, n), np.float32)
    p16 = ctypes.POINTER(ctypes.c_uint16)
    capi.check(capi.load().path_debug_tc_gemm(ab.ctypes.data_as(p16), bb.ctypes.data_as(p16),
                                              k, n, _fptr(d)))
    return d, bf16_value(ab), bf16_value(bb)


def debug_tc_wait_timeout(polls=1 << 16):
    """path_debug_tc_wait_timeout: the status of a tensor-core wait made to
    run out (PATH_ERR_DEVICE_TIMEOUT expected)."""
    return int(capi.load().path_debug_tc_wait_timeout(int(polls)))


class RadianceCache:
    """Neural radiance cache (path_cache_*): hash-grid encoding + BF16 MLP on
    the tensor cores, trained online with Adam."""

    N_WEIGHTS = 20480
    LEVELS, TABLE = 16, 1 << 19

    def __init__(self, seed=1, learning_rate=1e-2):
        h = ctypes.c_void_p()
        capi.check(capi.load().path_cache_create(int(seed), float(learning_rate),
                                                 ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and capi._lib is not None:
            capi._lib.path_cache_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def set_bounds(self, lo, hi):
        lo = np.asarray(lo, np.float32)
        hi = np.asarray(hi, np.float32)
        capi.check(capi.load().path_cache_set_bounds(self._h, _fptr(lo), _fptr(hi)))

    def set_ema(self, decay):
        """Inference on a moving average of the parameters (path_cache_set_ema)."""
        capi.check(capi.load().path_cache_set_ema(self._h, float(decay)))

    def use_batch_cells(self):
        """Positions in batch-cell coordinates (path_cache_use_batch_cells)."""
        capi.check(capi.load().path_cache_use_batch_cells(self._h))

    def query(self, queries):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 12)
        out = np.zeros((q.shape[0], 3), np.float32)
        capi.check(capi.load().path_cache_query(self._h, _fptr(q), q.shape[0], _fptr(out)))
        return out

    def train(self, records, update=True):
        r = np.ascontiguousarray(records, np.float32).reshape(-1, 16)
        loss = np.zeros(1, np.float32)
        capi.check(capi.load().path_cache_train(self._h, _fptr(r), r.shape[0], int(update),
                                                _fptr(loss)))
        return float(loss[0])

    def get(self, grads=False):
        w = np.zeros(self.N_WEIGHTS, np.float32)
        t = np.zeros((self.LEVELS, self.TABLE, 2), np.float32)
        gw = np.zeros_like(w) if grads else None
        gt = np.zeros_like(t) if grads else None
        capi.check(capi.load().path_cache_access(
            self._h, _fptr(w), _fptr(t), None if gw is None else _fptr(gw),
            None if gt is None else _fptr(gt), 0))
        return (w, t, gw, gt) if grads else (w, t)

    def set(self, weights=None, table=None):
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        t = None if table is None else np.ascontiguousarray(table, np.float32)
        capi.check(capi.load().path_cache_access(self._h, None if w is None else _fptr(w),
                                                 None if t is None else _fptr(t), None, None,
                                                 1))
