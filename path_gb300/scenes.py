"""Seeded synthetic scenes of the render-path workloads.

* ``cornell_box``: the small Cornell box -- 36 triangles: five walls of two
  triangles over [-1, 1]^3 with the front (+z) open, a 0.5 x 0.5 ceiling light
  (emission 15) facing down, and two boxes 0.6 and 1.2 tall rotated +-18
  degrees about y; Lambertian white 0.73, red (0.65, 0.05, 0.05) and green
  (0.12, 0.45, 0.15); pinhole camera at z = 3.5 with a 40 degree vertical
  field of view.
* ``large_mesh_room``: the same room and light holding an icosphere
  subdivided ``subdivisions`` times (8 -> 1,310,720 triangles) with radial
  displacement by 4-octave value noise (amplitude 0.08, seed 1) and a GGX
  material (roughness 0.2, F0 0.04), beside a latitude-longitude glass
  sphere of about 20k triangles (dielectric, IOR 1.5).

Triangles are wound so that face normals point into the room (walls) or out
of the objects; the light faces down so back-face culled emission is seen
from below.  All geometry is generated here; no third-party asset is used.
"""

import math

import numpy as np

from . import api

WHITE = (0.73, 0.73, 0.73)
RED = (0.65, 0.05, 0.05)
GREEN = (0.12, 0.45, 0.15)
LIGHT_EMISSION = (15.0, 15.0, 15.0)


def _quad(a, b, c, d):
    """Two triangles (a, b, c), (a, c, d); normal = (b - a) x (c - a)."""
    return [np.array([a, b, c], np.float32), np.array([a, c, d], np.float32)]


def room_triangles():
    """Walls [-1, 1]^3 (front open) and the ceiling light, inward facing."""
    p = lambda x, y, z: (x, y, z)  # noqa: E731
    walls = {
        "floor": _quad(p(-1, -1, -1), p(-1, -1, 1), p(1, -1, 1), p(1, -1, -1)),
        "ceiling": _quad(p(-1, 1, -1), p(1, 1, -1), p(1, 1, 1), p(-1, 1, 1)),
        "back": _quad(p(-1, -1, -1), p(1, -1, -1), p(1, 1, -1), p(-1, 1, -1)),
        "left": _quad(p(-1, -1, -1), p(-1, 1, -1), p(-1, 1, 1), p(-1, -1, 1)),
        "right": _quad(p(1, -1, -1), p(1, -1, 1), p(1, 1, 1), p(1, 1, -1)),
    }
    h = 0.25
    y = 0.999
    light = _quad(p(-h, y, -h), p(h, y, -h), p(h, y, h), p(-h, y, h))
    return walls, light


def _box(width, height, depth, angle_deg, centre_xz):
    """Axis box on the floor (y = -1) rotated about y; outward normals."""
    w, d = width / 2, depth / 2
    y0, y1 = -1.0, -1.0 + height
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)
    cx, cz = centre_xz

    def v(x, y, z):
        return (cx + ca * x + sa * z, y, cz - sa * x + ca * z)

    c = [v(-w, y0, -d), v(w, y0, -d), v(w, y0, d), v(-w, y0, d),
         v(-w, y1, -d), v(w, y1, -d), v(w, y1, d), v(-w, y1, d)]
    faces = [
        (c[0], c[1], c[2], c[3]),  # bottom, normal -y
        (c[4], c[7], c[6], c[5]),  # top, +y
        (c[0], c[4], c[5], c[1]),  # -z
        (c[3], c[2], c[6], c[7]),  # +z
        (c[0], c[3], c[7], c[4]),  # -x
        (c[1], c[5], c[6], c[2]),  # +x
    ]
    out = []
    for f in faces:
        out += _quad(*f)
    return np.stack(out)


class ArrayScene:
    """The same scene description as api.Scene (scene::TriangleConstructor),
    held in NumPy arrays instead of the library: add_material / add_mesh /
    sizes / export behave as path_scene_add_material / path_scene_add_mesh /
    path_scene_sizes / path_scene_export, bit for bit (face normals in
    float32 without contraction, one emissive cluster per emissive
    triangle, one identity instance per mesh).  For callers that must not
    load libpath_gb300.so: the CPU oracle's timed baseline builds its scenes
    with it."""

    def __init__(self):
        self._mats = []
        self._tris, self._normals, self._tri_mat = [], [], []
        self._mesh_ends, self._cluster_ends, self._clusters, self._xforms = [], [], [], []
        self._n = 0

    def add_material(self, m):
        self._mats.append(m)
        return len(self._mats) - 1

    @staticmethod
    def _emissive(m):
        e = [np.float32(v) for v in m.emission]
        return ((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2]) > np.float32(1e-9)

    @staticmethod
    def _face_normals(tris):
        t = tris.reshape(-1, 3, 3)
        a, b = t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]
        n = np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                      a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                      a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1)
        n2 = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
        with np.errstate(invalid="ignore", divide="ignore"):
            unit = n / np.sqrt(n2)[:, None]
        unit = np.where((n2 > 0)[:, None], unit, n).astype(np.float32)
        return np.tile(unit, (1, 3))

    def add_mesh(self, triangles, material_idx, normals=None, object_to_world=None):
        tris = np.ascontiguousarray(triangles, np.float32).reshape(-1, 9)
        mats = np.ascontiguousarray(material_idx, np.uint32).reshape(-1)
        if mats.size == 1 and len(tris) > 1:
            mats = np.full(len(tris), mats[0], np.uint32)
        if len(mats) != len(tris) or (len(mats) and int(mats.max()) >= len(self._mats)):
            raise ValueError("material index out of range")
        nrm = self._face_normals(tris) if normals is None else \
            np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
        emissive = np.array([self._emissive(m) for m in self._mats], bool)
        for i in np.nonzero(emissive[mats])[0] if len(mats) else []:
            self._clusters.append((int(mats[i]), self._n + int(i), self._n + int(i) + 1))
        self._tris.append(tris)
        self._normals.append(nrm)
        self._tri_mat.append(mats)
        self._n += len(tris)
        self._mesh_ends.append(self._n)
        self._cluster_ends.append(len(self._clusters))
        xf = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32) if object_to_world is \
            None else np.ascontiguousarray(object_to_world, np.float32).reshape(12)
        self._xforms.append(xf)

    def sizes(self):
        return {"triangles": self._n, "meshes": len(self._mesh_ends),
                "instances": len(self._xforms), "clusters": len(self._clusters),
                "materials": len(self._mats)}

    def export(self):
        from . import capi
        cat = (lambda xs, shape, dt: np.concatenate(xs).astype(dt) if xs else
               np.zeros(shape, dt))
        mats = (capi.PathMaterial * max(len(self._mats), 1))(*self._mats)
        return {
            "triangles": cat(self._tris, (0, 9), np.float32),
            "normals": cat(self._normals, (0, 9), np.float32),
            "tri_material": cat(self._tri_mat, (0,), np.uint32),
            "mesh_ends": np.array(self._mesh_ends, np.uint32),
            "cluster_ends_per_mesh": np.array(self._cluster_ends, np.uint32),
            "instance_xforms": np.array(self._xforms, np.float32).reshape(-1, 12),
            "instance_mesh": np.arange(len(self._xforms), dtype=np.uint32),
            "clusters": np.array(self._clusters, np.uint32).reshape(-1, 3),
            "materials": mats, "n_materials": len(self._mats),
        }


def cornell_camera(x_dim, y_dim, transform=None):
    """film_to_world of the pinhole camera at z = 3.5 looking down -z with a
    40 degree vertical field of view; transform defaults to
    api.camera_transform (any function of the same signature will do)."""
    return (transform or api.camera_transform)((0, 0, -1), (0, 1, 0), (0, 0, 3.5), 40.0,
                                               x_dim / y_dim)


def _add_room(scene, with_boxes):
    white = scene.add_material(api.material("Diffuse", diffuse=WHITE))
    red = scene.add_material(api.material("Diffuse", diffuse=RED))
    green = scene.add_material(api.material("Diffuse", diffuse=GREEN))
    light = scene.add_material(api.material("Diffuse", diffuse=(0.78, 0.78, 0.78),
                                            emission=LIGHT_EMISSION))
    walls, light_tris = room_triangles()
    tris, mats = [], []
    for name, ts in walls.items():
        m = red if name == "left" else green if name == "right" else white
        tris += ts
        mats += [m] * len(ts)
    tris += light_tris
    mats += [light] * len(light_tris)
    if with_boxes:
        short = _box(0.6, 0.6, 0.6, -18.0, (0.33, 0.37))
        tall = _box(0.6, 1.2, 0.6, 18.0, (-0.33, -0.3))
        for b in (short, tall):
            tris += list(b)
            mats += [white] * len(b)
    scene.add_mesh(np.stack(tris).reshape(-1, 9), np.array(mats, np.uint32))
    return white


def cornell_box(scene_cls=None):
    """The 36-triangle Cornell box (an api.Scene, or scene_cls())."""
    scene = (scene_cls or api.Scene)()
    _add_room(scene, with_boxes=True)
    return scene


# ---------------------------------------------------------------------------
# procedural meshes

def icosphere(subdivisions):
    """Unit icosphere by repeated midpoint subdivision (20 * 4^n triangles)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                      [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                      [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                      [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                      [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                      [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(subdivisions):
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        edges = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)])
        key = np.sort(edges, axis=1)
        uniq, inv = np.unique(key[:, 0] * (len(verts) + 1) + key[:, 1], return_inverse=True)
        e0 = uniq // (len(verts) + 1)
        e1 = uniq % (len(verts) + 1)
        mids = verts[e0] + verts[e1]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = len(verts)
        verts = np.concatenate([verts, mids])
        nf = len(faces)
        ab = base + inv[:nf]
        bc = base + inv[nf:2 * nf]
        ca = base + inv[2 * nf:]
        faces = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                                np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return verts, faces


def _hash3(ix, iy, iz, seed):
    """Integer lattice hash to [-1, 1] (MurmurHash3's 32-bit finaliser)."""
    h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ \
        (iy.astype(np.uint32) * np.uint32(0xD8163841)) ^ \
        (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32(seed * 0x9E3779B9 & 0xffffffff)
    h ^= h >> np.uint32(16)
    h *= np.uint32(0x85EBCA6B)
    h ^= h >> np.uint32(13)
    h *= np.uint32(0xC2B2AE35)
    h ^= h >> np.uint32(16)
    return h.astype(np.float64) / 4294967295.0 * 2.0 - 1.0


def value_noise(p, seed, octaves=4, base_frequency=2.0):
    """Fractal value noise in [-1, 1]: smoothstep-interpolated lattice values,
    frequency doubling and amplitude halving per octave."""
    total = np.zeros(len(p))
    norm = 0.0
    amp = 1.0
    freq = base_frequency
    with np.errstate(over="ignore"):
        for o in range(octaves):
            q = p * freq
            i = np.floor(q).astype(np.int64)
            f = q - i
            w = f * f * (3.0 - 2.0 * f)
            acc = np.zeros(len(p))
            for dx in (0, 1):
                for dy in (0, 1):
                    for dz in (0, 1):
                        val = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed + 7919 * o)
                        wx = w[:, 0] if dx else 1 - w[:, 0]
                        wy = w[:, 1] if dy else 1 - w[:, 1]
                        wz = w[:, 2] if dz else 1 - w[:, 2]
                        acc += val * wx * wy * wz
            total += amp * acc
            norm += amp
            amp *= 0.5
            freq *= 2.0
    return total / norm


def _vertex_normals(verts, faces):
    fn = np.cross(verts[faces[:, 1]] - verts[faces[:, 0]], verts[faces[:, 2]] - verts[faces[:, 0]])
    vn = np.zeros_like(verts)
    for k in range(3):
        np.add.at(vn, faces[:, k], fn)
    return vn / np.linalg.norm(vn, axis=1, keepdims=True)


def displaced_icosphere(subdivisions=8, radius=0.5, centre=(0.35, -0.4, -0.25),
                        amplitude=0.08, seed=1):
    verts, faces = icosphere(subdivisions)
    disp = radius + amplitude * value_noise(verts, seed)
    pos = verts * disp[:, None] + np.asarray(centre)
    normals = _vertex_normals(pos, faces)
    tris = pos[faces].reshape(-1, 9).astype(np.float32)
    nrm = normals[faces].reshape(-1, 9).astype(np.float32)
    return tris, nrm


def uv_sphere(n_lat=100, n_lon=100, radius=0.3, centre=(-0.45, -0.7, 0.3)):
    """Latitude-longitude sphere with analytic vertex normals (outward)."""
    th = np.linspace(0, np.pi, n_lat + 1)
    ph = np.linspace(0, 2 * np.pi, n_lon + 1)
    tris, nrm = [], []
    c = np.asarray(centre)

    def unit(t, p):
        return np.array([np.sin(t) * np.cos(p), np.cos(t), np.sin(t) * np.sin(p)])

    for i in range(n_lat):
        for j in range(n_lon):
            a, b = unit(th[i], ph[j]), unit(th[i], ph[j + 1])
            cc, d = unit(th[i + 1], ph[j + 1]), unit(th[i + 1], ph[j])
            if i > 0:
                tris.append([a, b, d])
            if i < n_lat - 1:
                tris.append([b, cc, d])
    n = np.array(tris)
    # wind outward: normal must agree with the position direction
    fn = np.cross(n[:, 1] - n[:, 0], n[:, 2] - n[:, 0])
    flip = np.einsum("ij,ij->i", fn, n.mean(axis=1)) < 0
    n[flip] = n[flip][:, ::-1]
    pos = n * radius + c
    return pos.reshape(-1, 9).astype(np.float32), n.reshape(-1, 9).astype(np.float32)


def large_mesh_room(subdivisions=8, glass_lat=100, glass_lon=100, scene_cls=None):
    """Room + light, displaced GGX icosphere and a glass sphere (an
    api.Scene, or scene_cls())."""
    scene = (scene_cls or api.Scene)()
    _add_room(scene, with_boxes=False)
    ggx = scene.add_material(api.material("GGX", specular=(0.04, 0.04, 0.04), roughness=0.2))
    glass = scene.add_material(api.material("DielectricRefractive", specular=(1, 1, 1), ior=1.5))
    tris, nrm = displaced_icosphere(subdivisions)
    scene.add_mesh(tris, np.full(len(tris), ggx, np.uint32), normals=nrm)
    gt, gn = uv_sphere(glass_lat, glass_lon)
    scene.add_mesh(gt, np.full(len(gt), glass, np.uint32), normals=gn)
    return scene


def path_settings(max_depth, traversal="wide"):
    """Settings for 'max depth D, no Russian roulette, Sobol': NIters{D-1}."""
    s = api.Settings()
    s.set_term_prob("NIters", iters=max_depth - 1)
    s.max_sample_size = 256
    s.back_cull_emission = 1
    s.traversal = 1 if traversal == "wide" else 0
    return s


# ---------------------------------------------------------------------------
# batched workload

def _sphere_grid(m, radius, centre):
    """Latitude-longitude sphere with m x m cells (vectorised): positions and
    analytic normals, outward winding; 2 m (m - 1) triangles."""
    th = np.linspace(0, np.pi, m + 1)
    ph = np.linspace(0, 2 * np.pi, m + 1)
    t, p = np.meshgrid(th, ph, indexing="ij")
    u = np.stack([np.sin(t) * np.cos(p), np.cos(t), np.sin(t) * np.sin(p)], -1)
    a, b = u[:-1, :-1], u[:-1, 1:]
    c, d = u[1:, 1:], u[1:, :-1]
    upper = np.stack([a, b, d], 2)[1:].reshape(-1, 3, 3)        # skip the north cap row
    lower = np.stack([b, c, d], 2)[:-1].reshape(-1, 3, 3)       # skip the south cap row
    n = np.concatenate([upper, lower])
    fn = np.cross(n[:, 1] - n[:, 0], n[:, 2] - n[:, 0])
    flip = np.einsum("ij,ij->i", fn, n.mean(axis=1)) < 0
    n[flip] = n[flip][:, ::-1]
    pos = n * radius + np.asarray(centre)
    return pos.reshape(-1, 9).astype(np.float32), n.reshape(-1, 9).astype(np.float32)


def batch_scene(rng):
    """One scene of the batched workload: the room, one ceiling light with
    emission U[5, 20], and 1-40 random boxes and tessellated spheres whose
    triangles total about T (log-uniform in [50k, 200k]); each object's
    material is diffuse, GGX (roughness U[0.05, 0.8]) or dielectric (IOR
    U[1.3, 1.7]) with equal probability.  Returns (scene, x_dim, y_dim, spp)
    with a square resolution from {64, 128, 192, 256} and spp log-uniform in
    [8, 128]."""
    scene = api.Scene()
    white = scene.add_material(api.material("Diffuse", diffuse=WHITE))
    red = scene.add_material(api.material("Diffuse", diffuse=RED))
    green = scene.add_material(api.material("Diffuse", diffuse=GREEN))
    e = float(rng.uniform(5, 20))
    light = scene.add_material(api.material("Diffuse", diffuse=(0.78, 0.78, 0.78),
                                            emission=(e, e, e)))
    walls, light_tris = room_triangles()
    tris, mats = [], []
    for name, ts in walls.items():
        m = red if name == "left" else green if name == "right" else white
        tris += ts
        mats += [m] * len(ts)
    tris += light_tris
    mats += [light] * len(light_tris)
    scene.add_mesh(np.stack(tris).reshape(-1, 9), np.array(mats, np.uint32))

    def random_material():
        k = rng.integers(3)
        if k == 0:
            return scene.add_material(api.material("Diffuse",
                                                   diffuse=tuple(rng.uniform(0.1, 0.9, 3))))
        if k == 1:
            return scene.add_material(api.material("GGX", specular=(0.04, 0.04, 0.04),
                                                   roughness=float(rng.uniform(0.05, 0.8))))
        return scene.add_material(api.material("DielectricRefractive", specular=(1, 1, 1),
                                               ior=float(rng.uniform(1.3, 1.7))))

    target = math.exp(rng.uniform(math.log(50e3), math.log(200e3)))
    n_obj = int(rng.integers(1, 41))
    is_sphere = rng.random(n_obj) < 0.5
    is_sphere[0] = True  # at least one sphere carries the triangle budget
    n_sph = int(is_sphere.sum())
    budget = max(target - 12 * (n_obj - n_sph), 2 * 4 * 3 * n_sph)
    m = max(4, int(round(math.sqrt(budget / (2 * n_sph)))))
    for k in range(n_obj):
        mat = random_material()
        if is_sphere[k]:
            r = float(rng.uniform(0.08, 0.3))
            c = (rng.uniform(-1 + r, 1 - r), rng.uniform(-1 + r, 0.6 - r), rng.uniform(-1 + r, 0.9))
            t, nrm = _sphere_grid(m, r, c)
            scene.add_mesh(t, np.full(len(t), mat, np.uint32), normals=nrm)
        else:
            w, h, d = rng.uniform(0.1, 0.5, 3)
            b = _box(w, h, d, float(rng.uniform(0, 90)),
                     (rng.uniform(-0.8, 0.8), rng.uniform(-0.8, 0.8)))
            scene.add_mesh(b.reshape(-1, 9), np.full(len(b), mat, np.uint32))
    res = int(rng.choice([64, 128, 192, 256]))
    spp = int(round(math.exp(rng.uniform(math.log(8), math.log(128)))))
    return scene, res, res, spp


def batch_scenes(n=256, seed=0):
    """The batched workload: n seeded scenes (see batch_scene), depth 6."""
    rng = np.random.default_rng(seed)
    return [batch_scene(rng) for _ in range(n)]


# ---------------------------------------------------------------------------
# differentiation workload

def _grid_quad(a, b, c, d, n):
    """Quad a-b-c-d as an n x n grid of quads: (triangles [2n^2, 9],
    cell centres [2n^2, 3])."""
    a, b, c, d = (np.asarray(v, np.float64) for v in (a, b, c, d))
    tris, cen = [], []
    for i in range(n):
        for j in range(n):
            u0, u1, v0, v1 = i / n, (i + 1) / n, j / n, (j + 1) / n

            def at(u, v):
                return (1 - u) * (1 - v) * a + u * (1 - v) * b + u * v * c + (1 - u) * v * d
            p = [at(u0, v0), at(u1, v0), at(u1, v1), at(u0, v1)]
            for t in ([p[0], p[1], p[2]], [p[0], p[2], p[3]]):
                tris.append(np.concatenate(t))
                cen.append(np.mean(t, axis=0))
    return np.array(tris, np.float32), np.array(cen)


def patch_cornell(seed=1, n_materials=16):
    """The Cornell geometry with walls and boxes split into patches of
    n_materials materials: floor, ceiling, left and right walls in two
    halves, the back wall in three strips, each box's top and sides, and the
    ceiling light.  Patch materials alternate Diffuse and GGX with albedo /
    F0 U[0.1, 0.9] and roughness U[0.1, 0.7]; the light emits 15.  Returns
    (scene, materials as capi.PathMaterial list)."""
    assert n_materials == 16
    rng = np.random.default_rng(seed)
    scene = api.Scene()
    mats = []

    def add(kind, **kw):
        m = api.material(kind, **kw)
        mats.append(m)
        return scene.add_material(m)

    patch_ids = []
    for k in range(15):
        refl = tuple(float(v) for v in rng.uniform(0.1, 0.9, 3))
        if k % 2 == 0:
            patch_ids.append(add("Diffuse", diffuse=refl))
        else:
            patch_ids.append(add("GGX", specular=refl, roughness=float(rng.uniform(0.1, 0.7))))
    light = add("Diffuse", diffuse=(0.78, 0.78, 0.78), emission=LIGHT_EMISSION)
    p = lambda x, y, z: (x, y, z)  # noqa: E731
    walls = [
        (p(-1, -1, -1), p(-1, -1, 1), p(1, -1, 1), p(1, -1, -1), 0, 2),   # floor: x halves
        (p(-1, 1, -1), p(1, 1, -1), p(1, 1, 1), p(-1, 1, 1), 2, 2),       # ceiling
        (p(-1, -1, -1), p(1, -1, -1), p(1, 1, -1), p(-1, 1, -1), 4, 3),   # back: 3 strips
        (p(-1, -1, -1), p(-1, 1, -1), p(-1, 1, 1), p(-1, -1, 1), 7, 2),   # left: z halves
        (p(1, -1, -1), p(1, -1, 1), p(1, 1, 1), p(1, 1, -1), 9, 2),       # right
    ]
    for a, b, c, d, first, parts in walls:
        tris, cen = _grid_quad(a, b, c, d, 6)
        axis = 2 if first in (7, 9) else 0
        x = (cen[:, axis] + 1.0) / 2.0
        idx = np.minimum((x * parts).astype(int), parts - 1)
        scene.add_mesh(tris, np.array([patch_ids[first + i] for i in idx], np.uint32))
    for (w, h, d, ang, cxz), first in (((0.6, 0.6, 0.6, -18.0, (0.33, 0.37)), 11),
                                       ((0.6, 1.2, 0.6, 18.0, (-0.33, -0.3)), 13)):
        b = _box(w, h, d, ang, cxz)
        # faces: bottom, top, then four sides (two triangles each)
        m = [patch_ids[first]] * 2 + [patch_ids[first + 1]] * 2 + [patch_ids[first]] * 8
        scene.add_mesh(b.reshape(-1, 9), np.array(m, np.uint32))
    _, light_tris = room_triangles()
    scene.add_mesh(np.stack(light_tris).reshape(-1, 9), np.full(2, light, np.uint32))
    return scene, mats


def perturbed_params(params, materials, seed=2, scale=0.1):
    """Target parameters: each active parameter scaled by U[1 - scale,
    1 + scale] (roughness and reflectance kept in [0.05, 0.95])."""
    from . import capi
    rng = np.random.default_rng(seed)
    out = np.array(params, np.float64)
    for i, m in enumerate(materials):
        f = rng.uniform(1 - scale, 1 + scale, 7)
        if m.type in (capi.BSDF["Diffuse"], capi.BSDF["GGX"]):
            out[i, 0:3] = np.clip(out[i, 0:3] * f[0:3], 0.05, 0.95)
        if m.type == capi.BSDF["GGX"]:
            out[i, 3] = np.clip(out[i, 3] * f[3], 0.05, 0.95)
        out[i, 4:7] = out[i, 4:7] * f[4:7]
    return out
