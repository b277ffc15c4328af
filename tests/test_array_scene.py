"""The NumPy scene description (scenes.ArrayScene) against the library's.

The CPU oracle's timed baseline builds its scenes with scenes.ArrayScene and
its camera with the oracle's own get_camera_transform, so that the reference
arm of the benchmark never loads libpath_gb300.so.  These checks hold both
to the library's scene export and camera bit for bit, and run the reference
arm's scene construction in a fresh process to check that the library is
not loaded there.
"""

import os
import subprocess
import sys

import numpy as np
import pytest

from path_gb300 import api, scenes
from oracle import oracle_lib as ol

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _same_export(a, b):
    for k in ("triangles", "normals", "tri_material", "mesh_ends", "cluster_ends_per_mesh",
              "instance_xforms", "instance_mesh", "clusters"):
        assert a[k].shape == b[k].shape, k
        assert np.array_equal(np.ascontiguousarray(a[k]).view(np.uint32),
                              np.ascontiguousarray(b[k]).view(np.uint32)), k
    assert a["n_materials"] == b["n_materials"]
    for i in range(a["n_materials"]):
        assert bytes(a["materials"][i]) == bytes(b["materials"][i])


@pytest.mark.parametrize("case", ["cornell", "large_mesh", "batch"])
def test_array_scene_exports_what_the_library_exports(lib, case):
    if case == "cornell":
        a, b = scenes.cornell_box(), scenes.cornell_box(scene_cls=scenes.ArrayScene)
    elif case == "large_mesh":
        a = scenes.large_mesh_room(subdivisions=3, glass_lat=20, glass_lon=20)
        b = scenes.large_mesh_room(subdivisions=3, glass_lat=20, glass_lon=20,
                                   scene_cls=scenes.ArrayScene)
    else:
        # face normals of arbitrary triangles, and a mesh without emitters
        rng = np.random.default_rng(4)
        tris = rng.normal(size=(500, 9)).astype(np.float32)
        tris[7] = 0  # degenerate: the zero normal is kept
        a, b = api.Scene(), scenes.ArrayScene()
        for sc in (a, b):
            m0 = sc.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5)))
            m1 = sc.add_material(api.material("Diffuse", emission=(1e-6, 0, 0)))
            sc.add_mesh(tris, np.where(np.arange(500) % 3 == 0, m1, m0).astype(np.uint32))
            sc.add_mesh(tris[:5], m0)
    assert a.sizes() == b.sizes()
    _same_export(a.export(), b.export())


def test_oracle_camera_equals_the_library_camera(lib):
    for w, h in ((256, 256), (1024, 1024), (64, 48), (37, 211)):
        assert np.array_equal(scenes.cornell_camera(w, h).view(np.uint32),
                              scenes.cornell_camera(w, h, ol.camera_transform).view(np.uint32))
    args = ((0.3, -0.2, -1), (0.1, 1, 0.2), (1, 2, 3), 55.0, 1.7)
    assert np.array_equal(api.camera_transform(*args), ol.camera_transform(*args))


@pytest.mark.parametrize("depth", [4, 5, 8])
def test_oracle_workload_settings_equal_the_library_settings(lib, depth):
    a = ol.workload_settings(depth, reduce_order=1, n_threads=3)
    b = ol.settings_from(scenes.path_settings(depth, "binary"), reduce_order=1, n_threads=3)
    assert bytes(a) == bytes(b)


def test_reference_arm_scene_does_not_load_the_library(oracle):
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "from path_gb300 import scenes\n"
        "from oracle import oracle_lib as ol\n"
        "sc = scenes.cornell_box(scene_cls=scenes.ArrayScene)\n"
        "arr = ol.SceneArrays(sc.export())\n"
        "f2w = scenes.cornell_camera(64, 64, ol.camera_transform)\n"
        "st = ol.workload_settings(5)\n"
        "img, _ = ol.Prepared(arr, st).render(st, 2, 64, 64, f2w, rows=(0, 64), stride=16)\n"
        "assert img[0].sum() > 0\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libpath_gb300' not in maps, 'library loaded'\n"
        "assert 'liboracle' in maps\n" % ROOT)
    proc = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stderr
