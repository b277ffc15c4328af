"""The reference's own scenes rendered on the GPU against the oracle.

Four scenes of the reference's scenes/ folder (the Cornell box with diffuse
walls, with a Phong-glossy sphere, with a mirror box and with a glass box),
as this library's loader reads their XML / OBJ / MTL files
(tests/golden/reference_scenes.npz, made by
tests/golden/make_reference_scene_fixtures.py; the CPU tests hold the
loader to these arrays), rendered with the reference's camera at 64 x 64,
16 spp, depth 5: bit for bit through the binary traversal, and within 1e-4
relative RMSE (and here bit for bit as well, no exact ties occurring)
through the 8-wide streaming path.
"""

import os

import numpy as np
import pytest

from path_gb300 import api, capi, scenes
from oracle import oracle_lib as ol

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ["cornell-diffuse", "cornell-glossy-sphere", "cornell-mirror", "cornell-glass-box"]


def _scene(g, name):
    sc = api.Scene()
    for rec in g[f"{name}/materials"]:
        m = capi.PathMaterial.from_buffer_copy(rec.tobytes())
        sc.add_material(m)
    sc.add_mesh(g[f"{name}/triangles"], g[f"{name}/tri_material"], normals=g[f"{name}/normals"],
                object_to_world=g[f"{name}/object_to_world"])
    return sc, g[f"{name}/film_to_world"]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("path", ["binary_mega", "wide_streaming"])
def test_reference_scene_matches_oracle(lib, oracle, name, path):
    g = np.load(os.path.join(HERE, "golden", "reference_scenes.npz"))
    sc, f2w = _scene(g, name)
    w = h = 64
    spp = 16
    s = scenes.path_settings(5, "binary" if path == "binary_mega" else "wide")
    s.kernel_approach = 0 if path == "binary_mega" else 1
    got = np.zeros((h, w, 3), np.float32)
    r = api.Renderer()
    r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w), got, sc, spp, s)
    assert r.stats()["device_status"] == 0
    st = ol.settings_from(scenes.path_settings(5, "binary"), reduce_order=1,
                          tie_rule=0 if path == "binary_mega" else 1)
    want, _ = ol.render(ol.SceneArrays(sc.export()), st, spp, w, h, f2w)
    assert float(want.mean()) > 0.0
    err = float(np.linalg.norm(got.astype(np.float64) - want) / np.linalg.norm(want))
    print(f"{name} {path}: rel RMSE {err:.2e}")
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
