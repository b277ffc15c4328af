"""In-kernel limits report through the device status word, with no fault
and no hang.

A path that never ends -- rays inside a closed box of perfect mirrors, with
no termination before 10000 vertices -- is cut at 4096 vertices (the bound
the reference does not have); the render returns PATH_ERR_DEVICE_TIMEOUT
with device status 4 (path too long), and the same renderer then renders a
normal scene cleanly.  The work is bounded: 64 paths of 4096 vertices."""

import numpy as np
import pytest

from path_gb300 import api, capi, scenes

pytestmark = pytest.mark.gpu

PATH_ERR_DEVICE_TIMEOUT = 4
STATUS_PATH_TOO_LONG = 4


def _mirror_box():
    """The cube [-1, 1]^3, 12 triangles facing inward, all perfect mirrors."""
    sc = api.Scene()
    mirror = sc.add_material(api.material("Mirror", specular=(1, 1, 1)))
    v = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], np.float32)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for a, b, c, d in quads:
        tris += [v[[a, b, c]].ravel(), v[[a, c, d]].ravel()]
    tris = np.array(tris, np.float32)
    sc.add_mesh(tris, np.full(len(tris), mirror, np.uint32))
    return sc


@pytest.mark.parametrize("approach,traversal", [(0, "binary"), (0, "wide"), (1, "wide")])
def test_endless_path_is_cut_and_reported(lib, approach, traversal):
    rng = np.random.default_rng(4)
    d = rng.normal(size=(64, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([rng.uniform(-0.5, 0.5, (64, 3)), d], 1).astype(np.float32)
    s = scenes.path_settings(10001, traversal)
    s.light_sampler = 1  # no emitters to sample
    s.kernel_approach = approach
    out = np.zeros((64, 3), np.float32)
    r = api.Renderer()
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, api.InitialRays(rays), out, _mirror_box(), 1, s)
    assert e.value.status == PATH_ERR_DEVICE_TIMEOUT
    assert r.stats()["device_status"] == STATUS_PATH_TOO_LONG
    # the renderer (and its context) stay usable
    sc = scenes.cornell_box()
    s2 = scenes.path_settings(5, traversal)
    s2.kernel_approach = approach
    img = np.zeros((16, 16, 3), np.float32)
    r.render(api.ExecutionModel.GPU, api.SquareImage(16, 16, scenes.cornell_camera(16, 16)),
             img, sc, 4, s2)
    assert r.stats()["device_status"] == 0
    assert float(img.mean()) > 0.0


PATH_ERR_OOM = 3


@pytest.mark.parametrize("approach", [0, 1])
def test_allocation_failure_is_reported_and_the_renderer_recovers(lib, approach):
    # An allocation cap (host-side fault injection: the allocation a full
    # device would refuse is refused before cudaMalloc is called) forces the
    # out-of-memory path in the middle of a render: the call returns
    # PATH_ERR_OOM with a message, and with the cap lifted the same renderer
    # renders the image a fresh renderer renders.
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "wide")
    s.kernel_approach = approach
    w = h = 32
    spec = api.SquareImage(w, h, scenes.cornell_camera(w, h))
    want = np.zeros((h, w, 3), np.float32)
    api.Renderer().render(api.ExecutionModel.GPU, spec, want, sc, 4, s)
    r = api.Renderer()
    out = np.zeros((h, w, 3), np.float32)
    try:
        capi.load().path_debug_set_device_alloc_cap(64 * 1024)
        with pytest.raises(capi.PathError) as e:
            r.render(api.ExecutionModel.GPU, spec, out, sc, 4, s)
        assert e.value.status == PATH_ERR_OOM
        assert "memory" in str(e.value).lower() or "alloc" in str(e.value).lower()
    finally:
        capi.load().path_debug_set_device_alloc_cap(0)
    r.render(api.ExecutionModel.GPU, spec, out, sc, 4, s)
    assert r.stats()["device_status"] == 0
    assert np.array_equal(out.view(np.uint32), want.view(np.uint32))
