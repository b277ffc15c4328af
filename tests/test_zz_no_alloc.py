"""path_render_noalloc: rendering without any device allocation.

Callers that cannot call cudaMalloc -- a host framework that owns all device
memory through its own allocator, or a real-time loop that must not allocate
after start-up because allocation can synchronise the device -- render
through path_render_noalloc once the scene is resident.  Its scratch (status
word, counters, per-sample-block partial sums and the reduction's second
buffer) lives in one fixed device array inside the library.

These checks call it through the C ABI twice in a row and compare each image
bit for bit with path_render's on the same scene (the binary traversal is
bit-exact, the tolerance the parity tests hold it to), with the image written
straight to the output, with partial sums reduced through the scratch array
and for a progressive frame (a nonzero sample_offset).  Around each call
after the first, the device's free memory (cudaMemGetInfo) must not change:
the property the entry point exists for.  The file is named to be collected
last so that a run stopping at the first failure has already run every other
test.
"""

import ctypes

import numpy as np
import pytest

from path_gb300 import api, capi, scenes

pytestmark = pytest.mark.gpu


def _noalloc(renderer, spec, out, scene, spp, settings):
    o = capi.Output()
    o.type = capi.OUTPUT_BGRA if out.dtype.is_floating_point is False else capi.OUTPUT_FLOAT_RGB
    o.data = out.data_ptr()
    o.on_device = 1
    c_spec = spec.to_c()
    secs = ctypes.c_double()
    return capi.load().path_render_noalloc(renderer._h, ctypes.byref(c_spec), ctypes.byref(o),
                                           scene.handle, spp, ctypes.byref(settings.raw),
                                           ctypes.byref(secs))


def _sample_block_settings():
    s = scenes.path_settings(5, "binary")
    s.render_work_division.block_size = 32
    s.render_work_division.force_target_samples = 1
    s.render_work_division.forced_target_samples_per_thread = 1
    return s


@pytest.mark.parametrize("case", ["direct", "sample_blocks", "bgra", "uniform_rng",
                                  "sample_offset"])
def test_noalloc_matches_path_render_twice(lib, case):
    torch = pytest.importorskip("torch")
    scene = scenes.cornell_box()
    w, h = 64, 48
    spp = 128 if case == "sample_blocks" else 16
    settings = _sample_block_settings() if case == "sample_blocks" else \
        scenes.path_settings(5, "binary")
    if case == "uniform_rng":
        settings.rng = 1
    offset = 48 if case == "sample_offset" else 0
    spec = api.SquareImage(w, h, scenes.cornell_camera(w, h), sample_offset=offset)
    r = api.Renderer()
    if case == "bgra":
        ref = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
    else:
        ref = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    r.render(api.ExecutionModel.GPU, spec, ref, scene, spp, settings)
    torch.cuda.synchronize()
    expect = ref.cpu().numpy()
    if offset:
        # a frame of later samples is a different image
        r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, spec.film_to_world), ref, scene,
                 spp, settings)
        assert not np.array_equal(ref.cpu().numpy(), expect)
    outs = [torch.full_like(ref, 7) for _ in range(3)]
    torch.cuda.synchronize()
    free_after_first = None
    for k, out in enumerate(outs):
        free_before = torch.cuda.mem_get_info()[0]
        capi.check(_noalloc(r, spec, out, scene, spp, settings))
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if k == 0:
            free_after_first = free_after
        else:
            # the first call on a device may load the library's module (and
            # with it the scratch array); later calls allocate nothing
            assert free_after == free_before == free_after_first
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint8), expect.view(np.uint8))
        assert r.stats()["device_status"] == 0


def test_noalloc_rejects_what_it_cannot_do(lib):
    torch = pytest.importorskip("torch")
    scene = scenes.cornell_box()
    r = api.Renderer()
    s = _sample_block_settings()
    w = h = 1024
    spec = api.SquareImage(w, h, scenes.cornell_camera(w, h))
    out = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    # not resident yet
    status = _noalloc(r, spec, out, scene, 128, s)
    assert status == 1 and "resident" in capi.load().path_last_error().decode()
    r.render(api.ExecutionModel.GPU, spec, out, scene, 128, s)
    # four sample blocks of partial sums for 1024 x 1024 pixels exceed the array
    status = _noalloc(r, spec, out, scene, 128, s)
    msg = capi.load().path_last_error().decode()
    assert status == 1 and "bytes of scratch" in msg, msg
    # host output is refused
    o = capi.Output()
    o.type = capi.OUTPUT_FLOAT_RGB
    host = np.zeros((h, w, 3), np.float32)
    o.data = host.ctypes.data
    o.on_device = 0
    c_spec = spec.to_c()
    status = capi.load().path_render_noalloc(r._h, ctypes.byref(c_spec), ctypes.byref(o),
                                             scene.handle, 128, ctypes.byref(s.raw), None)
    assert status == 1
