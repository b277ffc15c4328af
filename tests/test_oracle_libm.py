"""How far the shared transcendental polynomials move an image from the C
library's arithmetic.

The kernels and the oracle evaluate sin, cos, asin, acos and pow with the
same polynomials (path_gb300/csrc/pmath.h), so that CPU and GPU round every
bounce direction identically; the reference calls std::sin, std::cos,
std::asin, std::acos and std::pow (include/bsdf/diffuse.h:30-45,
glossy.h:26-49, dielectric_refractive.h:24-33, lib/projection.h:9-32,
term_prob/multiplier_func/multiplier_func.h:19-30).  liboracle_libm.so is
the same oracle built to call the C library's functions there.  These tests
render the same workloads with both builds and bound the difference, which
is the part of the image parity that rests on the shared polynomials rather
than on the reference's own arithmetic (measured: 3.3e-6 relative RMSE on
the small Cornell box at 256 x 256 x 16 spp, 7.0e-6 on the large-mesh room
at 128 x 128 x 16 spp; the reference's -Ofast build is itself not
reproducible at that level).
"""

import numpy as np
import pytest

from path_gb300 import scenes
from oracle import oracle_lib as ol


def _gap(scene, depth, size, spp):
    st = ol.workload_settings(depth, reduce_order=1)
    arr = ol.SceneArrays(scene.export())
    f2w = scenes.cornell_camera(size, size, ol.camera_transform)
    pm = ol.Prepared(arr, st)
    lm = ol.Prepared(arr, st, libm=True)
    a, _ = pm.render(st, spp, size, size, f2w)
    b, _ = lm.render(st, spp, size, size, f2w)
    rel = float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(a.astype(np.float64)))
    # per-sample view: how many paths changed at all, and how many by more
    # than 1e-3 (a diverged path rather than a rounding difference)
    sa = pm.sample_values(st, spp, size, size, f2w, rows=(0, size), stride=4)
    sb = lm.sample_values(st, spp, size, size, f2w, rows=(0, size), stride=4)
    d = np.abs(sa - sb).max(-1)
    return rel, float((d > 0).mean()), float((d > 1e-3).mean())


def test_libm_gap_small_cornell(oracle):
    rel, changed, diverged = _gap(scenes.cornell_box(scene_cls=scenes.ArrayScene), 5, 256, 16)
    print(f"Cornell 256x256x16: rel RMSE {rel:.2e}, samples changed {changed:.3f}, "
          f"diverged {diverged:.2e}")
    assert rel < 1e-4
    assert diverged < 1e-3


def test_libm_gap_large_mesh(oracle):
    scene = scenes.large_mesh_room(subdivisions=8, scene_cls=scenes.ArrayScene)
    rel, changed, diverged = _gap(scene, 8, 128, 16)
    print(f"large mesh 128x128x16: rel RMSE {rel:.2e}, samples changed {changed:.3f}, "
          f"diverged {diverged:.2e}")
    assert rel < 1e-4
    assert diverged < 1e-3


if __name__ == "__main__":
    pytest.main([__file__, "-q", "-s"])
