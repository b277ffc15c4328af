"""Writes tests/golden/cornell_fp64_4096spp.npz: the 4096-sample FP64 error
reference of the small Cornell box, computed by the CPU oracle.

The workload is the small Cornell box at 256 x 256, max depth 5 (NIters 4),
Sobol sampling, back-face-culled emission.  The reference image is the mean
of samples 16 .. 16 + 4095 of every pixel (the samples after the 16 a timed
16-spp render uses), each sample's radiance computed by the oracle exactly
as in its FP32 renders and summed per pixel in double precision.  Rows 2, 6,
10, ..., 254 are stored (64 of 256, as float32: the stored rounding is 6e-8
relative, far below the agreement the tests ask for).

Run from the repository root: python tests/golden/make_fp64_reference.py
(about two minutes on 8 cores).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "cornell_fp64_4096spp.npz")
SIZE, SPP, DEPTH, REF_SPP = 256, 16, 5, 4096
ROW_START, ROW_STRIDE = 2, 4


def main():
    from path_gb300 import scenes
    from oracle import oracle_lib as ol
    scene = scenes.cornell_box()
    settings = ol.settings_from(scenes.path_settings(DEPTH, "binary"), reduce_order=1)
    f2w = scenes.cornell_camera(SIZE, SIZE)
    prep = ol.Prepared(ol.SceneArrays(scene.export()), settings)
    img, secs = prep.render_f64(settings, REF_SPP, SIZE, SIZE, f2w, rows=(ROW_START, SIZE),
                                stride=ROW_STRIDE, sample_offset=SPP)
    rows = np.arange(ROW_START, SIZE, ROW_STRIDE)
    np.savez_compressed(OUT, rows=rows, image=img[rows].astype(np.float32),
                        size=SIZE, spp=SPP, depth=DEPTH, ref_spp=REF_SPP, sample_offset=SPP)
    print(f"wrote {OUT}: {len(rows)} rows, {secs:.1f} s of oracle time")


if __name__ == "__main__":
    main()
