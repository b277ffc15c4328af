"""Row-band sharding of one image over ranks, gathered on rank 0 (CPU,
gloo, world size 2; the bands are rendered by the oracle here, by the GPU
render in a real multi-GPU run)."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_band_rows_partition_every_row():
    from path_gb300.shard import band_rows
    for y_dim in (1, 7, 64, 100, 1024):
        for yb in (1, 4, 8):
            for world in (1, 2, 3, 8):
                bands = [band_rows(r, world, y_dim, yb) for r in range(world)]
                rows = [y for lo, hi in bands for y in range(lo, hi)]
                assert rows == list(range(y_dim))
                assert all(lo % yb == 0 for lo, hi in bands if hi > lo)


def _worker(rank, world, port, result_path):
    import torch.distributed as dist
    from path_gb300 import api, scenes
    from path_gb300.shard import band_rows, gather_bands
    from oracle import oracle_lib as ol
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc = scenes.cornell_box()
        s = scenes.path_settings(5, "binary")
        w = h = 24
        f2w = scenes.cornell_camera(w, h)
        wd = api.work_division(s.render_work_division, 4, w, h)
        lo, hi = band_rows(rank, world, h, wd["y_block_size"])
        arr = ol.SceneArrays(sc.export())
        img, _ = ol.render(arr, ol.settings_from(s, reduce_order=1, n_threads=1), 4, w, h, f2w,
                           (lo, hi))
        img[:lo] = 0
        img[hi:] = 0
        full = gather_bands(img, (lo, hi), rank, world)
        if rank == 0:
            np.save(result_path, full)
    finally:
        dist.destroy_process_group()


def test_gather_bands_reassembles_the_single_process_image(tmp_path):
    import torch.multiprocessing as mp
    from path_gb300 import scenes
    from oracle import oracle_lib as ol
    ol.load()
    out = str(tmp_path / "full.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "binary")
    ref, _ = ol.render(ol.SceneArrays(sc.export()), ol.settings_from(s, reduce_order=1), 4, 24,
                       24, scenes.cornell_camera(24, 24))
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
