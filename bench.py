"""Benchmark of the render hot path (one JSON line on rank 0).

Workload (default): the large-mesh scene -- Cornell room with a 1,310,720-
triangle displaced icosphere (GGX, roughness 0.2, F0 0.04) and a 19,800-
triangle glass sphere (IOR 1.5) -- rendered at 1024 x 1024, 64 spp, max depth
8 (NIters 7, no Russian roulette), Sobol sampling, FP32 accumulation.  One
step is one full render.

* value: Msamples/s of the integration + reduction kernels, timed with CUDA
  events on the renderer's stream (path_render_stats.kernel_ms), scene
  resident in HBM, image written to device memory.  L2 is flushed (512 MB
  write) before every timed step.
* e2e: the same metric through the C ABI call a user makes (path_render) with
  host buffers: every step re-copies the scene's device arrays from pinned
  host memory and copies the image back to the host, all inside the timed
  wall-clock region.
* roofline: the dominant kernel (the persistent trace) against both sides of
  the path's roofline -- algorithmic bytes (wide nodes x 80 B + triangles
  tested x 48 B + rays x 40 B, counted by a counting run of the same render)
  against the measured HBM copy bandwidth, and the instructions it issues
  (per node visit, from the committed ncu summary) against the SMs' issue
  rate -- with `bound` the side that is nearer its peak.
* parity_vs_oracle: the timed image against the CPU oracle (a restatement
  of the reference's CPU path) on spread rows of the same render.
* error_vs_4096spp_fp64: the timed image against 4096 samples per pixel
  summed in FP64, by the GPU (whole image) and by the oracle (spread rows).
* time_to_0.02_rmse, adjoint_forward_ratio: the other two parts of the
  metric (the radiance-cache and adjoint workloads, smaller runs than
  --workload cache / the adjoint tests).
* cpu_baseline: the CPU oracle on the spread rows, all host threads.

``--impl reference`` times that CPU restatement alone, on the same spread
rows, with the scene built in NumPy (scenes.ArrayScene) so that the
library is not loaded (the reference itself cannot be built here: it needs
clang as its CUDA compiler and libraries that are not installed).  N > 1
runs independent replicas, one per GPU (the render has no data-path
exchange).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _profiled_traffic(kernel, args, shape, alg_bytes_per_launch):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary of this workload (profiles/<kernel>_dram_<workload>.txt): its
    measured DRAM bytes per algorithmic byte ('dram_per_algorithmic_byte:')
    times this run's algorithmic bytes per launch, or its
    'dram_bytes_per_launch:' line; None when the summary is missing or was
    taken at another launch shape (its 'launch_shape:' line)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_dram_{args.workload}.txt")
    traffic, ratio, profiled_shape = None, None, None
    try:
        with open(path) as f:
            for ln in f:
                if ln.startswith("dram_bytes_per_launch:"):
                    traffic = float(ln.split(":", 1)[1])
                elif ln.startswith("dram_per_algorithmic_byte:"):
                    ratio = float(ln.split(":", 1)[1])
                elif ln.startswith("launch_shape:"):
                    profiled_shape = ln.split(":", 1)[1].strip()
    except OSError:
        pass
    if profiled_shape != shape:
        return None
    return ratio * alg_bytes_per_launch if ratio is not None else traffic


def _profiled_issue(kernel, args, shape):
    """Instructions the dominant kernel issues per wide-node visit (warp and
    thread level) from the committed ncu summary of this workload's kernel
    (lines 'warp_inst_per_node_visit: N', 'thread_inst_per_node_visit: N'
    and 'launch_shape:' in profiles/<kernel>_issue_<workload>.txt), or None
    when it is missing or was taken at another launch shape."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_issue_{args.workload}.txt")
    vals, profiled_shape = {}, None
    try:
        with open(path) as f:
            for ln in f:
                key, _, val = ln.partition(":")
                if key in ("warp_inst_per_node_visit", "thread_inst_per_node_visit"):
                    vals[key] = float(val)
                elif key == "launch_shape":
                    profiled_shape = val.strip()
    except (OSError, ValueError):
        return None
    return vals if profiled_shape == shape and len(vals) == 2 else None


def make_workload(name, size=None, spp_override=None, scene_cls=None):
    from path_gb300 import scenes
    if name == "large_mesh":
        scene = scenes.large_mesh_room(subdivisions=8, scene_cls=scene_cls)
        w = h = size or 1024
        spp, depth = spp_override or 64, 8
        desc = ("large-mesh room: 1,310,720-tri displaced icosphere (GGX a=0.2 F0=0.04) + "
                f"19,800-tri glass sphere (IOR 1.5), {w}x{h}, {spp} spp, depth 8")
    else:
        scene = scenes.cornell_box(scene_cls=scene_cls)
        w = h = size or 256
        spp, depth = spp_override or 16, 5
        desc = f"Cornell box: 36 triangles, {w}x{h}, {spp} spp, depth 5"
    return scene, w, h, spp, depth, desc


def spread_rows(h, rows):
    """`rows` rows spread over the image: every (h // rows)-th row, starting
    half a stride in."""
    stride = max(1, h // max(1, rows))
    start = stride // 2
    return start, stride, np.arange(start, h, stride)


def oracle_prepare(scene_arrays, settings, reduce_order, threads):
    from oracle import oracle_lib as ol
    s = ol.settings_from(settings, reduce_order=reduce_order, n_threads=threads)
    return ol.Prepared(scene_arrays, s), s


def cpu_sample(prep, s, spp, w, h, f2w, rows):
    """The oracle on spread rows; returns (image with those rows, row
    indices, samples, seconds)."""
    start, stride, sel = spread_rows(h, rows)
    img, secs = prep.render(s, spp, w, h, f2w, rows=(start, h), stride=stride)
    return img, sel, len(sel) * w * spp, secs


def run_reference(args, rank):
    if rank != 0:
        return
    from path_gb300 import scenes
    from oracle import oracle_lib as ol
    scene, w, h, spp, depth, desc = make_workload(args.workload, args.size, args.spp,
                                                  scene_cls=scenes.ArrayScene)
    f2w = scenes.cornell_camera(w, h, ol.camera_transform)
    threads = os.cpu_count() or 1
    # the reference's CPU execution model: lane-order reduction
    s = ol.workload_settings(depth, reduce_order=0, n_threads=threads)
    prep = ol.Prepared(ol.SceneArrays(scene.export()), s)
    rows = args.cpu_rows
    for _ in range(args.warmup):
        cpu_sample(prep, s, spp, w, h, f2w, rows)
    total_s, total_samples = 0.0, 0
    for _ in range(args.steps):
        _, sel, n, secs = cpu_sample(prep, s, spp, w, h, f2w, rows)
        total_s += secs
        total_samples += n
    value = total_samples / total_s / 1e6
    sample = (f"{len(sel)} rows spread over the image (1 in {h // rows}) x {w} px x {spp} "
              "spp per step")
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": desc, "sample": sample},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": sample + " (oracle: CPU restatement of the reference CPU "
                                            "path; scene built in NumPy, library not loaded)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batched(args, rank, world, local_rank):
    """The batched workload: seeded random scenes (room + 1-40 boxes and
    spheres, 50k-200k triangles, diffuse / GGX / dielectric, resolution in
    {64..256}^2, 8-128 spp, depth 6) in one path_render_batch call, launch
    shape from path_batch_autotune."""
    import torch
    import torch.distributed as dist
    from path_gb300 import api, scenes
    t0 = time.time()
    batch = scenes.batch_scenes(args.scenes, seed=0)
    gen_s = time.time() - t0
    settings = scenes.path_settings(6, "wide")
    settings.gpu_build = args.gpu_build
    outs = [np.zeros((h, w, 3), np.float32) for _, w, h, _ in batch]
    items = [(sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), o, spp)
             for (sc, w, h, spp), o in zip(batch, outs)]
    samples = sum(w * h * spp for _, w, h, spp in batch)
    tris = sum(sc.sizes()["triangles"] for sc, _, _, _ in batch)
    r = api.Renderer()
    t0 = time.time()
    tuning = r.autotune_batch(items, settings)
    setup_s = time.time() - t0
    build_s = r.stats()["bvh_build_seconds"]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        r.render_batch(items, settings, tuning)
    kernel_ms, wall, launches = [], [], 0
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t = time.perf_counter()
            r.render_batch(items, settings, tuning)
            wall.append(time.perf_counter() - t)
            st = r.stats()
            kernel_ms.append(st["kernel_ms"])
            launches += st["gpu_launches"]
    torch.cuda.synchronize()
    total_ms, e2e_total = sum(kernel_ms), sum(wall)
    if world > 1:
        t = torch.tensor([total_ms, e2e_total], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, e2e_total = float(t[0]), float(t[1])
    line = {
        "metric": METRIC, "value": world * samples * args.steps / (total_ms / 1e3) / 1e6,
        "unit": METRIC, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched: {len(batch)} seeded scenes, {tris} triangles, "
                               f"{samples} samples, depth 6",
                   "tuning": tuning, "l2": "flushed (512 MB write) before every timed step",
                   "bvh": ("GPU PLOC BVH" + (" over split references" if args.gpu_build == 2
                                             else "")) if args.gpu_build else "SBVH (host)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * samples * args.steps / e2e_total / 1e6, "unit": METRIC,
                "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(sum(o.nbytes for o in outs))},
        "gpu_launches": int(launches),
        "setup_s": setup_s, "bvh_build_s": build_s, "scene_generation_s": gen_s,
        "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def time_to_rmse(r, scene, w, h, f2w, settings, ref, cfg, max_frames, base, target=0.02):
    """Frames of 4 new samples each (from Sobol sample `base` on),
    accumulated in FP64 until the relative RMSE against `ref` is <= target:
    plain renders (cfg None) or radiance-cache frames (cfg: the vertex where
    paths end into the cache, training records and Adam steps per frame,
    training-only frames first).  Wall time of the render + training calls."""
    import torch
    from path_gb300 import api
    ref_norm = float(torch.linalg.norm(ref))
    out = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    cache = api.RadianceCache(seed=1) if cfg is not None else None
    if cache is not None and cfg.get("ema", 0.0) > 0.0:
        cache.set_ema(cfg["ema"])
    acc = torch.zeros_like(ref)
    wall, frames, err, curve = 0.0, 0, None, []

    def frame(offset):
        spec = api.SquareImage(w, h, f2w, sample_offset=offset)
        if cache is None:
            r.render(api.ExecutionModel.GPU, spec, out, scene, 4, settings)
        else:
            r.render_cached(cache, spec, out, scene, 4, settings,
                            cache_depth=cfg["cache_depth"], train_paths=cfg["train_paths"],
                            train_steps=cfg["train_steps"])

    if cfg is not None and cfg["pretrain_frames"] > 0:
        torch.cuda.synchronize()
        t = time.perf_counter()
        for f in range(cfg["pretrain_frames"]):
            frame(base + 4 * (max_frames + f))
        torch.cuda.synchronize()
        wall += time.perf_counter() - t
    while frames < max_frames:
        torch.cuda.synchronize()
        t = time.perf_counter()
        frame(base + 4 * frames)
        torch.cuda.synchronize()
        wall += time.perf_counter() - t
        frames += 1
        acc += out.double()
        err = float(torch.linalg.norm(acc / frames - ref)) / ref_norm
        if frames in (1, 2, 4, 8, 16, 32, 64, 128, 256) or err <= target:
            curve.append((frames, round(wall, 4), round(err, 5)))
        if err <= target:
            break
    res = {"frames": frames, "seconds": wall, "rel_rmse": err,
           "reached": err is not None and err <= target, "curve": curve}
    if cfg is not None:
        res["cache_bias"] = cache_bias(r, scene, settings, cache, cfg["cache_depth"])
        res["cache"] = (
            "hash grid 16x2x2^19, MLP 48-64x5-3 BF16 tcgen05, Adam 1e-2, "
            f"paths end into the cache at vertex {cfg['cache_depth']}, "
            f"{cfg['train_paths']} records x {cfg['train_steps']} steps per frame, "
            f"{cfg['pretrain_frames']} training-only frames first"
            + (f", inference on a moving average of the parameters (decay {cfg['ema']} "
               "per Adam step)" if cfg.get("ema", 0.0) > 0.0 else ""))
    return res


def cache_bias(r, scene, settings, cache, depth, n_queries=4096, ref_spp=1024):
    """The trained cache against converged radiance at its own queries: of
    the last frame's paths that ended into the cache (a spread sample of
    them), the network's prediction against the radiance the rest of the
    path carries on average, estimated by ref_spp paths traced from each
    query point (InitialRays from just in front of the point towards it,
    with the depth the path had left) in two halves, whose difference
    gives the estimate's own noise.  Queries on the light are left out (the
    traced estimate counts the light's emission, the cache's target does
    not)."""
    from path_gb300 import api
    q, beta = r.cached_frame_queries(max_n=n_queries, stride=997)
    if len(q) == 0:
        return None
    pos, wo = q[:, 0:3], q[:, 3:6]
    off_light = ~((pos[:, 1] > 0.99) & (np.abs(pos[:, 0]) < 0.26) & (np.abs(pos[:, 2]) < 0.26))
    q, beta, pos, wo = q[off_light], beta[off_light], pos[off_light], wo[off_light]
    rays = np.concatenate([pos + 1e-3 * wo, -wo], 1).astype(np.float32)
    s = settings.copy()
    s.set_term_prob("NIters", iters=max(0, int(settings.term_prob_iters) - depth))
    out = np.zeros((len(rays), 3), np.float32)
    r.render(api.ExecutionModel.GPU, api.InitialRays(rays), out, scene, ref_spp // 2, s)
    half = out.astype(np.float64)  # the first half of the samples
    r.render(api.ExecutionModel.GPU, api.InitialRays(rays), out, scene, ref_spp, s)
    ref = out.astype(np.float64)
    # ref - half = (second half - first half) / 2: the standard error of ref
    pred = cache.query(q).astype(np.float64)
    norm = np.linalg.norm(ref)
    wnorm = np.linalg.norm(beta * ref)
    rel = np.abs(pred - ref).sum(1) / (np.abs(ref).sum(1) + 1e-3)
    return {
        "queries": int(len(q)), "reference_spp": ref_spp,
        "rel_l2": float(np.linalg.norm(pred - ref) / norm),
        "rel_l2_throughput_weighted": float(np.linalg.norm(beta * (pred - ref)) / wnorm),
        "mean_rel_bias": float(np.sum(pred - ref) / np.sum(ref)),
        "median_rel_err": float(np.median(rel)), "p90_rel_err": float(np.percentile(rel, 90)),
        "reference_noise_rel_l2": float(np.linalg.norm(ref - half) / norm),
    }


def gpu_reference(r, scene, w, h, f2w, settings, first_sample, n_samples=4096, per_render=64):
    """n_samples samples per pixel from Sobol sample first_sample on, each
    render of per_render samples summed into an FP64 image (mean)."""
    import torch
    from path_gb300 import api
    out = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    ref = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
    n = max(1, n_samples // per_render)
    for f in range(n):
        r.render(api.ExecutionModel.GPU,
                 api.SquareImage(w, h, f2w, sample_offset=first_sample + per_render * f), out,
                 scene, per_render, settings)
        ref += out.double()
    return ref / n


def cache_study(r, scene, w, h, f2w, settings, ref, args, ref_note):
    """Time to 0.02 relative RMSE of the plain tracer and of the radiance
    cache (the configuration on the command line -- by default the
    specified one: paths end at vertex 2, 2^16 records x 4 Adam steps per
    frame -- and a tuned one with its untrained control), frames starting
    after the reference's samples."""
    base = 64 + 4096 + 64
    plain = time_to_rmse(r, scene, w, h, f2w, settings, ref, None, args.max_frames, base)
    spec_cfg = {"cache_depth": args.cache_depth, "train_paths": args.train_paths,
                "train_steps": args.train_steps, "pretrain_frames": args.pretrain_frames}
    runs = {"cached": time_to_rmse(r, scene, w, h, f2w, settings, ref, spec_cfg,
                                   args.max_frames, base),
            "cached_ema": time_to_rmse(r, scene, w, h, f2w, settings, ref,
                                       dict(spec_cfg, ema=0.99), args.max_frames, base)}
    controls = {}
    if not args.no_tuned_cache:
        tuned = {"cache_depth": 3, "train_paths": 1 << 14, "train_steps": 2,
                 "pretrain_frames": 0}
        runs["cached_tuned"] = time_to_rmse(r, scene, w, h, f2w, settings, ref, tuned,
                                            args.max_frames, base)
        runs["cached_tuned_ema"] = time_to_rmse(r, scene, w, h, f2w, settings, ref,
                                                dict(tuned, ema=0.9), args.max_frames, base)
        controls["cached_tuned_untrained"] = time_to_rmse(
            r, scene, w, h, f2w, settings, ref, dict(tuned, train_steps=0), args.max_frames,
            base)
    reached = [k for k in runs if runs[k]["reached"]]
    best = min(reached, key=lambda k: runs[k]["seconds"]) if reached else None
    return {
        "value": runs[best]["seconds"] if best else None, "unit": "s", "value_from": best,
        "ratio_cached_over_plain": (runs[best]["seconds"] / plain["seconds"]
                                    if plain["reached"] and best else None),
        "target_ratio": 0.25, "reference": ref_note,
        "plain": plain, **runs, **controls,
    }


def adjoint_study(steps=5):
    """Adjoint / forward cost on the 16-material Cornell patches (128 x 128,
    64 spp, depth 4, L2 loss to a target from parameters perturbed by up to
    10%, seed 2), kernel time of each, plus the adjoint's agreement with
    central differences (step 1e-3, common random numbers) on four
    reflectance / emission parameters."""
    from path_gb300 import api, diff, scenes
    w = h = 128
    sc, mats = scenes.patch_cornell(seed=1)
    s = scenes.path_settings(4, "wide")
    s.kernel_approach = 1
    rend = diff.Renderable(sc, mats, api.SquareImage(w, h, scenes.cornell_camera(w, h)), 64, s)
    p0 = diff.params_of(mats)
    target = rend.render(scenes.perturbed_params(p0, mats, seed=2)).astype(np.float64)
    img = rend.render(p0)
    d_img = (2.0 * (img.astype(np.float64) - target)).astype(np.float32)
    r = rend.renderer
    fwd, adj = [], []
    for _ in range(steps):
        rend.render(p0)
        fwd.append(r.stats()["kernel_ms"])
        g = rend.adjoint(p0, d_img)
        adj.append(r.stats()["kernel_ms"])

    def loss(p):
        d = rend.render(p).astype(np.float64) - target
        return float((d * d).sum())

    pairs = [(0, 0), (3, 1), (15, 4), (8, 2)]
    fd, ad = [], []
    for i, j in pairs:
        hi, lo = p0.copy(), p0.copy()
        hi[i, j] += 1e-3
        lo[i, j] -= 1e-3
        fd.append((loss(hi) - loss(lo)) / 2e-3)
        ad.append(g[i, j])
    fd, ad = np.array(fd), np.array(ad)
    return {"value": float(np.median(adj) / np.median(fwd)), "unit": "x", "target": 3.0,
            "forward_ms": float(np.median(fwd)), "adjoint_ms": float(np.median(adj)),
            "fd_rel_err": float(np.linalg.norm(ad - fd) / np.linalg.norm(fd)),
            "workload": "16-material Cornell patches, 128x128, 64 spp, depth 4, L2 loss; "
                        "adjoint = forward render + path replay"}


def run_cache(args, rank, world, local_rank):
    """Time to 0.02 relative RMSE, plain tracer against the radiance cache,
    on the large-mesh room at 1024 x 1024 in frames of 4 spp (depth 8)
    against 4096 spp of the plain tracer accumulated in FP64."""
    from path_gb300 import api, scenes
    size = args.size or 1024
    scene, w, h, _, depth, desc = make_workload("large_mesh", size, 4)
    settings = scenes.path_settings(8, "wide")
    settings.kernel_approach = 1
    f2w = scenes.cornell_camera(w, h)
    r = api.Renderer()
    t0 = time.time()
    ref = gpu_reference(r, scene, w, h, f2w, settings, 64)
    ref_s = time.time() - t0
    study = cache_study(r, scene, w, h, f2w, settings, ref, args,
                        "4096 spp (samples 64..4159), FP64 sum")
    line = {
        "metric": "seconds to 0.02 relative RMSE", "unit": "s", "higher_is_better": False,
        "value": study.pop("value"), "n_gpus": 1, "dtype": "f32 render, bf16 cache MLP",
        "data": "synthetic",
        "config": {"workload": f"{desc} in 4-spp frames; reference 4096 spp FP64",
                   "value_from": study["value_from"]},
        **study, "reference_seconds": ref_s,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_time_to_rmse(r, batch, settings, refs, cfg, max_frames, base, tuning, target=0.02):
    """time_to_rmse over a batch: frames of 4 new samples of every item (one
    path_render_batch or path_render_batch_cached call each), accumulated in
    FP64, until the relative RMSE of the whole batch (all items' pixels)
    against refs is <= target."""
    import torch
    from path_gb300 import api, scenes
    outs = [torch.zeros((h, w, 3), dtype=torch.float32, device="cuda") for _, w, h, _ in batch]
    accs = [torch.zeros_like(ref) for ref in refs]
    ref_norm = float(sum(float(torch.sum(ref * ref)) for ref in refs)) ** 0.5
    cache = api.RadianceCache(seed=1) if cfg is not None else None
    wall, frames, err, curve = 0.0, 0, None, []

    def frame(offset):
        items = [(sc, api.SquareImage(w, h, scenes.cornell_camera(w, h), sample_offset=offset),
                  o, 4) for (sc, w, h, _), o in zip(batch, outs)]
        if cache is None:
            r.render_batch(items, settings, tuning)
        else:
            r.render_batch_cached(cache, items, settings, tuning,
                                  cache_depth=cfg["cache_depth"], train_paths=cfg["train_paths"],
                                  train_steps=cfg["train_steps"])

    while frames < max_frames:
        torch.cuda.synchronize()
        t = time.perf_counter()
        frame(base + 4 * frames)
        torch.cuda.synchronize()
        wall += time.perf_counter() - t
        frames += 1
        sq = 0.0
        for acc, o, ref in zip(accs, outs, refs):
            acc += o.double()
            d = acc / frames - ref
            sq += float(torch.sum(d * d))
        err = sq ** 0.5 / ref_norm
        if frames in (1, 2, 4, 8, 16, 32, 64, 128, 256) or err <= target:
            curve.append((frames, round(wall, 4), round(err, 5)))
        if err <= target:
            break
    res = {"frames": frames, "seconds": wall, "rel_rmse": err,
           "reached": err is not None and err <= target, "curve": curve}
    if cfg is not None:
        res["cache"] = (
            "one cache for the batch (a cell per item), hash grid 16x2x2^19, MLP 48-64x5-3 "
            f"BF16 tcgen05, Adam 1e-2, paths end into the cache at vertex {cfg['cache_depth']}, "
            f"{cfg['train_paths']} records (random items) x {cfg['train_steps']} steps per frame")
    return res


def run_batched_cache(args, rank, world, local_rank):
    """Time to 0.02 relative RMSE of the batched render, plain against the
    batched + cache form (path_render_batch_cached): the first
    args.cache_scenes scenes of the batched workload in frames of 4 spp,
    against 4096 spp per item of the plain batch accumulated in FP64."""
    import torch
    from path_gb300 import api, scenes
    batch = scenes.batch_scenes(args.cache_scenes, seed=0)
    settings = scenes.path_settings(6, "wide")
    tuning = {"slots_log2": 24}
    r = api.Renderer()
    t0 = time.time()
    refs = [torch.zeros((h, w, 3), dtype=torch.float64, device="cuda") for _, w, h, _ in batch]
    outs = [torch.zeros((h, w, 3), dtype=torch.float32, device="cuda") for _, w, h, _ in batch]
    n_ref = 64
    for f in range(n_ref):
        items = [(sc, api.SquareImage(w, h, scenes.cornell_camera(w, h), sample_offset=64 + 64 * f),
                  o, 64) for (sc, w, h, _), o in zip(batch, outs)]
        r.render_batch(items, settings, tuning)
        for ref, o in zip(refs, outs):
            ref += o.double()
    refs = [ref / n_ref for ref in refs]
    ref_s = time.time() - t0
    base = 64 + 4096 + 64
    plain = batch_time_to_rmse(r, batch, settings, refs, None, args.max_frames, base, tuning)
    cfg = {"cache_depth": args.cache_depth, "train_paths": args.train_paths,
           "train_steps": args.train_steps}
    cached = batch_time_to_rmse(r, batch, settings, refs, cfg, args.max_frames, base, tuning)
    control = batch_time_to_rmse(r, batch, settings, refs, dict(cfg, train_steps=0),
                                 args.max_frames, base, tuning)
    pixels = sum(w * h for _, w, h, _ in batch)
    line = {
        "metric": "seconds to 0.02 relative RMSE (batch)", "unit": "s",
        "higher_is_better": False,
        "value": cached["seconds"] if cached["reached"] else None, "n_gpus": 1,
        "dtype": "f32 render, bf16 cache MLP", "data": "synthetic",
        "config": {"workload": f"batched + cache: the first {len(batch)} scenes of the batched "
                               f"workload ({pixels} pixels), depth 6, 4-spp frames; reference "
                               "4096 spp per item, FP64 sum",
                   "tuning": tuning},
        "ratio_cached_over_plain": (cached["seconds"] / plain["seconds"]
                                    if plain["reached"] and cached["reached"] else None),
        "target_ratio": 0.25, "plain": plain, "cached": cached, "cached_untrained": control,
        "reference_seconds": ref_s,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_sobol_draws(args, rank):
    """Cost of the integrator's Sobol draws read from the table against the
    same values formed from the direction vectors in registers
    (path_debug_sobol_draws), on the large-mesh workload's draw count: 67.1 M
    paths (1024 x 1024 x 64 spp) of 48 draws (six per vertex over the eight
    vertices of a depth-8 path)."""
    from path_gb300 import api
    n_paths, spp, draws = 1024 * 1024 * 64, 64, 48
    modes = {0: "table (the integrator's)", 1: "direction vectors via L1, XOR in registers",
             2: "direction vectors in shared memory, XOR in registers"}
    res, sums = {}, set()
    for m, name in modes.items():
        ms, cs = api.debug_sobol_draws(m, n_paths, spp, draws)
        res[name] = {"ms": ms, "ns_per_draw": ms * 1e6 / (n_paths * draws)}
        sums.add(cs)
    line = {"metric": "Sobol draw cost", "unit": "ms per 3.2 G draws", "n_gpus": 1,
            "config": {"workload": f"{n_paths} paths x {draws} draws, spp {spp}, 256 dims"},
            "modes": res, "same_values": len(sums) == 1}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_mesh",
                    choices=["large_mesh", "cornell", "batched", "cache", "batched_cache",
                             "sobol_draws"])
    ap.add_argument("--max-frames", type=int, default=400,
                    help="cache workload: frames before giving up on the error target")
    ap.add_argument("--cache-depth", type=int, default=2,
                    help="cache workload: the vertex where paths end into the cache")
    ap.add_argument("--train-paths", type=int, default=1 << 16,
                    help="cache workload: training records per frame")
    ap.add_argument("--train-steps", type=int, default=4,
                    help="cache workload: Adam steps per frame")
    ap.add_argument("--pretrain-frames", type=int, default=0,
                    help="cache workload: training-only frames before the first image")
    ap.add_argument("--no-tuned-cache", action="store_true",
                    help="cache workload: skip the tuned cache configuration")
    ap.add_argument("--scenes", type=int, default=256, help="batched workload: scene count")
    ap.add_argument("--cache-scenes", type=int, default=16,
                    help="batched_cache workload: scene count")
    ap.add_argument("--traversal", default="wide", choices=["wide", "binary"])
    ap.add_argument("--approach", default="streaming", choices=["streaming", "mega"],
                    help="wavefront (streaming) or megakernel integration")
    ap.add_argument("--cpu-rows", type=int, default=128,
                    help="image rows (spread over the image) in the CPU baseline sample: "
                         "about 7 s on 16 cores")
    ap.add_argument("--fp64-oracle-rows", type=int, default=8,
                    help="rows (spread) of the oracle's 4096-spp FP64 reference: about 25 s "
                         "on 16 cores")
    ap.add_argument("--no-extra-metrics", action="store_true",
                    help="skip the time-to-0.02-RMSE and adjoint/forward legs")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-megakernel", action="store_true",
                    help="skip the megakernel comparison render")
    ap.add_argument("--no-reference-error", action="store_true",
                    help="skip the 4096-spp FP64 reference render and the error against it")
    ap.add_argument("--size", type=int, default=None,
                    help="image width = height (profiling cases; default: the workload's)")
    ap.add_argument("--spp", type=int, default=None, help="samples per pixel override")
    ap.add_argument("--slots-log2", type=int, default=0,
                    help="streaming: paths in flight = 2^this (0 = default 26)")
    ap.add_argument("--gpu-build", type=int, nargs="?", const=1, default=0,
                    help="build the 8-wide BVH on the GPU instead of the SBVH: 1 PLOC, "
                         "2 PLOC over split triangle references")
    ap.add_argument("--trace-min-blocks", type=int, default=0,
                    help="streaming trace kernel variant (resident blocks per SM, 3..6)")
    ap.add_argument("--staged-nodes", type=int, default=None,
                    help="streaming trace: top BVH nodes staged in shared memory per CTA "
                         "(default: the library's)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)

    from path_gb300 import api, build, scenes
    build.build()
    if args.workload == "batched":
        run_batched(args, rank, world, local_rank)
        return
    if args.workload == "cache":
        run_cache(args, rank, world, local_rank)
        return
    if args.workload == "batched_cache":
        run_batched_cache(args, rank, world, local_rank)
        return
    if args.workload == "sobol_draws":
        run_sobol_draws(args, rank)
        return
    scene, w, h, spp, depth, desc = make_workload(args.workload, args.size, args.spp)
    settings = scenes.path_settings(depth, args.traversal)
    settings.kernel_approach = 1 if args.approach == "streaming" else 0
    settings.trace_min_blocks = args.trace_min_blocks
    settings.gpu_build = args.gpu_build
    settings.wavefront_slots_log2 = args.slots_log2
    if args.staged_nodes is not None:
        settings.trace_staged_nodes = args.staged_nodes
    f2w = scenes.cornell_camera(w, h)
    spec = api.SquareImage(w, h, f2w)
    r = api.Renderer()
    dev_out = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    t0 = time.time()
    r.render(api.ExecutionModel.GPU, spec, dev_out, scene, spp, settings)
    setup_s = time.time() - t0
    st0 = r.stats()

    # counting run: rays, wide nodes and triangles of one render
    cs = settings.copy()
    cs.count_work = 1
    r.render(api.ExecutionModel.GPU, spec, dev_out, scene, spp, cs)
    counts = r.stats()

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    streaming = args.approach == "streaming"
    settings.time_kernels = 1 if streaming else 0
    for _ in range(args.warmup):
        r.render(api.ExecutionModel.GPU, spec, dev_out, scene, spp, settings)
    kernel_ms, trace_ms, trace_launches, launches = [], [], 0, 0
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            r.render(api.ExecutionModel.GPU, spec, dev_out, scene, spp, settings)
            st = r.stats()
            kernel_ms.append(st["kernel_ms"])
            trace_ms.append(st["trace_ms"])
            trace_launches += st["trace_launches"]
            launches += st["gpu_launches"]
        torch.cuda.synchronize()
        # end to end through the C ABI with host buffers
        host_out = np.zeros((h, w, 3), np.float32)
        es = settings.copy()
        es.upload_scene_every_render = 1
        es.time_kernels = 0
        for _ in range(2):
            r.render(api.ExecutionModel.GPU, spec, host_out, scene, spp, es)
        e2e_s, h2d, d2h = [], 0, 0
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t = time.perf_counter()
            r.render(api.ExecutionModel.GPU, spec, host_out, scene, spp, es)
            e2e_s.append(time.perf_counter() - t)
            st = r.stats()
            h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
            launches += st["gpu_launches"]
    torch.cuda.synchronize()
    total_ms = sum(kernel_ms)
    if world > 1:
        t = torch.tensor([total_ms, sum(e2e_s)], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, e2e_total = float(t[0]), float(t[1])
    else:
        e2e_total = sum(e2e_s)
    samples = w * h * spp
    value = world * samples * args.steps / (total_ms / 1e3) / 1e6
    e2e_value = world * samples * args.steps / e2e_total / 1e6

    peak, peak_kind = _peaks()
    mean_ms = total_ms / args.steps
    timed_img = dev_out.cpu().numpy()
    if streaming:
        # dominant kernel: the persistent trace.  Per ray it reads its origin
        # and direction (32 B) and writes its hit (8 B); per visit 80 B of
        # wide node, per test 48 B of triangle.
        alg_bytes = counts["nodes_visited"] * 80 + counts["triangles_tested"] * 48 + \
            counts["rays_traced"] * 40
        launches_per_render = trace_launches / args.steps
        kern_ms = sum(trace_ms) / args.steps
        kernel_name = "k_wf_trace"
    else:
        # the megakernel does everything: traversal plus 96 B of shading data
        # (triangle normals + material) per traced ray
        alg_bytes = counts["nodes_visited"] * 80 + counts["triangles_tested"] * 48 + \
            counts["rays_traced"] * 96
        launches_per_render = 1
        kern_ms = mean_ms
        kernel_name = "k_render"
    clock_summary = clocks.summary()
    launch_s = kern_ms / launches_per_render / 1e3
    achieved = alg_bytes / (kern_ms / 1e3) / 1e9
    shape = (f"slots_log2={args.slots_log2 or 26} trace_min_blocks={args.trace_min_blocks or 4} "
             f"bvh={'gpu' + str(args.gpu_build) if args.gpu_build else 'sbvh'} "
             f"staged_nodes={settings.trace_staged_nodes}")
    full_size = args.size is None and args.spp is None
    traffic = (_profiled_traffic(kernel_name, args, shape, alg_bytes / launches_per_render)
               if full_size else None)
    issue = _profiled_issue(kernel_name, args, shape) if full_size and streaming else None
    # the other side of the roofline: FP32 work (22 operations per box test,
    # 8 box tests per wide node, 45 per Moller-Trumbore test) against the
    # FP32 lanes' issue rate, and -- from the ncu summary -- the warp
    # instructions the kernel actually issues against the schedulers' rate
    n_sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
    clk_hz = (clock_summary.get("sm_mhz") or 2070.0) * 1e6
    nodes_per_launch = counts["nodes_visited"] / launches_per_render
    fp32_ops = (22 * 8 * counts["nodes_visited"] + 45 * counts["triangles_tested"]) / \
        launches_per_render
    fp32_peak = n_sms * 128 * clk_hz / 1e12
    sides = {
        "hbm": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind, "bytes": "algorithmic (node, triangle and ray bytes "
                                                 "the traversal reads and writes)",
                "dram_frac": (traffic / launch_s / 1e9 / peak) if traffic else None},
        "fp32": {"achieved": fp32_ops / launch_s / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                 "frac": fp32_ops / launch_s / 1e12 / fp32_peak,
                 "peak_kind": f"{n_sms} SMs x 128 FP32 lanes x sampled SM clock",
                 "ops_per_launch": fp32_ops},
    }
    if issue is not None:
        winst = issue["warp_inst_per_node_visit"] * nodes_per_launch
        issue_peak = n_sms * 4 * clk_hz / 1e9
        sides["issue"] = {
            "achieved": winst / launch_s / 1e9, "peak": issue_peak, "unit": "Ginst/s",
            "frac": winst / launch_s / 1e9 / issue_peak,
            "peak_kind": f"{n_sms} SMs x 4 schedulers x 1 warp instruction per clock",
            "warp_inst_per_node_visit": issue["warp_inst_per_node_visit"],
            "thread_inst_per_node_visit": issue["thread_inst_per_node_visit"],
            "lanes_active": issue["thread_inst_per_node_visit"] /
            issue["warp_inst_per_node_visit"]}
    bound = max(("hbm", "issue"), key=lambda k: sides[k]["frac"] if k in sides else -1)
    b = sides[bound]
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": desc, "triangles": int(scene.sizes()["triangles"]),
            "width": w, "height": h, "spp": spp,
            "max_depth": depth, "traversal": args.traversal, "approach": args.approach,
            "trace_min_blocks": args.trace_min_blocks or 4,
            "slots_log2": args.slots_log2 or 26,
            "staged_nodes": int(settings.trace_staged_nodes),
            "bvh": ("GPU PLOC BVH" + (" over split references" if args.gpu_build == 2 else "") +
                    " collapsed to 8-wide") if args.gpu_build else
                   "SBVH (host) collapsed to 8-wide",
            "l2": "flushed (512 MB write) before every timed step",
            "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": {"bound": bound, "achieved": b["achieved"], "peak": b["peak"],
                     "unit": b["unit"], "frac": b["frac"], "traffic": traffic,
                     "peak_kind": b["peak_kind"], "kernel": kernel_name,
                     "launches_per_step": launches_per_render,
                     "kernel_ms_per_step": kern_ms,
                     "algorithmic_bytes_per_launch": alg_bytes / launches_per_render,
                     "sides": sides},
        "mrays_per_s": counts["rays_traced"] / (mean_ms / 1e3) / 1e6,
        "work_counts": {"rays": counts["rays_traced"], "wide_nodes": counts["nodes_visited"],
                        "triangles": counts["triangles_tested"]},
        "setup_s": setup_s, "bvh_build_s": st0["bvh_build_seconds"],
        "clocks": clock_summary,
    }
    rs = settings.copy()
    rs.time_kernels = 0
    ref = None
    if not args.no_reference_error and rank == 0:
        # the timed image's error against 4096 samples per pixel (samples
        # spp .. spp + 4095) accumulated in FP64 by the GPU
        ref = gpu_reference(r, scene, w, h, f2w, rs, spp)
        err = float(np.linalg.norm(timed_img - ref.cpu().numpy()) /
                    float(torch.linalg.norm(ref)))
        line["error_vs_4096spp_fp64"] = {
            "rel_rmse": err, "reference": "4096 spp (samples spp..spp+4095), FP64 sum, GPU",
            "image": f"the timed {spp}-spp render"}
    if streaming and full_size and not args.no_megakernel:
        # the same render through the megakernel (identical image), for the
        # wavefront-versus-megakernel comparison of this workload
        ms = settings.copy()
        ms.kernel_approach = 0
        ms.time_kernels = 0
        r.render(api.ExecutionModel.GPU, spec, dev_out, scene, spp, ms)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        r.render(api.ExecutionModel.GPU, spec, dev_out, scene, spp, ms)
        mk = r.stats()["kernel_ms"]
        line["megakernel"] = {"value": samples / (mk / 1e3) / 1e6, "unit": METRIC,
                              "ms_per_step": mk, "steps": 1,
                              "same_image": bool(np.array_equal(dev_out.cpu().numpy(),
                                                                timed_img))}
    if rank == 0 and world == 1 and ref is not None and full_size and \
            args.workload == "large_mesh" and not args.no_extra_metrics:
        # the other two parts of the metric
        cs = scenes.path_settings(8, "wide")
        cs.kernel_approach = 1
        line["time_to_0.02_rmse"] = cache_study(
            r, scene, w, h, f2w, cs, ref, args,
            "4096 spp (samples 64..4159), FP64 sum, GPU; frames from sample 4224")
        line["adjoint_forward_ratio"] = adjoint_study()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle_lib as ol
        threads = os.cpu_count() or 1
        t0 = time.time()
        # summed in the GPU path's shuffle-tree order, so that the band is
        # comparable with the timed image bit for bit
        prep, os_ = oracle_prepare(ol.SceneArrays(scene.export()), settings, 1, threads)
        prep_s = time.time() - t0
        band, sel, n, secs = cpu_sample(prep, os_, spp, w, h, f2w, args.cpu_rows)
        line["cpu_baseline"] = {
            "value": n / secs / 1e6, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{len(sel)} rows spread over the image (1 in {h // len(sel)}) x {w} px "
                      f"x {spp} spp (oracle: CPU restatement of the reference CPU path, "
                      f"{threads} threads; SBVH build {prep_s:.1f} s not timed)"}
        a, o = timed_img[sel].astype(np.float64), band[sel].astype(np.float64)
        line["parity_vs_oracle"] = {
            "rel_rmse": float(np.linalg.norm(a - o) / np.linalg.norm(o)),
            "bit_exact_pixels": float(np.mean(np.all(timed_img[sel] == band[sel], axis=-1))),
            "rows": f"{len(sel)} rows (1 in {h // len(sel)} from row {sel[0]}) of the timed image",
            "tolerance": 1e-4,
            "oracle": "CPU restatement of the reference CPU path, binary SBVH traversal with "
                      "the reference's tie rule"}
        if ref is not None and args.fp64_oracle_rows > 0:
            # 4096 samples per pixel summed in FP64 by the oracle, on spread rows
            start, stride, fsel = spread_rows(h, args.fp64_oracle_rows)
            f64, fsecs = prep.render_f64(os_, 4096, w, h, f2w, rows=(start, h), stride=stride,
                                         sample_offset=spp)
            g = ref.cpu().numpy()
            o64 = f64[fsel]
            line["error_vs_4096spp_fp64"]["oracle"] = {
                "rel_rmse": float(np.linalg.norm(timed_img[fsel] - o64) / np.linalg.norm(o64)),
                "gpu_reference_vs_oracle_reference": float(np.linalg.norm(g[fsel] - o64) /
                                                           np.linalg.norm(o64)),
                "gpu_reference_same_rows": float(np.linalg.norm(timed_img[fsel] - g[fsel]) /
                                                 np.linalg.norm(g[fsel])),
                "rows": f"{len(fsel)} rows (1 in {stride} from row {start})",
                "reference": "4096 spp (samples spp..spp+4095), every sample summed in FP64 "
                             "by the CPU oracle",
                "oracle_seconds": fsecs}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
