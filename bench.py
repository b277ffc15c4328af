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
* roofline: algorithmic bytes of the render kernel (wide nodes x 80 B +
  triangles tested x 48 B + rays x 96 B of shading data, counted by a
  counting run of the same render) over the kernel's event time, against the
  measured HBM copy bandwidth.
* cpu_baseline: the CPU oracle (a restatement of the reference's CPU path:
  OpenMP over WorkDivision blocks) on a band of image rows of the same
  workload, all host threads.

``--impl reference`` times that CPU restatement alone (the reference itself
cannot be built here: it needs clang as its CUDA compiler and libraries that
are not installed).  N > 1 runs independent
replicas, one per GPU (the render has no data-path exchange).
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


def _profiled_traffic(kernel, args, shape):
    """DRAM bytes per launch of the dominant kernel, from the committed ncu
    summary of this workload (a line 'dram_bytes_per_launch: N' in
    profiles/<kernel>_dram_<workload>.txt), or None when the summary is
    missing or was taken at another launch shape (its 'launch_shape:'
    line)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_dram_{args.workload}.txt")
    traffic, profiled_shape = None, None
    try:
        with open(path) as f:
            for ln in f:
                if ln.startswith("dram_bytes_per_launch:"):
                    traffic = float(ln.split(":", 1)[1])
                elif ln.startswith("launch_shape:"):
                    profiled_shape = ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return traffic if profiled_shape == shape else None


def make_workload(name, size=None, spp_override=None):
    from path_gb300 import scenes
    if name == "large_mesh":
        scene = scenes.large_mesh_room(subdivisions=8)
        w = h = size or 1024
        spp, depth = spp_override or 64, 8
        desc = ("large-mesh room: 1,310,720-tri displaced icosphere (GGX a=0.2 F0=0.04) + "
                f"19,800-tri glass sphere (IOR 1.5), {w}x{h}, {spp} spp, depth 8")
    else:
        scene = scenes.cornell_box()
        w = h = size or 256
        spp, depth = spp_override or 16, 5
        desc = f"Cornell box: 36 triangles, {w}x{h}, {spp} spp, depth 5"
    return scene, w, h, spp, depth, desc


def cpu_sample(scene, settings, spp, w, h, f2w, rows, threads):
    """The oracle on a band of rows; returns (samples, seconds)."""
    from oracle import oracle_lib as ol
    arr = ol.SceneArrays(scene.export())
    s = ol.settings_from(settings, reduce_order=0, n_threads=threads)
    r0 = h // 2 - rows // 2
    _, secs = ol.render(arr, s, spp, w, h, f2w, rows=(r0, r0 + rows))
    return rows * w * spp, secs


def run_reference(args, rank):
    if rank != 0:
        return
    from path_gb300 import scenes
    scene, w, h, spp, depth, desc = make_workload(args.workload, args.size, args.spp)
    settings = scenes.path_settings(depth, "binary")
    f2w = scenes.cornell_camera(w, h)
    threads = os.cpu_count() or 1
    rows = args.cpu_rows
    for _ in range(args.warmup):
        cpu_sample(scene, settings, spp, w, h, f2w, rows, threads)
    total_s, total_samples = 0.0, 0
    for _ in range(args.steps):
        n, secs = cpu_sample(scene, settings, spp, w, h, f2w, rows, threads)
        total_s += secs
        total_samples += n
    value = total_samples / total_s / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": desc, "sample": f"{rows} rows x {w} px x {spp} spp per step"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{rows} rows of {w} px at {spp} spp per step (oracle: CPU "
                                   "restatement of the reference CPU path)"},
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
    settings.gpu_build = 1 if args.gpu_build else 0
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
                   "bvh": "GPU linear BVH" if args.gpu_build else "SBVH (host)",
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


def run_cache(args, rank, world, local_rank):
    """Time to 0.02 relative RMSE, plain tracer against the radiance cache,
    on the large-mesh room at 1024 x 1024 in frames of 4 spp (depth 8).
    Reference: 4096 spp of the plain tracer accumulated in FP64 (64 frames
    of 64 spp).  Plain: frames of 4 new samples each, accumulated in FP64
    until the error is <= 0.02.  Cache: frames whose paths end into the
    cache after 2 bounces, each followed by 4 Adam steps on 2^16 records
    from fresh full-length paths, accumulated the same way (the first
    frames, with an untrained cache, included).  Then a tuned cache (paths
    end at vertex 3, 2^14 records x 2 steps per frame) and, as its control,
    the same truncation with the cache left untrained (what ending the paths
    early does without the network).  Wall time of render +
    training calls."""
    import torch
    from path_gb300 import api, scenes
    size = args.size or 1024
    scene, w, h, _, depth, desc = make_workload("large_mesh", size, 4)
    settings = scenes.path_settings(8, "wide")
    settings.kernel_approach = 1
    f2w = scenes.cornell_camera(w, h)
    r = api.Renderer()
    out = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    t0 = time.time()
    ref = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
    ref_frames = 64
    for f in range(ref_frames):
        r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w, sample_offset=64 * f), out,
                 scene, 64, settings)
        ref += out.double()
    ref /= ref_frames
    ref_s = time.time() - t0
    ref_norm = float(torch.linalg.norm(ref))

    def run(cached, cfg=None, target=0.02):
        cache = api.RadianceCache(seed=1) if cached else None
        acc = torch.zeros_like(ref)
        wall, frames, err = 0.0, 0, None
        curve = []
        base = 64 * ref_frames  # samples the reference did not use
        if cached and cfg["pretrain_frames"] > 0:
            # training-only frames (their images are not kept; time counted)
            torch.cuda.synchronize()
            t = time.perf_counter()
            for f in range(cfg["pretrain_frames"]):
                spec = api.SquareImage(w, h, f2w, sample_offset=base + 4 * (args.max_frames + f))
                r.render_cached(cache, spec, out, scene, 4, settings,
                                cache_depth=cfg["cache_depth"], train_paths=cfg["train_paths"],
                                train_steps=cfg["train_steps"])
            torch.cuda.synchronize()
            wall += time.perf_counter() - t
        while frames < args.max_frames:
            spec = api.SquareImage(w, h, f2w, sample_offset=base + 4 * frames)
            torch.cuda.synchronize()
            t = time.perf_counter()
            if cached:
                r.render_cached(cache, spec, out, scene, 4, settings,
                                cache_depth=cfg["cache_depth"], train_paths=cfg["train_paths"],
                                train_steps=cfg["train_steps"])
            else:
                r.render(api.ExecutionModel.GPU, spec, out, scene, 4, settings)
            torch.cuda.synchronize()
            wall += time.perf_counter() - t
            frames += 1
            acc += out.double()
            err = float(torch.linalg.norm(acc / frames - ref)) / ref_norm
            if frames in (1, 2, 4, 8, 16, 32, 64, 128, 256) or err <= target:
                curve.append((frames, round(wall, 4), round(err, 5)))
            if err <= target:
                break
        out_d = {"frames": frames, "seconds": wall, "rel_rmse": err,
                 "reached": err is not None and err <= target, "curve": curve}
        if cfg is not None:
            out_d["cache"] = (
                "hash grid 16x2x2^19, MLP 48-64x5-3 BF16 tcgen05, Adam 1e-2, "
                f"paths end into the cache at vertex {cfg['cache_depth']}, "
                f"{cfg['train_paths']} records x {cfg['train_steps']} steps per frame, "
                f"{cfg['pretrain_frames']} training-only frames first")
        return out_d

    plain = run(False)
    # the configuration on the command line (defaults: the specified one),
    # then a tuned one (picked by a search on this scene over the depth, the
    # records and the steps per frame) and its untrained control
    spec_cfg = {"cache_depth": args.cache_depth, "train_paths": args.train_paths,
                "train_steps": args.train_steps, "pretrain_frames": args.pretrain_frames}
    runs = {"cached": run(True, spec_cfg)}
    controls = {}
    if not args.no_tuned_cache:
        tuned = {"cache_depth": 3, "train_paths": 1 << 14, "train_steps": 2,
                 "pretrain_frames": 0}
        runs["cached_tuned"] = run(True, tuned)
        controls["cached_tuned_untrained"] = run(True, dict(tuned, train_steps=0))
    reached = [k for k in runs if runs[k]["reached"]]
    best = min(reached, key=lambda k: runs[k]["seconds"]) if reached else None
    line = {
        "metric": "seconds to 0.02 relative RMSE", "unit": "s", "higher_is_better": False,
        "value": runs[best]["seconds"] if best else None,
        "n_gpus": 1, "dtype": "f32 render, bf16 cache MLP", "data": "synthetic",
        "config": {"workload": f"{desc} in 4-spp frames; reference 4096 spp FP64",
                   "value_from": best,
                   "cache": runs[best]["cache"] if best else runs["cached"]["cache"]},
        "plain": plain, **runs, **controls,
        "ratio_cached_over_plain": (runs[best]["seconds"] / plain["seconds"]
                                    if plain["reached"] and best else None),
        "reference_seconds": ref_s,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_mesh",
                    choices=["large_mesh", "cornell", "batched", "cache"])
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
    ap.add_argument("--traversal", default="wide", choices=["wide", "binary"])
    ap.add_argument("--approach", default="streaming", choices=["streaming", "mega"],
                    help="wavefront (streaming) or megakernel integration")
    ap.add_argument("--cpu-rows", type=int, default=128,
                    help="image rows (centred) in the CPU baseline sample: about 7 s on 16 cores")
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
    ap.add_argument("--gpu-build", action="store_true",
                    help="build the 8-wide BVH on the GPU (linear BVH) instead of the SBVH")
    ap.add_argument("--trace-min-blocks", type=int, default=0,
                    help="streaming trace kernel variant (resident blocks per SM, 3..6)")
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
    scene, w, h, spp, depth, desc = make_workload(args.workload, args.size, args.spp)
    settings = scenes.path_settings(depth, args.traversal)
    settings.kernel_approach = 1 if args.approach == "streaming" else 0
    settings.trace_min_blocks = args.trace_min_blocks
    settings.gpu_build = 1 if args.gpu_build else 0
    settings.wavefront_slots_log2 = args.slots_log2
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
    achieved = alg_bytes / (kern_ms / 1e3) / 1e9
    shape = (f"slots_log2={args.slots_log2 or 26} trace_min_blocks={args.trace_min_blocks or 4} "
             f"bvh={'gpu' if args.gpu_build else 'sbvh'}")
    traffic = _profiled_traffic(kernel_name, args, shape) if args.size is None and \
        args.spp is None else None
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
            "bvh": "GPU linear BVH collapsed to 8-wide" if args.gpu_build else
                   "SBVH (host) collapsed to 8-wide",
            "l2": "flushed (512 MB write) before every timed step",
            "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind, "kernel": kernel_name,
                     "launches_per_step": launches_per_render,
                     "kernel_ms_per_step": kern_ms,
                     "algorithmic_bytes_per_launch": alg_bytes / launches_per_render},
        "mrays_per_s": counts["rays_traced"] / (mean_ms / 1e3) / 1e6,
        "work_counts": {"rays": counts["rays_traced"], "wide_nodes": counts["nodes_visited"],
                        "triangles": counts["triangles_tested"]},
        "setup_s": setup_s, "bvh_build_s": st0["bvh_build_seconds"],
        "clocks": clocks.summary(),
    }
    if not args.no_reference_error and rank == 0:
        # the timed image's error against a 4096-spp render of the same
        # scene accumulated in FP64 (64 renders of 64 new samples each)
        ref = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
        rs = settings.copy()
        rs.time_kernels = 0
        n_ref = max(1, 4096 // 64)
        for f in range(n_ref):
            r.render(api.ExecutionModel.GPU,
                     api.SquareImage(w, h, f2w, sample_offset=spp + 64 * f), dev_out, scene,
                     64, rs)
            ref += dev_out.double()
        ref /= n_ref
        r.render(api.ExecutionModel.GPU, spec, dev_out, scene, spp, rs)
        err = float(torch.linalg.norm(dev_out.double() - ref) / torch.linalg.norm(ref))
        line["error_vs_4096spp_fp64"] = {
            "rel_rmse": err, "reference": "4096 spp (samples spp..spp+4095), FP64 sum",
            "image": f"the timed {spp}-spp render"}
    if streaming and args.size is None and args.spp is None and not args.no_megakernel:
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
                              "ms_per_step": mk, "steps": 1}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n, secs = cpu_sample(scene, settings, spp, w, h, f2w, args.cpu_rows, threads)
        line["cpu_baseline"] = {
            "value": n / secs / 1e6, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{args.cpu_rows} rows of {w} px at {spp} spp (oracle: CPU restatement "
                      f"of the reference CPU path, {threads} threads)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
