"""Benchmark: Mrays/s of the GB300 path tracer on the large-mesh workload.

Workload (one "step" = one full frame): the 327,692-triangle scene (icosphere
subdivided 7 times, radius 1.5, 5-octave value-noise displacement, amplitude
0.08, base frequency 4, inside the open-front box room), 1920x1080, 16 pixel
samples, max depth 3, 1 Monte Carlo sample per bounce, one point light.
Synthetic, seeded geometry; the tree is the reference's SAH kd-tree (built on
the host, identical node words).

Metric: Mrays/s with the reference's ray count (pathtracer.cpp:21: traced rays
at depth <= max depth, misses included, shadow rays excluded).

  value   frame time on the device (CUDA events on the library's stream) with
          the scene resident in HBM, output image in device memory
  e2e     the same through the public C ABI with host buffers: the scene is
          uploaded from host memory, rendered and the image read back, every
          step (turner_upload_scene + turner_render + turner_free_scene)

`--impl reference` times the reference's CPU path tracer (the oracle
restatement of pathtracer.cpp / kdtree.cpp, all host threads) on interleaved
row sets of the same frame, one set per step, without loading the GPU library.

Multi-GPU (torchrun, one rank per GPU): the frame is partitioned by rows
(turner_job.row_begin/row_end), every rank holding the whole scene; no
collective on the data path; value = all ranks' rays / max over ranks of the
time (strong scaling: the frame is fixed).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WIDTH, HEIGHT, SPP, DEPTH, MC = 1920, 1080, 16, 3, 1
WORKLOAD = "sphere_room_327k_1920x1080_16spp_d3"
METRIC = "Mrays/s (reference ray count: primary + bounce rays incl. misses, excl. shadow rays)"
PEAKS = ROOT / "MEASURED_PEAKS.json"
TRAFFIC = ROOT / "profiles" / "k_trace_traffic.json"
# training objectives of the learned proposal (turner_guide_set_objective)
OBJECTIVES = {"kl": 0, "variance": 1}


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def sample_clocks(stop: threading.Event, out: list, device: int):
    q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    try:
        p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                              "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except OSError:
        return
    try:
        while not stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            out.append(line.strip())
    finally:
        p.terminate()
        try:
            p.wait(timeout=2)
        except subprocess.TimeoutExpired:
            p.kill()


def summarize_clocks(lines: list[str]) -> dict:
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        parts = [x.strip() for x in ln.split(",")]
        if len(parts) < 7:
            continue
        try:
            sm.append(float(parts[0]))
            mx.append(float(parts[1]))
        except ValueError:
            continue
        for name, val in zip(names, parts[3:7]):
            if val.lower() == "active":
                reasons.add(name)
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


class Clocks:
    """nvidia-smi clock samples while the `with` body runs; .summary after."""

    def __init__(self, device: int = 0):
        self.device = device
        self.lines: list[str] = []
        self.summary: dict | None = None

    def __enter__(self):
        self.stop = threading.Event()
        self.thread = threading.Thread(target=sample_clocks, args=(self.stop, self.lines, self.device), daemon=True)
        self.thread.start()
        return self

    def __exit__(self, *exc):
        self.stop.set()
        self.thread.join(timeout=5)
        self.summary = summarize_clocks(self.lines)
        return False


def make_workload():
    import turner_gb300 as tg

    mesh = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=7, aspect=16 / 9)
    t0 = time.perf_counter()
    tree = tg.KDTree.from_mesh(mesh)
    build_s = time.perf_counter() - t0
    return mesh, tree, build_s


def row_sets(threads: int, height: int = None) -> tuple[int, list[int]]:
    """Interleaved row sets of the frame: set k holds rows k, k + stride, ...
    with stride = height // (4 x threads), so a set has about 4 rows per
    thread (threads take one row at a time, as the reference's pool takes one
    task per row, main.cpp:193-226, and every core stays busy). The order is
    van der Corput's, so that any prefix of the sets is spread over the frame;
    all sets together are the whole frame."""
    h = height or HEIGHT
    stride = max(1, h // (4 * max(1, threads)))
    bits = max(1, (stride - 1).bit_length())
    order = sorted(range(stride), key=lambda k: int(format(k, f"0{bits}b")[::-1], 2))
    return stride, order


def cpu_baseline(mesh, tree, seed: int, budget_s: float = 12.0):
    """Oracle render of interleaved row sets of the same frame (spread over
    the whole frame), all host threads, until about budget_s of wall time.
    Returns (Mrays/s, rows, stats, threads, seconds); stats also count the
    reference traversal's node visits and triangle tests of those rays."""
    from oracle import oracle as orc

    nodes, tris, box = tree.export()
    sc = orc.Scene(nodes, tris, box)
    threads = os.cpu_count() or 1
    stride, order = row_sets(threads)
    stats = np.zeros(7, np.uint64)
    rows = 0
    t0 = time.perf_counter()
    for k in order:
        if time.perf_counter() - t0 >= budget_s:
            break
        _, st = sc.render(mesh.camera, mesh.light, WIDTH, HEIGHT, SPP, DEPTH, mc=MC, seed=seed, threads=threads,
                          rows=(k, HEIGHT), row_step=stride)
        stats += st
        rows += len(range(k, HEIGHT, stride))
    dt = time.perf_counter() - t0
    return float(stats[0]) / dt / 1e6, rows, stats, threads, dt, stride


def headline_mse(ctx, sid, mesh, seed: int, traversal: int, rows: int = 8, ref_spp: int = 16384) -> dict:
    """MSE of the headline frame against a converged render: `rows` rows
    through the middle of the frame rendered with the frame's own seed and
    sample count (bit-identical to those rows of the timed frame before tone
    mapping), against the same rows accumulated in FP64 over ref_spp samples
    (independent streams); linear RGB radiance."""
    import turner_gb300 as tg

    r0 = HEIGHT // 2 - rows // 2
    band = (r0, r0 + rows)
    t0 = time.perf_counter()
    rj = tg.make_job(sid, mesh, WIDTH, HEIGHT, pixel_samples=256, max_depth=DEPTH, monte_carlo_samples=MC,
                     seed=0xC0FFEE, traversal=tg.TRAVERSAL_PARITY, rows=band)
    rj.linear_output = 1
    ref, n = ctx.accumulate(rj, ref_spp // 256)
    ref_s = time.perf_counter() - t0
    fj = tg.make_job(sid, mesh, WIDTH, HEIGHT, pixel_samples=SPP, max_depth=DEPTH, monte_carlo_samples=MC,
                     seed=seed, traversal=traversal, rows=band)
    fj.linear_output = 1
    (img,), _ = ctx.render([fj])
    err = float(((img[..., :3].astype(np.float64) - ref[..., :3]) ** 2).mean())
    return {"value": err, "space": "linear RGB radiance", "rows": f"{band[0]}-{band[1]}",
            "frame_spp": SPP, "reference_spp": int(n), "reference_accumulation": "FP64",
            "reference_s": round(ref_s, 2)}


def run_reference(args) -> None:
    """The reference's CPU path tracer (the oracle restatement of
    pathtracer.cpp / kdtree.cpp, all host threads) on the same frame: each
    step renders one interleaved row set (about 4 rows per thread, spread
    over the whole frame); successive steps take successive sets. Its input
    (the synthetic scene and the reference's tree) comes from
    oracle/libinputs.so: this arm loads no GPU library."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    from oracle import oracle as orc

    inp = orc.SceneInputs(1, detail=7, aspect=16 / 9)   # the sphere room
    sc = orc.Scene(inp.nodes, inp.tris, inp.box)
    threads = os.cpu_count() or 1
    stride, order = row_sets(threads)

    def step(i):
        k = order[i % len(order)]
        _, st = sc.render(inp.camera, inp.light, WIDTH, HEIGHT, SPP, DEPTH, mc=MC, seed=1, threads=threads,
                          rows=(k, HEIGHT), row_step=stride)
        return int(st[0]), len(range(k, HEIGHT, stride))

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    rays = rows = 0
    for i in range(args.warmup, args.warmup + args.steps):
        r, n = step(i)
        rays += r
        rows += n
    dt = time.perf_counter() - t0
    value = rays / dt / 1e6
    sample = (f"{rows} rows of the {WIDTH}x{HEIGHT} frame in {args.steps} interleaved sets (row step "
              f"{stride}, {rows * WIDTH * SPP} paths), one set per step")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": sample, "threads": threads,
                   "triangles": inp.n_triangles, "nodes": int(inp.nodes.size)},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_batch64(args) -> None:
    """The batched workload: 64 independent scenes in one launch sequence.

    Each scene is a seeded clustered triangle soup in the room, triangle count
    log-uniform in [1k, max], image side uniform in [128, 1024], pixel samples
    from {1, 4, 16, 64}, max depth 1-5, its own streams. Reports Mrays/s over
    the whole batch (one CUDA graph launch per step); not the headline line."""
    import torch

    import turner_gb300 as tg

    rng = np.random.default_rng(2026)
    n = args.batch_scenes
    counts = np.exp(rng.uniform(np.log(1000), np.log(args.batch_max_tris), n)).astype(int)
    sides = rng.integers(128, 1025, n)
    spps = rng.choice([1, 4, 16, 64], n)
    depths = rng.integers(1, 6, n)
    ctx = tg.Context(0)
    t0 = time.perf_counter()
    jobs, tris, scenes = [], 0, []
    for k in range(n):
        m = tg.make_scene(tg.SCENE_SOUP, count=int(counts[k]), seed=1000 + k)
        tree = tg.KDTree.build_gpu(ctx, m) if args.gpu_build else tg.KDTree.from_mesh(m)
        sid = ctx.upload_tree(tree)
        tris += m.n_triangles
        scenes.append((m, tree))
        jobs.append(tg.make_job(sid, m, int(sides[k]), int(sides[k]), pixel_samples=int(spps[k]),
                                max_depth=int(depths[k]), seed=77 + k))
    build_s = time.perf_counter() - t0
    tuning = ctx.autotune(jobs, force=True).as_dict() if args.autotune else ctx.get_tuning().as_dict()
    outs = [torch.empty((j.height, j.width, 4), dtype=torch.float32, device="cuda") for j in jobs]
    ptrs = [o.data_ptr() for o in outs]
    for _ in range(args.warmup):
        ctx.render(jobs, ptrs, tg.DEVICE_BUFFERS)
    torch.cuda.synchronize()
    g0, l0 = ctx.graph_launch_count(), ctx.launch_count()
    dev_ms, rays = 0.0, 0
    with Clocks(0) as clk:
        for _ in range(args.steps):
            _, stats = ctx.render(jobs, ptrs, tg.DEVICE_BUFFERS)
            dev_ms += stats[0].device_ms
            rays += sum(s.rays for s in stats)
        torch.cuda.synchronize()
    print(json.dumps({
        "metric": "Mrays/s, 64-scene batch (reference ray count)", "value": round(rays / (dev_ms / 1000) / 1e6, 3),
        "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dev_ms / args.steps, 3), "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batch of {n} soups", "triangles_total": int(tris),
                   "paths_per_step": int(sum(j.width * j.height * j.pixel_samples for j in jobs)),
                   "rays_per_step": int(rays // args.steps),
                   "tree_build": "GPU (turner_kdtree_build_gpu)" if args.gpu_build else "host (reference node words)",
                   "setup_s": round(build_s, 2),   # scene generation + tree builds + uploads
                   "graph_launches_per_step": (ctx.graph_launch_count() - g0) / args.steps,
                   "kernel_launches_per_step": (ctx.launch_count() - l0) / args.steps, "tuning": tuning},
        "mse_vs_fp64": batch_mse(ctx, jobs[:4]) if not args.no_mse else None,
        "cpu_baseline": None if args.no_cpu else batch_cpu_baseline(scenes, jobs, args.cpu_budget),
        "clocks": clk.summary,
    }))
    ctx.close()


def batch_cpu_baseline(scenes, jobs, budget_s: float) -> dict:
    """The oracle restatement of the reference on the batch's scenes in
    order, one interleaved row set (about 4 rows per host thread, spread
    over the image) per scene, until about budget_s of wall time."""
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    rays, done, t_total = 0, 0, 0.0
    for (m, tree), j in zip(scenes, jobs):
        if t_total >= budget_s:
            break
        nodes, tris, box = tree.export()
        sc = orc.Scene(nodes, tris, box)
        step = max(1, j.height // (4 * threads))
        t0 = time.perf_counter()
        _, st = sc.render(m.camera, m.light, j.width, j.height, j.pixel_samples, j.max_depth, seed=j.seed,
                          threads=threads, rows=(0, j.height), row_step=step)
        t_total += time.perf_counter() - t0
        rays += int(st[0])
        done += 1
    return {"value": round(rays / t_total / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"one interleaved row set of each of the first {done} scenes ({t_total:.1f} s, oracle "
                      f"restatement of the reference, {threads} host threads)"}


def batch_mse(ctx, jobs, rows: int = 8, ref_spp: int = 4096) -> list:
    """MSE of batch jobs against converged renders: a band of `rows` rows
    through the middle of each image at the job's own sample count (linear
    radiance, its own seed) against the same band accumulated in FP64 over
    ref_spp samples."""
    import copy

    out = []
    for j in jobs:
        r0 = j.height // 2 - rows // 2
        fj = copy.copy(j)
        fj.row_begin, fj.row_end, fj.linear_output = r0, r0 + rows, 1
        (img,), _ = ctx.render([fj])
        rj = copy.copy(fj)
        rj.pixel_samples, rj.seed = 64, j.seed ^ 0x5EED
        ref, n = ctx.accumulate(rj, ref_spp // 64)
        out.append({"scene": int(j.scene_id), "spp": int(j.pixel_samples), "depth": int(j.max_depth),
                    "mse": float(((img[..., :3].astype(np.float64) - ref[..., :3]) ** 2).mean()),
                    "reference_spp": int(n)})
    return out


def run_guide(args) -> None:
    """Equal-time MSE of the learned proposal vs the plain cosine tracer.

    Scene: the indirect-lit room (walls tessellated 64x64 per wall, a 1.5x1.5
    baffle 0.3 below the point light, 40,998 triangles), side x side pixels,
    max depth 5. Reference: FP64-accumulated cosine render with ref_spp samples,
    in two independent halves whose difference estimates the reference's own
    variance (reported, and removed in value_reference_noise_removed).
    Both tracers accumulate passes of pass_spp samples in FP64 until the same
    wall-clock budget is spent; the learned tracer trains online inside that
    budget (--guide-steps Adam steps per pass over about --guide-records of
    the pass's bounces, lr --guide-lr) and its training passes count toward
    its image."""
    import turner_gb300 as tg

    side, depth = args.guide_side, 5
    ctx = tg.Context(0)
    ctx.set_guide_depth(args.guide_depth)
    ctx.set_guide_weighting(args.guide_weighting)
    mesh = tg.make_scene(tg.SCENE_BAFFLE_ROOM, detail=64)
    sid = ctx.upload_tree(tg.KDTree.from_mesh(mesh))

    def job(sampling, spp, seed):
        j = tg.make_job(sid, mesh, side, side, pixel_samples=spp, max_depth=depth, seed=seed, sampling=sampling)
        j.linear_output = 1
        return j

    # reference: two independent halves; their difference estimates the
    # reference's own variance, which inflates both MSEs by the same amount
    t0 = time.perf_counter()
    half = max(1, args.ref_spp // 512)
    cache = Path(args.ref_cache) if args.ref_cache else None
    cache_key = f"{side}-{depth}-{half}"
    if cache is not None and cache.exists() and str(np.load(cache)["key"]) == cache_key:
        z = np.load(cache)
        ref_a, ref_b, spp_a, spp_b = z["a"], z["b"], int(z["spp_a"]), int(z["spp_b"])
    else:
        ref_a, spp_a = ctx.accumulate(job(tg.SAMPLING_COSINE, 256, 424242), half)
        ref_b, spp_b = ctx.accumulate(job(tg.SAMPLING_COSINE, 256, 525252), half)
        if cache is not None:
            np.savez(cache, a=ref_a, b=ref_b, spp_a=spp_a, spp_b=spp_b, key=cache_key)
    ref_s = time.perf_counter() - t0
    ref, ref_spp = 0.5 * (ref_a + ref_b), spp_a + spp_b
    ref_var = float(((ref_a[..., :3] - ref_b[..., :3]) ** 2).mean() / 4)

    def mse(img):
        return float(((img[..., :3] - ref[..., :3]) ** 2).mean())

    def run(sampling, seed, guide=None):
        # passes of pass_spp samples accumulate on the device (no copy back
        # per pass) until the budget is spent; the learned tracer trains on
        # its passes for the first train_fraction of the budget
        if guide is not None:
            ctx.set_guide(guide, train=False)
        ctx.accumulate(job(sampling, args.pass_spp, seed), 1, readback=False)   # warm-up pass (workspace)
        if guide is not None:
            ctx.set_guide(guide, train=True, lr=args.guide_lr, records=args.guide_records,
                          steps_per_pass=args.guide_steps)
        training = guide is not None
        t = time.perf_counter()
        train_s = args.train_fraction * args.budget
        while True:
            if training and time.perf_counter() - t > train_s:
                ctx.set_guide(guide, train=False)   # the rest of the budget renders with the trained network
                training = False
            elif training and args.guide_lr_end > 0:
                # exponential learning-rate decay over the training window
                frac = min(1.0, (time.perf_counter() - t) / train_s)
                ctx.set_guide(guide, train=True, lr=args.guide_lr * (args.guide_lr_end / args.guide_lr) ** frac,
                              records=args.guide_records, steps_per_pass=args.guide_steps)
            ctx.accumulate(job(sampling, args.pass_spp, seed + 1), 1, readback=False)
            if time.perf_counter() - t >= args.budget:
                break
        wall = time.perf_counter() - t
        img, total = ctx.accumulate(job(sampling, args.pass_spp, seed + 1), 0)   # read the mean back
        return img, total, wall

    reps = []
    with Clocks(0) as clk:
        for rep in range(args.guide_repeats):
            seed = 7 + 1000 * rep
            plain, plain_spp, plain_s = run(tg.SAMPLING_COSINE, seed)
            guide = tg.Guide(ctx, seed=11 + rep)
            guide.set_objective(OBJECTIVES[args.guide_objective])
            learned, learned_spp, learned_s = run(tg.SAMPLING_GUIDED, seed, guide)
            steps, loss, train_ms = ctx.guide_stats()
            ctx.set_guide(None)
            guide.close()
            m_plain, m_learned = mse(plain), mse(learned)
            reps.append({"seed": seed, "ratio": round(m_plain / m_learned, 4),
                         "ratio_reference_noise_removed": round((m_plain - ref_var) / (m_learned - ref_var), 4),
                         "plain": {"mse": m_plain, "spp": int(plain_spp), "wall_s": round(plain_s, 3)},
                         "learned": {"mse": m_learned, "spp": int(learned_spp), "wall_s": round(learned_s, 3),
                                     "adam_steps": int(steps), "last_loss": round(loss, 4),
                                     "train_ms": round(train_ms, 1)}})
    ratios = [r["ratio"] for r in reps]
    print(json.dumps({
        "metric": "equal-time MSE vs FP64 reference, learned proposal vs cosine (indirect-lit room)",
        "value": round(float(np.mean(ratios)), 4), "unit": "MSE ratio (plain / learned, higher is better)",
        "min": min(ratios), "max": max(ratios), "std": round(float(np.std(ratios)), 4),
        "value_reference_noise_removed": round(float(np.mean([r["ratio_reference_noise_removed"] for r in reps])), 4),
        "reference_variance": ref_var,
        "higher_is_better": True, "n_gpus": 1, "dtype": "bf16 MLP / f32 tracing", "data": "synthetic",
        "config": {"workload": f"baffle room 40,998 triangles {side}x{side} depth {depth}",
                   "reference_spp": int(ref_spp), "reference_s": round(ref_s, 2), "budget_s": args.budget,
                   "pass_spp": args.pass_spp, "train_fraction": args.train_fraction,
                   "records_per_pass": args.guide_records, "steps_per_pass": args.guide_steps,
                   "lr": args.guide_lr, "repeats": args.guide_repeats, "guide_depth": args.guide_depth,
                   "guide_weighting": args.guide_weighting, "guide_objective": args.guide_objective,
                   "lr_end": args.guide_lr_end},
        "repeats": reps,
        "clocks": clk.summary,
    }))
    ctx.close()


def run_views16(args) -> None:
    """Learned proposal + batching: the 327,680-triangle displaced icosphere
    inside the baffled room (wall tessellation 64 per side), 16 camera views
    on a circle around the sphere at height 1.5 (radius --views-radius),
    1920x1080 each, max depth 5, one batch per render call (one CUDA graph when
    not training). One shared proposal is trained online across all views,
    then the guided and the cosine tracer each render --views-spp samples per
    view. Also an equal-time MSE comparison on the 1920x1080 views, cropped
    to a band of rows of each, against an FP64-accumulated cosine reference
    of those bands, over --guide-repeats seeds."""
    import torch

    import turner_gb300 as tg

    ctx = tg.Context(0)
    t0 = time.perf_counter()
    mesh = tg.make_scene(tg.SCENE_BAFFLE_SPHERE, detail=7, count=64, aspect=16 / 9)
    sid = ctx.upload_tree(tg.KDTree.from_mesh(mesh))
    build_s = time.perf_counter() - t0
    center = (2.78, 1.65, -3.5)
    cams = []
    for k in range(16):
        a = 2 * np.pi * k / 16
        pos = (center[0] + args.views_radius * np.cos(a), 1.5, center[2] + args.views_radius * np.sin(a))
        cams.append(tg.look_at_camera(pos, center, 16 / 9))

    def jobs(w, h, spp, sampling, seed):
        out = []
        for k, cam in enumerate(cams):
            j = tg.make_job(sid, mesh, w, h, pixel_samples=spp, max_depth=5, seed=seed * 131 + k, sampling=sampling)
            j.camera = cam
            j.linear_output = 1
            out.append(j)
        return out

    W, H = 1920, 1080
    outs = [torch.empty((H, W, 4), dtype=torch.float32, device="cuda") for _ in cams]
    ptrs = [o.data_ptr() for o in outs]
    guide = tg.Guide(ctx, seed=11)
    guide.set_objective(OBJECTIVES[args.guide_objective])
    ctx.set_guide(guide, train=True, lr=args.guide_lr, records=args.guide_records, steps_per_pass=args.guide_steps)
    t = time.perf_counter()
    calls = 0
    while time.perf_counter() - t < args.views_train_s:
        ctx.render(jobs(W, H, 1, tg.SAMPLING_GUIDED, 1000 + calls), ptrs, tg.DEVICE_BUFFERS)
        calls += 1
    train_wall = time.perf_counter() - t
    steps, loss, train_ms = ctx.guide_stats()
    ctx.set_guide(guide, train=False)
    thr = {}
    thr_clk = Clocks(0)
    thr_clk.__enter__()
    for name, sampling in (("guided", tg.SAMPLING_GUIDED), ("cosine", tg.SAMPLING_COSINE)):
        ctx.render(jobs(W, H, 1, sampling, 7), ptrs, tg.DEVICE_BUFFERS)   # workspace, graph shapes
        torch.cuda.synchronize()
        g0 = ctx.graph_launch_count()
        _, stats = ctx.render(jobs(W, H, args.views_spp, sampling, 11), ptrs, tg.DEVICE_BUFFERS)
        rays = sum(st.rays for st in stats)
        ctx.set_profiling(True)
        ctx.set_graph_mode(tg.GRAPH_NEVER)   # per-kernel events need uncaptured launches
        ctx.kernel_times(reset=True)
        ctx.render(jobs(W, H, 2, sampling, 13), ptrs, tg.DEVICE_BUFFERS)
        kt = ctx.kernel_times(reset=True)
        ctx.set_graph_mode(tg.GRAPH_AUTO)
        ctx.set_profiling(False)
        total = sum(v[0] for v in kt.values())
        thr[name] = {"mrays_per_s": round(rays / stats[0].device_ms / 1e3, 2), "ms": round(stats[0].device_ms, 1),
                     "rays": int(rays), "graph_launches": ctx.graph_launch_count() - g0,
                     "kernel_share": {k: round(v[0] / total, 4) for k, v in kt.items() if v[1]}}
    thr_clk.__exit__(None, None, None)

    # equal-time MSE on the configured 1920x1080 views, cropped to a band of
    # rows through the middle of every view (a converged 16k-spp reference of
    # 16 whole frames would take hours); both tracers render the same band
    r0 = H // 2 - args.views_eq_rows // 2
    band = (r0, r0 + args.views_eq_rows)
    bh = band[1] - band[0]
    small = [torch.empty((bh, W, 4), dtype=torch.float32, device="cuda") for _ in cams]
    sptr = [o.data_ptr() for o in small]

    def band_jobs(spp, sampling, seed):
        out = jobs(W, H, spp, sampling, seed)
        for j in out:
            j.row_begin, j.row_end = band
        return out

    def accumulate(sampling, spp, seed, calls=None, budget=None, train_fraction=0.0, guide=None):
        # running FP64 sum on the device: no host copy per pass
        acc = torch.zeros((16, bh, W, 3), dtype=torch.float64, device="cuda")
        n, t = 0, time.perf_counter()
        training = train_fraction > 0
        while (calls is not None and n < calls) or (budget is not None and time.perf_counter() - t < budget):
            if training and time.perf_counter() - t > train_fraction * budget:
                ctx.set_guide(guide, train=False)
                training = False
            ctx.render(band_jobs(spp, sampling, seed + n), sptr, tg.DEVICE_BUFFERS)
            for k, o in enumerate(small):
                acc[k] += o[..., :3]
            n += 1
        torch.cuda.synchronize()
        return (acc / n).cpu().numpy(), n * spp, time.perf_counter() - t

    t0 = time.perf_counter()
    half = max(1, args.views_ref_spp // 128)
    ref_a, _, _ = accumulate(tg.SAMPLING_COSINE, 64, 500000, calls=half)
    ref_b, _, _ = accumulate(tg.SAMPLING_COSINE, 64, 600000, calls=half)
    ref_s = time.perf_counter() - t0
    ref = 0.5 * (ref_a + ref_b)
    ref_var = float(((ref_a - ref_b) ** 2).mean() / 4)
    reps = []
    with Clocks(0) as clk:
        for rep in range(args.guide_repeats):
            seed = 7 + 1000 * rep
            plain, plain_spp, plain_s = accumulate(tg.SAMPLING_COSINE, args.pass_spp, seed, budget=args.budget)
            g2 = tg.Guide(ctx, seed=12 + rep)
            g2.set_objective(OBJECTIVES[args.guide_objective])
            ctx.set_guide(g2, train=False)
            ctx.render(band_jobs(args.pass_spp, tg.SAMPLING_GUIDED, 3), sptr, tg.DEVICE_BUFFERS)   # workspace
            ctx.set_guide(g2, train=True, lr=args.guide_lr, records=args.guide_records,
                          steps_per_pass=args.guide_steps)
            learned, learned_spp, learned_s = accumulate(tg.SAMPLING_GUIDED, args.pass_spp, seed, budget=args.budget,
                                                         train_fraction=args.views_train_fraction, guide=g2)
            ctx.set_guide(None)
            g2.close()
            m_plain = float(((plain - ref) ** 2).mean())
            m_learned = float(((learned - ref) ** 2).mean())
            reps.append({"seed": seed, "ratio": round(m_plain / m_learned, 4),
                         "ratio_reference_noise_removed": round((m_plain - ref_var) / (m_learned - ref_var), 4),
                         "plain": {"mse": m_plain, "spp": plain_spp, "wall_s": round(plain_s, 2)},
                         "learned": {"mse": m_learned, "spp": learned_spp, "wall_s": round(learned_s, 2)}})
    ratios = [r["ratio"] for r in reps]
    print(json.dumps({
        "metric": "Mrays/s, 16 views with the online-trained learned proposal (reference ray count)",
        "value": thr["guided"]["mrays_per_s"], "unit": "Mrays/s", "higher_is_better": True, "n_gpus": 1,
        "dtype": "bf16 MLP / f32 tracing", "data": "synthetic",
        "config": {"workload": f"baffled room + displaced icosphere, 16 views 1920x1080 x {args.views_spp} spp, depth 5",
                   "triangles": int(mesh.n_triangles), "views_radius": args.views_radius,
                   "host_tree_build_s": round(build_s, 2), "guide_objective": args.guide_objective},
        "guided": thr["guided"], "cosine": thr["cosine"],
        "training": {"calls": calls, "wall_s": round(train_wall, 2), "adam_steps": int(steps),
                     "last_loss": round(loss, 4), "train_ms": round(train_ms, 1)},
        "throughput_clocks": thr_clk.summary,
        "equal_time": {"views": f"16 x 1920x1080, rows {band[0]}-{band[1]} of each (crop: a 16k-spp reference "
                                f"of whole frames would take hours)",
                       "budget_s": args.budget, "train_fraction": args.views_train_fraction,
                       "reference_spp": 2 * half * 64,
                       "reference_s": round(ref_s, 1), "reference_variance": ref_var,
                       "mse_ratio": round(float(np.mean(ratios)), 4), "min": min(ratios), "max": max(ratios),
                       "std": round(float(np.std(ratios)), 4),
                       "mse_ratio_reference_noise_removed":
                           round(float(np.mean([r["ratio_reference_noise_removed"] for r in reps])), 4),
                       "repeats": reps, "clocks": clk.summary},
    }))
    guide.close()
    ctx.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--traversal", default="parity", choices=["parity", "fast"])
    ap.add_argument("--chunk-paths", type=int, default=1 << 24)
    ap.add_argument("--speculative", action="store_true", help="speculative traversal rounds")
    ap.add_argument("--no-packet", action="store_true", help="camera-ray warps traverse lane by lane, not as packets")
    ap.add_argument("--ring", type=int, default=0, choices=[0, 4, 8],
                    help="traversal stack entries kept in shared memory (0: all in local memory)")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mse", action="store_true", help="skip the converged-reference MSE of the headline frame")
    ap.add_argument("--small", action="store_true",
                    help="480x270 frame of the same scene (for profiler captures; not a bench line)")
    ap.add_argument("--workload", default="frame", choices=["frame", "batch64", "guide", "views16"])
    ap.add_argument("--views-radius", type=float, default=4.0)
    ap.add_argument("--views-spp", type=int, default=64)
    ap.add_argument("--views-train-s", type=float, default=3.0)
    ap.add_argument("--views-ref-spp", type=int, default=16384)
    ap.add_argument("--views-eq-rows", type=int, default=8, help="views16: rows of each view in the equal-time crop")
    ap.add_argument("--views-train-fraction", type=float, default=0.2,
                    help="views16: share of the equal-time budget the learned tracer trains for (measured best: 0.2 "
                         "here, 0.1 for the single view)")
    # guide workload defaults: the indirect-lit room at 1024x1024 against a
    # 16,384-spp FP64 reference, 10 s of equal wall time in 1-spp passes
    ap.add_argument("--guide-side", type=int, default=1024)
    ap.add_argument("--ref-spp", type=int, default=16384)
    ap.add_argument("--pass-spp", type=int, default=1)
    ap.add_argument("--budget", type=float, default=10.0)
    ap.add_argument("--ref-cache", default="", help="guide: .npz file that keeps the FP64 reference between runs")
    ap.add_argument("--train-fraction", type=float, default=0.1,
                    help="guide: share of the budget the learned tracer trains for (its passes count toward its image)")
    ap.add_argument("--guide-records", type=int, default=1 << 18)
    ap.add_argument("--guide-lr", type=float, default=1e-3)
    ap.add_argument("--guide-steps", type=int, default=16, help="Adam steps per training pass")
    ap.add_argument("--guide-lr-end", type=float, default=0.0,
                    help="guide: decay the learning rate exponentially to this value over the training window (0: constant)")
    ap.add_argument("--guide-repeats", type=int, default=3, help="guide: independent seeds (fresh networks)")
    ap.add_argument("--guide-depth", type=int, default=64, help="guided sampling at hits of depth < this")
    ap.add_argument("--guide-objective", default="kl", choices=sorted(OBJECTIVES),
                    help="training objective of the proposal: KL divergence or the 50/50 estimator's variance")
    ap.add_argument("--guide-weighting", type=int, default=0, choices=[0, 1, 2],
                    help="training-record weights: 0 incident radiance, 1 x path throughput, 2 x its square root")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-max-tris", type=int, default=500_000)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--gpu-build", action="store_true", help="batch64: build the 64 trees on the GPU")
    args = ap.parse_args()
    if args.workload == "batch64":
        run_batch64(args)
        return
    if args.workload == "guide":
        run_guide(args)
        return
    if args.workload == "views16":
        run_views16(args)
        return
    if args.small:
        global WIDTH, HEIGHT, WORKLOAD
        WIDTH, HEIGHT = 480, 270
        WORKLOAD = "sphere_room_327k_480x270_16spp_d3 (profiling case)"
    if args.impl == "reference":
        run_reference(args)
        return

    rank, world, local = rank_info()
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if world > 1 else 0
    torch.cuda.set_device(device)

    import turner_gb300 as tg

    from turner_gb300.shard import row_range

    mesh, tree, build_s = make_workload()
    ctx = tg.Context(device)
    ctx.set_chunk_paths(args.chunk_paths)
    ctx.set_traversal_ring(args.ring)
    ctx.set_traversal_speculative(args.speculative)
    ctx.set_traversal_packet(0 if args.no_packet else tg.PACKET_CAMERA)
    sid = ctx.upload_tree(tree)
    nodes, tris, box = tree.export()
    traversal = tg.TRAVERSAL_FAST if args.traversal == "fast" else tg.TRAVERSAL_PARITY
    seed = 1
    # one frame, partitioned by rows over the ranks (the reference's unit of
    # work is one row, main.cpp:193-226); every rank holds the whole scene
    y0, y1 = row_range(HEIGHT, rank, world)
    job = tg.make_job(sid, mesh, WIDTH, HEIGHT, pixel_samples=SPP, max_depth=DEPTH, monte_carlo_samples=MC,
                      seed=seed, traversal=traversal, rows=(y0, y1))
    out = torch.empty((y1 - y0, WIDTH, 4), dtype=torch.float32, device=f"cuda:{device}")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")   # > L2 (126 MiB)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up
    for _ in range(args.warmup):
        ctx.render([job], [out.data_ptr()], tg.DEVICE_BUFFERS)

    # timed, device-resident: L2 flushed between steps (outside the timed kernels)
    ctx.set_profiling(True)
    ctx.kernel_times(reset=True)
    launches0 = ctx.launch_count()
    clock_lines: list[str] = []
    stop = threading.Event()
    sampler = threading.Thread(target=sample_clocks, args=(stop, clock_lines, device), daemon=True)
    sampler.start()
    barrier()
    t0 = time.perf_counter()
    dev_ms, rays, shadow = 0.0, 0, 0
    for _ in range(args.steps):
        flush.zero_()
        _, (st,) = ctx.render([job], [out.data_ptr()], tg.DEVICE_BUFFERS)
        dev_ms += st.device_ms
        rays += st.rays
        shadow += st.shadow_rays
    barrier()
    wall = time.perf_counter() - t0
    stop.set()
    sampler.join(timeout=5)
    launches = ctx.launch_count() - launches0
    ktimes = ctx.kernel_times(reset=True)
    ctx.set_profiling(False)

    # end to end through the C ABI with host buffers
    img_host = np.empty((y1 - y0, WIDTH, 4), np.float32)
    h2d = nodes.nbytes + 2 * 64 * tris.shape[0]   # node words + intersection and shading records
    d2h = img_host.nbytes
    barrier()
    e0 = time.perf_counter()
    e_rays = 0
    for _ in range(args.steps):
        s2 = ctx.upload(nodes, tris, box)
        j2 = tg.make_job(s2, mesh, WIDTH, HEIGHT, pixel_samples=SPP, max_depth=DEPTH, monte_carlo_samples=MC,
                         seed=seed, traversal=traversal, rows=(y0, y1))
        (img,), (st,) = ctx.render([j2])
        e_rays += st.rays
        ctx.free_scene(s2)
    barrier()
    e_wall = time.perf_counter() - e0

    t_max = dev_ms / 1000.0
    if dist is not None:
        t = torch.tensor([t_max, e_wall], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max, e_wall = float(t[0]), float(t[1])
        r = torch.tensor([rays, e_rays], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(r, op=dist.ReduceOp.SUM)
        rays_all, e_rays_all = float(r[0]), float(r[1])
    else:
        rays_all, e_rays_all = float(rays), float(e_rays)
    value = rays_all / t_max / 1e6

    result = None
    if rank == 0:
        # roofline of the dominant kernel (closest-hit traversal): algorithmic
        # bytes per ray from the oracle's count of the reference's traversal
        # (every overlapped leaf, no early exit) on the CPU sample of this
        # frame (interleaved row sets spread over the whole frame)
        peaks = json.loads(PEAKS.read_text()) if PEAKS.exists() else {}
        hbm = peaks.get("hbm_gbs", 6800.0)
        cpu = None
        visits_per_ray = tests_per_ray = None
        if not args.no_cpu:
            cpu_mrays, cpu_rows, cst, threads, cdt, stride = cpu_baseline(mesh, tree, seed, budget_s=args.cpu_budget)
            visits_per_ray = float(cst[3]) / float(cst[0])
            tests_per_ray = float(cst[4]) / float(cst[0])
            cpu = {"value": round(cpu_mrays, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                   "sample": f"{cpu_rows} rows of the same frame in interleaved sets (row step {stride}, "
                             f"{cpu_rows * WIDTH * SPP} paths, {cdt:.1f} s, oracle restatement of the reference, "
                             f"{threads} host threads taking one row at a time)"}
        kt_ms, kt_n = ktimes["k_trace"]
        dominant = max(ktimes, key=lambda k: ktimes[k][0])
        roof = roof_l2 = None
        if visits_per_ray is not None and kt_ms > 0:
            node_b = 8 * visits_per_ray
            tri_b = 64 * tests_per_ray
            ray_b = 32 + 16   # ray in, hit out
            bytes_per_ray = node_b + tri_b + ray_b
            per_launch_bytes = bytes_per_ray * rays / max(kt_n, 1)
            avg_launch_s = kt_ms / 1000.0 / max(kt_n, 1)
            achieved = per_launch_bytes / avg_launch_s / 1e9
            traffic = None
            if TRAFFIC.exists():
                tr = json.loads(TRAFFIC.read_text())
                traffic = tr.get("dram_bytes_per_ray", 0) * rays / max(kt_n, 1)
            roof = {"kernel": "k_trace", "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                    "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": traffic,
                    "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if PEAKS.exists() else "fallback",
                    "bytes_per_ray": round(bytes_per_ray, 1), "node_visits_per_ray": round(visits_per_ray, 2),
                    "triangle_tests_per_ray": round(tests_per_ray, 2),
                    "counted_on": "the CPU sample's rays (interleaved rows over the whole frame)"}
            # the roof the traversal actually meets: random gathers served by
            # L2 (the scene is L2-resident), measured by the probe kernel:
            # node words at the 8-byte gather rate, records at the 32-byte one
            g8 = ctx.probe_gather(64 << 20, 8)
            g32 = ctx.probe_gather(64 << 20, 32)
            mix = bytes_per_ray / (node_b / g8 + tri_b / g32 + ray_b / hbm)
            roof_l2 = {"kernel": "k_trace", "bound": "l2", "achieved": round(achieved, 1), "peak": round(mix, 1),
                       "unit": "GB/s", "frac": round(achieved / mix, 4),
                       "probe": {"gather8_gbs": round(g8, 1), "gather32_gbs": round(g32, 1), "buffer_mib": 64,
                                 "peak_is": "bytes / (node bytes / gather8 + record bytes / gather32 + "
                                            "ray bytes / hbm)"},
                       "note": "algorithmic bytes count every node and record load; L1 hits (the tree's top "
                               "levels) make them cheaper than an L2 gather, so frac can pass 1"}
        mse = headline_mse(ctx, sid, mesh, seed, traversal) if not args.no_mse else None
        clocks = summarize_clocks(clock_lines)
        result = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000 * t_max / args.steps, 3), "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "triangles": int(tris.shape[0]), "nodes": int(nodes.size),
                       "width": WIDTH, "height": HEIGHT, "pixel_samples": SPP, "max_depth": DEPTH,
                       "monte_carlo_samples": MC, "traversal": args.traversal, "chunk_paths": args.chunk_paths,
                       "stack_ring": args.ring, "speculative": args.speculative, "camera_ray_packets": not args.no_packet,
                       "l2": "flushed between steps (512 MiB write outside the timed kernels)",
                       "parallelism": f"rows of one frame over {world} ranks" if world > 1 else "single GPU",
                       "kdtree_build_s": round(build_s, 3)},
            "e2e": {"value": round(e_rays_all / e_wall / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "rays_per_step": int(rays // args.steps), "shadow_rays_per_step": int(shadow // args.steps),
            # the same timed region, counted other ways (this rank's counts)
            "mpaths_per_s": round((y1 - y0) * WIDTH * SPP * args.steps / (dev_ms / 1000.0) / 1e6, 3),
            # shadow rays are traced only where the light is in front of the
            # surface (cos > 0): the reference traces one at every hit
            "mrays_incl_traced_shadow_per_s": round((rays + shadow) / (dev_ms / 1000.0) / 1e6, 3),
            "wall_ms_per_step": round(1000 * wall / args.steps, 3),
            "kernels_ms_per_step": {k: round(v[0] / args.steps, 3) for k, v in ktimes.items() if v[1]},
            "dominant_kernel": dominant,
            "roofline": roof,
            "roofline_l2": roof_l2,
            "mse_vs_fp64": mse,
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
        print(json.dumps(result))
    ctx.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
