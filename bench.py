"""Benchmark of the plain PatchMatch stereo path on one GB300 (or N replicas).

Workload (one step): PMHuberStereo::depthMap on one rectified pair of
1242x375 RGBA float32 (16 slanted planes, disparity 0-128 px, 2% salt noise,
+/-5% gain/bias between the views), 35x35 window, 8 iterations, LR threshold
1 px with fill-in, 250 PD steps per view and iteration.  Synthetic, seeded.

Metric: Mpix-iter/s = W*H*iterations / time of the whole depthMap (both views,
init through the final fill).  `value` is device-timed with the inputs
resident in HBM; `e2e` is the same metric through the C ABI on pinned host
buffers (cvtpm_depthmap_host: H2D of both images, the run, D2H of the map).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's algorithm on the host cores: the
CPU restatement of pmhstereo.cl/PDHuberWeighted.cl/RNG.cl and the depthMap
schedule (oracle/), EXACT arithmetic with MWC64X streams, all host threads,
each step a bounded crop of the same workload (the top-left 640x48 pixels of
the pair, all 8 iterations, so the theta ramp and the view candidates match
the timed run).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_CFG, H_CFG, DMAX, ITERS, PATCH = 1242, 375, 128.0, 8, 17
WORKLOAD = "plain PatchMatch depthMap, 1 pair 1242x375 RGBA f32, 16 planes, dmax 128, 2% salt, +/-5% gain/bias, 35x35 ASW, 8 iterations, LR 1px + fill"
METRIC = "PatchMatch Mpix-iter/s (plain depthMap, 1242x375, 8 iterations)"
FLOPS_PER_TAP = 55.0          # per (pixel, candidate) window tap: plane, lerp, truncated L1, accumulate
FLOPS_PER_WEIGHT_TAP = 20.0   # bilateral weight of a tap, once per pixel and launch
RECORD_BYTES_PER_TAP = 56.0   # the other view's value/difference records one evaluated tap reads (FAST)
L1_BYTES_PER_CLK_SM = 128.0   # L1/shared data path of one SM
FP32_LANES_PER_SM = 128       # FP32 CUDA cores per SM (FMA = 2 flops)
QUALITY_PAIRS = 8
PD_BYTES_PER_PX = 116.0       # u 16 + p 32 + f 16 + w 4 read; u 16 + p 32 written


def params_for(impl: str):
    from cvt_gb300.params import default_params, PRESET_BASELINE, ARITH_EXACT, RNG_MWC64X
    p = default_params(PRESET_BASELINE, patchsize=PATCH, depthmax=DMAX, iterations=ITERS, maxdispdiff=1.0)
    if impl == "reference":
        p = p.replace(arith=ARITH_EXACT, rng=RNG_MWC64X)
    return p


def scene_for(rank: int):
    from cvt_gb300 import scenes
    return scenes.config_scene(2, pair=rank)


def in_image_taps(W: int, H: int, P: int) -> int:
    xs = np.arange(W)
    nx = np.minimum(xs + P, W - 1) - np.maximum(xs - P, 0) + 1
    ys = np.arange(H)
    ny = np.minimum(ys + P, H - 1) - np.maximum(ys - P, 0) + 1
    return int(nx.sum()) * int(ny.sum())


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def read_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if "Active" in v and "Not" not in v:
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_baseline(params, sc, rows: int, cols: int, iters: int):
    """The oracle (CPU restatement) on the top-left `cols` x `rows` crop of
    the pair for `iters` iterations: Mpix-iter/s of the reference's algorithm
    on this host.  A left crop keeps every match of its pixels (x' = x - d
    < x), so the crop is a smaller pair of the same scene."""
    from oracle import oracle as orc
    p = params.replace(iterations=iters)
    L = np.ascontiguousarray(sc.left[:rows, :cols])
    R = np.ascontiguousarray(sc.right[:rows, :cols])
    t0 = time.perf_counter()
    orc.depthmap(p, L, R)
    dt = time.perf_counter() - t0
    return L.shape[1] * rows * iters / dt / 1e6, dt, orc.max_threads()


def cpu_sample_text(sc, rows, cols, iters):
    return (f"top-left {min(cols, sc.width)}x{rows} crop of the {sc.width}x{sc.height} pair (rows 0-{rows - 1}, "
            f"columns 0-{min(cols, sc.width) - 1}), {iters} iterations per step, exact arithmetic + MWC64X")


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from oracle import oracle as orc
    orc.lib()
    p = params_for("reference")
    sc = scene_for(0)
    rows, cols, iters = args.ref_rows, args.ref_cols, args.ref_iters
    for _ in range(args.warmup):              # loads and warms the library: one iteration of the crop
        cpu_baseline(p, sc, rows, cols, 1)
    vals, secs = [], 0.0
    for _ in range(args.steps):
        v, dt, cores = cpu_baseline(p, sc, rows, cols, iters)
        vals.append(v)
        secs += dt
    value = float(np.mean(vals))
    sample = cpu_sample_text(sc, rows, cols, iters) + "; warm-up steps run 1 iteration of the crop"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix-iter/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Voronoi slanted planes, blurred noise texture)",
            "config": {"workload": WORKLOAD, "arith": "exact (reference operation order)", "rng": "MWC64X"},
            "cpu_baseline": {"value": value, "unit": "Mpix-iter/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Mpix-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(x: float, dist: bool, device) -> float:
    """The largest value of x over all ranks (the slowest rank sets the time)."""
    if not dist:
        return x
    import torch
    import torch.distributed as tdist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, W: int, H: int, iters: int, seconds: float) -> float:
    """Whole-job Mpix-iter/s of `world` replicas, one W x H pair each."""
    return world * W * H * iters / seconds / 1e6


def run_ours(args, rank, world, local_rank):
    import torch
    from cvt_gb300 import scenes, _lib
    from cvt_gb300.stereo import PMHuberStereo
    dist = world > 1
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if dist:
        import torch.distributed as tdist

    def barrier():
        if dist:
            tdist.barrier()
        torch.cuda.synchronize()

    p = params_for("ours")
    sc = scene_for(rank)
    W, H = sc.width, sc.height
    st = PMHuberStereo(local_rank, p)
    L = torch.from_numpy(sc.left).to(dev)
    R = torch.from_numpy(sc.right).to(dev)
    dmap = torch.empty((H, W), device=dev)
    flush = torch.empty(64 * 1024 * 1024, device=dev)          # 256 MB > 129 MB L2
    stream = torch.cuda.current_stream(dev)

    fp32 = _lib.ctypes.c_float()
    rc = _lib.lib().cvtpm_tool_fp32_peak(local_rank, _lib.ctypes.c_void_p(stream.cuda_stream), _lib.ctypes.byref(fp32))
    fp32_tflops = float(fp32.value) if rc == 0 else None

    for _ in range(args.warmup):
        st.depthMap(dmap, L, R, PATCH, DMAX, ITERS, 4)
    barrier()
    st.reset_stats()
    st.set_timing(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local_rank) as clk:
        barrier()
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            st.depthMap(dmap, L, R, PATCH, DMAX, ITERS, 4)
            ev[i][1].record(stream)
        barrier()
        wall = time.perf_counter() - t0
    st.set_timing(False)
    stats = st.stats()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = max_over_ranks(float(np.mean(step_ms)), dist, dev)
    value = replica_rate(world, W, H, ITERS, ms * 1e-3)
    bad1 = scenes.bad_pixel_rate(dmap.cpu().numpy() * DMAX, sc)
    epe = scenes.end_point_error(dmap.cpu().numpy() * DMAX, sc)

    # ---- end to end through the C ABI on pinned host buffers
    hl = torch.from_numpy(sc.left).pin_memory()
    hr = torch.from_numpy(sc.right).pin_memory()
    hd = torch.empty((H, W), dtype=torch.float32).pin_memory()
    for _ in range(max(1, args.warmup // 2)):
        st.depthMapHost(hl.numpy(), hr.numpy(), PATCH, DMAX, ITERS, 4, dmap=hd.numpy())
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st.depthMapHost(hl.numpy(), hr.numpy(), PATCH, DMAX, ITERS, 4, dmap=hd.numpy())
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, dist, dev)
    e2e = replica_rate(world, W, H, ITERS, e2e_s)

    if rank != 0:
        return 0
    # ---- quality, untimed: this configuration and the reference's algorithm
    # (EXACT arithmetic + MWC64X, full runs bit-identical to the reference's
    # code) on pairs 0-7 of the same scene family
    qual = {"ours": [], "reference": []}
    qms = {"ours": [], "reference": []}
    for pair in range(QUALITY_PAIRS):
        qs = scene_for(pair)
        ql, qr = torch.from_numpy(qs.left).to(dev), torch.from_numpy(qs.right).to(dev)
        for name in ("ours", "reference"):
            st.set_params(params_for(name))
            q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            q0.record(stream)
            st.depthMap(dmap, ql, qr, PATCH, DMAX, ITERS, 4)
            q1.record(stream)
            qual[name].append(scenes.bad_pixel_rate(dmap.cpu().numpy() * DMAX, qs))
            qms[name].append(q0.elapsed_time(q1))
    st.set_params(p)
    exact_ms = float(np.mean(qms["reference"]))
    exact = {"value": W * H * ITERS / 1e6 / (exact_ms * 1e-3), "unit": "Mpix-iter/s", "ms_per_step": exact_ms,
             "fast_ms_per_step_same_runs": float(np.mean(qms["ours"])),
             "note": "the reference's arithmetic on the GPU (EXACT operation order + MWC64X; results bit-identical "
                     "to the reference's code): mean over the untimed quality runs, pairs 0-7, L2 not flushed"}
    # ---- roofline of the dominant kernel (propagation: FP32 CUDA cores)
    nprop = max(1, stats["propagate_launches"])
    prop_ms = stats["propagate_ms"] / nprop
    flops_launch = (stats["cost_taps"] * FLOPS_PER_TAP) / nprop + in_image_taps(W, H, PATCH) * FLOPS_PER_WEIGHT_TAP
    achieved = flops_launch / (prop_ms * 1e-3) / 1e12
    traffic = read_traffic()
    roofline = {"kernel": "k_propagate<fast>", "bound": "fp32", "achieved": achieved,
                "peak": fp32_tflops, "unit": "TFLOP/s",
                "frac": (achieved / fp32_tflops) if fp32_tflops else None,
                "traffic": traffic.get("k_propagate_bytes_per_launch"),
                "peak_source": "FFMA-chain probe run in this process (cvtpm_tool_fp32_peak), FMA = 2 flops",
                "flops_per_launch": flops_launch, "launch_ms": prop_ms,
                "share_of_step": stats["propagate_ms"] / max(1e-9, sum(step_ms))}
    hbm_peak, hbm_src = peaks()
    # the PD kernel alone (depthMap runs the two views' smoothers concurrently,
    # so its phase timers overlap): 248 steps on the last call's left input
    pd_us = _lib.ctypes.c_float()
    rc = _lib.lib().cvtpm_tool_pd_time(st._h, 248, _lib.ctypes.c_void_p(stream.cuda_stream), _lib.ctypes.byref(pd_us))
    pd_ms = float(pd_us.value) * 1e-3 if rc == 0 else float("nan")   # per PD step (a launch runs up to 4)
    pd_bytes = PD_BYTES_PER_PX * W * H
    roofline_pd = {"kernel": "k_pd_block", "bound": "hbm", "achieved": pd_bytes / (pd_ms * 1e-3) / 1e9,
                   "peak": hbm_peak, "unit": "GB/s", "frac": pd_bytes / (pd_ms * 1e-3) / 1e9 / hbm_peak,
                   "traffic": (traffic["k_pd_block_bytes_per_launch"] / traffic.get("k_pd_block_steps_per_launch", 4)
                               if "k_pd_block_bytes_per_launch" in traffic else None),
                   "traffic_per": "PD step (DRAM bytes of one 4-step launch / 4)", "peak_source": hbm_src,
                   "per": "PD step (algorithmic bytes of one step / time of one step)",
                   "steps_per_launch": stats["pd_steps"] / max(1, stats["pd_launches"]),
                   "timed": "the blocked PD kernel alone, 248 steps on the bench pair's left smoother input "
                            "(cvtpm_tool_pd_time); inside depthMap the two views' smoothers run concurrently",
                   "note": "the blocked kernel keeps 4 steps in shared memory, so it moves fewer bytes than one step's algorithmic count"}
    # the propagation's limiter is the L1 data path: its record bytes against
    # 128 B per clock and SM at the sampled clock
    clocks = clk.summary()
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    l1_peak = (n_sm * L1_BYTES_PER_CLK_SM * clocks["sm_mhz"] * 1e6 / 1e9) if clocks.get("sm_mhz") else None
    fp32_derived = (n_sm * FP32_LANES_PER_SM * 2 * clocks["sm_mhz"] * 1e6 / 1e12) if clocks.get("sm_mhz") else None
    roofline["peak_derived"] = fp32_derived
    roofline["frac_of_derived"] = (achieved / fp32_derived) if fp32_derived else None
    roofline["peak_derived_source"] = (f"{n_sm} SMs x {FP32_LANES_PER_SM} FP32 lanes x 2 flops x the median SM clock "
                                       "sampled during the timed region")
    l1_achieved = stats["cost_taps"] / nprop * RECORD_BYTES_PER_TAP / (prop_ms * 1e-3) / 1e9
    roofline_l1 = {"kernel": "k_propagate<fast> + k_nbcost (the propagation pass)", "bound": "l1",
                   "achieved": l1_achieved, "peak": l1_peak, "unit": "GB/s",
                   "frac": (l1_achieved / l1_peak) if l1_peak else None,
                   "per": "pass: device-counted evaluated taps x 56 record bytes (a lower bound: image-1 reads, "
                          "weights and misaligned 128-byte lines come on top; ncu measures the L1 data pipe at "
                          "81-88 % busy) / pass time",
                   "peak_source": f"{n_sm} SMs (from the device) x 128 B/clk x the median SM clock sampled during "
                                  "the timed region"}
    cpu = None
    if not args.no_cpu_baseline:
        from cvt_gb300.params import ARITH_EXACT, RNG_MWC64X
        pv, dt, cores = cpu_baseline(p.replace(arith=ARITH_EXACT, rng=RNG_MWC64X), sc, args.ref_rows, args.ref_cols,
                                     args.ref_iters)
        cpu = {"value": pv, "unit": "Mpix-iter/s", "cores": cores, "kind": "port",
               "sample": cpu_sample_text(sc, args.ref_rows, args.ref_cols, args.ref_iters) + f", {dt:.1f} s"}
    line = {"metric": METRIC, "value": value, "unit": "Mpix-iter/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Voronoi slanted planes, blurred noise texture); replica r uses pair seed 2000+r",
            "config": {"workload": WORKLOAD, "arith": "fast (FMA, fixed-point tap positions; mirrored bit-exactly by the oracle)",
                       "rng": "Philox4x32-10", "preset": "BASELINE (gamma 10, alpha 0.9, tau 10/255 and 2/255)",
                       "l2": "flushed between steps (256 MB write)", "parallelism": "replicas" if world > 1 else "1 GPU"},
            "e2e": {"value": e2e, "unit": "Mpix-iter/s", "h2d_bytes_per_step": 2 * W * H * 16,
                    "d2h_bytes_per_step": W * H * 4},
            "roofline": roofline, "roofline_l1": roofline_l1, "roofline_pd": roofline_pd, "cpu_baseline": cpu,
            "exact_arithmetic": exact,
            "quality": {"bad1_nonocc_pct": bad1, "epe_nonocc_px": epe,
                        "pairs": QUALITY_PAIRS,
                        "bad1_nonocc_pct_mean": float(np.mean(qual["ours"])),
                        "reference_algorithm_bad1_nonocc_pct_mean": float(np.mean(qual["reference"])),
                        "note": "first two: the timed pair; means over pairs 0-7 (untimed); reference algorithm = "
                                "EXACT arithmetic + MWC64X; a different RNG stream moves one pair's bad-1px by ~0.3 pp"},
            "clocks": clocks, "gpu_launches": stats["launches"], "wall_s": wall}
    if not args.no_extras:
        line["adjoint"] = adjoint_record(max(3, args.steps // 4))
        line["batch"] = batch_record(args.pairs, args.batch_iters)
    print(json.dumps(line), flush=True)
    return 0


def run_profile(args):
    """A short run for ncu: one warm-up and one timed depthMap with
    --profile-iters iterations on the same pair (device memory ~0.2 GB)."""
    import torch
    from cvt_gb300.stereo import PMHuberStereo
    p = params_for("ours").replace(iterations=args.profile_iters)
    sc = scene_for(0)
    st = PMHuberStereo(0, p)
    L = torch.from_numpy(sc.left).cuda()
    R = torch.from_numpy(sc.right).cuda()
    dmap = torch.empty((sc.height, sc.width), device="cuda")
    for _ in range(2):
        st.depthMap(dmap, L, R, PATCH, DMAX, args.profile_iters, 4)
    torch.cuda.synchronize()
    print(json.dumps({"profile_run": "ok", "iterations": args.profile_iters, "launches_per_step": st.stats()["launches"] // 2}))
    return 0


def batch_record(npairs: int, iters: int) -> dict:
    """The batched workload: `npairs` uneven pairs (widths 320-1920, heights
    240-1080, disparity ranges 32-256, 4-24 planes; seeded), `iters`
    iterations, FAST + Philox.  Times a loop of plain per-pair depthMap calls
    and the batched graph (tuned and captured on its first call, then
    replayed) on the same pairs, device-timed with CUDA events on the
    launching stream; checks that both give the same bits and reports
    bad-1px."""
    import multiprocessing as mp
    import torch
    from cvt_gb300 import scenes
    from cvt_gb300.stereo import PMHuberStereo
    shapes = scenes.batch_shapes(npairs)
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 4)) as pool:
        scs = pool.map(scenes.batch_scene, shapes)
    p = params_for("ours").replace(iterations=iters)
    dev = torch.device("cuda", torch.cuda.current_device())
    pairs = [(torch.from_numpy(sc.left).to(dev), torch.from_numpy(sc.right).to(dev), sh[2]) for sc, sh in zip(scs, shapes)]
    npx = sum(sh[0] * sh[1] for sh in shapes)
    mpix_iter = npx * p.iterations / 1e6
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    plain = PMHuberStereo(dev.index, p)
    outs_plain = [torch.empty(sc.left.shape[:2], device=dev) for sc in scs]
    big = max(range(len(pairs)), key=lambda i: shapes[i][0] * shapes[i][1])
    plain.depthMap(outs_plain[big], pairs[big][0], pairs[big][1], PATCH, pairs[big][2], p.iterations, 4)  # sizes scratch

    def loop():
        for (left, right, dmax), d in zip(pairs, outs_plain):
            plain.depthMap(d, left, right, PATCH, dmax, p.iterations, 4)
    t_plain = timed(loop)

    bat = PMHuberStereo(dev.index, p)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    outs = bat.depthMapBatched(pairs)
    torch.cuda.synchronize()
    first = time.perf_counter() - t0
    t_bat = timed(lambda: bat.depthMapBatched(pairs, outs=outs))
    info = bat.batch_info()
    same = all(torch.equal(a.view(torch.int32), b.view(torch.int32)) or
               bool(((a == b) | (torch.isnan(a) & torch.isnan(b))).all()) for a, b in zip(outs, outs_plain))
    bad = [scenes.bad_pixel_rate(d.cpu().numpy() * sh[2], sc) for d, sh, sc in zip(outs, shapes, scs)]
    bad_plain = [scenes.bad_pixel_rate(d.cpu().numpy() * sh[2], sc) for d, sh, sc in zip(outs_plain, shapes, scs)]
    return {"metric": f"PatchMatch Mpix-iter/s ({len(pairs)} uneven pairs, {p.iterations} iterations)",
            "workload": "batch", "unit": "Mpix-iter/s", "n_gpus": 1, "dtype": "f32", "data": "synthetic, seeded",
            "config": {"workload": f"{len(pairs)} pairs, W 320-1920, H 240-1080, dmax 32-256, 4-24 planes, "
                                   f"35x35 ASW, {p.iterations} iterations, BASELINE preset, FAST + Philox",
                       "pixels": npx},
            "plain_loop": {"value": mpix_iter / t_plain, "seconds": t_plain,
                           "launches": plain.stats()["launches"]},
            "batched": {"value": mpix_iter / t_bat, "seconds": t_bat, "first_call_seconds": first,
                        "mode": "phase-batched" if info["phased"] else f"{info['lanes']} lanes",
                        "launches": info["launches"], "graph_nodes": info["graph_nodes"],
                        "knobs": {"grid_mult": info["grid_mult"], "pd_rows": info["pd_rows"],
                                  "pd_halo": info["pd_halo"]},
                        "tuning_ms": info["tune_ms"], "tuning": info["candidates"],
                        "mode_proxy_ms": info["mode_ms"],
                        "shared_windows": info["shared_windows"]},
            "speedup": t_plain / t_bat, "bit_identical_to_plain": same,
            "timing": "CUDA events on the launching stream, one run each (inputs in HBM)",
            "quality": {"bad1_nonocc_pct_mean": float(np.mean(bad)),
                        "plain_bad1_nonocc_pct_mean": float(np.mean(bad_plain))}}


def run_batch(args):
    print(json.dumps(batch_record(args.pairs, args.batch_iters)), flush=True)
    return 0


def _disparity(planes, W, H):
    import torch
    yy, xx = torch.meshgrid(torch.arange(H, device=planes.device), torch.arange(W, device=planes.device), indexing="ij")
    return planes[..., 0] * xx + planes[..., 1] * yy + planes[..., 2]


def adjoint_record(steps: int) -> dict:
    """The differentiation workload: forward + adjoint (planes and both
    images) of the aggregated cost for 8 pairs at 640x480, plane fields =
    ground truth + N(0, 0.01) on a, b and N(0, 1) on c, clamped to
    a, b in [-0.3, 0.3], c in [0, 64]; dL/dcost ~ N(0, 1).  Device-timed with
    CUDA events over `steps` repetitions after one warm-up."""
    import torch
    from cvt_gb300 import scenes
    from cvt_gb300.stereo import PMHuberStereo
    from cvt_gb300.params import default_params, PRESET_BASELINE
    st = PMHuberStereo(torch.cuda.current_device(), default_params(PRESET_BASELINE, patchsize=PATCH))
    rng = np.random.default_rng(4)
    items = []
    for i in range(8):
        sc = scenes.make_scene(640, 480, 8, 64.0, seed=4000 + i)
        pf = sc.plane_field().astype(np.float64)
        pl = np.zeros((480, 640, 4), np.float32)
        pl[..., 0] = np.clip(pf[..., 0] + rng.normal(0, 0.01, pf.shape[:2]), -0.3, 0.3)
        pl[..., 1] = np.clip(pf[..., 1] + rng.normal(0, 0.01, pf.shape[:2]), -0.3, 0.3)
        pl[..., 2] = np.clip(pf[..., 2] + rng.normal(0, 1.0, pf.shape[:2]), 0.0, 64.0)
        items.append((torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda(), torch.from_numpy(pl).cuda(),
                      torch.randn(480, 640, device="cuda")))
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    fwd = timed(lambda: [st.cost_adjoint(a, b, p, 1) for a, b, p, g in items], steps)
    full = timed(lambda: [st.cost_adjoint(a, b, p, 1, dcost=g) for a, b, p, g in items], steps)
    mpx = 8 * 640 * 480 / 1e6
    return {"workload": "adjoint", "config": {"workload": "8 pairs 640x480 RGBA f32, 35x35 ASW, BASELINE preset, "
                                                          "perturbed ground-truth planes, forward + adjoint w.r.t. "
                                                          "planes and both images"},
            "forward_ms": fwd, "forward_plus_adjoint_ms": full,
            "forward_mpix_per_s": mpx / (fwd * 1e-3), "forward_plus_adjoint_mpix_per_s": mpx / (full * 1e-3),
            "unit": "Mpix/s", "steps": steps, "timing": "CUDA events on the launching stream, inputs in HBM"}


def run_adjoint(args):
    print(json.dumps(adjoint_record(args.steps)), flush=True)
    return 0


def run_combined(args):
    """The combined workload: 16 uneven pairs (up to 1920x1080, disparity up
    to 256) in one batched graph with 8 iterations, then 4 plane-polishing
    steps per pixel of the left views; bad-1px and EPE against ground truth
    and against the plain output."""
    import multiprocessing as mp
    import torch
    from cvt_gb300 import scenes
    from cvt_gb300.stereo import PMHuberStereo
    shapes = scenes.batch_shapes(args.pairs, seed=5000)
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 4)) as pool:
        scs = pool.map(scenes.batch_scene, shapes)
    p = params_for("ours").replace(iterations=8)
    pairs = [(torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda(), sh[2]) for sc, sh in zip(scs, shapes)]
    bat = PMHuberStereo(0, p)
    outs = bat.depthMapBatched(pairs)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    bat.depthMapBatched(pairs, outs=outs)
    e1.record()
    torch.cuda.synchronize()
    t_batch = e0.elapsed_time(e1) / 1e3
    plain = PMHuberStereo(0, p)
    t_polish = 0.0
    rows = []
    for (left, right, dmax), sc, d_b in zip(pairs, scs, outs):
        H, W = left.shape[:2]
        tr = {}
        d_plain = plain.depthMap(None, left, right, PATCH, dmax, p.iterations, 4, trace=tr)
        s = tr["states"][0]
        planes = torch.zeros_like(s)
        planes[..., 0], planes[..., 1], planes[..., 2] = 1 - s[..., 0], -s[..., 1], -s[..., 2]
        planes = planes.contiguous()
        a0 = _disparity(planes, W, H)
        torch.cuda.synchronize()
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record()
        plain.polish_planes(left, right, planes, 1, 4)
        q1.record()
        torch.cuda.synchronize()
        t_polish += q0.elapsed_time(q1) / 1e3
        valid = tr["valid"].bool()
        dp = d_plain * dmax
        d_pol = torch.where(valid, _disparity(planes, W, H), dp)
        gt = torch.from_numpy(sc.disp_left).cuda()
        m = ~torch.from_numpy(sc.occluded).cuda()
        same = bool((d_b == d_plain).all())
        rows.append({"bad1_plain": float(((dp - gt).abs() > 1)[m].float().mean()) * 100,
                     "bad1_polished": float(((d_pol - gt).abs() > 1)[m].float().mean()) * 100,
                     "epe_plain": float((dp - gt).abs()[m].mean()), "epe_polished": float((d_pol - gt).abs()[m].mean()),
                     "epe_vs_plain": float((d_pol - dp).abs()[m].mean()), "batched_equals_plain": same,
                     "pixels": W * H})
    npx = sum(r["pixels"] for r in rows)
    wavg = lambda k: sum(r[k] * r["pixels"] for r in rows) / npx
    print(json.dumps({"workload": "combined",
                      "config": {"workload": f"{len(pairs)} pairs up to 1920x1080, dmax up to 256, 8 iterations batched, "
                                             "then 4 plane-polishing steps, BASELINE preset, FAST + Philox",
                                 "pixels": npx},
                      "batched_seconds": t_batch, "batched_mpix_iter_per_s": npx * 8 / t_batch / 1e6,
                      "polish_seconds": t_polish, "lanes": bat.batch_info()["lanes"],
                      "quality": {k: wavg(k) for k in ("bad1_plain", "bad1_polished", "epe_plain", "epe_polished",
                                                       "epe_vs_plain")},
                      "batched_equals_plain": all(r["batched_equals_plain"] for r in rows)}), flush=True)
    return 0


def cpu_port_ms(fn, reps=1):
    """Wall time of the oracle port on the host cores (OpenMP, all threads):
    the CPU baseline of the input/output-side workloads."""
    import time
    fn()
    t = time.perf_counter()
    for _ in range(reps):
        fn()
    return (time.perf_counter() - t) * 1e3 / reps


def run_rectify(args):
    """Input-side workload: a 3840x2160 RGBA8 stereo pair undistorted and
    rectified (two warp maps, IWarp::apply's 8-bit sampler), about 264 MB of
    traffic per step (beyond L2).  Algorithmic bytes per output pixel: map 8 +
    source 4 (each texel read about once) + destination 4."""
    import torch
    from cvt_gb300 import imageio, rectify
    W, H = 3840, 2160
    K0 = np.array([[2800.0, 0, 1915.0], [0, 2795.0, 1082.0], [0, 0, 1]], np.float32)
    K1 = np.array([[2790.0, 0, 1925.0], [0, 2788.0, 1076.0], [0, 0, 1]], np.float32)
    c0 = {"K": K0, "radial": np.array([-0.12, 0.04, 0.0], np.float32), "tangential": np.array([1e-4, -2e-4], np.float32)}
    c1 = {"K": K1, "radial": np.array([-0.11, 0.035, 0.0], np.float32), "tangential": np.array([-1e-4, 1e-4], np.float32)}
    a, t = 0.01, np.array([-0.12, 0.001, 0.002])
    E = np.eye(4, dtype=np.float32)
    E[:3, :3] = [[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]]
    E[:3, 3] = t
    rng = np.random.default_rng(5)
    left = torch.from_numpy(rng.integers(0, 256, (H, W, 4), dtype=np.uint8)).cuda()
    right = torch.from_numpy(rng.integers(0, 256, (H, W, 4), dtype=np.uint8)).cuda()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r = rectify.StereoRectification(c0, c1, E, W, H)
    torch.cuda.synchronize()
    e0.record(stream)
    r = rectify.StereoRectification(c0, c1, E, W, H)
    e1.record(stream)
    torch.cuda.synchronize()
    maps_ms = e0.elapsed_time(e1)
    outl, outr = torch.empty_like(left), torch.empty_like(right)
    for _ in range(max(3, args.warmup)):
        r.undistortLeft(left, imageio.RGBA_UINT8, outl)
        r.undistortRight(right, imageio.RGBA_UINT8, outr)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        r.undistortLeft(left, imageio.RGBA_UINT8, outl)
        r.undistortRight(right, imageio.RGBA_UINT8, outr)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    npx = 2 * W * H
    peak, src = peaks()
    gbs = 16.0 * npx / (ms * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle
        hl, hr = left.cpu().numpy(), right.cpu().numpy()
        ml, mr = r.maps[0].cpu().numpy(), r.maps[1].cpu().numpy()
        cms = cpu_port_ms(lambda: (oracle.warp(imageio.RGBA_UINT8, hl, ml), oracle.warp(imageio.RGBA_UINT8, hr, mr)))
        cpu = {"value": npx / 1e6 / (cms * 1e-3), "unit": "Mpix/s", "ms_per_step": cms, "cores": os.cpu_count(),
               "kind": "port", "sample": "the full step: both views warped by the oracle (IWarp::apply's 8-bit "
                                         "sampler restated), OpenMP over rows"}
    print(json.dumps({"workload": "rectify", "metric": "rectified Mpix/s (IWarp::apply, RGBA8, both views)",
                      "value": npx / 1e6 / (ms * 1e-3), "unit": "Mpix/s", "ms_per_step": ms, "steps": args.steps,
                      "maps_ms": maps_ms, "config": {"workload": f"{W}x{H} RGBA8 pair, radial + tangential distortion, "
                                                                 "undistort + rectify both views per step"},
                      "roofline": {"kernel": "k_warp_apply<U8C4>", "bound": "hbm", "achieved": gbs, "peak": peak,
                                   "unit": "GB/s", "frac": gbs / peak, "peak_source": src,
                                   "bytes_per_px": 16}, "cpu_baseline": cpu}), flush=True)
    return 0


def run_tsdf(args):
    """Output-side workload: TSDF fusion into a 512^3 volume of 1 cm voxels
    (1 GB of (tsdf, weight)), per step 4 depth maps of 640x480 integrated and
    one ray cast of 640x480.  Bytes: clear writes 8 per voxel; integration
    reads 8 and writes 8 per voxel inside the truncation band and projects
    every voxel (the depth-map reads stay in L2)."""
    import torch
    from cvt_gb300 import scenes, tsdf
    N = 512
    g2w = np.eye(4, dtype=np.float32)
    g2w[:3, :3] *= 0.01
    g2w[:3, 3] = [-2.56, -2.56, 0.5]
    K = np.array([[525.0, 0, 319.5], [0, 525.0, 239.5], [0, 0, 1]], np.float32)
    spheres = ((0.0, 0.0, 2.6, 0.8), (0.9, -0.4, 2.2, 0.35))
    planes = ((0.0, 0.0, 1.0, 4.5), (0.0, -1.0, 0.0, -1.4))

    def pose(angle, tx):
        E = np.eye(4, dtype=np.float32)
        E[:3, :3] = [[np.cos(angle), 0, np.sin(angle)], [0, 1, 0], [-np.sin(angle), 0, np.cos(angle)]]
        E[:3, 3] = [tx, 0.0, 0.0]
        return E
    poses = [pose(a, tx) for a, tx in ((0.0, 0.0), (0.05, -0.1), (-0.05, 0.1), (0.1, -0.2))]
    depths = [torch.from_numpy(scenes.render_depth(K, E, 640, 480, spheres, planes)).cuda() for E in poses]
    vol = tsdf.TSDFVolume(g2w, N, N, N, truncation=0.04)
    out = torch.empty((480, 640), device="cuda")
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    clear_ms = timed(lambda: vol.clear(), args.steps)
    vol.clear()
    add_ms = timed(lambda: [vol.addDepthMap(K, E, d, 1.0) for E, d in zip(poses, depths)], args.steps) / 4
    ray_ms = timed(lambda: vol.rayCastDepthMap(K, poses[0], 640, 480, -1.0, out=out), args.steps)
    v = vol.volume()
    band = int((v[..., 1] > 0).sum())
    hit = float((out > 0).float().mean())
    err = float(((out - depths[0]).abs()[(out > 0) & (depths[0] > 0)]).median())
    peak, src = peaks()
    nvox = N ** 3
    clear_gbs = 8.0 * nvox / (clear_ms * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle
        hv = oracle.tsdf_clear(N, N, N, 0.0)
        T0, _ = oracle.tsdf_matrices(tsdf.projection(K, poses[0]), g2w)
        hd = depths[0].cpu().numpy()
        cms = cpu_port_ms(lambda: oracle.tsdf_add(hv, hd, 1.0, T0, 0.04))
        cpu = {"value": nvox / (cms * 1e-3) / 1e9, "unit": "Gvoxel/s", "add_ms": cms, "cores": os.cpu_count(),
               "kind": "port", "sample": "one depth map integrated into the 512^3 volume by the oracle "
                                         "(TSDFVolume_add restated), OpenMP over z"}
    print(json.dumps({"workload": "tsdf", "metric": "TSDF integration Gvoxel/s (512^3, 640x480 depth maps)",
                      "value": nvox / (add_ms * 1e-3) / 1e9, "unit": "Gvoxel/s", "steps": args.steps,
                      "add_ms": add_ms, "raycast_ms": ray_ms, "clear_ms": clear_ms,
                      "raycast_mpix_per_s": 640 * 480 / 1e6 / (ray_ms * 1e-3),
                      "voxels_with_weight": band, "raycast_hit_fraction": hit,
                      "raycast_median_abs_error_m": err,
                      "config": {"workload": "512^3 volume of 1 cm voxels, truncation 4 cm, 4 depth maps 640x480 "
                                             "(2 spheres, 2 planes, 4 poses) per step, ray cast from the first pose"},
                      "roofline_clear": {"kernel": "k_tsdf_clear", "bound": "hbm", "achieved": clear_gbs, "peak": peak,
                                         "unit": "GB/s", "frac": clear_gbs / peak, "peak_source": src},
                      "add_bytes_per_launch_algorithmic": 16 * band / 4.0, "cpu_baseline": cpu}), flush=True)
    return 0


def run_gcv(args):
    """The comparison baseline (cvt::StereoGCVFilter) on the headline pair:
    1242x375, disparities 0..127 in steps of 1, both views and the fused
    check (apply), against PatchMatch's bad-1px on the same pair."""
    import torch
    from cvt_gb300 import gcv, scenes
    sc = scene_for(0)
    H, W = sc.left.shape[:2]
    left, right = torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda()
    f = gcv.StereoGCVFilter()
    plan = gcv.plan(W, H, 0.0, DMAX, 1.0)
    stream = torch.cuda.current_stream()
    for _ in range(max(1, args.warmup)):
        f.apply(right, left, 0.0, DMAX, 1.0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        out, d0, d1 = f.apply(right, left, 0.0, DMAX, 1.0)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    disp = d0.cpu().numpy() * DMAX
    bad = scenes.bad_pixel_rate(disp, sc)
    nd = int(DMAX)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle
        cms = cpu_port_ms(lambda: oracle.gcv_apply(sc.right, sc.left, 0.0, DMAX, 1.0), reps=1)
        cpu = {"value": cms, "unit": "ms", "cores": os.cpu_count(), "kind": "port",
               "sample": "the full apply (128 disparities, both views, check) by the oracle's restatement of the "
                         "reference's kernels, OpenMP over rows"}
    print(json.dumps({"workload": "gcv", "metric": "StereoGCVFilter::apply ms (1242x375, 128 disparities, both views)",
                      "value": ms, "unit": "ms", "steps": args.steps,
                      "mpix_disp_per_s": 2 * W * H * nd / 1e6 / (ms * 1e-3),
                      "launches_per_apply": 2 * plan["launches"] + 1, "disparities_per_batch": plan["batch"],
                      "bad1_nonocc_pct_left_view": bad, "cpu_baseline": cpu,
                      "config": {"workload": "pair 0 of the headline scene family (1242x375, dmax 128), point cost, "
                                             "guided filter r 9, eps 1e-3; right image as cam0, left as cam1"}}), flush=True)
    return 0


def run_pipeline(args):
    """The product path from files, per step: a 1242x375 8-bit RGB PNG pair
    decoded on the host, copied to the device, rectified (undistort + rectify
    maps, IWarp::apply's 8-bit sampler), PatchMatch depthMap on the 8-bit
    images (read as read_imagef reads them), disparityToDepthmap and TSDF
    integration into a 256^3 volume.  Host stages by wall clock, device
    stages by CUDA events on the launching stream."""
    import tempfile
    import torch
    from cvt_gb300 import imageio, rectify, scenes, tsdf, vision
    from cvt_gb300.stereo import PMHuberStereo
    sc = scene_for(0)
    H, W = sc.left.shape[:2]
    tmp = tempfile.mkdtemp()
    paths = []
    for name, img in (("left", sc.left), ("right", sc.right)):
        a = np.round(np.clip(img, 0.0, 1.0) * 255).astype(np.uint8)
        path = os.path.join(tmp, name + ".png")
        imageio.write_png(path, np.ascontiguousarray(a), imageio.RGBA_UINT8)
        paths.append(path)
    f = 700.0
    K = np.array([[f, 0, W / 2 - 0.5], [0, f, H / 2 - 0.5], [0, 0, 1]], np.float32)
    cam = {"K": K, "radial": np.array([-1e-3, 0.0, 0.0], np.float32), "tangential": np.zeros(2, np.float32)}
    # a 54 cm baseline with the small misalignment of a real rig: the
    # reference's rectification is NaN for a baseline exactly along x (the
    # axis of its zero alignment rotation), and so is this mirror of it
    a = 0.002
    E = np.eye(4, dtype=np.float32)
    E[:3, :3] = [[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]]
    E[:3, 3] = [-0.54, 0.004, 0.002]
    rect = rectify.StereoRectification(cam, cam, E, W, H)
    st = PMHuberStereo(0, params_for("ours"))
    g2w = np.eye(4, dtype=np.float32)
    g2w[:3, :3] *= 0.05
    g2w[:3, 3] = [-6.4, -3.2, 2.0]
    vol = tsdf.TSDFVolume(g2w, 256, 256, 256, truncation=0.2)
    stream = torch.cuda.current_stream()
    dmap = torch.empty((H, W), device="cuda")
    stages = {k: [] for k in ("png_decode", "h2d", "rectify", "depthmap", "depth", "tsdf_add", "total")}

    def step(record):
        t0 = time.perf_counter()
        hl, _ = imageio.read_png(paths[0])
        hr, _ = imageio.read_png(paths[1])
        t1 = time.perf_counter()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        ev[0].record(stream)
        dl, dr = torch.from_numpy(hl).cuda(non_blocking=False), torch.from_numpy(hr).cuda(non_blocking=False)
        ev[1].record(stream)
        rl = rect.undistortLeft(dl, imageio.RGBA_UINT8)
        rr = rect.undistortRight(dr, imageio.RGBA_UINT8)
        ev[2].record(stream)
        st.depthMapImage(dmap, rl, imageio.RGBA_UINT8, rr, imageio.RGBA_UINT8, PATCH, DMAX, ITERS, 4)
        ev[3].record(stream)
        depth = vision.disparityToDepthmap(dmap, DMAX, f, 0.54)
        ev[4].record(stream)
        vol.addDepthMap(K, np.eye(4, dtype=np.float32), depth, 1.0)
        ev[5].record(stream)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if record:
            stages["png_decode"].append((t1 - t0) * 1e3)
            for k, (a, b) in zip(("h2d", "rectify", "depthmap", "depth", "tsdf_add"), zip(ev, ev[1:])):
                stages[k].append(a.elapsed_time(b))
            stages["total"].append((t2 - t0) * 1e3)

    vol.clear()
    for _ in range(max(1, args.warmup)):
        step(False)
    for _ in range(args.steps):
        step(True)
    ms = {k: float(np.mean(v)) for k, v in stages.items()}
    v = vol.volume()
    print(json.dumps({"workload": "pipeline", "metric": "pairs/s from PNG files to a fused TSDF volume",
                      "value": 1e3 / ms["total"], "unit": "pairs/s", "steps": args.steps,
                      "ms_per_stage": ms, "voxels_with_weight": int((v[..., 1] > 0).sum()),
                      "config": {"workload": f"{W}x{H} 8-bit RGBA PNG pair (the headline scene), rectification "
                                             "maps of a 0.54 m rig with radial distortion, PatchMatch 35x35 / dmax 128 / 8 "
                                             "iterations (FAST + Philox), f 700 px, baseline 0.54 m, "
                                             "256^3 TSDF of 5 cm voxels"}}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--ref-rows", type=int, default=48)
    ap.add_argument("--ref-cols", type=int, default=640)
    ap.add_argument("--ref-iters", type=int, default=ITERS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batch and adjoint sub-records")
    ap.add_argument("--profile", action="store_true", help="short run for ncu captures")
    ap.add_argument("--profile-iters", type=int, default=1)
    ap.add_argument("--workload", choices=["pair", "batch", "adjoint", "combined", "rectify", "tsdf", "gcv", "pipeline"],
                    default="pair",
                    help="pair: the 1242x375 headline; batch: uneven pairs, plain loop vs batched graph; "
                         "adjoint: forward + adjoint, 8 x 640x480; combined: 16 pairs batched + plane polishing")
    ap.add_argument("--pairs", type=int, default=64)
    ap.add_argument("--batch-iters", type=int, default=5)
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "gcv":
        return run_gcv(args)
    if args.workload == "pipeline":
        return run_pipeline(args)
    if args.workload == "rectify":
        return run_rectify(args)
    if args.workload == "tsdf":
        return run_tsdf(args)
    if args.workload == "combined":
        if args.pairs == 64:
            args.pairs = 16
        return run_combined(args)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
    try:
        return run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as tdist
            tdist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
