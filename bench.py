#!/usr/bin/env python
"""BC1 encoder benchmark: Gpixel/s per quality level on the quality-sweep workload.

Workload (one "step"): the 4096x4096 RGBA8 quality-sweep image (seeded
gradients + 4-octave value noise + rectangles, 5% single-colour and 5%
near-black blocks, alpha from a second noise field) encoded at every quality
level 0..9 with color_weights {0.299, 0.587, 0.114}, input_weights =
alpha / 255, D3D10, three_color_mode = three_color_black = true.  The
headline value is the whole sweep's throughput: 10 x 16.8 Mpx / step time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU implementation of the same path (the C
restatement of the reference's scalar encoder, every host thread) on a bounded
sample of the same workload.  Under torchrun each rank encodes its own replica
(the path has no exchange step); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import gc
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

METRIC = "BC1 Gpixel/s per quality level, batched vs plain, bit-exact; serving p50/p99 ms"
UNIT = "Gpixel/s"
CW = (0.299, 0.587, 0.114)
LEVELS = list(range(10))

# Algorithmic FP32 operations per unit of work, counted from the reference's
# scalar encoder (icbc.h v1.05): one op per float add/sub/mul/div/compare/
# min/max/abs/convert executed by the ICBC_SIMD=0 build.
OPS_PER_UNIT = {
    "cf4_combos": 140,     # cluster_fit_four iteration, icbc.h:2650-2733
    "cf3_combos": 123,     # cluster_fit_three iteration, icbc.h:2273-2335
    "refine_steps": 996,   # refine_endpoints step: palette, compute_indices, evaluate_mse, icbc.h:3614-3648
    "out4_blocks": 950,    # output_block4: 565 quantise, palette, compute_indices4, evaluate_mse
    "out3_blocks": 915,    # output_block3
    "single_blocks": 283,  # single-colour path + evaluate_mse, icbc.h:3761-3764
    "sat_builds": 151,     # compute_sat fixed part: power iterations, normalisation
    "sat_points": 37,      # compute_sat per colour: centroid, covariance, projection, prefix sums
    "reduce_pairs": 9,     # reduce_colors equal() test
    "reduce_merges": 13,   # reduce_colors weighted merge
    "box_fits": 41,        # inset_bbox + select_diagonal fixed part
    "box_points": 13,      # fit_colors_bbox + select_diagonal per colour
    "lsq_fits": 378,       # optimize_end_points4
}
REDUCE_PER_BLOCK = 64      # reduce_colors per-texel tests (levels 2..9)


# DRAM bytes per level call (dram__bytes_read.sum + dram__bytes_write.sum of
# its launches: the first pass, the listed pass and, at level 9, the
# refinement pass) from one ncu capture of this workload without cache
# flushes between kernels, as a timed call runs.  Level 8's
# figure includes ~46 MB of write-backs of the buffer that flushes L2 before
# the step; level 9's is its own traffic (the image is read once, through L2).
NCU_TRAFFIC_BYTES = {8: (67.18e6 + 48.94e6) + (20.45e6 + 12.09e6),
                     9: (15.97e6 + 9.10e6) + (21.56e6 + 7.68e6) + (11.61e6 + 7.52e6)}
TRAFFIC_SOURCE = "one ncu capture of this workload with --cache-control none: dram__bytes_read.sum + " \
                 "dram__bytes_write.sum summed over the level call's launches"


def launches_per_level(level: int) -> int:
    """Kernel launches of one level call on the RGBA8 image: levels 2-9 run in
    two passes (blocks of 0 or 1 colours, then the listed rest), level 9 adds
    its refinement pass."""
    return 1 if level < 2 else 3 if level == 9 else 2


def level_kernels(level: int) -> str:
    """The launches of one level call on the RGBA8 image with alpha weights
    (the default shapes: a CTA-wide listed pass from level 4 on)."""
    if level < 2:
        return "k_encode_image<%d>" % level
    listed = "k_image_listed<%d>" % level if level < 4 else "k_image_listed_cta<%d, %d, 16>" % (level, level == 9)
    return "k_image_trivial<%d> + %s" % (level, listed) + (" + k_refine<1>" if level == 9 else "")


def algorithmic_ops(stats: dict, level: int) -> float:
    ops = sum(OPS_PER_UNIT[k] * stats.get(k, 0) for k in OPS_PER_UNIT)
    if level >= 2:
        ops += REDUCE_PER_BLOCK * stats["blocks"]
    return float(ops)


def load_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        p["source"] = "measured"
        return p
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "fallback"}


def fp32_peak_tops(peaks: dict, sms: int) -> float:
    """Non-FMA FP32 peak: 128 lanes per SM x SMs x max SM clock (ops/s / 1e12)."""
    return 128 * sms * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""
    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self.proc = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            time.sleep(0.5)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [x.strip() for x in line.split(",")]))

    def mark(self, begin: bool):
        if begin:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.2)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        inside = [r for t, r in self.rows if self.t0 and self.t1 and self.t0 <= t <= self.t1 + 0.05]
        if not inside:
            inside = [r for _, r in self.rows]
        sm = [float(r[1]) for r in inside if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in inside if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in inside:
            if len(r) > 8:
                for name, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(inside)}


def sample_rows(img: np.ndarray, stride: int) -> np.ndarray:
    """Every stride-th row of 4x4 blocks (whole blocks, same width)."""
    h = img.shape[0]
    rows = [img[y:y + 4] for y in range(0, h - h % 4, 4 * stride)]
    return np.ascontiguousarray(np.concatenate(rows, axis=0))


# The two CPU forms of the reference encoder that are timed: the scalar build
# (ICBC_SIMD=0, the oracle's plain loops; what the reference compiles to when
# its SIMD detection finds nothing) and the NEON build (ICBC_SIMD=-1) with its
# cluster loops run as 4-lane vector code, as that build runs them.
CPU_FORMS = {"scalar": {"profile": 0, "vector": False, "build": "scalar build (ICBC_SIMD=0)"},
             "neon-vector": {"profile": 6, "vector": True,
                             "build": "NEON build (ICBC_SIMD=-1): cluster loops as 4-lane vectors"}}


def cpu_sweep(img_sample: np.ndarray, nthreads: int, levels=None, form: str = "scalar"):
    """Times a CPU form of the reference encoder (the oracle, a C restatement)
    on the sample."""
    from oracle import oracle as O
    O.lib()  # build/load outside the timed region
    levels = LEVELS if levels is None else levels
    f = CPU_FORMS[form]
    times, stats, outs = {}, {}, {}
    for lv in levels:
        t0 = time.perf_counter()
        b, _, st = O.encode_image(img_sample, lv, 0, CW, 1, None, True, True, nthreads=nthreads, with_stats=True,
                                  profile=f["profile"], vector=f["vector"])
        times[lv] = time.perf_counter() - t0
        stats[lv] = st
        outs[lv] = b
    return times, stats, outs


def block_texels(img: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """RGBA8 texels (len(idx), 64) of blocks idx (row-major block order) with
    edge replication, as the encoder reads them."""
    h, w = img.shape[:2]
    bw = (w + 3) // 4
    by, bx = np.asarray(idx) // bw, np.asarray(idx) % bw
    ys = np.minimum(by[:, None] * 4 + np.arange(4)[None, :], h - 1)
    xs = np.minimum(bx[:, None] * 4 + np.arange(4)[None, :], w - 1)
    return np.ascontiguousarray(img[ys[:, :, None], xs[:, None, :]].reshape(len(idx), 64))


def parity(gpu: np.ndarray, ref: np.ndarray, img: np.ndarray, decoder: int) -> dict:
    """Bit-exactness of every block against the oracle: the mismatch count and,
    over mismatching blocks, the worst relative difference of their
    evaluate_bc1_error (icbc.h:3030-3046) from the oracle block's."""
    from oracle import oracle as O
    bad = np.flatnonzero((gpu.reshape(-1, 8) != ref.reshape(-1, 8)).any(1))
    worst = 0.0
    if bad.size:
        tex = block_texels(img, bad)
        eg = O.evaluate_bc1_error(tex, gpu.reshape(-1, 8)[bad], decoder).astype(np.float64)
        er = O.evaluate_bc1_error(tex, ref.reshape(-1, 8)[bad], decoder).astype(np.float64)
        worst = float(np.max(np.abs(eg - er) / np.maximum(er, 1e-30)))
    return {"blocks_checked": int(gpu.size // 8), "mismatches": int(bad.size), "worst_rel_error_delta": worst}


def rmse_psnr(img: np.ndarray, blocks: np.ndarray, decoder: int):
    """RMSE and PSNR of an encoded image from the oracle's FP64 decode and
    compare over every block texel, as icbc_test.cpp:309-324 computes them:
    mse = sum of evaluate_bc1_error / (16 * blocks), PSNR clamped to
    [0, 300] dB (1e10 for an exact image)."""
    from oracle import oracle as O
    nb = blocks.size // 8
    mse = O.image_sse(img, blocks, decoder) / (16.0 * nb)
    rms = float(np.sqrt(mse))
    psnr = float(min(max(20.0 * np.log10(255.0 / rms), 0.0), 300.0)) if rms > 0 else 1e10
    return rms, psnr, mse


def max_over_ranks(value: float, device) -> float:
    """The largest of every rank's value (the job's time is its slowest rank)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gpix(world: int, pixels_per_rank: float, step_ms_max: float) -> float:
    """Whole-job Gpixel/s: every rank encodes its own replica of the step's
    pixels; the step takes as long as the slowest rank."""
    return world * pixels_per_rank / (step_ms_max * 1e-3) / 1e9


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def sample_text(stride: int, px: int) -> str:
    if stride == 1:
        return "the whole workload: all 10 levels of the image (%d px per level)" % px
    return "every %dth block row of the workload (%d px per level), all 10 levels" % (stride, px)


def sweep_config(size: int, ws: int) -> dict:
    """The workload's config, the same in both arms' lines."""
    return {"workload": "quality_sweep_%dx%d_L0-9" % (size, size), "levels": LEVELS, "color_weights": CW,
            "input_weights": "alpha/255", "decoder": "D3D10", "three_color_mode": True, "three_color_black": True,
            "form": "plain: one call per level (1 launch at levels 0-1, 2 at levels 2-8, 3 at level 9)",
            "l2": "flushed between steps (256 MB write outside the timed events)",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    from icbc_gb300 import synth
    img = synth.quality_sweep_image(args.size, args.size, seed=1)
    sample = sample_rows(img, args.cpu_stride)
    px = sample.shape[0] * sample.shape[1]
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sweep(sample, nthreads, levels=[0, 9], form=args.cpu_form)
    step_times = []
    per_level = {lv: [] for lv in LEVELS}
    for _ in range(args.steps):
        times, _, outs = cpu_sweep(sample, nthreads, levels=LEVELS, form=args.cpu_form)
        step_times.append(sum(times.values()))
        for lv in LEVELS:
            per_level[lv].append(times[lv])
    t = statistics.mean(step_times)
    value = len(LEVELS) * px / t / 1e9
    # The other form, one untimed-by-the-contract sweep, for comparison.
    other = "scalar" if args.cpu_form != "scalar" else "neon-vector"
    otimes, _, oouts = cpu_sweep(sample, nthreads, levels=LEVELS, form=other)
    # Blocks where the NEON form's output differs from the scalar build's.
    neon_outs, scalar_outs = (outs, oouts) if args.cpu_form != "scalar" else (oouts, outs)
    neon_diff = {str(lv): int((neon_outs[lv] != scalar_outs[lv]).any(1).sum()) for lv in LEVELS}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": sweep_config(args.size, ws),
        "per_level": {str(lv): len(per_level[lv]) and px / statistics.mean(per_level[lv]) / 1e9 for lv in LEVELS},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample_text(args.cpu_stride, px), "build": CPU_FORMS[args.cpu_form]["build"],
                         "ms_per_step_mean_min": [t * 1e3, min(step_times) * 1e3],
                         other: {"value": len(LEVELS) * px / sum(otimes.values()) / 1e9,
                                 "build": CPU_FORMS[other]["build"]},
                         "neon_blocks_differing_from_scalar": {"total": sum(neon_diff.values()),
                                                               "blocks_per_level": len(outs[LEVELS[0]]),
                                                               "per_level": neon_diff}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    import torch.distributed as dist

    import icbc_gb300 as ig
    from icbc_gb300 import synth

    ws, rank, local = dist_info()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    ig.init(ig.Decoder_D3D10)
    sms = ig.load().icbc_gpu_sm_count()
    if args.cta_warps:
        for lv in range(2, 10):
            g, p, _ = ig.get_launch_config(lv)
            ig.set_launch_config(lv, g, p, args.cta_warps)
    if args.only_hard:  # profiling runs of the hard-mixture leg alone
        peak = fp32_peak_tops(load_peaks(), sms)
        print(json.dumps({"hard": hard_leg(ig, torch, dev, args, peak), "profiling_run": True}))
        return

    img = synth.quality_sweep_image(args.size, args.size, seed=1)
    h, w = img.shape[:2]
    px = h * w
    nb = ig.blocks_of(w, h)
    d_img = torch.from_numpy(img).to(dev)
    outs = {lv: torch.zeros((nb, 8), dtype=torch.uint8, device=dev) for lv in LEVELS}
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def encode(lv):
        ig.compress_image(d_img, lv, ig.Decoder_D3D10, CW, weight_mode=ig.WEIGHTS_ALPHA, out=outs[lv], stream=stream)

    # Launch shapes per level picked by the autotuner on this workload (outside
    # the timed region).
    tuning = None
    if not args.no_autotune:
        table = ig.autotune(d_img, LEVELS, color_weights=CW, weight_mode=ig.WEIGHTS_ALPHA)
        tuning = {str(lv): "%d groups/warp, %s%s" % (t["groups_per_warp"], "persistent" if t["persistent"] else
                                                      "hw-balanced",
                                                      ", listed pass %d-warp CTAs" % t["cta_warps"] if lv >= 2 else "")
                  for lv, t in table.items()}

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            for lv in LEVELS:
                encode(lv)
    torch.cuda.synchronize()

    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in LEVELS]
          for _ in range(args.steps)]
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.mark(True)
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()  # L2 flush (256 MB written) between steps, outside the timed events
            for i, lv in enumerate(LEVELS):
                ev[k][i][0].record(stream)
                encode(lv)
                ev[k][i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clocks.mark(False)
    if ws > 1:
        dist.barrier()
    clk = clocks.stop()
    lvl_ms = {lv: statistics.mean(ev[k][i][0].elapsed_time(ev[k][i][1]) for k in range(args.steps))
              for i, lv in enumerate(LEVELS)}
    step_ms = sum(lvl_ms.values())
    step_ms = max_over_ranks(step_ms, dev) if ws > 1 else step_ms
    value = whole_job_gpix(ws, len(LEVELS) * px, step_ms)

    # End to end through the host-buffer C-ABI call: pinned image in, blocks out.
    e2e = None
    if not args.no_e2e:
        e2e = e2e_leg(ig, torch, img, nb, px, ws, args)
    if rank != 0:
        return
    batch = None if (args.no_batch or args.no_cpu_baseline) else batch_leg(ig, torch, dev, args)
    serving = None
    if not (args.no_serve or args.no_cpu_baseline):
        serving = serving_leg(ig, args, batch["batched"]["gpix_s"] if batch else None)
    if args.no_cpu_baseline:
        print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": step_ms, "levels": LEVELS,
                          "per_level_ms": lvl_ms, "e2e": e2e and e2e["value"], "clocks": clk,
                          "profiling_run": True}))
        return
    # CPU baseline, algorithmic op counts and complete parity: the oracle
    # encodes the workload (every block of every level; stride 1 by default)
    # on every host thread, timed as the CPU baseline, and every GPU block is
    # compared with it, outside the timed region.
    sample = img if args.cpu_stride == 1 else sample_rows(img, args.cpu_stride)
    sample_px = sample.shape[0] * sample.shape[1]
    nthreads = os.cpu_count() or 1
    ctimes, cstats, couts = cpu_sweep(sample, nthreads, levels=LEVELS)
    cpu_scalar = len(LEVELS) * sample_px / sum(ctimes.values()) / 1e9
    vtimes, _, vouts = cpu_sweep(sample, nthreads, levels=LEVELS, form="neon-vector")
    neon_diff = {str(lv): int((vouts[lv] != couts[lv]).any(1).sum()) for lv in LEVELS}
    cpu_value = len(LEVELS) * sample_px / sum(vtimes.values()) / 1e9
    bw = w // 4
    rows = list(range(0, h // 4, args.cpu_stride))
    checks, quality = {}, {}
    for lv in LEVELS:
        gpu = outs[lv].cpu().numpy()
        gsample = gpu.reshape(h // 4, bw, 8)[rows].reshape(-1, 8)
        checks[str(lv)] = parity(gsample, couts[lv], sample, 0)
        rms, psnr, _ = rmse_psnr(img, gpu, 0)
        quality[str(lv)] = {"rmse": rms, "psnr_db": psnr}
    scale = nb / cstats[LEVELS[0]]["blocks"]
    ops = {lv: algorithmic_ops(cstats[lv], lv) * scale for lv in LEVELS}
    peaks = load_peaks()
    peak = fp32_peak_tops(peaks, sms)
    hard = None if args.no_hard else hard_leg(ig, torch, dev, args, peak)
    top = max(LEVELS, key=lambda lv: lvl_ms[lv])
    achieved = ops[top] / (lvl_ms[top] * 1e-3) / 1e12
    per_level = {str(lv): {"gpix_s": px / (lvl_ms[lv] * 1e-3) / 1e9, "ms": lvl_ms[lv],
                           "fp32_frac": ops[lv] / (lvl_ms[lv] * 1e-3) / 1e12 / peak,
                           "cpu_gpix_s": sample_px / vtimes[lv] / 1e9,
                           "cpu_scalar_gpix_s": sample_px / ctimes[lv] / 1e9} for lv in LEVELS}
    hbm = peaks.get("hbm_gbs", 6800.0)
    l0_bytes = px * 4 + nb * 8
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": sweep_config(w, ws),
        "per_level": per_level,
        "parity": {"against": "oracle (C restatement of the reference's scalar encoder, pinned to the compiled "
                              "reference)", "per_level": checks,
                   "blocks_checked": sum(c["blocks_checked"] for c in checks.values()),
                   "mismatches": sum(c["mismatches"] for c in checks.values())},
        "quality": {"how": "FP64 decode-and-compare of the GPU blocks (oracle decode): RMSE and PSNR per level "
                           "image, icbc_test.cpp:309-324", "per_level": quality},
        "roofline": {"bound": "fp32", "kernel": level_kernels(top), "achieved": achieved, "peak": peak,
                     "unit": "Tops/s", "frac": achieved / peak, "traffic": NCU_TRAFFIC_BYTES.get(top),
                     "traffic_unit": "bytes per level call", "traffic_source": TRAFFIC_SOURCE,
                     "peak_source": "128 FP32 lanes x %d SMs x %s MHz (%s sm_max_mhz)" % (
                         sms, peaks.get("sm_max_mhz"), peaks["source"])},
        "roofline_hbm_level0": ({"bound": "hbm", "achieved": l0_bytes / (lvl_ms[0] * 1e-3) / 1e9, "peak": hbm,
                                 "unit": "GB/s", "frac": l0_bytes / (lvl_ms[0] * 1e-3) / 1e9 / hbm,
                                 "traffic": None} if 0 in lvl_ms else None),
        "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample_text(args.cpu_stride, sample_px),
                         "build": CPU_FORMS["neon-vector"]["build"],
                         "scalar": {"value": cpu_scalar, "build": CPU_FORMS["scalar"]["build"]},
                         "neon_blocks_differing_from_scalar": {"total": sum(neon_diff.values()),
                                                               "blocks_per_level": int(couts[LEVELS[0]].shape[0]),
                                                               "per_level": neon_diff}},
        "e2e": {"value": e2e["value"] if e2e else None, "unit": UNIT,
                "h2d_bytes_per_step": e2e["h2d"] if e2e else None, "d2h_bytes_per_step": e2e["d2h"] if e2e else None,
                "path": "icbc_gpu_compress_bc1_image_host, pinned host buffers, 10 calls per step",
                "steps": e2e["steps"] if e2e else None, "ms_per_step_min_max": e2e["min_max"] if e2e else None,
                "per_level_ms": e2e["per_level_ms"] if e2e else None},
        "autotune": tuning,
        "batch": batch,
        "serving": serving,
        "hard": hard,
        "gpu_launches": args.steps * sum(launches_per_level(lv) for lv in LEVELS),
        "clocks": clk,
        "wall_s_timed": wall,
    }
    print(json.dumps(line))


def e2e_leg(ig, torch, img, nb, px, ws, args):
    """Same metric through the host-buffer C-ABI call: pinned image in, blocks
    out, host<->device copies inside the timed region; as many steps as the
    device-timed leg, each step's wall time taken separately."""
    pin = torch.from_numpy(img).pin_memory()
    host_img = pin.numpy()
    host_out = {lv: torch.zeros((nb, 8), dtype=torch.uint8).pin_memory().numpy() for lv in LEVELS}
    for lv in LEVELS:
        ig.compress_image_host(host_img, lv, ig.Decoder_D3D10, CW, ig.WEIGHTS_ALPHA, out=host_out[lv])
    steps = max(3, args.steps)
    times = []
    per_level = {lv: [] for lv in LEVELS}
    for _ in range(steps):
        t0 = time.perf_counter()
        for lv in LEVELS:
            tl = time.perf_counter()
            ig.compress_image_host(host_img, lv, ig.Decoder_D3D10, CW, ig.WEIGHTS_ALPHA, out=host_out[lv])
            per_level[lv].append(time.perf_counter() - tl)
        times.append(time.perf_counter() - t0)
    t = statistics.mean(times)
    if ws > 1:  # the job's time is its slowest rank's
        t = max_over_ranks(t * 1e3, torch.device("cuda", torch.cuda.current_device())) * 1e-3
    h2d = len(LEVELS) * img.nbytes + sum(nb * 8 for lv in LEVELS if lv >= 4)
    d2h = len(LEVELS) * nb * 8
    return {"value": ws * len(LEVELS) * px / t / 1e9, "h2d": h2d, "d2h": d2h, "steps": steps,
            "min_max": [min(times) * 1e3, max(times) * 1e3],
            "per_level_ms": {str(lv): statistics.mean(per_level[lv]) * 1e3 for lv in LEVELS}}


def batch_leg(ig, torch, dev, args):
    """Mixed-size batch: 2,000 images (sides log-uniform 64..2048, 10% not
    multiples of 4), random level 0..9 and decoder D3D10/NVIDIA/AMD, uniform
    weights, cw {1,1,1}.  Content: crops of gradient/noise/rectangle textures.
    Times the plain form (one launch per image) against the batched form
    (one persistent launch, replayed graph), checks both give the same bytes."""
    from icbc_gb300 import synth
    specs = synth.batch_specs(args.batch_images, seed=7)
    host_bases = [synth.gradient_noise_rects(2048, 2048, 100 + k) for k in range(4)]
    bases = [torch.from_numpy(b).to(dev) for b in host_bases]
    imgs, outs_plain, outs_batch, descs, crops = [], [], [], [], []
    px = 0
    for i, s in enumerate(specs):
        y0 = (s.seed * 131) % (2049 - s.height)
        x0 = (s.seed * 197) % (2049 - s.width)
        img = bases[i % len(bases)][y0:y0 + s.height, x0:x0 + s.width].contiguous()
        crops.append((i % len(bases), y0, x0))
        nb = ig.blocks_of(s.width, s.height)
        imgs.append(img)
        outs_plain.append(torch.zeros((nb, 8), dtype=torch.uint8, device=dev))
        ob = torch.zeros((nb, 8), dtype=torch.uint8, device=dev)
        outs_batch.append(ob)
        descs.append(ig.image_desc(img, s.level, ob, None, s.decoder))
        px += s.width * s.height
    del bases
    stream = torch.cuda.Stream(device=dev)
    plain_descs = [ig.image_desc(img, s.level, o, None, s.decoder) for s, img, o in zip(specs, imgs, outs_plain)]

    def plain():
        ig.compress_images_each(plain_descs, stream)

    # The batched form's CTA size, tuned on this batch (outside the timed region).
    tuned = ig.autotune_batch(descs, stream=stream) if not args.no_autotune else None
    batch = ig.Batch(descs)
    with torch.cuda.stream(stream):
        plain()
        batch.launch(stream)
    torch.cuda.synchronize()
    same = all(torch.equal(a, b) for a, b in zip(outs_plain, outs_batch))
    res = {}
    for name, fn in (("plain", plain), ("batched", lambda: batch.launch(stream))):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            fn()
            e0.record(stream)
            for _ in range(args.batch_steps):
                fn()
            e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.batch_steps
        res[name] = {"ms": ms, "gpix_s": px / (ms * 1e-3) / 1e9}
    batch.close()
    # Every image against the oracle (all blocks), and its RMSE / PSNR from
    # the FP64 decode-and-compare; one image per host thread at a time.
    from oracle import oracle as O
    O.lib()
    host_out = [o.cpu().numpy() for o in outs_batch]

    def check(i):
        s = specs[i]
        k, y0, x0 = crops[i]
        img = np.ascontiguousarray(host_bases[k][y0:y0 + s.height, x0:x0 + s.width])
        ob, _ = O.encode_image(img, s.level, s.decoder, (1, 1, 1), 0, None, True, True, nthreads=1)
        pr = parity(host_out[i], ob, img, s.decoder)
        rms, psnr, mse = rmse_psnr(img, host_out[i], s.decoder)
        return pr, rms, psnr, mse

    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        results = list(ex.map(check, range(len(specs))))
    mism = sum(r[0]["mismatches"] for r in results)
    worst = max(r[0]["worst_rel_error_delta"] for r in results)
    psnrs = np.array([r[2] for r in results])
    rmses = np.array([r[1] for r in results])
    nbs = np.array([ig.blocks_of(s.width, s.height) for s in specs], np.float64)
    agg_mse = float(np.sum([r[3] for r in results] * nbs) / nbs.sum())
    by_level = {}
    for lv in range(10):
        sel = [i for i, s in enumerate(specs) if s.level == lv]
        if sel:
            m = float(np.sum([results[i][3] * nbs[i] for i in sel]) / nbs[sel].sum())
            by_level[str(lv)] = {"images": len(sel), "rmse": float(np.sqrt(m)),
                                 "psnr_db": float(20 * np.log10(255.0 / np.sqrt(m))) if m > 0 else 1e10}
    q = lambda a, p: float(np.percentile(a, p))  # noqa: E731
    return {"workload": "mixed_batch_%d_images" % len(specs), "pixels": px,
            "plain": res["plain"], "batched": res["batched"],
            "speedup_batched_over_plain": res["plain"]["ms"] / res["batched"]["ms"],
            "batched_equals_plain": bool(same),
            "parity": {"images_checked": len(specs), "blocks_checked": int(nbs.sum()), "mismatches": mism,
                       "worst_rel_error_delta": worst},
            "quality": {"how": "FP64 decode-and-compare per image (icbc_test.cpp:309-324), aggregate weighted by "
                               "blocks as the reference driver sums it",
                        "rmse": float(np.sqrt(agg_mse)), "psnr_db": float(20 * np.log10(255.0 / np.sqrt(agg_mse))),
                        "per_image_rmse_min_p50_max": [float(rmses.min()), q(rmses, 50), float(rmses.max())],
                        "per_image_psnr_min_p1_p50_p99_max": [float(psnrs.min()), q(psnrs, 1), q(psnrs, 50),
                                                              q(psnrs, 99), float(psnrs.max())],
                        "per_level": by_level},
            "launches_plain": len(specs), "launches_batched": 1,
            "autotune": tuned and {"batch_cta_warps": tuned["batch_cta_warps"],
                                   "candidates_ms": {str(k): v for k, v in tuned["candidates"].items()}}}


def serving_leg(ig, args, batched_gpix):
    """Serving workload: Poisson arrivals, sides {64..2048} with probabilities
    {.30,.25,.20,.15,.07,.03}, level uniform 0..9, D3D10, 40 GB HBM budget.
    Latency is submit -> blocks in the caller's host buffer."""
    from icbc_gb300 import synth
    bases = [synth.gradient_noise_rects(2048, 2048, 300 + k) for k in range(2)]
    pool = {}
    for side in synth.SERVING_SIDES:
        crops = []
        for k in range(3):
            y0, x0 = (k * 389) % (2049 - side), (k * 211) % (2049 - side)
            crops.append(np.ascontiguousarray(bases[k % 2][y0:y0 + side, x0:x0 + side]))
        pool[side] = crops
    # Untimed warm-up: one request of every side and level through a server
    # (first launches, callback and delivery threads, allocator state).
    warm = ig.Server(40 << 30, max_inflight=args.serve_inflight, max_batch_images=1024)
    wids = [warm.submit(pool[side][0], lv, ig.Decoder_D3D10,
                        out=np.zeros((ig.blocks_of(side, side), 8), np.uint8))
            for side in synth.SERVING_SIDES for lv in range(10)]
    for rid in wids:
        warm.wait(rid, 120000)
    warm.close()
    def run_once(rate):
        n = int(min(args.serve_max_requests, max(400, rate * args.serve_seconds)))
        reqs = synth.serving_requests(n, rate, seed=int(rate))
        # The callers' result buffers exist, touched, before the requests
        # arrive (a client reuses its buffers): fresh pages would put the
        # kernel's first-touch faults and zeroing on the delivery path.
        outs = [np.empty((ig.blocks_of(r.side, r.side), 8), np.uint8) for r in reqs]
        for o in outs:
            o.fill(0)
        srv = ig.Server(40 << 30, max_inflight=args.serve_inflight, max_batch_images=1024)
        ids = [None] * n
        nthreads = args.serve_threads

        def submitter(k, t0):
            # Thread k submits requests k, k + nthreads, ... at their arrival
            # times (ctypes releases the GIL inside the call).  Waits sleep
            # (releasing the GIL) down to 50 us instead of spinning, so the
            # submitting threads do not hold each other up by a switch interval.
            for i in range(k, n, nthreads):
                r = reqs[i]
                while True:
                    dt = r.arrival_s - (time.perf_counter() - t0)
                    if dt <= 0:
                        break
                    if dt > 5e-5:
                        time.sleep(dt * 0.8)
                ids[i] = srv.submit(pool[r.side][i % 3], r.level, ig.Decoder_D3D10, out=outs[i])

        # No garbage-collector pause inside the timed run: one would hold the
        # submitting threads and release their requests in a burst.
        gc.collect()
        gc.disable()
        t0 = time.perf_counter()
        threads = [threading.Thread(target=submitter, args=(k, t0)) for k in range(nthreads)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        submit_span = time.perf_counter() - t0
        for rid in ids:
            srv.wait(rid, 120000)
        wall = time.perf_counter() - t0
        gc.enable()
        st = srv.stats()
        srv.close()
        px = sum(r.side * r.side for r in reqs)
        return {"rate_req_s": rate, "requests": n, "offered_gpix_s": px / reqs[-1].arrival_s / 1e9,
                "achieved_submit_rate_req_s": n / submit_span, "submit_threads": nthreads,
                "gpix_s": st["pixels_completed"] / wall / 1e9, "p50_ms": st["latency_p50_ms"],
                "p99_ms": st["latency_p99_ms"], "mean_ms": st["latency_mean_ms"], "max_ms": st["latency_max_ms"],
                "batches": st["batches"], "arena_peak_bytes": st["arena_peak"], "completed": st["completed"]}

    # Each rate runs serve_repeats times (a fresh server each time); the
    # line reports the run with the median p99 and lists every run's
    # Gpixel/s, p50 and p99 (the host is shared, so a run can catch a stall
    # of the machine's other work).
    runs = []
    for rate in args.serve_rates:
        reps = [run_once(rate) for _ in range(max(1, args.serve_repeats))]
        med = sorted(reps, key=lambda r: r["p99_ms"])[(len(reps) - 1) // 2]
        med = dict(med, repeats=len(reps), gpix_s_all=[r["gpix_s"] for r in reps],
                   p50_ms_all=[r["p50_ms"] for r in reps], p99_ms_all=[r["p99_ms"] for r in reps])
        runs.append(med)
    return {"workload": "poisson_serving", "hbm_budget_bytes": 40 << 30, "max_inflight": args.serve_inflight,
            "batched_offline_gpix_s": batched_gpix, "runs": runs,
            "saturation": {"rate_req_s": runs[-1]["rate_req_s"], "gpix_s": runs[-1]["gpix_s"],
                           "offered_gpix_s": runs[-1]["offered_gpix_s"]} if runs else None}


def hard_leg(ig, torch, dev, args, peak_tops):
    """Hard-distribution batch: args.hard_images images of args.hard_side^2
    drawn from the block mixture (30% noise, 20% two-colour dither, 15% single
    colour, 15% near-black, 20% gradient+noise; 25% zero-weight texels via
    alpha), Quality_Max, both three-colour modes, weights = alpha/255.
    Batched (one persistent launch) against plain (one launch per image);
    sampled bit-exactness against the oracle, per-image RMSE/PSNR from an FP64
    decode-and-compare, and the FP32 fraction."""
    from icbc_gb300 import synth
    from oracle import oracle as O
    n, side = args.hard_images, args.hard_side
    nb = ig.blocks_of(side, side)
    imgs = [synth.hard_mixture_torch(side, side, 1000 + i, dev) for i in range(n)]
    outs_b = [torch.zeros((nb, 8), dtype=torch.uint8, device=dev) for _ in range(n)]
    outs_p = [torch.zeros((nb, 8), dtype=torch.uint8, device=dev) for _ in range(n)]
    cw = (1.0, 1.0, 1.0)
    descs_b = [ig.image_desc(im, 9, o, None, ig.Decoder_D3D10, cw, ig.WEIGHTS_ALPHA) for im, o in zip(imgs, outs_b)]
    descs_p = [ig.image_desc(im, 9, o, None, ig.Decoder_D3D10, cw, ig.WEIGHTS_ALPHA) for im, o in zip(imgs, outs_p)]
    stream = torch.cuda.Stream(device=dev)
    batch = ig.Batch(descs_b)
    res = {}
    for name, fn in (("batched", lambda: batch.launch(stream)), ("plain", lambda: ig.compress_images_each(descs_p, stream))):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            fn()
            e0.record(stream)
            for _ in range(args.hard_steps):
                fn()
            e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.hard_steps
        res[name] = {"ms": ms, "gpix_s": n * side * side / (ms * 1e-3) / 1e9}
    batch.close()
    same = all(torch.equal(a, b) for a, b in zip(outs_b, outs_p))
    if args.no_parity:
        del imgs, outs_b, outs_p
        torch.cuda.empty_cache()
        return {"workload": "hard_mixture_%dx%d^2_L9" % (n, side), "blocks": n * nb, "batched": res["batched"],
                "plain": res["plain"], "batched_equals_plain": bool(same)}
    # Oracle parity + op counts: every block of image 0, and every 97th block
    # row of every 8th image after it.
    nthreads = os.cpu_count() or 1
    host0 = imgs[0].cpu().numpy()
    ob, _, stats = O.encode_image(host0, 9, 0, cw, 1, None, True, True, nthreads=nthreads, with_stats=True)
    full = parity(outs_b[0].cpu().numpy(), ob, host0, 0)
    mism, sampled, worst = full["mismatches"], full["blocks_checked"], full["worst_rel_error_delta"]
    for i in range(8, n, 8):
        host = imgs[i].cpu().numpy()
        rows = sample_rows(host, 97)
        ob, _, st = O.encode_image(rows, 9, 0, cw, 1, None, True, True, nthreads=nthreads, with_stats=True)
        gpu = outs_b[i].cpu().numpy().reshape(side // 4, side // 4, 8)[::97].reshape(-1, 8)
        pr = parity(gpu, ob, rows, 0)
        mism += pr["mismatches"]
        sampled += pr["blocks_checked"]
        worst = max(worst, pr["worst_rel_error_delta"])
        stats = {k: stats[k] + st[k] for k in st}
    ops = algorithmic_ops(stats, 9) * (n * nb) / stats["blocks"]
    # FP64 decode-and-compare on the GPU: exact per-block integer SSE, FP64 sums
    psnr = []
    sse_total = 0.0
    for im, o in zip(imgs, outs_b):
        tex = im.view(side // 4, 4, side // 4, 4, 4).permute(0, 2, 1, 3, 4).reshape(nb, 64).contiguous()
        e = ig.evaluate_errors(tex, o, ig.Decoder_D3D10)
        sse = float(e.double().sum())
        sse_total += sse
        mse = sse / (16 * nb)
        psnr.append(20 * np.log10(255.0 / np.sqrt(mse)) if mse > 0 else 300.0)
    # the GPU SSE equals the oracle's FP64 decode-and-compare on one image
    sse0 = O.image_sse(imgs[0].cpu().numpy(), outs_b[0].cpu().numpy(), 0)
    ev0 = float(ig.evaluate_errors(imgs[0].view(side // 4, 4, side // 4, 4, 4).permute(0, 2, 1, 3, 4)
                                   .reshape(nb, 64).contiguous(), outs_b[0], 0).double().sum())
    mse = sse_total / (16 * n * nb)
    del imgs, outs_b, outs_p
    torch.cuda.empty_cache()
    return {"workload": "hard_mixture_%dx%d^2_L9" % (n, side), "blocks": n * nb,
            "batched": res["batched"], "plain": res["plain"],
            "speedup_batched_over_plain": res["plain"]["ms"] / res["batched"]["ms"],
            "batched_equals_plain": bool(same),
            "parity": {"blocks_checked": sampled, "mismatches": mism, "worst_rel_error_delta": worst,
                       "images_checked_whole": 1, "full_image_0": full,
                       "also": "every 97th block row of images 8, 16, ..., %d" % (8 * ((n - 1) // 8))},
            "rmse": float(np.sqrt(mse)), "psnr_db": float(20 * np.log10(255.0 / np.sqrt(mse))),
            "psnr_db_per_image_min_max": [float(min(psnr)), float(max(psnr))],
            "fp64_sse_image0_gpu_vs_oracle": [ev0, sse0],
            "fp32_frac": ops / (res["batched"]["ms"] * 1e-3) / 1e12 / peak_tops}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--cpu-stride", type=int, default=1,
                    help="the CPU legs encode every n-th block row (1: the whole workload)")
    ap.add_argument("--levels", type=int, nargs="+", default=None,
                    help="encode only these levels (profiling); the headline uses all ten")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU leg (profiling runs)")
    ap.add_argument("--cpu-form", default="neon-vector", choices=sorted(CPU_FORMS),
                    help="CPU form of the reference encoder the reference arm times")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-vs-plain leg")
    ap.add_argument("--batch-images", type=int, default=2000)
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-hard", action="store_true", help="skip the hard-distribution leg")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--cta-warps", type=int, default=0, choices=[0, 4, 8, 16],
                    help="the listed pass's CTA size at levels 2-9 (the autotuner, unless off, may change it)")
    ap.add_argument("--hard-images", type=int, default=64)
    ap.add_argument("--hard-side", type=int, default=8192)
    ap.add_argument("--hard-steps", type=int, default=2)
    ap.add_argument("--only-hard", action="store_true", help="run the hard-mixture leg alone (profiling)")
    ap.add_argument("--no-parity", action="store_true",
                    help="with --only-hard: skip the oracle checks and op counts (profiling)")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[500, 2000, 5000, 20000, 80000],
                    help="Poisson arrival rates; the last (80,000/s, above what the GPU encodes) measures saturation")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--serve-max-requests", type=int, default=8000)
    ap.add_argument("--serve-threads", type=int, default=4)
    ap.add_argument("--serve-repeats", type=int, default=3,
                    help="runs per serving rate; the line reports the median-p99 run and lists all")
    ap.add_argument("--serve-inflight", type=int, default=8, help="batched launches the server keeps on the GPU")
    args = ap.parse_args()
    if args.levels:
        global LEVELS
        LEVELS = sorted(set(args.levels))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
