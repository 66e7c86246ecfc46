"""Benchmark: rotations/s of the exhaustive 6D LCC search on one GB300.

Workload (default ``lcc128_filtered``): a seeded synthetic 128^3 map at 1.5 A
per voxel holding 6 copies of a 4,000-atom chain at 6 A resolution, SNR 3;
Laplace pre-filter and core-weighted LCC; 70,728 rotations (the size of the
reference's 4.71 degree set; its Karney file is not available on the GPU host,
so a super-Fibonacci SO(3) set of the same size stands in).

A step scans one eighth of the rotation set (8,841 rotations), accumulating
the running best, so the default 8 timed steps are one full search.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank scans its own rotations (weak scaling) and
the per-voxel results are merged on rank 0 after the timed region.
``--impl reference`` times the reference's CPU correlator path (the oracle
restatement: numpy.fft, as the reference runs without pyFFTW) on all host
cores instead.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "rotations/s at 128^3 LCC (1 GB300)"


def metric_for(shape):
    return "rotations/s at %d^3 LCC (1 GB300)" % shape[0] if len(set(shape)) == 1 else \
        "rotations/s at %dx%dx%d LCC (1 GB300)" % tuple(shape)
UNIT = "rotations/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="lcc128_filtered")
    ap.add_argument("--rotations", type=int, default=0, help="rotation-set size (default: the config's set)")
    ap.add_argument("--per-step", type=int, default=0, help="rotations per step (default: set size / 8)")
    ap.add_argument("--cpu-rot-per-core", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--learned-maps", type=int, default=10,
                    help="held-out 128^3 maps for the learned-proposal leg (0: skip)")
    ap.add_argument("--queue-steps", type=int, default=2,
                    help="timed steps of the uneven-map queue leg in the default line (0: skip)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the float64-normalisation leg")
    ap.add_argument("--pairs", type=int, default=0)
    ap.add_argument("--precision", action="store_true",
                    help="precision study: GPU variants vs the float64 oracle on a rotation subset")
    ap.add_argument("--precision-rotations", type=int, default=32)
    ap.add_argument("--precision-timed", type=int, default=2048, help="rotations of each variant's speed run")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def workload(name, nrot_override=0):
    from powerfit_gb300 import synth
    from powerfit_gb300.rotations import rotation_set
    from powerfit_gb300.correlator import determine_core_indices
    cfg = synth.CONFIGS[name]
    case = synth.make_config(name, seed=0)
    mask = determine_core_indices(case.mask) if cfg["core_weighted"] else case.mask
    rot, desc = rotation_set(cfg["angle"], data_dir=os.environ.get("POWERFIT_ROTATION_DATA") or "/nonexistent")
    if nrot_override:
        rot = rot[:nrot_override]
    return cfg, case.target.astype(np.float64), case.template, mask, rot, desc


def workload_config(name, cfg, shape, nset, per_step, l2):
    """The `config` object of a bench line: the same keys in both arms (the
    GPU search and the reference's CPU path), so the two lines describe one
    workload."""
    return {"workload": name, "grid": list(shape), "voxelspacing": cfg["voxelspacing"], "laplace": cfg["laplace"],
            "core_weighted": cfg["core_weighted"], "rotation_set_size": int(nset),
            "rotations_per_step": int(per_step), "l2": l2}


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU side: the reference correlator path (oracle restatement) on host cores
# ---------------------------------------------------------------------------

def make_pool(n):
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(n)


def cpu_sample(pool, nproc, target, template, mask, rot, laplace, per_core):
    """Time the reference's _cpu_scan structure on nproc processes over the
    first nproc*per_core rotations of `rot`.  Every process times its set-up
    (the correlator's Laplace filter and target spectra, done once per process
    in a whole search) apart from its rotation loop, so the rate is the steady
    state of a whole search: the sample's rotations over the slowest process's
    loop.  Returns a summary dict and the sample's (lcc, rot)."""
    from oracle import oracle as O
    sample = rot[: nproc * per_core]
    t0 = time.perf_counter()
    lcc, r, parts = O.cpu_scan_timed(target, template, mask, sample, laplace, nproc=nproc, pool=pool)
    wall = time.perf_counter() - t0
    loop = max(pt[1] for pt in parts)
    n = int(sample.shape[0])
    return {"value": n / loop, "rotations": n, "loop_s": loop, "wall_s": wall,
            "prepare_s": statistics.mean(pt[0] for pt in parts), "with_prepare": n / wall}, (lcc, r)


def warm_pool(pool, nproc, target, template, mask, rot, laplace):
    """One untimed round of one rotation per process: the processes start and
    import numpy / scipy before the timed sample."""
    cpu_sample(pool, nproc, target, template, mask, rot, laplace, 1)


def sample_rotations(cfg, rot, count):
    """Rotations of the CPU sample (and of the precision check on it): the
    reference's own 4.71 degree set where the workload uses that set -- the
    committed strided slice of c48u2947.npy in tests/golden/rotset_471.npz --
    else the workload's set."""
    path = os.path.join(ROOT, "tests", "golden", "rotset_471.npz")
    if abs(cfg["angle"] - 4.71) < 1e-6 and os.path.exists(path):
        with np.load(path) as d:
            ref = d["rotmats"]
        if ref.shape[0] >= count:
            return ref[:count], "the reference's 4.71 deg set (every 34th row of c48u2947.npy)"
    return rot[:count], "the workload's set"


def precision_vs_oracle(ftarget, base, sample, ref, device, flags=0):
    """The GPU search on the CPU baseline's rotation sample against the
    oracle's result for it (float64): max |dLCC| and argmax agreement."""
    from powerfit_gb300 import _lib
    ctx = _lib.Context(ftarget.shape, device)
    ctx.set_target(ftarget, base._lcc_mask)
    ctx.set_template_mask(base._template, base._mask, float(base._norm_factor), base._rmax)
    lcc, rot = ctx.scan(sample, flags=flags)
    ctx.close()
    ref_lcc, ref_rot = ref
    fin = np.isfinite(ref_lcc)
    hit = fin & (ref_lcc > 0)
    return {"max_abs_dlcc": float(np.max(np.abs(lcc[fin] - ref_lcc[fin]))),
            "argmax_agreement": float(np.mean(rot[hit] == ref_rot[hit])) if hit.any() else 1.0,
            "voxels": int(hit.sum()), "rotations": int(sample.shape[0]), "tolerance": 1e-4,
            "reference": "float64 oracle (restated CPUCorrelator) on the CPU baseline's sample; argmax over "
                         "every voxel with a positive best LCC, near-ties included"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    pool = make_pool(cores)
    cfg, target, template, mask, rot, desc = workload(args.config, args.rotations)
    per_core = args.cpu_rot_per_core
    sample, sample_src = sample_rotations(cfg, rot, cores * per_core)
    if args.warmup > 0:
        warm_pool(pool, cores, target, template, mask, sample, cfg["laplace"])
    runs = [cpu_sample(pool, cores, target, template, mask, sample, cfg["laplace"], per_core)[0]
            for _ in range(args.steps)]
    pool.close()
    tot_rot = sum(r["rotations"] for r in runs)
    value = tot_rot / sum(r["loop_s"] for r in runs)
    line = {
        "impl": "reference", "metric": metric_for(target.shape), "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(r["wall_s"] for r in runs) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded map, template, mask; %s)" % desc,
        "config": workload_config(args.config, cfg, target.shape, int(rot.shape[0]), cores * per_core,
                                  "not applicable (host cores)"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d rotations per step (%d per core) from %s, _cpu_scan structure, numpy.fft; "
                                   "rate over the rotation loops (the per-process set-up, once per process in a "
                                   "whole search, timed apart)" % (cores * per_core, per_core, sample_src),
                         "prepare_s": statistics.mean(r["prepare_s"] for r in runs),
                         "with_prepare": tot_rot / sum(r["wall_s"] for r in runs)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

def bytes_per_rotation(n, B):
    """Compulsory HBM traffic of the three-pass fused pipeline per rotation
    (F = 3 spectra, complex64 spectra, B rotations sharing target spectra and
    the running max): 8N + 8H(2F+6) + (16H + 17N)/B, H = n*n*(n/2+1)."""
    N = n ** 3
    H = n * n * (n // 2 + 1)
    return 8 * N + 8 * H * (2 * 3 + 6) + (16 * H + 17 * N) / B


def dram_traffic(kernel, n, pairs_per_launch):
    """DRAM bytes per launch of ``kernel`` at grid n^3 from the committed ncu
    summary (read + write of one captured launch), scaled from the captured
    launch's rotation pairs to this run's; (None, reason) without an entry."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        with open(path) as f:
            lines = f.readlines()
        for ln in lines:
            parts = ln.split()
            if len(parts) >= 5 and not ln.startswith("#") and parts[0] == kernel and int(parts[1]) == n:
                cap_pairs, rd, wr = int(parts[2]), float(parts[3]), float(parts[4])
                scale = pairs_per_launch / cap_pairs
                note = "ncu dram__bytes_read.sum + dram__bytes_write.sum, profiles/dram_traffic.txt"
                if abs(scale - 1.0) > 1e-9:
                    note += " (captured at %d pairs per launch, scaled to %g)" % (cap_pairs, pairs_per_launch)
                return (rd + wr) * scale, note
    except (OSError, ValueError):
        pass
    return None, "no ncu capture for %s at %d^3" % (kernel, n)


def run_ours(args, rank, world, local_rank):
    import torch
    cores = os.cpu_count() or 1
    pool = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        pool = make_pool(cores)          # spawn before any CUDA work
    torch.cuda.set_device(local_rank)
    from powerfit_gb300 import _lib
    from powerfit_gb300.correlator import BaseCorrelator

    cfg, target, template, mask, rot_all, desc = workload(args.config, args.rotations)
    nset = rot_all.shape[0]
    per_step = args.per_step or -(-nset // 8)
    # weak scaling: every rank scans nset rotations of its own, a contiguous
    # shard of one set of world * nset rotations, stored with their indices in
    # that set (the shard's first index as the rotation offset)
    if world > 1:
        from powerfit_gb300.distributed import weak_scaling_shard
        from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
        rot_rank, rank_first = weak_scaling_shard(lambda c: quat_to_rotmat(super_fibonacci(c)), nset, rank, world)
    else:
        rot_rank, rank_first = rot_all, 0

    base = BaseCorrelator(target, laplace=cfg["laplace"])
    base.template = template
    base.mask = mask
    ftarget = base._laplace_filter(base._target) if cfg["laplace"] else base._target
    shape = target.shape
    n = shape[0]

    ctx = _lib.Context(shape, local_rank)
    if args.pairs:
        ctx.set_tuning(pairs=args.pairs)
    # a dedicated (non-default) stream made current: the library launches on it
    # and the CUDA events below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_target(ftarget, base._lcc_mask)
    ctx.set_template_mask(base._template, base._mask, float(base._norm_factor), base._rmax)
    ctx.set_rotations(rot_rank)
    if args.pairs:
        tuned = {"pairs": args.pairs, "source": "--pairs"}
    else:
        tuned = ctx.autotune(512)
        tuned["source"] = "autotuner (512-rotation trials)"
    pairs, ty1, ty3 = ctx.get_tuning()
    geo = ctx.get_geometry()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step(k, first, flags=0):
        f = (k * per_step) % nset
        cnt = min(per_step, nset - f)
        ctx.scan_resident(f, cnt, rank_first, flags | (0 if first else _lib.PF_FLAG_ACCUMULATE))
        return cnt

    def timed(profile, flags=0):
        ctx.set_profiling(profile)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        done = 0
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            done += step(k, k == 0, flags)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        kms, kl = ctx.kernel_times()
        ctx.set_profiling(False)
        return done, sum(a.elapsed_time(b) for a, b in ev) / 1e3, wall, kms, kl

    for w in range(args.warmup):
        step(w, w == 0)
    torch.cuda.synchronize()

    # timed region: device-resident inputs, L2 flushed before each step, no
    # per-kernel instrumentation
    clocks = ClockSampler(local_rank)
    clocks.start()
    done, dev_s, wall, _, _ = timed(False)
    clk = clocks.stop()
    # the same steps again with CUDA events around every kernel launch (the
    # per-kernel durations for the roofline)
    _, prof_s, _, kms, klaunch = timed(True)
    # the same steps with the local variance and the LCC normalisation in
    # float64 (PF_FLAG_FP64_NORM), the literal precision specification
    fp64 = None
    if not args.no_fp64:
        for w in range(min(args.warmup, 1)):
            step(w, True, _lib.PF_FLAG_FP64_NORM)
        torch.cuda.synchronize()
        f_done, f_s, _, _, _ = timed(False, _lib.PF_FLAG_FP64_NORM)
        fp64 = {"value": f_done * world / f_s, "unit": UNIT, "ms_per_step": 1e3 * f_s / args.steps,
                "flags": "PF_FLAG_FP64_NORM",
                "note": "same workload, steps and timing as the headline; local variance Nm*ave2 - ave^2 and "
                        "the LCC division in float64 on the GPU (the headline: float-float with FMA products)"}
    t = torch.tensor([dev_s], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
    dev_s = float(t.item())
    value = done * world / dev_s

    # end-to-end through the reference-facing API with host buffers: per step
    # the whole correlator job for that step's rotations (target and template
    # upload + spectra, rotations H2D, scan, LCC and rotation volumes D2H)
    e2e_steps = max(1, min(args.steps, 3))
    out_lcc = np.empty(shape, np.float32)
    out_rot = np.empty(shape, np.int32)
    rot_host = [np.ascontiguousarray(rot_rank[(k * per_step) % nset:(k * per_step) % nset + per_step])
                for k in range(e2e_steps)]
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0 = time.perf_counter()
    for k in range(e2e_steps):
        ctx.set_target(ftarget, base._lcc_mask)
        ctx.set_template_mask(base._template, base._mask, float(base._norm_factor), base._rmax)
        ctx.set_rotations(rot_host[k])
        ctx.scan_resident(0, rot_host[k].shape[0], rank_first, 0)
        ctx.get_results(out_lcc, out_rot)
    e2e_s = time.perf_counter() - e0
    te = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
    e2e_value = sum(r.shape[0] for r in rot_host) * world / float(te.item())
    N = int(np.prod(shape))
    h2d = N * 4 + N + N * 4 * 2 + per_step * 9 * 8
    d2h = N * 8

    # multi-rank: merge per-voxel results on rank 0 (outside the timed region)
    merged_rot_range = None
    if world > 1:
        from powerfit_gb300 import distributed as D
        lcc_r, rot_r = ctx.get_results()
        merged = D.gather_and_merge(lcc_r, rot_r, rank_offset=0)   # indices already global
        if merged is not None:
            lo, hi = int(merged[1].min()), int(merged[1].max())
            if lo < 0 or hi >= world * nset:
                raise RuntimeError("merged rotation indices [%d, %d] outside [0, %d)" % (lo, hi, world * nset))
            merged_rot_range = [lo, hi]

    if rank != 0:
        return 0

    # roofline of the dominant kernel: algorithmic bytes per launch / average launch time
    names = ["pass1_rotate_fwdx", "pass2_yz_product", "pass3_invx_lcc"]
    kernels = ["k_pass1_ct", "k_pass2_ct", "k_pass3_ct"]
    dom = int(np.argmax(kms))
    launches = int(klaunch.sum())
    nz, ny, nx = shape
    re = min(geo["rmax"], geo["reff"])
    cz = np.where(2 * np.arange(nz) <= nz, np.arange(nz), np.arange(nz) - nz)
    cy = np.where(2 * np.arange(ny) <= ny, np.arange(ny), np.arange(ny) - ny)
    disk = int(np.sum(cz[:, None] ** 2 + cy[None, :] ** 2 <= re * re))   # (z, y) rows the rotation reaches
    pairs_per_launch = done / 2.0 / max(int(klaunch[dom]), 1)
    B = 2.0 * pairs_per_launch                                         # rotations per launch
    H = nz * ny * (nx // 2 + 1)
    F = 3
    # the streaming pipeline model 8N + 8H(2F+6) + (16H+17N)/B, split by the pass that moves the bytes
    per_rot = {
        0: 8 * N + 8 * H * F,                     # template + mask read, F forward spectra written
        1: 8 * H * F + 8 * H * 3 + 16 * H / B,    # F spectra read, 3 product spectra written, target spectra once
        2: 8 * H * 3 + 17 * N / B,                # 3 product spectra read; lcc mask, lcc, rot once per launch
    }
    # what the pruned kernels move (complex64 full planes of a rotation pair, rows outside the reach disk skipped)
    pruned_per_pair = {
        0: 8 * N / pairs_per_launch + 3 * 8 * disk * nx,      # template + mask once, disk rows of 3 spectra written
        1: 3 * nx * 8 * (disk + nz * ny) + 16 * N / pairs_per_launch,
        2: 3 * 8 * N + (17 * N) / pairs_per_launch,
    }
    alg_bytes = per_rot[dom] * B
    avg_s = kms[dom] / 1e3 / max(int(klaunch[dom]), 1)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg_bytes / avg_s / 1e9
    traffic, traffic_src = dram_traffic(kernels[dom], n, pairs_per_launch)
    pipe_bytes = bytes_per_rotation(n, 2 * pairs)
    pruned_bytes = sum(pruned_per_pair.values()) / 2.0
    line = {
        "metric": metric_for(shape), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 FFT / float-float LCC",
        "data": "synthetic (seeded map, template, mask; %s)" % desc,
        "config": workload_config(args.config, cfg, shape, nset, per_step,
                                  "flushed (256 MiB write) before every timed step"),
        # the search's own shapes (the reference arm has none): batch and
        # tiles from the autotuner, and the pruning geometry of this template
        "search": {"pairs_per_batch": pairs, "rows_pass1": ty1, "rows_pass3": ty3, "tuning": tuned,
                   "reach_radius": re, "planes": geo["valid_planes"], "disk_rows": disk,
                   "full_search_s": nset / (value / world)},
        "clocks": clk,
        "wall_s": wall,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "steps": e2e_steps, "note": "per step: target+template upload and spectra, rotations H2D, "
                                             "scan, lcc+rot D2H"},
        "gpu_launches": launches,
        "kernel_ms": {names[i]: float(kms[i]) for i in range(3)},
        "kernel_launches": {names[i]: int(klaunch[i]) for i in range(3)},
        "kernel_share": {names[i]: float(kms[i] / kms.sum()) for i in range(3)},
        "profiled_pass_s": prof_s,
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "bytes_per_launch": alg_bytes, "pruned_bytes_per_launch": pruned_per_pair[dom] * pairs_per_launch,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s"},
        "pipeline_roofline": {"model": "streaming 3-pass, unpruned: 8N + 8H(2F+6) + (16H+17N)/B",
                              "bytes_per_rotation": pipe_bytes, "achieved_gbs": pipe_bytes * value / world / 1e9,
                              "frac": pipe_bytes * value / world / 1e9 / peak,
                              "pruned_bytes_per_rotation": pruned_bytes,
                              "pruned_frac": pruned_bytes * value / world / 1e9 / peak},
    }
    if merged_rot_range is not None:
        line["merged_rotation_range"] = merged_rot_range
    if fp64 is not None:
        line["fp64_norm"] = fp64
    if pool is not None:
        sample, sample_src = sample_rotations(cfg, rot_all, cores * args.cpu_rot_per_core)
        warm_pool(pool, cores, target, template, mask, sample, cfg["laplace"])
        cs, cres = cpu_sample(pool, cores, target, template, mask, sample, cfg["laplace"], args.cpu_rot_per_core)
        pool.close()
        line["cpu_baseline"] = {"value": cs["value"], "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": "%d rotations (%d per core) from %s, same map, template and mask; "
                                          "_cpu_scan structure with numpy.fft; rate over the rotation loops (%.1f s), "
                                          "the per-process set-up (once per process in a whole search) timed apart"
                                          % (cs["rotations"], args.cpu_rot_per_core, sample_src, cs["loop_s"]),
                                "prepare_s": cs["prepare_s"], "with_prepare": cs["with_prepare"],
                                "wall_s": cs["wall_s"]}
        line["precision"] = precision_vs_oracle(ftarget, base, sample, cres, local_rank)
        line["precision"]["rotations_from"] = sample_src
        if fp64 is not None:
            fp64["precision"] = precision_vs_oracle(ftarget, base, sample, cres, local_rank, _lib.PF_FLAG_FP64_NORM)
    if args.queue_steps > 0 and world == 1:
        line["queue"] = queue_leg(args.queue_steps, max(1, min(args.warmup, 1)))
    if args.learned_maps > 0 and world == 1:
        line["learned"] = learned_leg(args.learned_maps)
    print(json.dumps(line), flush=True)
    return 0


def learned_leg(nmaps):
    """Time to best fit, learned proposal against exhaustive search, on held-out
    seeded 128^3 maps with the 207,576-rotation set (the trained network shipped
    in powerfit_gb300/data)."""
    from powerfit_gb300 import proposal as PR, proposal_train as T
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    rotmats = quat_to_rotmat(super_fibonacci(T.SET_SIZE))
    nbr = PR.rotation_neighbours(rotmats)
    net = PR.ProposalNet.load(PR.default_weights())
    fractions = T.operating_fractions(PR.default_weights())
    rows = T.evaluate(net, [T.EVAL_SEED0 + i for i in range(nmaps)], 128, rotmats, nbr, fractions=fractions,
                      log=lambda m: None)
    summ = T.summarise(rows)
    return {"metric": "time to best fit, learned proposal vs exhaustive search (128^3, 1 GB300)",
            "value": summ["network"]["time_vs_exhaustive"], "unit": "fraction of exhaustive time",
            "higher_is_better": False,
            "recall": summ["network"]["recall"], "recall_at": summ["network"]["recall_at"],
            "fraction": fractions["network"],
            "learned_s": summ["network"]["time_s"], "exhaustive_s": summ["exhaustive_s"],
            "coarse_only": {"recall": summ["coarse_only"]["recall"], "recall_at": summ["coarse_only"]["recall_at"],
                            "fraction": fractions["coarse_only"],
                            "time_vs_exhaustive": summ["coarse_only"]["time_vs_exhaustive"],
                            "median_rank_fraction": summ["coarse_only"]["median_rank_fraction"],
                            "worst_rank_fraction": summ["coarse_only"]["worst_rank_fraction"]},
            "median_rank_fraction": summ["network"]["median_rank_fraction"],
            "worst_rank_fraction": summ["network"]["worst_rank_fraction"],
            "config": {"maps": nmaps, "seeds": "held-out %d.." % T.EVAL_SEED0, "grid": [128, 128, 128],
                       "rotation_set_size": T.SET_SIZE,
                       "operating_fractions": "chosen on validation maps when the network was trained "
                                              "(stored with its weights), for each ranking on its own",
                       "coarse_grid": [PR.COARSE_EDGE] * 3, "data": "synthetic"}}


def queue_leg(steps, warmup, nrot=0):
    """Uneven-map queue (16 seeded maps of 48^3-160^3, the 9.72 degree set's
    size each): every map's scan queued on its own stream before any is
    awaited; batch and tile shapes from the autotuner, run once per grid size
    during the warm-up and reused for every later map of that size.  Also the
    same queue captured once into one CUDA graph and replayed."""
    import torch
    from powerfit_gb300.queue import MapJob, QueueGraph, make_queue, scan_queue
    from powerfit_gb300.rotations import rotation_set
    rot, desc = rotation_set(10.0, data_dir=os.environ.get("POWERFIT_ROTATION_DATA") or "/nonexistent")
    if nrot:
        rot = rot[:nrot]
    cases = make_queue(16, seed=0)
    mk = lambda: [MapJob(c.target.astype(np.float64), c.template, c.mask, rot) for c in cases]
    tuning = {}
    t0 = time.perf_counter()
    for _ in range(max(1, warmup)):
        scan_queue(mk(), autotune_trial=512, tuning=tuning)
    torch.cuda.synchronize()
    warm_s = time.perf_counter() - t0
    times = []
    for _ in range(steps):
        jobs = mk()
        t0 = time.perf_counter()
        scan_queue(jobs, tuning=tuning)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    total_rot = rot.shape[0] * len(cases)
    qg = QueueGraph(mk(), tuning=tuning)
    for _ in range(max(1, warmup)):
        qg.replay()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        qg.replay()
    torch.cuda.synchronize()
    graph_s = time.perf_counter() - t0
    qg.close()
    return {"metric": "map-rotations/s, queue of 16 uneven maps (1 GB300)",
            "value": total_rot * len(times) / sum(times), "unit": "map-rotations/s", "steps": steps,
            "ms_per_step": 1e3 * sum(times) / len(times), "data": "synthetic (%s)" % desc,
            "grids": [c.target.shape[0] for c in cases], "rotations_per_map": int(rot.shape[0]),
            "tuning": {"x".join(str(v) for v in k): {kk: vv for kk, vv in t.items() if kk != "trial_ms"}
                       for k, t in tuning.items()},
            "tuning_source": "autotuner (512-rotation trials), once per grid size in the warm-up (%.1f s)" % warm_s,
            "timing": "host wall clock per step: per-map setup (spectra, template, rotations) + all scans",
            "graph": {"value": total_rot * steps / graph_s, "unit": "map-rotations/s",
                      "ms_per_replay": 1e3 * graph_s / steps,
                      "timing": "one CUDA graph of all 16 maps' scans (captured once), host wall clock per replay"}}


def run_queue(args):
    """The uneven-map queue on its own line (``--config queue16``)."""
    q = queue_leg(args.steps, args.warmup, args.rotations)
    line = {"metric": q["metric"], "value": q["value"], "unit": q["unit"], "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": q["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 FFT / float-float LCC", "data": q["data"],
            "config": {"workload": "queue16", "grids": q["grids"], "rotations_per_map": q["rotations_per_map"],
                       "tuning": q["tuning"], "tuning_source": q["tuning_source"], "timing": q["timing"]},
            "graph": q["graph"]}
    print(json.dumps(line), flush=True)
    return 0


def run_precision(args):
    """Precision study: max |dLCC| and argmax agreement of the GPU variants
    against the float64 oracle, on a rotation subset of the configuration:
    float32 FFTs with float-float or float64 normalisation, and the DFT stages
    on the tensor cores in split-bf16x3 (PF_FLAG_TENSOR_DFT with mma.sync;
    runtime-planned kernels).  Each variant's search speed is timed on a larger slice, next to
    the float32 runtime-planned kernels it replaces.  With
    PF_FLAG_TENSOR_TC05 the plane pass's stages run on tcgen05; grids whose
    plane does not fit one block's shared memory report it unsupported."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(cores)
    from powerfit_gb300 import CUDACorrelator, _lib
    from oracle import oracle as O
    cfg, target, template, mask, rot, desc = workload(args.config, args.rotations)
    sub = rot[:: max(1, rot.shape[0] // args.precision_rotations)][:args.precision_rotations]
    t0 = time.perf_counter()
    # oracle with the top-two gap, one rotation slice per process (merged with _combine semantics)
    per = -(-sub.shape[0] // cores)
    jobs = [(target, template, mask, cfg["laplace"], sub[i:i + per]) for i in range(0, sub.shape[0], per)]
    parts = pool.map(_oracle_top2, jobs)
    pool.close()
    lcc = np.zeros(target.shape)
    second = np.zeros(target.shape)
    rrot = np.zeros(target.shape)
    for k, (pl, pr, ps) in enumerate(parts):
        off = k * per
        better = pl > lcc
        with np.errstate(invalid="ignore"):
            sec_new = np.where(better, np.maximum(lcc, ps), np.maximum(second, np.where(pl > second, pl, second)))
        second = sec_new
        lcc = np.where(better, pl, lcc)
        rrot = np.where(better, pr + off, rrot)
    oracle_s = time.perf_counter() - t0
    res = {}
    timed = rot[:min(rot.shape[0], args.precision_timed)]
    variants = (("fp32_fft+floatfloat_norm", 0), ("fp32_fft+fp64_norm", _lib.PF_FLAG_FP64_NORM),
                ("fp32_fft_runtime_planned+floatfloat_norm", _lib.PF_FLAG_GENERIC),
                ("bf16x3_tensor_dft+floatfloat_norm", _lib.PF_FLAG_TENSOR_DFT),
                ("bf16x3_tensor_dft_tcgen05_plane+floatfloat_norm",
                 _lib.PF_FLAG_TENSOR_DFT | _lib.PF_FLAG_TENSOR_TC05))
    for name, flags in variants:
        corr = CUDACorrelator(target, laplace=cfg["laplace"], flags=flags)
        corr.template = template
        corr.mask = mask
        corr.rotations = sub
        try:
            corr.scan()
        except _lib.PowerFitError as e:        # a variant this grid does not support
            res[name] = {"unsupported": str(e)}
            continue
        fin = np.isfinite(lcc)
        err = float(np.max(np.abs(corr.lcc[fin] - lcc[fin])))
        clear = fin & ((lcc - second) > 1e-4) & (lcc > 0)
        agree = float(np.mean(corr.rot[clear] == rrot[clear])) if clear.any() else 1.0
        res[name] = {"max_abs_dlcc": err, "argmax_agreement_where_gap_gt_1e-4": agree,
                     "clear_voxels": int(clear.sum())}
        ctx = corr.context            # speed on a larger slice (device-resident, one warm-up)
        ctx.set_rotations(timed)
        ctx.scan_resident(0, min(64, timed.shape[0]), flags=flags)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.scan_resident(0, timed.shape[0], flags=flags)
        ctx.synchronize()
        res[name]["rotations_per_s"] = timed.shape[0] / (time.perf_counter() - t0)
    line = {"metric": "precision vs float64 oracle", "config": {"workload": args.config, "grid": list(target.shape),
            "rotations": int(sub.shape[0]), "laplace": cfg["laplace"], "core_weighted": cfg["core_weighted"]},
            "variants": res, "oracle_s": oracle_s, "oracle_cores": cores, "timed_rotations": int(timed.shape[0])}
    print(json.dumps(line), flush=True)
    return 0


def _oracle_top2(job):
    from oracle import oracle as O
    target, template, mask, laplace, rots = job
    p = O.prepare(target, template, mask, laplace)
    return O.scan(p, rots, track_second=True)


def run_kernels(args):
    """One launch of every kernel outside the fast search passes, at 128^3:
    GPU preprocessing (splat, dilation, Laplace, core weights), the
    runtime-planned search passes and target spectra (PF_FLAG_GENERIC), the
    same passes with the DFT stages on the tensor cores (PF_FLAG_TENSOR_DFT:
    mma.sync; with PF_FLAG_TENSOR_TC05 the plane pass's stages on tcgen05),
    the float64 unit mirrors, the shard merge, the proposal network's kernels
    and the learned proposal's coarse 32^3 search (2,048 rotations).
    Wall time per call (synchronised); meant as the command an ncu capture
    of these kernels runs."""
    import torch
    from powerfit_gb300 import _lib, proposal as PR
    from powerfit_gb300.correlator import BaseCorrelator
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    torch.cuda.set_device(0)
    cfg, target, template, mask, rot_all, desc = workload("lcc128_filtered")
    from powerfit_gb300 import synth
    case = synth.make_config("lcc128_filtered", seed=0)
    n = target.shape[0]
    times = {}

    def timed(name, fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        times[name] = time.perf_counter() - t0
        return out

    pts = (case.chain / case.voxelspacing).T
    grid = np.zeros(target.shape)
    timed("blur_points", lambda: _lib.blur_points(pts, case.elements.astype(np.float64),
                                                  synth.res_to_sigma(case.resolution) / case.voxelspacing, grid))
    m = np.zeros(target.shape)
    timed("dilate_points", lambda: _lib.dilate_points(pts, 5.0 / case.voxelspacing, m))
    timed("laplace_wrap", lambda: _lib.laplace_wrap(target))
    timed("core_indices", lambda: _lib.core_indices(m))
    # runtime-planned search passes and spectra
    base = BaseCorrelator(target, laplace=True)
    base.template = template
    base.mask = mask
    ctx = _lib.Context(target.shape)
    timed("set_target (spectra)", lambda: ctx.set_target(_lib.laplace_wrap(base._target), base._lcc_mask))
    ctx.set_template_mask(base._template, base._mask, float(base._norm_factor), base._rmax)
    rot = quat_to_rotmat(super_fibonacci(8))
    timed("scan generic", lambda: ctx.scan(rot, flags=_lib.PF_FLAG_GENERIC))
    timed("scan tensor-core DFT", lambda: ctx.scan(rot, flags=_lib.PF_FLAG_TENSOR_DFT))
    timed("scan tensor-core DFT, tcgen05 plane pass",
          lambda: ctx.scan(rot, flags=_lib.PF_FLAG_TENSOR_DFT | _lib.PF_FLAG_TENSOR_TC05))
    lcc, r = ctx.scan(rot[:2])
    timed("combine", lambda: _lib.combine_into(lcc.copy(), r.copy(), lcc, r, 0))
    timed("fft3d", lambda: ctx.fft3d(target.astype(np.float32)))
    ctx.close()
    out = np.zeros(target.shape)
    timed("rotate_grid3d", lambda: _lib.rotate_grid3d(base._template, rot[1], n // 2, out, False))
    a = np.random.default_rng(0).normal(size=n * n * (n // 2 + 1)) + 0j
    timed("conj_multiply", lambda: _lib.conj_multiply(a, a, np.empty_like(a)))
    timed("calc_lcc", lambda: _lib.calc_lcc(target, target, target * target + 1, base._lcc_mask,
                                            np.empty(target.shape)))
    # proposal network on the 207,576-rotation set
    rows = 207576
    x = torch.randn(rows, PR.FEATURES, device="cuda")
    t = torch.randn(rows, device="cuda")
    w = torch.ones(rows, device="cuda")
    net = PR.ProposalNet.load(PR.default_weights())
    timed("mlp forward", lambda: net.forward(x))
    timed("mlp grad", lambda: _lib.mlp_grad(x, t, w, net.nin, net.nh, net.pb, 1.0 / rows, net.grad, net.loss))
    timed("mlp adam", lambda: _lib.mlp_adam(net.p, net.pb, net.grad, net.m, net.v, 1e-3, 1))
    # the learned proposal's coarse search: the map brought to 32^3, 2,048
    # rotations with per-rotation maxima (the 32^3 fast kernels: 128-thread
    # plane-pass blocks, pass 3 split over four pair parts per tile and merged
    # by k_combine_parts)
    ct, ctm, cm, _, _ = PR.coarsen(target, template, mask, case.voxelspacing, case.resolution)
    cb = BaseCorrelator(ct)
    cb.template = ctm
    cb.mask = cm
    cctx = _lib.Context(ct.shape)
    cctx.set_target(cb._target, cb._lcc_mask)
    cctx.set_template_mask(cb._template, cb._mask, float(cb._norm_factor), cb._rmax)
    cctx.set_tuning(pairs=128, rows1=32, rows3=16)
    cctx.set_rotations(quat_to_rotmat(super_fibonacci(2048)))
    timed("coarse 32^3 search (2,048 rotations)",
          lambda: (cctx.scan_resident(0, 2048, 0, _lib.PF_FLAG_ROT_MAX), cctx.synchronize()))
    cctx.close()
    print(json.dumps({"metric": "per-call wall time of the auxiliary kernels (128^3)", "unit": "s",
                      "values": times, "config": {"workload": "kernels", "grid": list(target.shape)}}), flush=True)
    return 0


def main():
    args = parse()
    if args.precision:
        return run_precision(args)
    if args.config == "queue16":
        return run_queue(args)
    if args.config == "kernels":
        return run_kernels(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group(backend)
    try:
        if args.impl == "reference":
            return run_reference(args, rank, world)
        return run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
