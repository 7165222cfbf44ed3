"""Benchmark: exact-DBSCAN points/sec on one GB300 (replicas on N GPUs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload zipf2d_10m|aniso3d_20m|blobs2d_100k|batch4096|serve]
                  [--precision fp64|fp32band] [--no-extras]

Default workload: 10,000,000 2D float64 points (500 Zipf-sized Gaussian blobs +
5% uniform noise), eps=0.3, minpts=8, every distance test in float64 -- the
single-instance GPU configuration the headline metric is quoted on.

A step is one full exact-DBSCAN pass (index build, core flags, union-find,
cluster numbering, borders, labels in caller order) over the whole point set.
  value  points/s with the points already in HBM (CUDA events on the stream the
         library launches on, L2 flushed between steps with a 512 MiB write)
  e2e    points/s through gd_dbscan with pinned HOST input and output: the
         host->device copy of the points and the device->host copy of the
         labels are inside the timed region
The JSON line also carries a float32-band run of the same workload, per-phase
device times, the roofline of the pipeline, the CPU baseline (the CPU
restatement of the reference's exact DBSCAN on this host's cores, bounded
sample) and the SM clocks sampled during the timed region.

On one GPU the default run attaches the rest of the metric ("batched/FP32-band
vs plain; p50/p99 serve latency") as extra keys of the same line, each with its
own clock samples and label checks (--no-extras leaves them out):
  c3  20M 3D points, float32 filter + float64 band (aniso3d_20m)
  c4  4,096 independent instances in one gd_batch_dbscan run, autotuned, against
      the single-instance path once per instance; labels of a sample of 256
      instances are checked against the oracle in that key's CPU-baseline leg
  c5  the served request stream (Poisson arrivals at 200/s, sizes log-uniform in
      [1e3, 2e6], 150 GB admission budget) through gd_server_*, p50/p99 against
      one-at-a-time solves, and a second open-loop run near the one-at-a-time
      saturation rate

--workload batch4096 / serve run those alone, as the headline.
--impl reference times the reference's exact CPU DBSCAN path on this host: the
reference's own R-tree program (oracle/_ref) where it was built, otherwise the
CPU restatement (oracle/), with all host threads, on a bounded sample per step.
Multi-GPU: the path does not shard across GPUs here; --gpus N runs N
independent replicas (one per rank) and reports their aggregate.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib
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
PKG = "fast-cuda-gpu-dbscan_gb300"

ALGO_BYTES_PER_POINT = {2: 8 * 2 + 4, 3: 8 * 3 + 4}   # f64 coordinates in + int32 label out
METRIC = "points/sec at exact labels"

# kernels of each timed phase (the library records CUDA events between phases)
PHASE_KERNELS = {
    "ms_index": "k_bbox_init, k_bbox_chunk, k_params_inst, k_layout, k_keys, radix sort "
                "(k_rs_upsweep, k_scan_onepass, k_rs_downsweep per pass), k_gather, k_run_bits, "
                "k_scan_onepass, k_compact_bits, k_runs_finish, k_cell_counts, k_start_fill, "
                "k_scan_onepass, k_rank_off (k_row_hash for hashed grids)",
    "ms_core": "k_core_split, k_scan_onepass, k_compact_bits, k_core_point (3D: near rows, "
               "k_scan_onepass, k_compact_bits, far rows), k_core_heavy",
    "ms_union": "k_parent_init, k_scan_onepass, k_compact_bits, k_union_scan + k_union_heavy + "
                "k_compress per pass (2D: 2 passes, 3D: 3), k_asym_resolve",
    "ms_label": "k_roots, k_scan_onepass, k_cell_ids, k_label, k_scan_onepass, k_compact_bits, "
                "k_border_point, k_border_heavy, k_scatter_labels",
}


def phase_bytes_per_point(phase: str, dim: int, f32: bool) -> int:
    """Compulsory HBM bytes per point of a phase: its own inputs read once and
    outputs written once (re-reads of neighbour cells are cache traffic, not
    algorithmic).  Coordinates are read as float32 (centred copy) in the
    float32-band mode, float64 otherwise."""
    c = (4 if f32 else 8) * dim
    return {"ms_index": 8 * dim + 4 + 4 + 8 * dim + (4 * dim if f32 else 0),  # in, key, id, X(,Xf)
            "ms_core": c + 1,            # coordinates in, core flag out
            "ms_union": c + 1,           # coordinates + core flag in
            "ms_label": c + 1 + 4 + 4}[phase]  # coordinates, core flag, point id in; label out


def max_over_ranks(x: float, dist) -> float:
    """The largest x over all ranks (one process per GPU); x itself in a
    single-process run.  Step times are combined this way, so the job's rate is
    set by its slowest replica."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds: float, world: int) -> float:
    """Whole-job rate of `world` replicas that each process units_per_rank in
    `seconds` (the slowest replica's time): the work is fixed per GPU (weak
    scaling), so the total grows with the replica count."""
    return world * units_per_rank / seconds


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def recorded_traffic(workload: str, precision: str, n: int):
    """DRAM bytes recorded by an ncu capture for this workload (profiles/), used
    only when the capture was taken on the sources of this build and on the same
    point count; otherwise None and the reason."""
    build = importlib.import_module(PKG + ".build")
    path = os.path.join(ROOT, "profiles", f"traffic_{workload}_{precision}.json")
    if not os.path.exists(path):
        return None, "no capture recorded"
    with open(path) as f:
        tj = json.load(f)
    digest = build.source_digest()
    if tj.get("source_digest") != digest:
        return None, f"capture {os.path.basename(path)} was taken on other sources"
    if int(tj.get("points", -1)) != int(n):
        return None, f"capture {os.path.basename(path)} was taken on {tj.get('points')} points"
    return tj, f"profiles/{os.path.basename(path)} (sources {digest})"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 2 + i and r[2 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def make_workload(name: str, scale: float = 1.0):
    ds = importlib.import_module(PKG + ".datasets")
    if scale != 1.0:
        return getattr(ds, name)(seed=0, scale=scale)
    return getattr(ds, name)(seed=0)


def cpu_baseline(name: str, target_s: float = 12.0):
    """The CPU restatement of the reference's exact DBSCAN on all host cores,
    on a bounded sample of the same workload (density-preserving scale-down)."""
    from oracle import oracle
    ds = importlib.import_module(PKG + ".datasets")
    cores = os.cpu_count() or 1
    scale = 0.01
    while True:
        inst = getattr(ds, name)(seed=0, scale=scale)
        t0 = time.perf_counter()
        oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts, nthreads=cores)
        dt = time.perf_counter() - t0
        if dt * 3 > target_s or scale >= 1.0:
            break
        scale = min(1.0, scale * max(2.0, min(8.0, target_s / max(dt, 1e-3) / 2)))
    return {"value": inst.n / dt, "unit": "points/s", "cores": cores, "kind": "port",
            "sample": f"{name} scale {scale:g}: {inst.n} points, one full run, {dt:.2f} s"}


def batch_cpu_baseline(insts, gpu_labels, poffs, stride: int = 16):
    """CPU-baseline leg of the batched workload: the oracle (all host cores) on
    every `stride`-th instance, timed, and its labels compared with the batched
    GPU run's labels of the same instances."""
    from oracle import oracle
    cores = os.cpu_count() or 1
    picked = list(range(0, len(insts), stride))
    t = 0.0
    pts = 0
    mismatched = []
    for i in picked:
        inst = insts[i]
        t0 = time.perf_counter()
        want, _, _ = oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts, nthreads=cores)
        t += time.perf_counter() - t0
        pts += inst.n
        got = gpu_labels[int(poffs[i]): int(poffs[i]) + inst.n]
        if not np.array_equal(got, want):
            mismatched.append(i)
    return ({"value": pts / t, "unit": "points/s", "cores": cores, "kind": "port",
             "sample": f"every {stride}th instance ({len(picked)} instances, {pts} points), "
                       f"one oracle run each, {t:.2f} s"},
            {"instances": len(picked), "points": pts, "sample": f"every {stride}th instance",
             "identical": not mismatched, "mismatched_instances": mismatched[:16]})


def run_reference(args, rank):
    """--impl reference: the reference's exact CPU DBSCAN on this host."""
    if rank != 0:
        return None
    from oracle import build as obuild
    from oracle import oracle
    ds = importlib.import_module(PKG + ".datasets")
    cores = os.cpu_count() or 1
    use_ref = os.path.exists(obuild.REF_RTREE_SO)
    wl = args.workload if args.workload in ("zipf2d_10m", "aniso3d_20m", "blobs2d_100k") \
        else "zipf2d_10m"
    dim = 3 if wl.startswith("aniso3d") else 2
    if use_ref and dim != 2:
        use_ref = False
    # bounded sample: grow the scale until one run takes ~2 s
    scale, inst, dt = 0.002, None, 0.0
    while True:
        inst = getattr(ds, wl)(seed=0, scale=scale)
        t0 = time.perf_counter()
        if use_ref:
            oracle.ref_rtree_dbscan(inst.points, inst.eps, inst.minpts)
        else:
            oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts, nthreads=cores)
        dt = time.perf_counter() - t0
        if dt > 2.0 or scale >= 1.0:
            break
        scale = min(1.0, scale * 4)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        if use_ref:
            oracle.ref_rtree_dbscan(inst.points, inst.eps, inst.minpts)
        else:
            oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts, nthreads=cores)
        times.append(time.perf_counter() - t0)
    t = sum(times)
    value = inst.n * len(times) / t
    kind = "reference" if use_ref else "port"
    return {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": wl, "points": inst.n, "dim": dim, "eps": inst.eps,
                   "minpts": inst.minpts, "precision": "fp64", "sample_scale": scale},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": 1 if use_ref else cores,
                         "kind": kind,
                         "sample": f"{wl} scale {scale:g} ({inst.n} points) per step"},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------- single run
def run_single(args, world, local, dist, workload, precision, scale, steps, warmup,
               with_cpu, rank):
    """One instance per step: device-resident timing, the other precision on the
    same data (labels must agree), end to end through gd_dbscan with pinned host
    buffers, and the roofline of the dominant phase."""
    import torch
    gdm = importlib.import_module(PKG)
    api = importlib.import_module(PKG + ".api")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    inst = make_workload(workload, scale)
    n, dim = inst.n, inst.dim
    prec = gdm.GD_PREC_FP64 if precision == "fp64" else gdm.GD_PREC_FP32_BAND

    stream = torch.cuda.current_stream(dev)
    ctx = gdm.Context(local, precision=prec)
    ctx.set_stream(stream.cuda_stream)
    pts_dev = torch.from_numpy(inst.points).to(dev)
    lab_dev = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)

    def step_device():
        ctx.index_build(pts_dev, inst.eps)
        ctx.expand(inst.minpts)
        ctx.get_result(out=lab_dev)

    def timed_device(k, w):
        for _ in range(w):
            step_device()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        evs = []
        phases = []
        for _ in range(k):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step_device()
            b.record(stream)
            evs.append((a, b))
            phases.append(ctx.stats())
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms = [a.elapsed_time(b) for a, b in evs]
        return ms, phases

    # headline: device-resident input, chosen precision
    with ClockSampler(local) as clk:
        ms, phases = timed_device(steps, warmup)
    clocks = clk.summary()
    t_step = sum(ms) / len(ms)
    t_step = max_over_ranks(t_step, dist)
    value = job_rate(n, t_step / 1e3, world)
    st = phases[-1]
    ref_labels = lab_dev.cpu().numpy()

    # the other precision on the same workload (labels must agree bit for bit)
    other = gdm.GD_PREC_FP32_BAND if prec == gdm.GD_PREC_FP64 else gdm.GD_PREC_FP64
    ctx.set_precision(other)
    ms2, ph2 = timed_device(max(3, steps // 2), 1)
    other_labels_equal = bool(np.array_equal(lab_dev.cpu().numpy(), ref_labels))
    ctx.set_precision(prec)

    # end to end through gd_dbscan: pinned host points in, pinned host labels out
    host_pts = torch.from_numpy(inst.points).pin_memory().numpy()
    host_lab = torch.empty(n, dtype=torch.int32).pin_memory().numpy()
    ctx2 = gdm.Context(local, precision=prec)
    gp = api.GdPoints(host_pts.ctypes.data, n, dim, 0)
    gst = api.GdStats()

    def step_e2e():
        api._check(ctx2._lib.gd_dbscan(ctx2._ctx, ctypes.byref(gp), inst.eps, inst.minpts,
                                       host_lab.ctypes.data, ctypes.byref(gst)))

    for _ in range(warmup):
        step_e2e()
    e2e_times = []
    for _ in range(steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_e2e()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_times) / len(e2e_times)
    e2e_s = max_over_ranks(e2e_s, dist)
    e2e_equal = bool(np.array_equal(host_lab, ref_labels))
    ctx2.close()

    peak, peak_kind = peaks()
    algo = ALGO_BYTES_PER_POINT[dim] * n
    achieved = algo / (t_step / 1e3) / 1e9
    # dominant phase: its kernels timed live by the library's CUDA events on its
    # stream, averaged over the timed steps
    f32 = int(st["precision_used"]) == 1
    ph_avg = {k: sum(p[k] for p in phases) / len(phases) for k in PHASE_KERNELS}
    dom = max(ph_avg, key=ph_avg.get)
    dom_bytes = phase_bytes_per_point(dom, dim, f32) * n
    dom_achieved = dom_bytes / (ph_avg[dom] / 1e3) / 1e9
    tj, traffic_from = recorded_traffic(workload, precision, n)
    traffic = tj.get("dram_bytes_per_step") if tj else None
    dom_traffic = tj.get("phases", {}).get(dom) if tj else None

    cpu = None
    if with_cpu and rank == 0 and world == 1:
        cpu = cpu_baseline(workload)

    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": t_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == gdm.GD_PREC_FP64 else "f32+f64band", "data": "synthetic",
        "config": {"workload": workload + ("" if scale == 1.0 else f" scale {scale:g}"),
                   "points": n, "dim": dim, "eps": inst.eps,
                   "minpts": inst.minpts, "precision": precision,
                   "parallelism": f"replicas{world}",
                   "l2": "512 MiB flush write between timed steps; inputs 160+ MB > L2"},
        "e2e": {"value": job_rate(n, e2e_s, world), "unit": "points/s",
                "h2d_bytes_per_step": n * dim * 8, "d2h_bytes_per_step": n * 4,
                "ms_per_step": e2e_s * 1e3, "labels_equal_device_run": e2e_equal,
                "last_step_ms": {"h2d": gst.ms_h2d, "pipeline": gst.ms_total,
                                 "d2h": gst.ms_d2h}},
        "gpu_launches": int(st["launches"]) * steps,
        "roofline": {"bound": "hbm", "achieved": dom_achieved, "peak": peak, "unit": "GB/s",
                     "frac": dom_achieved / peak, "traffic": dom_traffic,
                     "traffic_from": traffic_from,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)",
                     "kernel": f"{dom[3:]} phase: {PHASE_KERNELS[dom]}",
                     "ms_per_launch": ph_avg[dom], "algorithmic_bytes": dom_bytes,
                     "algorithmic_bytes_per_point": phase_bytes_per_point(dom, dim, f32)},
        "pipeline_roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                              "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                              "traffic_from": traffic_from,
                              "kernel": "whole single-instance pipeline (one step)",
                              "algorithmic_bytes": algo,
                              "algorithmic_bytes_per_point": ALGO_BYTES_PER_POINT[dim]},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "phases_ms": {k: sum(p[k] for p in phases) / len(phases)
                      for k in ("ms_index", "ms_core", "ms_union", "ms_label", "ms_total")},
        "counts": {k: st[k] for k in ("n_clusters", "n_noise", "n_core", "n_border", "n_cells",
                                      "n_dense_cells", "tests_fp64", "tests_fp32",
                                      "band_retests", "asym_pairs", "key_bits")},
        "other_precision": {"precision": "fp32band" if other == gdm.GD_PREC_FP32_BAND else "fp64",
                            "value": job_rate(n, max_over_ranks(sum(ms2) / len(ms2), dist) / 1e3,
                                              world),
                            "ms_per_step": sum(ms2) / len(ms2),
                            "labels_identical": other_labels_equal,
                            "tests_fp32": ph2[-1]["tests_fp32"],
                            "tests_fp64": ph2[-1]["tests_fp64"],
                            "band_retests": ph2[-1]["band_retests"],
                            "band_hit_rate": ph2[-1]["band_retests"] / max(1, ph2[-1]["tests_fp32"])},
    }
    ctx.close()
    del pts_dev, lab_dev, flush
    torch.cuda.empty_cache()
    return line


# ---------------------------------------------------------------- batched run
def run_batch(args, world, local, dist, steps, warmup, check_oracle, rank):
    """Batched workload: many independent instances (own eps, minpts, dim) in one
    gd_batch_dbscan run, against the single-instance path called once per
    instance on the same device-resident data (labels must agree)."""
    import torch
    gdm = importlib.import_module(PKG)
    api = importlib.import_module(PKG + ".api")
    ds = importlib.import_module(PKG + ".datasets")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    insts = ds.batch4096(seed=0, count=args.instances, workers=min(16, os.cpu_count() or 1))
    gen_s = time.perf_counter() - t0
    K = len(insts)
    desc = (api.GdInstance * K)()
    for i, inst in enumerate(insts):
        desc[i].n, desc[i].dim, desc[i].minpts, desc[i].eps = inst.n, inst.dim, inst.minpts, inst.eps
    flat = np.concatenate([inst.points.reshape(-1) for inst in insts])
    ntot = int(sum(inst.n for inst in insts))
    prec = gdm.GD_PREC_FP64 if args.precision_batch == "fp64" else gdm.GD_PREC_FP32_BAND
    stream = torch.cuda.current_stream(dev)
    ctx = gdm.Context(local, precision=prec)
    ctx.set_stream(stream.cuda_stream)
    tuning, tune_s, tune_ms = ctx.get_tuning(), 0.0, None
    if not args.no_autotune:
        # autotune on a sample: the first 256 instances (about 1/16 of the points)
        t0 = time.perf_counter()
        tuning, tune_ms = ctx.autotune([(i.points, i.eps, i.minpts) for i in insts[:256]])
        tune_s = time.perf_counter() - t0
    d_flat = torch.from_numpy(flat).to(dev)
    d_lab = torch.empty(ntot, dtype=torch.int32, device=dev)
    kc = np.zeros(K, dtype=np.int64)
    st = api.GdStats()

    def step_batch():
        api._check(ctx._lib.gd_batch_dbscan(ctx._ctx, K, desc, d_flat.data_ptr(), 1,
                                            d_lab.data_ptr(), kc.ctypes.data, ctypes.byref(st)))

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)
    for _ in range(warmup):
        step_batch()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = []
        for _ in range(steps):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step_batch()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
    t_batch = max_over_ranks(sum(ms) / len(ms), dist)
    batch_labels = d_lab.cpu().numpy()
    # the single-instance path once per instance, same device-resident data
    offs = np.cumsum([0] + [inst.n * inst.dim for inst in insts])
    poffs = np.cumsum([0] + [inst.n for inst in insts])
    loop_lab = torch.empty(ntot, dtype=torch.int32, device=dev)
    gp = api.GdPoints()

    def step_loop():
        for i, inst in enumerate(insts):
            gp.coords = d_flat.data_ptr() + int(offs[i]) * 8
            gp.n, gp.dim, gp.on_device = inst.n, inst.dim, 1
            api._check(ctx._lib.gd_dbscan(ctx._ctx, ctypes.byref(gp), inst.eps, inst.minpts,
                                          loop_lab.data_ptr() + int(poffs[i]) * 4, None))

    step_loop()
    torch.cuda.synchronize()
    loops = []
    for _ in range(max(1, min(args.loop_repeats, steps))):
        torch.cuda.synchronize()
        a = time.perf_counter()
        step_loop()
        torch.cuda.synchronize()
        loops.append(time.perf_counter() - a)
    t_loop = sum(loops) / len(loops)
    same = bool(np.array_equal(loop_lab.cpu().numpy(), batch_labels))
    # end to end with pinned host buffers
    h_flat = torch.from_numpy(flat).pin_memory().numpy()
    h_lab = torch.empty(ntot, dtype=torch.int32).pin_memory().numpy()

    def step_e2e():
        api._check(ctx._lib.gd_batch_dbscan(ctx._ctx, K, desc, h_flat.ctypes.data, 0,
                                            h_lab.ctypes.data, kc.ctypes.data, ctypes.byref(st)))

    step_e2e()
    e2e = []
    for _ in range(steps):
        torch.cuda.synchronize()
        a = time.perf_counter()
        step_e2e()
        e2e.append(time.perf_counter() - a)
    t_e2e = max_over_ranks(sum(e2e) / len(e2e), dist)
    same_e2e = bool(np.array_equal(h_lab, batch_labels))
    peak, peak_kind = peaks()
    algo = int(sum(inst.n * (8 * inst.dim + 4) for inst in insts))
    achieved = algo / (t_batch / 1e3) / 1e9
    value = job_rate(ntot, t_batch / 1e3, world)
    cpu, vs_oracle = None, None
    if check_oracle and rank == 0:
        cpu, vs_oracle = batch_cpu_baseline(insts, batch_labels, poffs)
    line = {
        "metric": METRIC + " (batched instances)", "value": value, "unit": "points/s",
        "n_gpus": world, "steps": steps, "warmup": warmup, "ms_per_step": t_batch,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == gdm.GD_PREC_FP64 else "f32+f64band", "data": "synthetic",
        "config": {"workload": "batch4096", "instances": K, "points": ntot,
                   "dims": {"2": int(sum(i.dim == 2 for i in insts)),
                            "3": int(sum(i.dim == 3 for i in insts))},
                   "precision": args.precision_batch, "parallelism": f"replicas{world}",
                   "generation_s": round(gen_s, 1),
                   "eps": "median exact 4th-NN distance over 2,048 sampled query points "
                          "(all points when fewer)",
                   "tuning": tuning, "autotune": None if args.no_autotune else
                   {"sample": "first 256 instances", "seconds": round(tune_s, 2),
                    "sample_device_ms": tune_ms},
                   "l2": "512 MiB flush write between timed steps"},
        "e2e": {"value": job_rate(ntot, t_e2e, world), "unit": "points/s",
                "h2d_bytes_per_step": int(flat.nbytes), "d2h_bytes_per_step": ntot * 4,
                "ms_per_step": t_e2e * 1e3, "labels_equal_device_run": same_e2e},
        "looped_single_instance": {"value": ntot / t_loop, "ms_per_batch": t_loop * 1e3,
                                   "repeats": len(loops),
                                   "speedup_batched": t_loop * 1e3 / t_batch,
                                   "labels_identical": same},
        "labels_vs_oracle": vs_oracle,
        "cpu_baseline": cpu,
        "gpu_launches": int(st.launches) * steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": "whole batched pipeline (one step)", "algorithmic_bytes": algo},
        "clocks": clk.summary(),
        "phases_ms": {k: getattr(st, k) for k in ("ms_index", "ms_core", "ms_union", "ms_label",
                                                  "ms_total")},
        "counts": {k: getattr(st, k) for k in ("n_clusters", "n_noise", "n_core", "n_cells",
                                               "tests_fp64", "tests_fp32", "band_retests")},
    }
    ctx.close()
    del d_flat, d_lab, loop_lab, flush
    torch.cuda.empty_cache()
    return line


def _pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if len(xs) else None


# ---------------------------------------------------------------- served run
def run_serve(args, world, local, dist, duration, hi_duration):
    """Served request stream through the request server (gd_server_*): Poisson
    arrivals, every request with its own points, eps, minpts and dimension, host
    buffers in and labels out.  Open loop at the stream's rate gives p50/p99
    latency; a closed loop (every request queued at once) gives the saturation
    throughput.  Both are compared with one-at-a-time plain solves (gd_dbscan
    per request, in arrival order) on the same requests, and every request's
    labels must be identical in both.  A second open loop runs at 80% of the
    one-at-a-time saturation rate, where requests arrive while others are on
    the GPU and batching has something to batch."""
    import torch
    gdm = importlib.import_module(PKG)
    ds = importlib.import_module(PKG + ".datasets")
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    pool, arrivals, which = ds.serve_stream(seed=0, rate=args.rate, duration=duration,
                                            pool=args.pool,
                                            workers=min(16, os.cpu_count() or 1))
    gen_s = time.perf_counter() - t0
    # pinned host copies: both arms read the same host buffers
    pts = [torch.from_numpy(np.ascontiguousarray(i.points)).pin_memory().numpy() for i in pool]
    prec = gdm.GD_PREC_FP64 if args.precision_serve == "fp64" else gdm.GD_PREC_FP32_BAND
    budget = int(args.hbm_budget_gb * (1 << 30))

    def open_loop_server(srv, arr, wh):
        nreq = len(arr)
        ids = [None] * nreq
        start = time.perf_counter()

        def submitter():
            for r in range(nreq):
                d = start + arr[r] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                inst = pool[wh[r]]
                ids[r] = srv.submit(pts[wh[r]], inst.eps, inst.minpts)

        th = threading.Thread(target=submitter)
        th.start()
        lat, labs, batch = [], [], []
        first = last = None
        for r in range(nreq):
            while ids[r] is None:
                time.sleep(0.0002)
            lab, info = srv.wait(ids[r])
            lat.append(info["done_ms"] - info["submit_ms"])
            batch.append(info["batch_size"])
            first = info["submit_ms"] if first is None else min(first, info["submit_ms"])
            last = info["done_ms"] if last is None else max(last, info["done_ms"])
            labs.append(lab)
        th.join()
        return lat, labs, batch, (last - first) / 1e3

    def open_loop_single(ctx, arr, wh):
        lat, labs = [], []
        start = time.perf_counter()
        for r in range(len(arr)):
            at = start + arr[r]
            d = at - time.perf_counter()
            if d > 0:
                time.sleep(d)
            inst = pool[wh[r]]
            labs.append(ctx.dbscan(pts[wh[r]], inst.eps, inst.minpts))
            lat.append((time.perf_counter() - at) * 1e3)
        return lat, labs, time.perf_counter() - start - arr[0]

    nreq = len(arrivals)
    sat_n = min(nreq, args.saturation_requests)

    def closed_loop_server(srv):
        a = time.perf_counter()
        ids = [srv.submit(pts[which[r]], pool[which[r]].eps, pool[which[r]].minpts)
               for r in range(sat_n)]
        for i in ids:
            srv.wait(i)
        return time.perf_counter() - a

    def closed_loop_single(ctx):
        torch.cuda.synchronize()
        a = time.perf_counter()
        for r in range(sat_n):
            ctx.dbscan(pts[which[r]], pool[which[r]].eps, pool[which[r]].minpts)
        return time.perf_counter() - a

    ctx = gdm.Context(local, precision=prec)
    srv = gdm.Server(local, workers=args.workers, max_batch=args.max_batch, precision=prec,
                     hbm_budget_bytes=budget)
    try:
        # warm-up: every pool instance once, so device buffers are grown
        for i in [srv.submit(p, inst.eps, inst.minpts) for p, inst in zip(pts, pool)]:
            srv.wait(i)
        for p, inst in zip(pts, pool):
            ctx.dbscan(p, inst.eps, inst.minpts)
        with ClockSampler(local) as clk:
            s_lat, s_labs, s_batch, s_span = open_loop_server(srv, arrivals, which)
        with ClockSampler(local) as clk1:
            o_lat, o_labs, o_span = open_loop_single(ctx, arrivals, which)
        sat_server = closed_loop_server(srv)
        sat_single = closed_loop_single(ctx)
        # open loop near the one-at-a-time saturation rate
        hi_rate = 0.8 * sat_n / sat_single
        hi_arr = ds.poisson_arrivals(5, hi_rate, hi_duration)
        hi_which = np.random.Generator(np.random.PCG64(6)).integers(0, len(pool),
                                                                     size=hi_arr.shape[0])
        with ClockSampler(local) as clk2:
            h_lat, h_labs, h_batch, h_span = open_loop_server(srv, hi_arr, hi_which)
            ho_lat, ho_labs, ho_span = open_loop_single(ctx, hi_arr, hi_which)
        sstats = srv.stats()
    finally:
        srv.close()
        ctx.close()
    same = all(np.array_equal(a, b) for a, b in zip(s_labs, o_labs))
    same_hi = all(np.array_equal(a, b) for a, b in zip(h_labs, ho_labs))
    npts = np.array([pool[w].n for w in which], dtype=np.int64)
    total = int(npts.sum())
    hi_total = int(sum(pool[w].n for w in hi_which))
    sat_pts = int(npts[:sat_n].sum())
    sat_server = max_over_ranks(sat_server, dist)
    value = job_rate(sat_pts, sat_server, world)
    return {
        "metric": METRIC + " (served request stream)", "value": value, "unit": "points/s",
        "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": sat_server * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == gdm.GD_PREC_FP64 else "f32+f64band", "data": "synthetic",
        "config": {"workload": "serve", "rate_per_s": args.rate, "duration_s": duration,
                   "requests": nreq, "points": total, "pool_instances": len(pool),
                   "sizes": "log-uniform [1000, 2000000]", "workers": args.workers,
                   "max_batch": args.max_batch, "hbm_budget_gb": args.hbm_budget_gb,
                   "precision": args.precision_serve, "parallelism": f"replicas{world}",
                   "generation_s": round(gen_s, 1),
                   "l2": "inputs stream from host memory every request"},
        "serve": {"p50_ms": _pct(s_lat, 50), "p99_ms": _pct(s_lat, 99),
                  "max_ms": max(s_lat), "throughput_points_s": total / s_span,
                  "mean_batch": float(np.mean(s_batch)), "max_batch": int(max(s_batch)),
                  "clocks": clk.summary()},
        "one_at_a_time": {"p50_ms": _pct(o_lat, 50), "p99_ms": _pct(o_lat, 99),
                          "max_ms": max(o_lat), "throughput_points_s": total / o_span,
                          "saturation_points_s": sat_pts / sat_single,
                          "clocks": clk1.summary()},
        "saturation": {"requests": sat_n, "points": sat_pts, "server_s": sat_server,
                       "one_at_a_time_s": sat_single, "speedup": sat_single / sat_server},
        "near_saturation": {"rate_per_s": hi_rate, "duration_s": hi_duration,
                            "requests": int(hi_arr.shape[0]), "points": hi_total,
                            "server": {"p50_ms": _pct(h_lat, 50), "p99_ms": _pct(h_lat, 99),
                                       "throughput_points_s": hi_total / h_span,
                                       "mean_batch": float(np.mean(h_batch)),
                                       "max_batch": int(max(h_batch))},
                            "one_at_a_time": {"p50_ms": _pct(ho_lat, 50),
                                              "p99_ms": _pct(ho_lat, 99),
                                              "throughput_points_s": hi_total / ho_span},
                            "labels_identical": same_hi, "clocks": clk2.summary()},
        "server_stats": {"batches": int(sstats["batches"]), "failed": int(sstats["failed"])},
        "labels_identical": same,
        "e2e": {"value": value, "unit": "points/s",
                "h2d_bytes_per_step": int(sum(pts[which[r]].nbytes for r in range(sat_n))),
                "d2h_bytes_per_step": sat_pts * 4},
        "clocks": clk.summary(),
    }


def _extra_c3(args, world, local, dist, rank):
    t0 = time.perf_counter()
    c3 = run_single(args, world, local, dist, "aniso3d_20m", "fp32band", 1.0,
                    args.extra_steps, 3, False, rank)
    keep = ("value", "unit", "ms_per_step", "steps", "warmup", "dtype", "config", "e2e",
            "clocks", "phases_ms", "counts", "roofline", "gpu_launches")
    out = {k: c3[k] for k in keep}
    op = c3["other_precision"]
    out["plain_fp64"] = {"value": op["value"], "ms_per_step": op["ms_per_step"],
                         "labels_identical": op["labels_identical"]}
    out["band_hit_rate"] = c3["counts"]["band_retests"] / max(1, c3["counts"]["tests_fp32"])
    out["speedup_vs_plain_fp64"] = c3["value"] / op["value"]
    out["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def _extra_c4(args, world, local, dist, rank):
    t0 = time.perf_counter()
    c4 = run_batch(args, world, local, dist, args.extra_steps, 3, True, rank)
    keep = ("value", "unit", "ms_per_step", "steps", "warmup", "dtype", "config", "e2e",
            "looped_single_instance", "labels_vs_oracle", "cpu_baseline", "clocks",
            "phases_ms", "counts", "roofline", "gpu_launches")
    out = {k: c4[k] for k in keep}
    out["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def _extra_c5(args, world, local, dist, rank):
    t0 = time.perf_counter()
    c5 = run_serve(args, world, local, dist, args.extra_serve_duration, args.hi_duration)
    keep = ("value", "unit", "dtype", "config", "serve", "one_at_a_time", "saturation",
            "near_saturation", "server_stats", "labels_identical", "e2e", "clocks")
    out = {k: c5[k] for k in keep}
    out["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def _extra_import():
    """Dataset import on the host (the reference's ImportDataset, main.cu:469-498,
    parses text): the same points read from the reference's CSV format and from
    the raw float64 ('.f64') format through gd_import_dataset, on a
    1,000,000-point sample of the 10M-point 2D workload (time grows linearly)."""
    import tempfile
    api = importlib.import_module(PKG + ".api")
    ds = importlib.import_module(PKG + ".datasets")
    inst = ds.zipf2d_10m(seed=0, scale=0.1)
    out = {"points": inst.n, "dim": inst.dim}
    with tempfile.TemporaryDirectory() as tmp:
        csv, raw = os.path.join(tmp, "pts.csv"), os.path.join(tmp, "pts.f64")
        ds.write_csv(csv, inst.points)
        np.ascontiguousarray(inst.points).tofile(raw)
        for name, path in (("csv", csv), ("f64", raw)):
            best = None
            for _ in range(2):
                t0 = time.perf_counter()
                pts = api.import_dataset(path, inst.dim)
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            out[name] = {"seconds": best, "points_per_s": inst.n / best,
                         "bytes": os.path.getsize(path),
                         "equal_to_source": bool(np.array_equal(pts, inst.points))}
    out["f64_speedup"] = out["csv"]["seconds"] / out["f64"]["seconds"]
    out["full_10m_estimate_s"] = {k: out[k]["seconds"] * 10 for k in ("csv", "f64")}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="zipf2d_10m",
                    choices=["zipf2d_10m", "aniso3d_20m", "blobs2d_100k", "batch4096", "serve"])
    ap.add_argument("--instances", type=int, default=4096,
                    help="batch4096 workload: number of instances")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32band"])
    ap.add_argument("--precision-batch", default="fp32band", choices=["fp64", "fp32band"],
                    help="batched and served workloads: precision mode")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default run: leave out the c3 / c4 / c5 keys")
    ap.add_argument("--extra-steps", type=int, default=5,
                    help="timed steps of the c3 and c4 keys")
    ap.add_argument("--extra-serve-duration", type=float, default=30.0,
                    help="c5 key: seconds of the 200 req/s stream")
    ap.add_argument("--hi-duration", type=float, default=10.0,
                    help="serve: seconds of the open loop near one-at-a-time saturation")
    ap.add_argument("--loop-repeats", type=int, default=1,
                    help="batch: timed repeats of the looped single-instance path")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batch4096: keep the default tuning instead of autotuning on a sample")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="single-instance workloads: density-preserving size factor (profiling)")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: stream seconds")
    ap.add_argument("--pool", type=int, default=512, help="serve: distinct request instances")
    ap.add_argument("--workers", type=int, default=2, help="serve: server worker streams")
    ap.add_argument("--max-batch", type=int, default=1024, help="serve: requests per batch")
    ap.add_argument("--hbm-budget-gb", type=float, default=150.0,
                    help="serve: admission budget for requests in flight")
    ap.add_argument("--saturation-requests", type=int, default=2000,
                    help="serve: requests of the closed-loop throughput run")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    args.precision_serve = args.precision_batch
    if args.workload in ("batch4096", "serve"):
        args.precision_batch = args.precision_serve = args.precision

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    if args.impl == "reference":
        line = run_reference(args, rank)
        if rank == 0:
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    gdm = importlib.import_module(PKG)
    gdm.load_library()
    if args.workload == "batch4096":
        line = run_batch(args, world, local, dist, args.steps, args.warmup,
                         not args.no_cpu_baseline, rank)
    elif args.workload == "serve":
        line = run_serve(args, world, local, dist, args.duration, args.hi_duration)
    else:
        line = run_single(args, world, local, dist, args.workload, args.precision, args.scale,
                          args.steps, args.warmup, not args.no_cpu_baseline, rank)
        if (world == 1 and not args.no_extras and args.workload == "zipf2d_10m"
                and args.scale == 1.0):
            line["c3"] = _extra_c3(args, world, local, dist, rank)
            line["c4"] = _extra_c4(args, world, local, dist, rank)
            line["c5"] = _extra_c5(args, world, local, dist, rank)
            line["import_io"] = _extra_import()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
