"""Benchmark: P+B boxes/s of the PBI4 estimator path on GB300.

Workload (one "step" = one box through the whole path): 2,097,152 particles
(128^3 lattice) displaced by the Zel'dovich approximation (P(k) ~ k^-1.5, rms
displacement 5 Mpc/h, RSD along z with f = 0.7) in L = 1000 Mpc/h; grid 256^3,
PCS with interlacing; P(k) multipoles l = 0,2,4 with dk = kf (128 bins);
bispectrum B0,B2,B4 over all (open) triangles with dk = 3 kf up to 0.5 k_Nyq
(21 shells, 1156 triangles).  Triangle counts depend only on the binning and
are computed once per plan (the reference caches them in its cfile).

Lines printed (rank 0): one JSON line for our arm, or for ``--impl reference``
the CPU restatement of the reference (oracle/, serial loops as in the Fortran,
FFTs on all host cores) timed on a bounded sample and extrapolated per box.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="zeldovich_256_pcs_interlaced_P024_B024", particles=128 ** 3, box=1000.0, grid=256,
                nintp=4, interlacing=True, multipoles=True, los=[0.0, 0.0, 1.0], kbin_ps=1.0, kcenter_ps=1.0,
                nbins_ps=128, kbin_bs=3.0, kcenter_bs=3.0, nbins_bs=21, iopen=True)
METRIC = "P+B boxes/s @256^3 PCS interlaced (P l=0,2,4 + B l=0,2,4)"


def make_positions(quick=False, small=False):
    from pbi4_gb300 import synthetic
    n = 32 if quick else (64 if small else 128)
    return synthetic.zeldovich_box(n, WORKLOAD["box"], n_s=-1.5, rms_disp=5.0, f_growth=0.7, seed=2)


def est_config(precision, grid=None):
    from pbi4_gb300.estimator import EstimatorConfig
    w = WORKLOAD
    return EstimatorConfig(grid=grid or w["grid"], box=w["box"], nintp=w["nintp"], interlacing=w["interlacing"],
                           multipoles=w["multipoles"], los=tuple(w["los"]), kbin_ps=w["kbin_ps"],
                           kcenter_ps=w["kcenter_ps"], nbins_ps=w["nbins_ps"] if grid is None else None,
                           do_bispectrum=True, kbin_bs=w["kbin_bs"], kcenter_bs=w["kcenter_bs"],
                           nbins_bs=w["nbins_bs"] if grid is None else None, iopen=w["iopen"], precision=precision)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 9 for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ------------------------------------------------------------ CPU legs ---
def oracle_params(grid=None):
    """The workload as a reference params dict (pbi4.py:86-119), with the
    bispectrum's own binning (kbin_bs, kcenter_bs, nbins_bisp, itot).  A smaller
    `grid` (the debug cases) keeps the binning widths and derives the bin counts."""
    from oracle import pbi4_oracle as O
    w = WORKLOAD
    g = grid or w["grid"]
    p = dict(grid=g, box=w["box"], interpolation=w["nintp"], interlacing=w["interlacing"],
             multipoles=w["multipoles"], kbin=w["kbin_ps"], kcenter=w["kcenter_ps"], iopen=w["iopen"], los=w["los"],
             cross=False, om=0.3, ol=0.7, z=0.5)
    p.update(O.derived_params(p))
    nb = w["nbins_bs"] if grid is None else int((g / 3 + w["kbin_bs"] - w["kcenter_bs"]) // w["kbin_bs"])
    p.update(kbin_bs=w["kbin_bs"], kcenter_bs=w["kcenter_bs"], nbins_bisp=nb,
             itot=O.itot(nb, w["kbin_bs"], w["kcenter_bs"], w["iopen"]))
    return p


def oracle_full_box(pos, workers, grid=None):
    """One whole box through the CPU restatement of the reference (every stage
    computed: assignment, density FFT + fcomb, the 22 multipole FFT passes, P
    binning, 63 shell-map FFTs, 1156 x 3 triangle sums), after the triangle
    counts (input independent, computed first like the reference's cfile).
    Returns (pout, bout, seconds of the box, seconds per cost class, counts
    seconds, the FP64 counts)."""
    from oracle import pbi4_oracle as O
    bp = O.BoxPipeline(pos, oracle_params(grid), workers=workers)
    t0 = time.perf_counter()
    bp.compute_counts()
    t_counts = time.perf_counter() - t0
    t0 = time.perf_counter()
    stages = bp.run_all()
    return bp.pout, bp.bout, time.perf_counter() - t0, stages, t_counts, bp.counts


ORACLE_SAMPLE = ("one whole 256^3 box, every stage computed (no extrapolation): serial assignment, density FFT + "
                 "fcomb, 1 ifftn + 21 fftn multipole passes, serial P binning, 63 shell-map FFTs, 1156 x 3 triangle "
                 "sums; triangle counts computed once before the box (input independent, the reference's cfile). "
                 "FFTs (scipy.fft) on %d threads (the reference: FFTW npool threads for the maps, single-threaded "
                 "scipy fftn for the density), triangle rows split over %d threads (each row the reference's serial "
                 "loop); assignment, fcomb and binning loops serial as in the Fortran")


def run_reference(args):
    """The reference's CPU path (the oracle restatement) on this host's cores.
    The warm-up computes the triangle counts and one whole box (which also
    measures the cost of each of the box's work items); the K timed steps then
    compute one more whole box, its work items split in order into K
    contiguous groups of about equal measured cost, one group per step.  The
    timed region is exactly one box: value = 1 / (sum of the K step times)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import pbi4_oracle as O
    O.build()
    pos = make_positions(quick=args.quick)
    cores = os.cpu_count() or 1
    p = oracle_params(64 if args.quick else None)
    # warm-up: counts + one whole box with per-item timing
    bp = O.BoxPipeline(pos, p, workers=cores)
    bp.compute_counts()
    cost = []
    for name, cls, fn in bp.items():
        t0 = time.perf_counter()
        fn()
        cost.append(time.perf_counter() - t0)
    # timed: one whole box in K contiguous groups of about equal cost
    bp2 = O.BoxPipeline(pos, p, counts=bp.counts, workers=cores)
    items = bp2.items()
    total = sum(cost)
    K = args.steps
    bounds, acc, k = [], 0.0, 0
    for idx, c in enumerate(cost):
        acc += c
        if acc >= total * (k + 1) / K and k < K - 1:
            bounds.append(idx + 1)
            k += 1
    bounds = [0] + bounds + [len(items)] * (K - len(bounds))
    step_s = []
    for k in range(K):
        t0 = time.perf_counter()
        for _, _, fn in items[bounds[k]: bounds[k + 1]]:
            fn()
        step_s.append(time.perf_counter() - t0)
    box_s = sum(step_s)
    value = 1.0 / box_s
    sample = ORACLE_SAMPLE % (cores, cores) + "; the timed steps are one box split into %d groups of its work items" % K
    line = {"metric": METRIC, "value": value, "unit": "boxes/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": box_s * 1e3 / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Zel'dovich box)",
            "config": bench_config(args.gpus), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "boxes/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "boxes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "box_seconds": box_s, "warmup_box_seconds": total,
            "step_seconds": [round(x, 3) for x in step_s]}
    print(json.dumps(line), flush=True)


def bench_config(world):
    """The workload's `config` (the same in both arms)."""
    return {**WORKLOAD, "parallelism": f"replicas{world}",
            "l2": "working set > L2 (a box's shell maps are 2.0 GB on the 200^3 map grid; the density grids 0.27 GB)",
            "triangle_counts": "computed once per binning, outside the timed region (input independent)"}


# ------------------------------------------------------------ GPU arm ---
DTYPE = {"fp32": "f32", "fp64": "f64", "fp16split": "fp16 hi+lo (f32 accumulate)", "bf16": "bf16 (f32 accumulate)",
         "tf32split": "tf32 hi+lo (f32 accumulate)"}


def error_report(pout, bout, pref, bref, tol, counts=None, counts_ref=None, grid=None):
    """Per-bin errors against a reference run (the oracle, or the FP64 GPU form).

    Plain relative errors |x / x_ref - 1| of every P_l and B_l bin: the maximum,
    and how many bins exceed `tol`.  Beside them the two normalised metrics:
    P2, P4 relative to P0 (the multipoles cross zero), and B_l relative to
    max(|B_l|, (2l+1)(P1P2 + P1P3 + P2P3)) (the reduced bispectrum where B_l
    itself is near zero).  Mode and triangle counts must be identical: with the
    oracle's FP64 counts (counts_ref = N^3 N_tri, an FFT sum) and this library's
    exact integers (counts), the integers are compared; the float32 N_tr column of
    the reference rounds its FP64 sum, so above 2^24 a count halfway between two
    float32 values may land on the other neighbour (Ntr_float32_ties)."""
    ok = pref[4] > 0
    e = {"tol": tol, "P_bins": int(ok.sum()), "B_bins": int(bref.shape[1]),
         "Nmodes_equal": bool(np.array_equal(pout[4], pref[4]))}
    if counts is not None and counts_ref is not None:
        exact_ref = np.round(np.asarray(counts_ref) / float(grid) ** 3).astype(np.int64)
        e["Ntr_integer_equal"] = bool(np.array_equal(np.asarray(counts, dtype=np.int64), exact_ref))
        e["Ntr_float32_ties"] = int((bout[8] != bref[8]).sum())
    else:
        e["Ntr_equal"] = bool(np.array_equal(bout[8], bref[8]))
    for name, r in (("P0", 1), ("P2", 2), ("P4", 3)):
        rel = np.abs(pout[r][ok] / pref[r][ok] - 1)
        e[name + "_max_rel"] = float(rel.max())
        e[name + "_bins_above_tol"] = int((rel > tol).sum())
        if r > 1:
            e[name + "_max_rel_to_P0"] = float(np.max(np.abs(pout[r][ok] - pref[r][ok]) / np.abs(pref[1][ok])))
    den = np.abs(bref[3] * bref[4]) + np.abs(bref[3] * bref[5]) + np.abs(bref[4] * bref[5])
    for name, r, f in (("B0", 6, 1.0), ("B2", 9, 5.0), ("B4", 10, 9.0)):
        rel = np.abs(bout[r] / bref[r] - 1)
        e[name + "_max_rel"] = float(rel.max())
        e[name + "_median_rel"] = float(np.median(rel))
        e[name + "_bins_above_tol"] = int((rel > tol).sum())
        e[name + "_max_rel_Q"] = float(np.max(np.abs(bout[r] - bref[r]) / np.maximum(np.abs(bref[r]), f * den)))
    e["shell_powers_max_rel"] = float(np.max(np.abs(bout[3:6] / bref[3:6] - 1)))
    return e


def run_ours(args):
    import torch
    import torch.distributed as dist

    from pbi4_gb300 import replicas
    from pbi4_gb300.estimator import Estimator

    # N GPUs: independent replicas, each rank runs whole boxes; no data-path collective
    world, rank, local = replicas.init("nccl")
    barrier = replicas.barrier

    pos = make_positions(quick=args.quick, small=args.small)
    npart = pos.shape[1]
    grid = 64 if args.quick else (128 if args.small else None)
    cfg = est_config(args.precision, grid=grid)
    est = Estimator(cfg)
    itot, map_grid, nmaps = est.itot, est.map_grid, est.nmaps
    dpos = torch.from_numpy(pos).cuda()
    pout, bout = est.alloc_outputs()

    def timed(e, po, bo, steps, clocks=False):
        """Device time of `steps` boxes on plan e (CUDA events on the plan's stream = torch's current)."""
        for _ in range(args.warmup):  # plan tables, triangle counts, cuFFT plans
            e.run_device(npart, dpos, po, bo)
        torch.cuda.synchronize()
        e.enable_timing(True)
        e.stage_times()
        l0 = e.launches
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            start.record()
            for _ in range(steps):
                e.run_device(npart, dpos, po, bo)
            stop.record()
            torch.cuda.synchronize()
        barrier()
        st = e.stage_times()
        e.enable_timing(False)
        return replicas.max_over_ranks(start.elapsed_time(stop)), e.launches - l0, st, clk.summary()

    # one box in flight: the per-stage times and the roofline come from this pass
    ms_one, launches_one, stages, clocks_one = timed(est, pout, bout, args.steps)
    tri_counts = est.triangle_counts()
    value_one = replicas.throughput(world * args.steps, ms_one / 1e3)
    map_work = est.map_work()
    tensor_units = est.tensor_units()

    # K boxes in flight (the batched form): K plans on K streams take the boxes
    # in turn, so one box's low-occupancy phases (kernel tails, the tile scan,
    # the small kernels) overlap the others' work
    K = max(1, args.boxes_in_flight)
    streams = [torch.cuda.Stream() for _ in range(K)]
    est.set_stream(streams[0])
    ests = [est] + [Estimator(cfg, stream=streams[k]) for k in range(1, K)]
    outs = [(pout, bout)] + [e.alloc_outputs() for e in ests[1:]]
    for e, (po, bo) in zip(ests, outs):
        for _ in range(args.warmup):
            e.run_device(npart, dpos, po, bo)
    torch.cuda.synchronize()
    l0 = sum(e.launches for e in ests)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    joined = [torch.cuda.Event() for _ in range(K)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(streams[0])
        for k in range(1, K):
            streams[k].wait_event(start)
        for i in range(args.steps):
            ests[i % K].run_device(npart, dpos, *outs[i % K])
        for k in range(1, K):
            joined[k].record(streams[k])
            streams[0].wait_event(joined[k])
        stop.record(streams[0])
        torch.cuda.synchronize()
    barrier()
    for e in ests:
        e.check()
    ms_max = replicas.max_over_ranks(start.elapsed_time(stop))
    launches = sum(e.launches for e in ests) - l0
    clocks = clk.summary()
    value = replicas.throughput(world * args.steps, ms_max / 1e3)

    # e2e: host (pinned) positions in, host results out, through the C-ABI call
    # (pbi4g_plan_run_host), C callers (host threads, one plan and stream each)
    # so one box's copies overlap the others' kernels
    import threading as _th
    C = max(1, args.e2e_callers)
    eps = ests[:C] + [Estimator(cfg, stream=torch.cuda.Stream()) for _ in range(C - len(ests))]
    hpos = torch.from_numpy(pos).pin_memory().numpy()
    for e in eps:
        for _ in range(2):
            e.run_host(hpos)
    e2e_steps = max(C, args.steps)
    results = [[] for _ in range(C)]

    def caller(k, n):
        for _ in range(n):
            results[k].append(eps[k].run_host(hpos))

    barrier()
    t0 = time.perf_counter()
    th = [_th.Thread(target=caller, args=(k, len(range(k, e2e_steps, C)))) for k in range(C)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0)
    e2e_value = replicas.throughput(world * e2e_steps, e2e_s)
    p_h, b_h = results[0][-1]
    est.set_stream(None)
    for e in set(ests[1:] + eps[1:]):
        e.close()

    # the plain FP32 GPU form on the same box; the errors of both forms against the
    # oracle (one whole box of the CPU restatement of the reference, which is also
    # the timed cpu_baseline) and against the FP64 GPU form
    plain = errors = errors64 = cpu = None
    tol = 1e-5 if args.precision in ("fp32", "fp64") else 1e-4
    if rank == 0 and not (args.no_compare and args.no_cpu_baseline):
        if not args.no_compare and args.precision != "fp32":
            e32 = Estimator(est_config("fp32", grid=grid))
            po32, bo32 = e32.alloc_outputs()
            ms32, _, _, _ = timed(e32, po32, bo32, max(3, args.steps // 4))
            plain = {"value": max(3, args.steps // 4) / (ms32 / 1e3), "unit": "boxes/s",
                     "ms_per_step": ms32 / max(3, args.steps // 4)}
            p32, b32 = e32.run_host(pos)
            e32.close()
        if not args.no_compare:
            e64 = Estimator(est_config("fp64", grid=grid))
            p64, b64 = e64.run_host(pos)
            e64.close()
            errors64 = error_report(p_h, b_h, p64, b64, tol)
            if plain is not None:
                plain["error_vs_fp64_gpu"] = error_report(p32, b32, p64, b64, 1e-5)
        cores = os.cpu_count() or 1
        pref, bref, box_s, cls_s, counts_s, counts_ref = oracle_full_box(pos, cores, grid=grid)
        if not args.no_cpu_baseline:
            cpu = {"value": 1.0 / box_s, "unit": "boxes/s", "cores": cores, "kind": "port",
                   "sample": ORACLE_SAMPLE % (cores, cores), "seconds_by_stage": {k: round(v, 3) for k, v in
                                                                                cls_s.items()},
                   "triangle_counts_seconds": round(counts_s, 3)}
        if not args.no_compare:
            g = grid or WORKLOAD["grid"]
            errors = error_report(p_h, b_h, pref, bref, tol, tri_counts, counts_ref, g)
            if plain is not None:
                plain["error_vs_oracle"] = error_report(p32, b32, pref, bref, 1e-5, tri_counts, counts_ref, g)

    # serving: a short Poisson stream of mixed boxes through the continuous-batching loop
    serving = None
    if args.serve_requests > 0 and rank == 0 and not args.quick and not args.small:
        from pbi4_gb300 import serve_workload
        est.close()
        torch.cuda.empty_cache()
        reqs = serve_workload.make_stream(n_requests=args.serve_requests, grids=(128, 192, 256, 384),
                                          npart_min=1e5, npart_max=args.serve_npart_max, rate_hz=args.serve_rate,
                                          precision=args.precision)
        live = serve_workload.run_stream(reqs, hbm_budget_gb=200.0, slots=3, batch=4, realtime=True)
        sat = serve_workload.run_stream(reqs, hbm_budget_gb=200.0, slots=3, batch=4, realtime=False)
        n_serial = min(len(reqs), 500)
        serial = serve_workload.run_serial_plain(reqs[:n_serial])
        r3 = lambda x: round(x, 3)
        serving = {"requests": live["n"], "offered_rate_hz": args.serve_rate,
                   "p50_ms": r3(live["p50_ms"]), "p99_ms": r3(live["p99_ms"]),
                   "queue_p50_ms": r3(live["queue_p50_ms"]), "queue_p99_ms": r3(live["queue_p99_ms"]),
                   "service_p50_ms": r3(live["service_p50_ms"]), "service_p99_ms": r3(live["service_p99_ms"]),
                   "p99_tail": {k: (r3(v) if isinstance(v, float) else v) for k, v in live["tail"].items()},
                   "plans_built_during_stream": live["plans_built"], "evictions": live["evictions"],
                   "failed_requests": live["failed_requests"] + sat["failed_requests"],
                   "errors": sorted(set(live["errors"] + sat["errors"])),
                   "boxes_per_s_offered_load": round(live["boxes_per_s"], 2),
                   "boxes_per_s_saturated": round(sat["boxes_per_s"], 2),
                   "p50_ms_saturated": r3(sat["p50_ms"]), "p99_ms_saturated": r3(sat["p99_ms"]),
                   "mean_graph_batch_saturated": round(sat["mean_batch"], 2),
                   "serial_plain_fp32_boxes_per_s": round(serial["boxes_per_s"], 2),
                   "serial_plain_fp32_sample": f"the first {n_serial} requests",
                   "workload": "Poisson arrivals; grid in {128,192,256,384}; npart log-uniform [1e5, %.0e]; uniform "
                               "or Zel'dovich (P~k^n, n in [-2,-1]) positions; CIC/TSC/PCS; interlacing on/off; P-only "
                               "or P+B (dk=2kf to 0.5 kNyq); plans warmed before the stream (resident plans); "
                               "same-configuration boxes batched into captured CUDA graphs (up to 4), 3 stream slots; "
                               "serial plain FP32 = the same boxes one by one on warm FP32 plans" % args.serve_npart_max}

    from pbi4_gb300 import roofline
    rl, rl_all = roofline.for_stages(stages, args.steps, cfg, npart, itot=itot, map_grid=map_grid, nmaps=nmaps,
                                     map_work=map_work, tensor_units=tensor_units)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "boxes/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[args.precision],
                "data": "synthetic (seeded Zel'dovich box, positions resident in HBM)",
                "config": bench_config(world),
                "form": {"precision": args.precision, "boxes_in_flight": K, "map_grid": map_grid, "maps": nmaps,
                         "triangles": itot},
                "e2e": {"value": e2e_value, "unit": "boxes/s", "callers": C, "h2d_bytes_per_step": int(pos.nbytes),
                        "d2h_bytes_per_step": int(p_h.nbytes + b_h.nbytes)},
                "gpu_launches": int(launches), "clocks": clocks, "roofline": rl, "roofline_stages": rl_all,
                "one_box_in_flight": {"value": value_one, "unit": "boxes/s", "ms_per_step": ms_one / args.steps,
                                      "gpu_launches": int(launches_one), "clocks": clocks_one,
                                      "note": "one plan, one stream: the stage times and the roofline"},
                "cpu_baseline": cpu,
                "plain_fp32": plain, "error_vs_oracle": errors, "error_vs_fp64_gpu": errors64, "serving": serving,
                "stages_ms_per_box": {k: round(v[0] / max(1, args.steps), 4) for k, v in stages.items()}}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


PRECISION_FORM = dict(workload="zeldovich_512_pcs_interlaced_P024_B024_76shells", lattice=256, box=2000.0, grid=512,
                      kbin_bs=2.0, kcenter_bs=2.0, nbins_bs=76, map_budget_mb=0)
# the 1024^3 single box: B with dk = 4 kf up to 0.4 k_Nyq (51 shells); the P multipoles
# switch on B2 and B4 as in the reference's multipole run (153 maps on the 640^3 map
# grid); the maps stream over z-slabs so the plan's working set stays under 150 GB
LARGE_BOX = dict(workload="zeldovich_1024_pcs_interlaced_P024_B024_51shells", lattice=512, box=3000.0, grid=1024,
                 kbin_bs=4.0, kcenter_bs=4.0, nbins_bs=51, map_budget_mb=24576)


def _forms_leg(w, dpos, forms, metric, data, ref="fp32", print_line=True):
    """Time each (precision, steps) of `forms` on the device-resident box dpos
    (after one untimed run that builds tables, counts and buffers) and report
    the errors of the other forms against the form `ref` (the plain FP32 form,
    or the FP64 GPU form)."""
    import torch
    from pbi4_gb300.estimator import Estimator, EstimatorConfig
    npart = int(dpos.shape[1])
    out, res = {}, {}
    for prec, steps in forms:
        cfg = EstimatorConfig(grid=w["grid"], box=w["box"], nintp=4, interlacing=True, multipoles=True,
                              los=(0.0, 0.0, 1.0), kbin_ps=1.0, kcenter_ps=1.0, do_bispectrum=True,
                              kbin_bs=w["kbin_bs"], kcenter_bs=w["kcenter_bs"], nbins_bs=w["nbins_bs"], iopen=True,
                              precision=prec, map_budget_mb=w["map_budget_mb"])
        est = Estimator(cfg)
        po, bo = est.alloc_outputs()
        t_setup = time.perf_counter()
        est.run_device(npart, dpos, po, bo)  # tables, triangle counts (cached), buffers
        torch.cuda.synchronize()
        t_setup = time.perf_counter() - t_setup
        est.enable_timing(True)
        est.stage_times()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(steps):
            est.run_device(npart, dpos, po, bo)
        t1.record()
        torch.cuda.synchronize()
        est.check()
        ms = t0.elapsed_time(t1) / steps
        st = est.stage_times()
        free, total = torch.cuda.mem_get_info()
        res[prec] = (po.cpu().numpy(), bo.cpu().numpy())
        zs, ns = est.map_slabs()
        out[prec] = {"boxes_per_s": round(1e3 / ms, 4), "ms_per_box": round(ms, 2), "steps": steps,
                     "first_run_s": round(t_setup, 2), "map_grid": est.map_grid, "maps": est.nmaps,
                     "triangles": est.itot, "map_slabs": ns, "slab_z_planes": zs,
                     "device_used_gb": round((total - free) / 1e9, 1),
                     "stages_ms_per_box": {k: round(v[0] / steps, 2) for k, v in st.items() if v[1]}}
        est.close()
        del po, bo
        torch.cuda.empty_cache()
    pr, br = res[ref]
    errs = {prec: error_report(res[prec][0], res[prec][1], pr, br, 1e-5 if prec == "fp32" else 1e-4)
            for prec, _ in forms if prec != ref}
    line = {"metric": metric, "unit": "boxes/s", "data": data,
            "config": {**w, "particles": npart, "nintp": 4, "interlacing": True, "multipoles": True},
            "forms": out, ("error_vs_plain_fp32" if ref == "fp32" else "error_vs_fp64_gpu"): errs}
    if print_line:
        print(json.dumps(line), flush=True)
    return line


def run_precision_form(args):
    """The 512^3 precision form: a 256^3-lattice Zel'dovich box in L = 2000 Mpc/h,
    grid 512^3, PCS interlaced, P l=0,2,4 (dk = kf), B l=0,2,4 with dk = 2 kf up to
    0.6 k_Nyq (76 shells, 228 maps on the 480^3 map grid).  The FP16 hi+lo and BF16
    tensor-core forms run beside the plain FP32 form, with their errors against
    it; then the FP16 hi+lo and plain FP32 forms run beside the FP64 GPU form on
    the first 40 shells (all 76 in FP64 would need about 200 GB of FP64 maps),
    with their errors against FP64."""
    import torch
    from pbi4_gb300 import synthetic
    w = PRECISION_FORM
    pos = synthetic.zeldovich_box(w["lattice"], w["box"], n_s=-1.5, rms_disp=5.0, f_growth=0.7, seed=2)
    dpos = torch.from_numpy(pos).cuda()
    data = "synthetic (seeded Zel'dovich box, positions resident in HBM)"
    full = _forms_leg(w, dpos, (("fp16split", 2), ("bf16", 2), ("fp32", 1)),
                      "P+B boxes/s @512^3 PCS interlaced, 76 shells (precision form)", data, print_line=False)
    # FP64 reference on a stated subset: the first 40 of the 76 shells (k up to
    # 0.32 k_Nyq; the FP64 maps of all 76 would need about 200 GB)
    sub = _forms_leg({**w, "nbins_bs": 40, "workload": w["workload"] + "_first40shells"}, dpos,
                     (("fp16split", 2), ("fp32", 1), ("fp64", 1)), "", data, ref="fp64", print_line=False)
    full["fp64_subset"] = {"shells": 40, "forms": sub["forms"], "error_vs_fp64_gpu": sub["error_vs_fp64_gpu"]}
    print(json.dumps(full), flush=True)


def run_large_box(args):
    """The 1024^3 single box: a 512^3-lattice Zel'dovich box (134,217,728 particles,
    generated on the device) in L = 3000 Mpc/h, grid 1024^3, PCS interlaced, P
    l=0,2,4 (dk = kf), B l=0,2,4 with dk = 4 kf up to 0.4 k_Nyq (51 shells).  The
    FP16 hi+lo form runs beside the plain FP32 form with a 24 GiB budget for the
    slab-sized map buffers, with its errors against the plain FP32 form; then both
    run beside the FP64 GPU form on the first 25 shells, with their errors against
    FP64."""
    import torch
    from pbi4_gb300 import synthetic
    w = LARGE_BOX
    dpos = synthetic.zeldovich_box_device(w["lattice"], w["box"], n_s=-1.5, rms_disp=5.0, f_growth=0.7, seed=4)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    data = "synthetic (seeded Zel'dovich box generated on the device, positions resident in HBM)"
    full = _forms_leg(w, dpos, (("fp16split", 2), ("fp32", 1)),
                      "P+B boxes/s @1024^3 PCS interlaced, 51 shells (large single box)", data, print_line=False)
    # FP64 reference on a stated subset: the first 25 of the 51 shells (k up to
    # 0.2 k_Nyq; the FP64 maps of all 51 would need over 300 GB)
    sub = _forms_leg({**w, "nbins_bs": 25, "workload": w["workload"] + "_first25shells"}, dpos,
                     (("fp16split", 2), ("fp32", 1), ("fp64", 1)), "", data, ref="fp64", print_line=False)
    full["fp64_subset"] = {"shells": 25, "forms": sub["forms"], "error_vs_fp64_gpu": sub["error_vs_fp64_gpu"]}
    print(json.dumps(full), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", default="fp16split", choices=["fp32", "fp64", "fp16split", "bf16", "tf32split"])
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-FP32 and FP64 comparison runs")
    ap.add_argument("--serve-requests", type=int, default=2000, help="requests in the serving leg (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="offered request rate of the serving leg (1/s)")
    ap.add_argument("--serve-npart-max", type=float, default=1e7, help="largest particle count of a served box")
    ap.add_argument("--boxes-in-flight", type=int, default=2,
                    help="plans (one stream each) taking the timed boxes in turn")
    ap.add_argument("--e2e-callers", type=int, default=4,
                    help="host threads (one plan and stream each) calling run_host in the e2e leg")
    ap.add_argument("--quick", action="store_true", help="small box (debug only)")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: 64^3 particles on a 128^3 grid (same kernels, a few hundred MB)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision-form", action="store_true",
                    help="only the 512^3 precision form (FP16 split, BF16, plain FP32; ~1 min)")
    ap.add_argument("--large-box", action="store_true",
                    help="only the 1024^3 single box (FP16 split and plain FP32, maps in z-slabs; ~1 min)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.precision_form:
        run_precision_form(args)
    elif args.large_box:
        run_large_box(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
