"""Synthetic request stream for the serving loop (the mixed-grid serving workload).

Requests arrive as a Poisson process.  Each draws a grid from `grids`, a particle
count log-uniform in [npart_min, npart_max], uniform or Zel'dovich-clustered
positions (P ~ k^n, n uniform in [-2, -1]) in L = 1000 Mpc/h, an assignment
order from {CIC, TSC, PCS}, interlacing on/off, and P-only or P+B with
dk = 2 kf up to 0.5 k_Nyq.  A small pool of particle sets is generated once and
sliced per request so that generation does not dominate the run.
"""
from __future__ import annotations

import time
from math import floor

import numpy as np

from . import synthetic
from .estimator import Estimator, EstimatorConfig
from .serve import Request, Server


def request_config(grid, nintp, interlacing, with_b, precision, box=1000.0):
    nb = floor((0.5 * grid / 2) / 2.0)   # dk = 2 kf up to 0.5 k_Nyq
    return EstimatorConfig(grid=grid, box=box, nintp=nintp, interlacing=interlacing, multipoles=False,
                           kbin_ps=1.0, kcenter_ps=1.0, do_bispectrum=with_b, kbin_bs=2.0, kcenter_bs=2.0,
                           nbins_bs=nb, iopen=True, precision=precision)


def make_stream(n_requests=64, grids=(128, 192, 256, 384), npart_min=1e5, npart_max=1e7, rate_hz=50.0, seed=3,
                precision="fp16split", pool=4, orders=(2, 3, 4)):
    rng = np.random.default_rng(seed)
    box = 1000.0
    # particle pool: uniform and clustered sets of the largest size, sliced per request
    nmax = int(npart_max)
    sets = []
    for k in range(pool):
        if k % 2 == 0:
            sets.append(synthetic.uniform_box(nmax, box, seed=1000 + k))
        else:
            side = int(round(nmax ** (1 / 3)))
            sets.append(synthetic.zeldovich_box(side, box, n_s=float(rng.uniform(-2, -1)), seed=2000 + k))
    t = 0.0
    reqs = []
    for rid in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        grid = int(rng.choice(grids))
        npart = int(np.exp(rng.uniform(np.log(npart_min), np.log(npart_max))))
        src = sets[int(rng.integers(len(sets)))]
        npart = min(npart, src.shape[1])
        off = int(rng.integers(0, src.shape[1] - npart + 1))
        pos = np.ascontiguousarray(src[:, off:off + npart])
        cfg = request_config(grid, int(rng.choice(orders)), bool(rng.integers(2)), bool(rng.integers(2)), precision)
        reqs.append((t, Request(cfg=cfg, pos=pos, rid=rid)))
    return reqs


def configs_of(reqs):
    seen = {}
    for _, r in reqs:
        seen.setdefault(r.cfg.key(), r.cfg)
    return list(seen.values())


def run_stream(reqs, hbm_budget_gb=200.0, slots=3, batch=4, max_npart=None, warm=True, realtime=True):
    """Replay the stream through a Server; realtime=False submits everything at
    once (throughput under saturation).  Returns its stats."""
    max_npart = max_npart or max(r.pos.shape[1] for _, r in reqs)
    srv = Server(hbm_budget_bytes=int(hbm_budget_gb * 1e9), slots=slots, max_npart=max_npart, batch=batch)
    if warm:
        srv.warm(configs_of(reqs))
    t0 = time.perf_counter()
    futs = []
    for t, r in reqs:
        if realtime:
            now = time.perf_counter() - t0
            if t > now:
                time.sleep(t - now)
        r.t_arrival = time.perf_counter()
        futs.append(srv.submit(r))
    errors = []
    for f in futs:
        try:
            f.result(timeout=1800)
        except Exception as e:  # a failed request is counted and reported, the stream goes on
            errors.append(f"{type(e).__name__}: {e}")
    st = srv.stats()
    srv.close()
    st["errors"] = sorted(set(errors))[:5]
    st["failed_requests"] = len(errors)
    return st


def run_serial_plain(reqs, repeat_warm=True):
    """The same boxes one after another on plain FP32 plans (one plan per configuration)."""
    import torch
    plans = {}
    total = 0.0
    for _, r in reqs:
        cfg = EstimatorConfig(**{**r.cfg.__dict__, "precision": "fp32"})
        key = cfg.key()
        if key not in plans:
            plans[key] = Estimator(cfg)
            if repeat_warm:
                plans[key].run_host(r.pos)  # tables, counts, cuFFT plans (cold start excluded)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plans[key].run_host(r.pos)
        total += time.perf_counter() - t0
    for p in plans.values():
        p.close()
    return {"n": len(reqs), "seconds": total, "boxes_per_s": len(reqs) / total}
