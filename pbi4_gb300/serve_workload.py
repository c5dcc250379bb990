"""Synthetic request stream for the serving loop (the mixed-grid serving workload).

Requests arrive as a Poisson process.  Each draws a grid from `grids`, a particle
count log-uniform in [npart_min, npart_max], uniform or Zel'dovich-clustered
positions (P ~ k^n, n uniform in [-2, -1]) in L = 1000 Mpc/h, an assignment
order from {CIC, TSC, PCS}, interlacing on/off, and P-only or P+B with
dk = 2 kf up to 0.5 k_Nyq.  A small pool of particle sets is generated once and
reused so that generation does not dominate the run.
"""
from __future__ import annotations

import time
from math import floor

import numpy as np

from . import synthetic
from .estimator import Estimator, EstimatorConfig
from .serve import Request, Server


def make_stream(n_requests=64, grids=(128, 192, 256), npart_min=1e5, npart_max=3e6, rate_hz=50.0, seed=3,
                precision="fp16split", pool=6):
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
        nintp = int(rng.choice([2, 3, 4]))
        inter = bool(rng.integers(2))
        with_b = bool(rng.integers(2))
        nb = floor((0.5 * grid / 2) / 2.0)   # dk = 2 kf up to 0.5 k_Nyq
        cfg = EstimatorConfig(grid=grid, box=box, nintp=nintp, interlacing=inter, multipoles=False,
                              kbin_ps=1.0, kcenter_ps=1.0, do_bispectrum=with_b, kbin_bs=2.0, kcenter_bs=2.0,
                              nbins_bs=nb, iopen=True, precision=precision)
        reqs.append((t, Request(cfg=cfg, pos=pos, rid=rid)))
    return reqs


def run_stream(reqs, hbm_budget_gb=120.0, slots=4, max_npart=None):
    """Replay the stream in real time through a Server; returns its stats."""
    max_npart = max_npart or max(r.pos.shape[1] for _, r in reqs)
    srv = Server(hbm_budget_bytes=int(hbm_budget_gb * 1e9), slots=slots, max_npart=max_npart)
    t0 = time.perf_counter()
    futs = []
    for t, r in reqs:
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        r.t_arrival = time.perf_counter()
        futs.append(srv.submit(r))
    for f in futs:
        f.result(timeout=600)
    st = srv.stats()
    srv.close()
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
