"""Roofline bookkeeping of the per-stage timings (algorithmic bytes / flops).

Algorithmic traffic per box (N grid, H = N^2 (N/2+1) half-spectrum cells,
G = 2 grids with interlacing, M shell maps, T triangles, S q-sets):
  assign          24 Np (float64 xyz read) + 8 G N^3 (int64 fixed-point grid write)
  grid_convert    8 G N^3 read + 4 G N^3 write
  fcomb           8 G H read + 8 H write
  pk_binning      8 H read
  shell_spectra   8 H read + 8 M H write
  triangle_sums   2 N^3 T S flops (tensor-core forms) / maps read 4 M N^3 bytes (CUDA-core FP32)
Peaks are the measured ones in MEASURED_PEAKS.json at the repository root
(HBM copy bandwidth, cuBLAS bf16 dense), else the documented fallback.
"""
from __future__ import annotations

import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "bf16_tflops_sustained": float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def traffic_table():
    """Per-launch DRAM bytes of each stage from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "dram_bytes.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


def stage_work(cfg, npart):
    N = int(cfg.grid)
    G = 2 if cfg.interlacing else 1
    H = N * N * (N // 2 + 1)
    nsets = 3 if cfg.multipoles else 1
    M = nsets * int(cfg.nbins_bs) if cfg.do_bispectrum else 0
    return {
        "assign": ("hbm", 24 * npart + 8 * G * N ** 3),
        "grid_convert": ("hbm", 12 * G * N ** 3),
        "fcomb": ("hbm", 8 * G * H + 8 * H),
        "pk_binning": ("hbm", 8 * H),
        "shell_spectra": ("hbm", 8 * H + 8 * M * H),
    }


def for_stages(stages, steps, cfg, npart, itot=None):
    """Roofline object of the dominant stage among this library's kernels (the
    cuFFT stages are library calls and are reported only in the stage times).
    Tensor-core triangle sums count the useful flops 2 N^3 itot S against the
    measured bf16 dense peak; HBM stages count their algorithmic bytes."""
    pk = peaks()
    work = dict(stage_work(cfg, npart))
    if itot and cfg.precision in ("fp16split", "bf16"):
        nsets = 3 if cfg.multipoles else 1
        work["triangle_sums"] = ("tensor", 2.0 * int(cfg.grid) ** 3 * itot * nsets)
    best = None
    for name, (bound, amount) in work.items():
        ms, calls = stages.get(name, (0.0, 0))
        if calls == 0 or ms <= 0:
            continue
        avg_ms = ms / calls
        if best is None or avg_ms > best[1]:
            best = (name, avg_ms, amount, bound)
    if best is None:
        return None
    name, avg_ms, amount, bound = best
    tt = traffic_table().get(name)
    if bound == "tensor":
        achieved = amount / (avg_ms * 1e-3) / 1e12
        peak = pk["bf16_tflops"]
        return {"kernel": "trisum_tc_kernel", "stage": name, "bound": "tensor", "achieved": round(achieved, 2),
                "peak": peak, "unit": "TFLOP/s", "frac": round(achieved / peak, 5), "traffic": tt,
                "algorithmic_flops": amount, "avg_ms": round(avg_ms, 4), "peak_source": pk["source"]}
    achieved = amount / (avg_ms * 1e-3) / 1e9
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": tt, "algorithmic_bytes": amount,
            "avg_ms": round(avg_ms, 4), "peak_source": pk["source"]}
