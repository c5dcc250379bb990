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


def for_stages(stages, steps, cfg, npart, tri_flops=None):
    """Roofline object of the dominant own-kernel HBM stage (library FFT stages excluded)."""
    pk = peaks()
    work = stage_work(cfg, npart)
    best = None
    for name, (bound, nbytes) in work.items():
        ms, calls = stages.get(name, (0.0, 0))
        if calls == 0 or ms <= 0:
            continue
        avg_ms = ms / calls
        if best is None or avg_ms > best[1]:
            best = (name, avg_ms, nbytes)
    if best is None:
        return None
    name, avg_ms, nbytes = best
    achieved = nbytes / (avg_ms * 1e-3) / 1e9
    tt = traffic_table().get(name)
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": tt, "algorithmic_bytes": nbytes,
            "avg_ms": round(avg_ms, 4), "peak_source": pk["source"]}
