"""Roofline bookkeeping of the per-stage timings (algorithmic bytes / flops).

Algorithmic traffic per box (N grid, H = N^2 (N/2+1) half-spectrum cells,
G = 2 grids with interlacing, Np particles; M shell maps on the map grid Nm;
FP32 forms: Tz, Uy complex elements of the pruned transform's z-column and
(z, y)-plane intermediates; T triangles, S = 3 multipole sets or 1):
  assign          FP32 forms (the owner-tile kernel): 32 R Np (R = records per particle,
                  (1 + (w-1)/16)^3 for a stencil w = nintp (+1 interlaced) wide) read + 4 G N^3
                  (FP32 grid write); FP64 form: 24 Np (float64 xyz read) + 8 G N^3 (int64)
  assign_sort     FP32 forms' counting sort: 24 Np (xyz) + 64 Np (record write, read) + 32 R Np
  grid_convert    8 G N^3 read + 4 G N^3 write (FP64 form only)
  fcomb           8 G H read + 8 H write
  pk_binning      8 H read
  shell_maps_z    FP32: 8 Tz write (the shell modes it gathers stay in L2);
                  FP64: 16 H read + 16 M Hm write (shell spectra)
  shell_maps_y    FP32: 8 Tz read + 8 Uy write (FP64: cuFFT Z2D, a library call)
  shell_maps_x    FP32: 8 Uy read + 4 M Nm^3 write (the real maps; the tensor-core forms
                  write their operand planes: 4 / 8 / 2 B per map and point for FP16 hi+lo /
                  TF32 hi+lo / BF16, plus 4 nb Nm^3 for the FP32 pair factors)
  triangle_sums   2 Nm^3 T S flops (tensor-core forms; useful sums only)
cuFFT stages (fft_r2c, the FP64 shell_maps_y) are library calls: timed, not given a roofline.
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
    """Per-launch DRAM bytes of each stage from the committed ncu summary, if present,
    keyed by "grid<N>_<precision>" of the workload it was measured (and scaled) for:
    {stage: {"bytes": B, "source": hash of the kernel's sources when captured}}."""
    p = os.path.join(ROOT, "profiles", "dram_bytes.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


# the source files each stage's kernels are built from (pbi4_gb300/csrc)
SOURCES = {"assign": ("assign_owner.cu", "assign_owner.cuh"), "assign_sort": ("assign_owner.cu", "assign_owner.cuh"),
           "fcomb": ("spectrum.cu",), "pk_binning": ("spectrum.cu",),
           "shell_maps_z": ("mapfft.cu", "fft_small.cuh"), "shell_maps_y": ("mapfft.cu", "fft_small.cuh"),
           "shell_maps_x": ("mapfft.cu", "fft_small.cuh"), "triangle_sums": ("trisum_tm.cu", "tc_ptx.cuh")}


def source_hash(stage):
    """First 16 hex digits of the SHA-256 of the stage's kernel sources (None if unknown)."""
    import hashlib
    files = SOURCES.get(stage)
    if not files:
        return None
    h = hashlib.sha256()
    for f in files:
        p = os.path.join(ROOT, "pbi4_gb300", "csrc", f)
        if not os.path.exists(p):
            return None
        with open(p, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def measured_traffic(table, stage):
    """The captured per-launch DRAM bytes of a stage, or None when there is none or
    the kernel's sources changed since the capture (the figure would be stale)."""
    t = table.get(stage)
    if isinstance(t, dict) and t.get("source") and t.get("source") == source_hash(stage):
        return t.get("bytes")
    return None


def stage_work(cfg, npart, map_grid=None, nmaps=None, map_work=None):
    N = int(cfg.grid)
    G = 2 if cfg.interlacing else 1
    H = N * N * (N // 2 + 1)
    nsets = 3 if cfg.multipoles else 1
    M = nmaps if nmaps is not None else (nsets * int(cfg.nbins_bs) if cfg.do_bispectrum else 0)
    Nm = map_grid or N
    Hm = Nm * Nm * (Nm // 2 + 1)
    gbytes = 8 if cfg.precision == "fp64" else 4
    w = int(cfg.nintp) + (1 if cfg.interlacing else 0)
    R = (1.0 + (w - 1) / 16.0) ** 3
    work = {
        "assign": ("hbm", (24 * npart + gbytes * G * N ** 3) if cfg.precision == "fp64"
                   else (32 * R * npart + 4 * G * N ** 3)),
        "assign_sort": ("hbm", 24 * npart + 64 * npart + 32 * R * npart),
        "grid_convert": ("hbm", 12 * G * N ** 3),
        "fcomb": ("hbm", 8 * G * H + 8 * H),
        "pk_binning": ("hbm", 8 * H),
    }
    if cfg.precision == "fp64":
        work["shell_maps_z"] = ("hbm", 16 * H + 16 * M * Hm)
    elif map_work and map_work[0] > 0:
        tz, uy = map_work
        work["shell_maps_z"] = ("hbm", 8 * tz)
        work["shell_maps_y"] = ("hbm", 8 * tz + 8 * uy)
        # the x pass writes 4 B per map and point (FP32 maps, or FP16 hi + lo), 8 B (TF32 hi + lo) or
        # 2 B (BF16), plus the FP32 set-0 maps (the pair factors) for the tensor-core forms
        per_map = {"fp16split": 4, "tf32split": 8, "bf16": 2}.get(cfg.precision, 4)
        extra = 4 * int(cfg.nbins_bs or 0) * Nm ** 3 if cfg.precision in ("fp16split", "tf32split", "bf16") else 0
        work["shell_maps_x"] = ("hbm", 8 * uy + per_map * M * Nm ** 3 + extra)
    return work


KERNEL = {"assign": "owner_tile_kernel", "assign_sort": "owner_count/scan/scatter_kernel",
          "grid_convert": "fixed_to_real_kernel",
          "fcomb": "fcomb_interlaced_half_kernel", "pk_binning": "pk_accum_kernel",
          "shell_maps_z": "map_zpass_kernel", "shell_maps_y": "map_ypass_kernel", "shell_maps_x": "map_xpass_kernel",
          "triangle_sums": "trisum_tm_kernel"}

def _entry(name, bound, amount, avg_ms, pk, traffic):
    if bound == "tensor":
        achieved = amount / (avg_ms * 1e-3) / 1e12
        return {"kernel": KERNEL.get(name, name), "stage": name, "bound": "tensor", "achieved": round(achieved, 2),
                "peak": pk["bf16_tflops"], "unit": "TFLOP/s", "frac": round(achieved / pk["bf16_tflops"], 5),
                "traffic": traffic, "algorithmic_flops": amount, "avg_ms": round(avg_ms, 4),
                "peak_source": pk["source"]}
    achieved = amount / (avg_ms * 1e-3) / 1e9
    return {"kernel": KERNEL.get(name, name), "stage": name, "bound": "hbm", "achieved": round(achieved, 1),
            "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": traffic,
            "algorithmic_bytes": amount, "avg_ms": round(avg_ms, 4), "peak_source": pk["source"]}


def for_stages(stages, steps, cfg, npart, itot=None, map_grid=None, nmaps=None, map_work=None, tensor_units=None):
    """(dominant, all): the roofline object of the slowest stage among this
    library's kernels and the list for every timed stage (per box: a stage that
    runs slab by slab adds its launches).  Tensor-core triangle sums count the
    useful flops 2 Nm^3 itot S against the measured bf16 dense peak; with
    tensor_units = (units, products) they also report the executed tensor work (every
    128-pair x 64-map tile of a unit over every point, times the split's products)
    and the fraction of the tiles' entries that is no triangle sum.  HBM stages count their
    algorithmic bytes.  `traffic` is the per-launch DRAM bytes of the committed ncu
    capture for this workload, if one exists and the kernel's sources are those it
    was captured from (else null)."""
    pk = peaks()
    work = dict(stage_work(cfg, npart, map_grid, nmaps, map_work))
    if itot and cfg.precision in ("fp16split", "bf16", "tf32split"):
        nsets = 3 if cfg.multipoles else 1
        work["triangle_sums"] = ("tensor", 2.0 * int(map_grid or cfg.grid) ** 3 * itot * nsets)
    table = traffic_table().get("grid%d_%s" % (int(cfg.grid), cfg.precision), {})
    out = []
    for name, (bound, amount) in work.items():
        ms, calls = stages.get(name, (0.0, 0))
        if calls == 0 or ms <= 0:
            continue
        e = _entry(name, bound, amount, ms / max(1, steps), pk, measured_traffic(table, name))
        if name == "shell_maps_z" and cfg.precision == "fp64":
            e["kernel"] = "build_map_spectra_kernel"
        if name == "triangle_sums" and tensor_units and tensor_units[0]:
            units, products = tensor_units
            executed = float(units) * int(map_grid or cfg.grid) ** 3 * 128 * 64 * 2 * products
            e["executed_flops"] = executed
            e["executed_tflops"] = round(executed / (e["avg_ms"] * 1e-3) / 1e12, 1)
            e["split_products"] = products
            # entries of the units' (pair, map) tiles that are no (triangle, set) slot
            e["gemm_recast_waste"] = round(1.0 - amount * products / executed, 4)
        out.append(e)
    if not out:
        return None, []
    best = max(out, key=lambda e: e["avg_ms"])
    return best, out
