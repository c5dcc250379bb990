"""Device-resident estimator: one resident plan per box configuration.

``Estimator`` wraps the ``pbi4g_plan_*`` C ABI.  Positions enter either as a
CUDA tensor / device pointer of shape (3, npart) float64 in [0, 1)
(``run_device``: the throughput path, everything stays in HBM) or as a host
numpy array (``run_host``: copies inside the call).  Outputs follow the
reference's Fortran arrays: ``pout`` is (5, nbins_ps) with rows
avgk, P0, P2, P4, Nmodes (measure_pk_multipoles, powerI4.f90:685-691; for real
space rows avgk, P, Nmodes as measure_pk, :589-592), ``bout`` is (9 or 11, itot)
as measure_bk / measure_bk_multipoles (bispectrumI4.f90:174-182, 490-500).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from math import floor

import numpy as np

from ._lib import PRECISIONS, Config, check, lib, ptr


@dataclass
class EstimatorConfig:
    grid: int
    box: float
    nintp: int = 4
    interlacing: bool = True
    multipoles: bool = False
    los: tuple = (0.0, 0.0, 1.0)      # already divided by (los . los), as IO.derived_params does
    kbin_ps: float = 1.0
    kcenter_ps: float = 1.0
    nbins_ps: int | None = None
    do_bispectrum: bool = True
    kbin_bs: float = 1.0
    kcenter_bs: float = 1.0
    nbins_bs: int | None = None
    iopen: bool = True
    precision: str = "fp32"
    # FP32 forms: MiB the real-space shell maps may hold at once (0: no bound);
    # above it the maps are made and contracted z-slab by z-slab
    map_budget_mb: int = 0
    extra: dict = field(default_factory=dict)

    def __post_init__(self):
        g = int(self.grid)
        if self.nbins_ps is None:   # pbi4.py:98
            self.nbins_ps = floor((g / 2 + self.kbin_ps - self.kcenter_ps) / self.kbin_ps)
        if self.nbins_bs is None:   # pbi4.py:99
            self.nbins_bs = floor((g / 3 + self.kbin_bs - self.kcenter_bs) / self.kbin_bs)

    @classmethod
    def from_params(cls, params: dict, precision: str = "fp32", do_bispectrum: bool = True, **over):
        """From a reference params dict after IO.derived_params (pbi4.py:86-119)."""
        kw = dict(grid=int(params["grid"]), box=float(params["box"]), nintp=int(params["interpolation"]),
                  interlacing=bool(params["interlacing"]), multipoles=bool(params["multipoles"]),
                  los=tuple(float(x) for x in np.asarray(params["los"], dtype=np.float64)),
                  kbin_ps=float(params["kbin"]), kcenter_ps=float(params["kcenter"]),
                  nbins_ps=int(params["nbins_ps"]), do_bispectrum=do_bispectrum,
                  kbin_bs=float(params["kbin"]), kcenter_bs=float(params["kcenter"]),
                  nbins_bs=int(params["nbins_bisp"]), iopen=bool(params["iopen"]), precision=precision)
        kw.update(over)
        return cls(**kw)

    def to_c(self) -> Config:
        c = Config()
        c.grid, c.box, c.nintp = int(self.grid), float(self.box), int(self.nintp)
        c.interlacing, c.multipoles = int(bool(self.interlacing)), int(bool(self.multipoles))
        for k in range(3):
            c.los[k] = float(self.los[k])
        c.kbin_ps, c.kcenter_ps, c.nbins_ps = float(self.kbin_ps), float(self.kcenter_ps), int(self.nbins_ps)
        c.do_bispectrum = int(bool(self.do_bispectrum))
        c.kbin_bs, c.kcenter_bs, c.nbins_bs = float(self.kbin_bs), float(self.kcenter_bs), int(self.nbins_bs)
        c.iopen = int(bool(self.iopen))
        c.precision = PRECISIONS[self.precision]
        c.map_budget_mb = int(self.map_budget_mb)
        return c

    def key(self):
        return (int(self.grid), float(self.box), int(self.nintp), bool(self.interlacing), bool(self.multipoles),
                tuple(self.los), float(self.kbin_ps), float(self.kcenter_ps), int(self.nbins_ps),
                bool(self.do_bispectrum), float(self.kbin_bs), float(self.kcenter_bs), int(self.nbins_bs),
                bool(self.iopen), self.precision, int(self.map_budget_mb))


def footprint(cfg: EstimatorConfig, npart_max: int) -> int:
    # (the captured form adds batch x 3 x npart_max float64 position slots)
    """Device bytes a plan for cfg needs (admission control); allocates nothing."""
    c = cfg.to_c()
    out = ctypes.c_int64()
    check(lib().pbi4g_plan_footprint(ctypes.byref(c), int(npart_max), ctypes.byref(out)))
    return int(out.value)


def uses_owner_work(cfg: EstimatorConfig) -> bool:
    """Whether a plan for cfg assigns with the owner-computes tiles, whose record
    buffers a shared AssignScratch can hold (the FP32 and tensor-core forms on
    grids that are multiples of 16 in [32, 2048])."""
    g = int(cfg.grid)
    return cfg.precision != "fp64" and g % 16 == 0 and 32 <= g <= 2048


def scratch_footprint(grid_max: int, npart_max: int, boxes: int = 0) -> int:
    """Device bytes of an AssignScratch for grids up to grid_max, npart_max particles
    and `boxes` graph position slots."""
    out = ctypes.c_int64()
    check(lib().pbi4g_scratch_footprint(int(grid_max), int(npart_max), int(boxes), ctypes.byref(out)))
    return int(out.value)


class AssignScratch:
    """Assignment buffers shared by plans that run one after another on one stream
    (a serving slot): the per-tile particle records, up to 8 per particle, that
    each plan otherwise owns, and `boxes` position slots for their captured graphs
    (pbi4g_scratch_*).  It never grows: a box above grid_max or npart_max fails.
    Plans that share one must not run concurrently."""

    def __init__(self, grid_max: int, npart_max: int, boxes: int = 0):
        h = ctypes.c_void_p()
        check(lib().pbi4g_scratch_create(int(grid_max), int(npart_max), int(boxes), ctypes.byref(h)))
        self._h = h
        self.grid_max, self.npart_max, self.boxes = int(grid_max), int(npart_max), int(boxes)
        self.bytes = scratch_footprint(grid_max, npart_max, boxes)

    def close(self):
        """Free the buffers; raises while a plan still uses them."""
        if getattr(self, "_h", None):
            check(lib().pbi4g_scratch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Estimator:
    stream = None  # the stream object last given to set_stream (serving bookkeeping)
    scratch = None  # the AssignScratch in use (None: the plan's own buffers)

    def __init__(self, cfg: EstimatorConfig, stream=None):
        self.cfg = cfg
        self._c = cfg.to_c()
        h = ctypes.c_void_p()
        check(lib().pbi4g_plan_create(ctypes.byref(self._c), ctypes.byref(h)))
        self._h = h
        if stream is not None:
            self.set_stream(stream)
        nb, it, br = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
        check(lib().pbi4g_plan_shape(self._h, ctypes.byref(nb), ctypes.byref(it), ctypes.byref(br)))
        self.nbins_ps, self.itot, self.brows = nb.value, it.value, br.value
        mg, nm = ctypes.c_int32(), ctypes.c_int32()
        check(lib().pbi4g_plan_map_grid(self._h, ctypes.byref(mg), ctypes.byref(nm)))
        self.map_grid, self.nmaps = mg.value, nm.value

    def map_work(self):
        """(z columns, y planes): complex elements of the FP32 map transform's
        intermediates, once a bispectrum has run (0, 0 before, and for FP64)."""
        t, u = ctypes.c_int64(), ctypes.c_int64()
        check(lib().pbi4g_plan_map_work(self._h, ctypes.byref(t), ctypes.byref(u)))
        return t.value, u.value

    def map_slabs(self):
        """(z-planes per slab, slabs per box) of the last bispectrum run."""
        z, n = ctypes.c_int32(), ctypes.c_int32()
        check(lib().pbi4g_plan_map_slabs(self._h, ctypes.byref(z), ctypes.byref(n)))
        return z.value, n.value

    def tensor_units(self):
        """(units, products per K step) of the tensor-core triangle sums of the last run."""
        u, k = ctypes.c_int32(), ctypes.c_int32()
        check(lib().pbi4g_plan_tensor_units(self._h, ctypes.byref(u), ctypes.byref(k)))
        return u.value, k.value

    # -- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            lib().pbi4g_plan_destroy(self._h)
            self._h = None
            self.scratch = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        """stream: a torch.cuda.Stream, an integer cudaStream_t, or None (legacy default)."""
        s = getattr(stream, "cuda_stream", stream)
        check(lib().pbi4g_plan_set_stream(self._h, s))

    def use_scratch(self, scratch):
        """Assign through a shared AssignScratch (None: the plan's own buffers).  The
        plan must be idle; its captured graphs follow the binding.  A no-op for the
        FP64 form, which has no such buffers."""
        if scratch is self.scratch:
            return
        check(lib().pbi4g_plan_use_scratch(self._h, scratch._h if scratch is not None else None))
        self.scratch = scratch  # keeps the scratch alive while the plan uses it

    def enable_timing(self, on: bool = True):
        check(lib().pbi4g_plan_enable_timing(self._h, int(bool(on))))

    def stage_times(self):
        """{stage: (summed ms, calls)} since the last query (synchronises the plan's stream)."""
        from ._lib import NSTAGES, STAGES
        ms = np.zeros(NSTAGES, dtype=np.float64)
        calls = np.zeros(NSTAGES, dtype=np.int64)
        check(lib().pbi4g_plan_stage_times(self._h, ms.ctypes.data, calls.ctypes.data))
        return {STAGES[k]: (float(ms[k]), int(calls[k])) for k in range(NSTAGES)}

    @property
    def launches(self) -> int:
        return int(lib().pbi4g_plan_kernel_launches(self._h))

    # -- stages (device pointers / CUDA tensors)
    def density(self, npart: int, pos, weight=None):
        check(lib().pbi4g_plan_density(self._h, int(npart), ptr(pos), ptr(weight)))

    def powerspectrum(self, pout):
        check(lib().pbi4g_plan_powerspectrum(self._h, ptr(pout)))

    def bispectrum(self, bout):
        check(lib().pbi4g_plan_bispectrum(self._h, ptr(bout)))

    def run_device(self, npart: int, pos, pout, bout=None, weight=None):
        check(lib().pbi4g_plan_run_device(self._h, int(npart), ptr(pos), ptr(weight), ptr(pout), ptr(bout)))

    def check(self):
        """Synchronise and raise if a bounded wait inside a tensor-core launch gave up."""
        check(lib().pbi4g_plan_check(self._h))

    # -- captured form
    graph_ready = False

    def graph_build(self, batch: int, npart_cap: int):
        """Hold `batch` box slots of up to npart_cap particles and capture the box
        pipeline as CUDA graphs on first use (needs a non-default stream)."""
        check(lib().pbi4g_plan_graph_build(self._h, int(batch), int(npart_cap)))
        self.graph_batch, self.graph_cap, self.graph_ready = int(batch), int(npart_cap), True

    def graph_run_host(self, pos_list, pout_list, bout_list=None):
        """One graph launch for len(pos_list) boxes: pos_list of (3, npart) float64
        C-contiguous host arrays, outputs preallocated host arrays shaped like
        alloc_outputs' ((5, nbins_ps) / (brows, itot), Fortran order, or the
        C-order transposes' buffers).  Asynchronous with pinned outputs: read them
        after the plan's stream completes."""
        n = len(pos_list)
        npart = (ctypes.c_int64 * n)(*[int(p.shape[1]) for p in pos_list])
        pp = (ctypes.c_void_p * n)(*[p.ctypes.data for p in pos_list])
        po = (ctypes.c_void_p * n)(*[o.ctypes.data for o in pout_list])
        bo = (ctypes.c_void_p * n)(*[o.ctypes.data for o in bout_list]) if bout_list else None
        check(lib().pbi4g_plan_graph_run_host(self._h, n, npart, pp, po, bo))

    def alloc_outputs(self, device="cuda"):
        """Device output tensors (pout (5, nbins_ps), bout (brows, itot)) in Fortran layout."""
        import torch
        pout = torch.empty((self.nbins_ps, 5), dtype=torch.float64, device=device).t()
        bout = None
        if self.itot:
            bout = torch.empty((self.itot, self.brows), dtype=torch.float64, device=device).t()
        return pout, bout

    # -- host path
    def run_host(self, pos: np.ndarray, weight: np.ndarray | None = None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        if pos.ndim != 2 or pos.shape[0] != 3:
            raise ValueError("pos must be (3, npart)")
        npart = pos.shape[1]
        w = None if weight is None else np.ascontiguousarray(weight, dtype=np.float64)
        pout = np.empty((5, self.nbins_ps), dtype=np.float64, order="F")
        bout = np.empty((self.brows, self.itot), dtype=np.float64, order="F") if self.itot else None
        check(lib().pbi4g_plan_run_host(self._h, npart, pos.ctypes.data, ptr(w), pout.ctypes.data,
                                        None if bout is None else bout.ctypes.data))
        return pout, bout

    def triangle_counts(self) -> np.ndarray:
        out = np.empty(self.itot, dtype=np.int64)
        check(lib().pbi4g_plan_triangle_counts(self._h, out.ctypes.data))
        return out

    def set_delta_half(self, npart: int, half: np.ndarray):
        h = np.ascontiguousarray(half, dtype=np.complex128)
        n = int(self.cfg.grid)
        if h.shape != (n, n, n // 2 + 1):
            raise ValueError(f"expected a ({n},{n},{n // 2 + 1}) half spectrum")
        check(lib().pbi4g_plan_set_delta_half(self._h, int(npart), h.ctypes.data))

    def set_counts(self, counts: np.ndarray):
        c = np.ascontiguousarray(counts, dtype=np.float64)
        if c.shape[0] < self.itot:
            raise ValueError(f"counts has {c.shape[0]} entries, itot={self.itot}")
        check(lib().pbi4g_plan_set_counts(self._h, c.ctypes.data))

    def delta_half(self) -> np.ndarray:
        n = int(self.cfg.grid)
        out = np.empty((n, n, n // 2 + 1), dtype=np.complex128)
        check(lib().pbi4g_plan_get_delta_half(self._h, out.ctypes.data))
        return out
