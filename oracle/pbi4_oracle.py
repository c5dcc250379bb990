"""FP64 CPU oracle for the PBI4 estimator path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import this module, and only as the checker (or, for
``bench.py --impl reference``, as the timed CPU restatement of the reference).
The product package ``pbi4_gb300`` never imports it.

It restates, routine by routine, the reference's f2py modules
(``pbi4/F90_modules/powerI4.f90``, ``pbi4/F90_modules/bispectrumI4.f90``,
compiled here from ``oracle/pbi4_oracle.c``) and the driver semantics of
``pbi4/pbi4.py`` (normalisation, FFT calls, output records).  The FFTs that the
reference takes from FFTW 3.3.10 (``bispectrumI4.f90:109-111,150``; not vendored,
version from the path in ``setup.py:12``) and scipy.fft (``pbi4.py:8,337,359``)
are scipy.fft FP64 here; both are exact DFTs up to ~1e-15 relative rounding.

Parity pin: the input-independent columns of ``Tutorials/testdata/ps.dat``
(k, avgk, Nmodes) and ``bs.dat`` (k1, k2, k3 order, N_tr) are reproduced
exactly by this oracle (tests/test_oracle_golden.py).  P/B values themselves
cannot be pinned to the reference's data: its input catalogue is missing.

Array conventions follow f2py: 3-D grids are numpy arrays of shape (N, N, N)
indexed ``a[ix-1, iy-1, iz-1]`` == Fortran ``a(ix, iy, iz)`` (Fortran order in
memory).  ``pos`` is numpy (3, npart) float64 in [0, 1).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from math import floor

import numpy as np
import scipy.fft

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libpbi4oracle.so")
_lib = None

_d = ctypes.POINTER(ctypes.c_double)
_f = ctypes.POINTER(ctypes.c_float)
_i32 = ctypes.POINTER(ctypes.c_int32)
_ci, _cl, _cf = ctypes.c_int, ctypes.c_int64, ctypes.c_float


def build() -> str:
    """Compile oracle/pbi4_oracle.c with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(os.path.join(_HERE, "pbi4_oracle.c")):
            build()
        L = ctypes.CDLL(_SO)
        L.or_assign_single_grid.argtypes = [_ci, _ci, _cl, _d, _d, _d]
        L.or_assign_double_grid.argtypes = [_ci, _ci, _cl, _d, _d, _d]
        L.or_fcomb.argtypes = [_ci, _ci, _ci, _cf, _d]
        L.or_reduce_array.argtypes = [_ci, _d, _ci, _d]
        L.or_compute_q2k.argtypes = [_ci, _cf, _d, _ci, _ci, _d]
        L.or_compute_q4k.argtypes = [_ci, _cf, _d, _ci, _ci, _ci, _ci, _d]
        L.or_measure_pk.argtypes = [_ci, _cf, _cf, _cf, _ci, _d, _d, _d]
        L.or_measure_pk_multipoles.argtypes = [_ci, _cf, _cf, _cf, _ci, _d, _d, _d, _d]
        L.or_shell_index.argtypes = [_ci, _cf, _cf, _ci, _i32]
        L.or_count_itot.argtypes = [_ci, _cf, _cf, _ci, _ci]
        L.or_count_itot.restype = ctypes.c_int64
        L.or_triangle_counts_sum.argtypes = [_ci, _cf, _cf, _ci, _ci, _cl, _d, _d]
        L.or_bk_last_sum.argtypes = [_ci, _cf, _cf, _ci, _cf, _cl, _cl, _f, _d, _d, _d]
        L.or_bk_multipoles_last_sum.argtypes = [_ci, _cf, _cf, _ci, _cf, _cl, _cl, _f, _d, _d, _d, _d, _d]
        L.or_bk_cross_last_sum.argtypes = [_ci, _cf, _cf, _ci, _cf, _cl, _f, _d, _d, _d]
        L.or_triangle_counts_sum_rows.argtypes = [_ci, _cf, _cf, _ci, _ci, _cl, _d, _d, _cl, _cl]
        L.or_bk_last_sum_rows.argtypes = [_ci, _cf, _cf, _ci, _cf, _cl, _cl, _f, _d, _d, _d, _cl, _cl]
        L.or_bk_multipoles_last_sum_rows.argtypes = [_ci, _cf, _cf, _ci, _cf, _cl, _cl, _f, _d, _d, _d, _d, _d,
                                                     _cl, _cl]
        L.or_bk_cross_last_sum_rows.argtypes = [_ci, _cf, _cf, _ci, _cf, _cl, _f, _d, _d, _d, _cl, _cl]
        _lib = L
    return _lib


def _p(a, t=_d):
    return a.ctypes.data_as(t)


def _rows(fn, nrows, workers, *args):
    """Run a triangle "Last sum" routine `fn(*args, m0, m1)` over the rows
    [0, nrows), split into contiguous blocks over `workers` threads (ctypes
    releases the GIL).  Each row is the same serial loop as in one pass, so the
    result does not depend on the split."""
    nrows = int(nrows)
    nw = max(1, min(int(workers or 1), nrows))
    if nw == 1:
        fn(*args, 0, nrows)
        return
    import concurrent.futures as cf
    # blocks of ~4 rows per task keep threads busy to the end (rows cost the same)
    step = max(1, min(4, nrows // nw))
    bounds = [(a, min(nrows, a + step)) for a in range(0, nrows, step)]
    with cf.ThreadPoolExecutor(max_workers=nw) as ex:
        list(ex.map(lambda b: fn(*args, b[0], b[1]), bounds))


def _cgrid(a):
    return np.asfortranarray(a, dtype=np.complex128)


def _cptr(a):
    return a.ctypes.data_as(_d)


# ---------------------------------------------------------------- powerI4 ---
def assign_single_grid(grid, nintp, npart, pos, weight):
    """powerI4.f90:68-140 -> float64 (N,N,N), Fortran order."""
    grid = int(grid)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    weight = np.ascontiguousarray(weight, dtype=np.float64)
    out = np.zeros((grid, grid, grid), dtype=np.float64, order="F")
    lib().or_assign_single_grid(grid, int(nintp), int(npart), _p(pos), _p(weight), _p(out))
    return out


def assign_double_grid(grid, nintp, npart, pos, weight):
    """powerI4.f90:142-249 -> complex128 (N,N,N), Re = grid, Im = interlaced grid."""
    grid = int(grid)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    weight = np.ascontiguousarray(weight, dtype=np.float64)
    out = np.zeros((grid, grid, grid), dtype=np.complex128, order="F")
    lib().or_assign_double_grid(grid, int(nintp), int(npart), _p(pos), _p(weight), _cptr(out))
    return out


def fcomb(grid, nintp, interlacing, box, fdcl):
    """powerI4.f90:251-378 (dcl = fdcl, then modified in place)."""
    dcl = np.array(fdcl, dtype=np.complex128, order="F", copy=True)
    lib().or_fcomb(int(grid), int(nintp), int(bool(interlacing)), float(box), _cptr(dcl))
    return dcl


def reduce_array(L, din, grid):
    """powerI4.f90:380-407."""
    din = _cgrid(din)
    out = np.zeros((int(grid),) * 3, dtype=np.complex128, order="F")
    lib().or_reduce_array(int(L), _cptr(din), int(grid), _cptr(out))
    return out


def compute_q2k(grid, box, deltak, i, j):
    """powerI4.f90:409-458 (i, j are 1-based)."""
    deltak = _cgrid(deltak)
    out = np.empty_like(deltak, order="F")
    lib().or_compute_q2k(int(grid), float(box), _cptr(deltak), int(i), int(j), _cptr(out))
    return out


def compute_q4k(grid, box, deltak, i, j, l, k):
    """powerI4.f90:460-508."""
    deltak = _cgrid(deltak)
    out = np.empty_like(deltak, order="F")
    lib().or_compute_q4k(int(grid), float(box), _cptr(deltak), int(i), int(j), int(l), int(k), _cptr(out))
    return out


def measure_pk(grid, box, kbin, kcenter, nbins, dcl1, dcl2):
    """powerI4.f90:510-594 -> pout (5, nbins)."""
    a, b = _cgrid(dcl1), _cgrid(dcl2)
    pout = np.zeros((5, int(nbins)), dtype=np.float64, order="F")
    lib().or_measure_pk(int(grid), float(box), float(kbin), float(kcenter), int(nbins), _cptr(a), _cptr(b), _p(pout))
    return pout


def measure_pk_multipoles(grid, box, kbin, kcenter, nbins, dcl, dcl2, dcl4):
    """powerI4.f90:596-693 -> pout (5, nbins)."""
    a, b, c = _cgrid(dcl), _cgrid(dcl2), _cgrid(dcl4)
    pout = np.zeros((5, int(nbins)), dtype=np.float64, order="F")
    lib().or_measure_pk_multipoles(int(grid), float(box), float(kbin), float(kcenter), int(nbins),
                                   _cptr(a), _cptr(b), _cptr(c), _p(pout))
    return pout


# ----------------------------------------------------------- bispectrumI4 ---
def shell_index(grid, kbin, kcenter, tiny_double=False):
    """Shell index of every full-grid mode (bispectrumI4.f90:66-77), as an
    (N,N,N) array s[i0, j0, l0] for dcl(i0+1, j0+1, l0+1)."""
    grid = int(grid)
    s = np.empty(grid ** 3, dtype=np.int32)
    lib().or_shell_index(grid, float(kbin), float(kcenter), int(tiny_double), _p(s, _i32))
    return s.reshape(grid, grid, grid)


def itot(nbins, kbin, kcenter, iopen, cross=False):
    return int(lib().or_count_itot(int(nbins), float(kbin), float(kcenter), int(bool(iopen)), int(bool(cross))))


def hermitian_full_grid(dcl):
    """The map1/map2 construction of bispectrumI4.f90:116-136: the kx >= 0 half
    of dcl is taken as is, the other half is its conjugate mirror, and the
    imaginary part is zeroed at the 8 self-conjugate points."""
    dcl = np.asarray(dcl)
    N = dcl.shape[0]
    neg = (-np.arange(N)) % N
    full = np.array(dcl, dtype=np.complex128, copy=True)
    mirror = np.conj(dcl[neg][:, neg][:, :, neg])
    full[N // 2 + 1:] = mirror[N // 2 + 1:]
    for a in (0, N // 2):
        for b in (0, N // 2):
            for c in (0, N // 2):
                full[a, b, c] = full[a, b, c].real
    return full


def shell_maps(dcl, nbins, kbin, kcenter, workers=None):
    """k-maps of bispectrumI4.f90:142-157: for each shell, FFTW FORWARD of the
    masked Hermitian grid, real part.  Returns (maps [nbins, N^3] FP64, nmodes).
    The reference lays the grid out transposed (x<->z) before its FFT; the
    triangle sums and shell powers it reports are sums over all x, which the
    transpose does not change."""
    N = np.asarray(dcl).shape[0]
    full = hermitian_full_grid(dcl)
    shell = shell_index(N, kbin, kcenter)
    maps = np.empty((nbins, N ** 3), dtype=np.float64)
    nmodes = np.zeros(nbins, dtype=np.int64)
    for b in range(1, nbins + 1):
        sel = shell == b
        nmodes[b - 1] = int(sel.sum())
        m = np.where(sel, full, 0.0)
        maps[b - 1] = scipy.fft.fftn(m, workers=workers).real.ravel()
    return maps, nmodes


def count_triangles(nbins, grid, kbin, kcenter, iopen, cross, npool, itot_, workers=None):
    """bispectrumI4.f90:763-915 -> counts[itot] float64 (= N^3 x N_tri)."""
    grid = int(grid)
    shell = shell_index(grid, kbin, kcenter, tiny_double=True)
    maps = np.empty((nbins, grid ** 3), dtype=np.float64)
    for b in range(1, nbins + 1):
        m = (shell == b).astype(np.complex128)
        maps[b - 1] = scipy.fft.fftn(m, workers=workers).real.ravel()
    counts = np.zeros(int(itot_), dtype=np.float64)
    _rows(lib().or_triangle_counts_sum_rows, itot_, workers, int(nbins), float(kbin), float(kcenter),
          int(bool(iopen)), int(bool(cross)), grid ** 3, _p(maps), _p(counts))
    return counts


def _shell_pow(maps, nmodes, kf, npart, gridD):
    """pow(i) of bispectrumI4.f90:151-156."""
    kf3 = float(np.float32(kf) * np.float32(kf) * np.float32(kf))
    powSN = 1.0 / float(npart) / kf3
    avg = np.einsum("ij,ij->i", maps, maps)
    return kf3 * avg / float(gridD) / nmodes.astype(np.float64) - powSN


def measure_bk(nbins, grid, kbin, kcenter, iopen, kf, npool, itot_, npart, counts, dcl, workers=None):
    """bispectrumI4.f90:1-198 -> bout (9, itot)."""
    grid = int(grid)
    maps, nmodes = shell_maps(dcl, nbins, kbin, kcenter, workers)
    pw = _shell_pow(maps, nmodes, kf, npart, grid ** 3)
    c32 = np.ascontiguousarray(counts, dtype=np.float32)
    bout = np.zeros((9, int(itot_)), dtype=np.float64, order="F")
    _rows(lib().or_bk_last_sum_rows, itot_, workers, int(nbins), float(kbin), float(kcenter), int(bool(iopen)),
          float(kf), int(npart), grid ** 3, _p(c32, _f), _p(maps), _p(pw), _p(bout))
    return bout


def measure_bk_multipoles(nbins, grid, kbin, kcenter, iopen, kf, npool, itot_, npart, counts, dcl, dcl2, dcl4,
                          workers=None):
    """bispectrumI4.f90:200-516 -> bout (11, itot)."""
    grid = int(grid)
    maps, nmodes = shell_maps(dcl, nbins, kbin, kcenter, workers)
    maps2, _ = shell_maps(dcl2, nbins, kbin, kcenter, workers)
    maps4, _ = shell_maps(dcl4, nbins, kbin, kcenter, workers)
    pw = _shell_pow(maps, nmodes, kf, npart, grid ** 3)
    c32 = np.ascontiguousarray(counts, dtype=np.float32)
    bout = np.zeros((11, int(itot_)), dtype=np.float64, order="F")
    _rows(lib().or_bk_multipoles_last_sum_rows, itot_, workers, int(nbins), float(kbin), float(kcenter),
          int(bool(iopen)), float(kf), int(npart), grid ** 3, _p(c32, _f), _p(maps), _p(maps2), _p(maps4), _p(pw),
          _p(bout))
    return bout


def measure_bk_cross(nbins, grid, kbin, kcenter, iopen, kf, npool, itot_, npart, counts, dcl1, dcl2, workers=None):
    """bispectrumI4.f90:518-761 -> bout (5, itot)."""
    grid = int(grid)
    maps, _ = shell_maps(dcl1, nbins, kbin, kcenter, workers)
    mapsB, _ = shell_maps(dcl2, nbins, kbin, kcenter, workers)
    c32 = np.ascontiguousarray(counts, dtype=np.float32)
    bout = np.zeros((5, int(itot_)), dtype=np.float64, order="F")
    _rows(lib().or_bk_cross_last_sum_rows, itot_, workers, int(nbins), float(kbin), float(kcenter),
          int(bool(iopen)), float(kf), grid ** 3, _p(c32, _f), _p(maps), _p(mapsB), _p(bout))
    return bout


# ------------------------------------------------------------ pbi4.py driver --
def derived_params(params):
    """pbi4.py:86-119."""
    p = dict(params)
    los = np.array(p["los"], dtype=np.float64)
    d = {
        "dk": p["kbin"] * 2.0 * np.pi / p["box"],
        "nbins_ps": floor((p["grid"] / 2 + p["kbin"] - p["kcenter"]) / p["kbin"]),
        "nbins_bisp": floor((p["grid"] / 3 + p["kbin"] - p["kcenter"]) / p["kbin"]),
        "kf": 2.0 * np.pi / p["box"],
        "kN": 2 * np.pi / p["box"] * p["grid"] / 2.0,
        "Hz": 100.0 * np.sqrt(p["om"] * (1.0 + p["z"]) ** 3 + p["ol"]),
        "los": los / (los @ los),
    }
    d["kvec"] = np.array([(i - 1) * d["dk"] + p["kcenter"] * 2.0 * np.pi / p["box"]
                          for i in range(1, d["nbins_ps"] + 1)])
    ishift = int(p["kcenter"] / p["kbin"]) + (1 if p["iopen"] else 0)
    n = 0
    for l in range(1, d["nbins_bisp"] + 1):
        for j in range(1, l + 1):
            imax = min(d["nbins_bisp"], j + l - 1 + ishift) if p["cross"] else j
            for i in range(max(1, l - j + 1 - ishift), imax + 1):
                n += 1
    d["itot"] = n
    return d


def assign_grid(pos, params, weight=None):
    """pbi4.py:290-302."""
    npart = len(pos.T)
    if weight is None:
        weight = np.ones(npart)
    if params["interlacing"]:
        dcl = assign_double_grid(params["grid"], params["interpolation"], npart, pos, weight)
    else:
        dcl = assign_single_grid(params["grid"], params["interpolation"], npart, pos, weight)
    return npart, dcl


def compute_density(npart, dcl, params, workers=None):
    """pbi4.py:336-339: dcl /= npart; fftn; fcomb."""
    dcl = dcl / npart
    dcl = scipy.fft.fftn(dcl, workers=workers)
    return fcomb(params["grid"], params["interpolation"], params["interlacing"], params["box"], dcl)


_Q4_FAC = {}


def _q4_fac(i, j, l, k):
    """Multiplicity of the symmetric 4-index term, pbi4.py:376-382."""
    if i == j and j == l and l == k:
        return 1
    if i == j and j == l and l > k:
        return 4
    if i == j and j > l and l == k:
        return 6
    if i > j and j == l and l == k:
        return 4
    if i == j and j > l and l > k:
        return 12
    if i > j and j == l and l > k:
        return 12
    if i > j and j > l and l == k:
        return 12
    raise AssertionError


def compute_density_multipoles(dcl, params, workers=None):
    """pbi4.py:343-388, literally: 1 ifftn + 6 fftn (delta_2) + 15 fftn (delta_4)."""
    los = params["los"]
    deltax = scipy.fft.ifftn(dcl, workers=workers)
    dcl2 = -0.5 * dcl
    for i in range(3):
        for j in range(i + 1):
            fac = 2.0 if i != j else 1.0
            deltak = scipy.fft.fftn(deltax * los[i] * los[j], workers=workers)
            dcl2 = dcl2 + fac * 1.5 * compute_q2k(params["grid"], params["box"], deltak, i + 1, j + 1)
    dcl4 = -7.0 / 8.0 * dcl - 2.5 * dcl2
    for i in range(3):
        for j in range(i + 1):
            for l in range(j + 1):
                for k in range(l + 1):
                    fac = _q4_fac(i, j, l, k)
                    deltak = scipy.fft.fftn(deltax * los[i] * los[j] * los[l] * los[k], workers=workers)
                    dcl4 = dcl4 + fac * (35.0 / 8.0) * compute_q4k(params["grid"], params["box"], deltak,
                                                                   i + 1, j + 1, l + 1, k + 1)
    return dcl2, dcl4


PS_DTYPE = [("k", np.float32), ("avgk", np.float32), ("P0+PSN", np.float32), ("P2", np.float32),
            ("P4", np.float32), ("Nmodes", np.float32), ("PSN", np.float32)]


def powerspectrum(npart, dcl, params, dcl2=None, dcl4=None):
    """pbi4.py:405-461 (auto spectra)."""
    out = np.zeros(len(params["kvec"]), dtype=PS_DTYPE)
    psn = 1.0 / (npart * (2.0 * np.pi / params["box"]) ** 3)
    if params["multipoles"]:
        pout = measure_pk_multipoles(params["grid"], params["box"], params["kbin"], params["kcenter"],
                                     params["nbins_ps"], dcl, dcl2, dcl4)
        out["P0+PSN"], out["P2"], out["P4"], out["Nmodes"] = pout[1], pout[2], pout[3], pout[4]
    else:
        if not params.get("cross", False) or dcl2 is None:
            dcl2 = dcl
        pout = measure_pk(params["grid"], params["box"], params["kbin"], params["kcenter"], params["nbins_ps"],
                          dcl, dcl2)
        out["P0+PSN"], out["Nmodes"] = pout[1], pout[2]
    out["k"] = params["kvec"]
    out["avgk"] = pout[0]
    out["PSN"] = psn
    return out


BS_DTYPE = [("k1", np.float32), ("k2", np.float32), ("k3", np.float32), ("Pk1", np.float32), ("Pk2", np.float32),
            ("Pk3", np.float32), ("B0+BSN", np.float32), ("BSN", np.float32), ("Ntr", np.float32)]
BS_MP_DTYPE = BS_DTYPE + [("B2", np.float32), ("B4", np.float32)]
BS_CROSS_DTYPE = [("k1", np.float32), ("k2", np.float32), ("k3", np.float32), ("B0", np.float32),
                  ("Ntr", np.float32)]


def bispectrum(npart, counts, dcl, params, dcl2=None, dcl4=None, workers=None):
    """pbi4.py:478-553."""
    a = (params["nbins_bisp"], params["grid"], params["kbin"], params["kcenter"], params["iopen"], params["kf"],
         params.get("npool", 1), params["itot"], npart, counts)
    if params.get("cross", False):
        bout = measure_bk_cross(*a, dcl, dcl2, workers=workers)
        dt = BS_CROSS_DTYPE
    elif not params["multipoles"]:
        bout = measure_bk(*a, dcl, workers=workers)
        dt = BS_DTYPE
    else:
        bout = measure_bk_multipoles(*a, dcl, dcl2, dcl4, workers=workers)
        dt = BS_MP_DTYPE
    out = np.zeros(bout.shape[1], dtype=dt)
    for r, (name, _) in enumerate(dt):
        out[name] = bout[r]
    return out


class BoxPipeline:
    """One box through the reference's call sequence (Tutorials/Script/test.py:7-13
    with pbi4.py:290-553): assign_grid -> compute_density -> compute_density_multipoles
    (the literal 1 ifftn + 21 fftn) -> measure_pk[_multipoles] -> measure_bk[_multipoles],
    with the triangle counts given (the reference loads them from its cfile when
    present, pbi4.py:466-470) or computed first.

    The box is a list of work items (`items()`: name, cost class, callable) run in
    order; running all of them computes the whole box.  FFTs use `workers` threads
    (the reference's FFTW npool threads for the maps; its scipy fftn calls are
    single-threaded) and the triangle sums split their rows over `workers`
    threads; the Fortran loops of assignment, fcomb and P binning stay serial.
    After the last item, `pout` and `bout` hold the f2py outputs."""

    def __init__(self, pos, params, counts=None, workers=None, tri_block=16):
        self.pos, self.p, self.workers = pos, params, workers
        self.counts = counts
        self.tri_block = int(tri_block)
        self.pout = self.bout = None

    # -- the counts (input independent; cached by the caller like the reference's cfile)
    def compute_counts(self):
        p = self.p
        self.counts = count_triangles(p["nbins_bisp"], p["grid"], p["kbin_bs"], p["kcenter_bs"], p["iopen"], False,
                                      1, p["itot"], workers=self.workers)
        return self.counts

    def items(self):
        p, w = self.p, self.workers
        N = int(p["grid"])
        mp = bool(p["multipoles"])
        nb, itot_ = int(p["nbins_bisp"]), int(p["itot"])
        kb, kc = float(p["kbin_bs"]), float(p["kcenter_bs"])
        st = {}
        out = []

        def assign():
            st["npart"], st["dcl"] = assign_grid(self.pos, p)

        def density():
            st["d"] = compute_density(st["npart"], st["dcl"], p, workers=w)
            st["dcl"] = None

        out += [("assign", "assign", assign), ("fft_fcomb", "fft", density)]
        los = p["los"]
        if mp:
            def inv():
                st["deltax"] = scipy.fft.ifftn(st["d"], workers=w)
                st["d2"] = -0.5 * st["d"]

            out.append(("multipoles_ifft", "fft", inv))
            for i in range(3):
                for j in range(i + 1):
                    def q2(i=i, j=j):
                        fac = 2.0 if i != j else 1.0
                        dk_ = scipy.fft.fftn(st["deltax"] * los[i] * los[j], workers=w)
                        st["d2"] = st["d2"] + fac * 1.5 * compute_q2k(N, p["box"], dk_, i + 1, j + 1)
                    out.append((f"q2k_{i}{j}", "fft", q2))

            def d4init():
                st["d4"] = -7.0 / 8.0 * st["d"] - 2.5 * st["d2"]
            out.append(("d4_init", "small", d4init))
            for i in range(3):
                for j in range(i + 1):
                    for l in range(j + 1):
                        for k in range(l + 1):
                            def q4(i=i, j=j, l=l, k=k):
                                dk_ = scipy.fft.fftn(st["deltax"] * los[i] * los[j] * los[l] * los[k], workers=w)
                                st["d4"] = st["d4"] + _q4_fac(i, j, l, k) * (35.0 / 8.0) * compute_q4k(
                                    N, p["box"], dk_, i + 1, j + 1, l + 1, k + 1)
                            out.append((f"q4k_{i}{j}{l}{k}", "fft", q4))

        def pk():
            if mp:
                st["deltax"] = None
                self.pout = measure_pk_multipoles(N, p["box"], p["kbin"], p["kcenter"], p["nbins_ps"], st["d"],
                                                  st["d2"], st["d4"])
            else:
                self.pout = measure_pk(N, p["box"], p["kbin"], p["kcenter"], p["nbins_ps"], st["d"], st["d"])
        out.append(("pk_binning", "small", pk))
        if not p.get("do_bispectrum", True) or itot_ == 0:
            return out

        sets = ("d", "d2", "d4") if mp else ("d",)
        shell = shell_index(N, kb, kc)
        st["maps"] = {s: np.empty((nb, N ** 3), dtype=np.float64) for s in sets}
        st["nmodes"] = np.array([int((shell == b).sum()) for b in range(1, nb + 1)], dtype=np.int64)
        for s in sets:
            def herm(s=s):
                st["full"] = hermitian_full_grid(st[s])
            out.append((f"hermitian_{s}", "small", herm))
            for b in range(1, nb + 1):
                def one_map(s=s, b=b):
                    m = np.where(shell == b, st["full"], 0.0)
                    st["maps"][s][b - 1] = scipy.fft.fftn(m, workers=w).real.ravel()
                out.append((f"map_{s}_{b}", "fft", one_map))

        def setup_sums():
            st["full"] = None
            st["pw"] = _shell_pow(st["maps"]["d"], st["nmodes"], p["kf"], st["npart"], N ** 3)
            st["c32"] = np.ascontiguousarray(self.counts, dtype=np.float32)
            st["bout"] = np.zeros((11 if mp else 9, itot_), dtype=np.float64, order="F")
        out.append(("shell_powers", "small", setup_sums))
        L = lib()
        for m0 in range(0, itot_, self.tri_block):
            m1 = min(itot_, m0 + self.tri_block)

            def tri(m0=m0, m1=m1):
                M = st["maps"]
                if mp:
                    fn, args = L.or_bk_multipoles_last_sum_rows, (
                        nb, kb, kc, int(bool(p["iopen"])), float(p["kf"]), int(st["npart"]), N ** 3,
                        _p(st["c32"], _f), _p(M["d"]), _p(M["d2"]), _p(M["d4"]), _p(st["pw"]), _p(st["bout"]))
                else:
                    fn, args = L.or_bk_last_sum_rows, (
                        nb, kb, kc, int(bool(p["iopen"])), float(p["kf"]), int(st["npart"]), N ** 3,
                        _p(st["c32"], _f), _p(M["d"]), _p(st["pw"]), _p(st["bout"]))
                # rows m0..m1 split over the threads, one row per task
                _rows_range(fn, m0, m1, w, *args)
                if m1 == itot_:
                    self.bout = st["bout"]
            out.append((f"triangles_{m0}", "triangles", tri))
        return out

    def run_all(self, timer=None):
        """Every item in order; returns {item cost class: seconds}."""
        import time
        if self.counts is None and self.p.get("do_bispectrum", True) and int(self.p["itot"]) > 0:
            self.compute_counts()
        t = {}
        for name, cls, fn in self.items():
            t0 = time.perf_counter()
            fn()
            t[cls] = t.get(cls, 0.0) + time.perf_counter() - t0
        return t


def _rows_range(fn, m0, m1, workers, *args):
    """Rows [m0, m1) of a "Last sum" routine, one row per thread task."""
    nw = max(1, min(int(workers or 1), m1 - m0))
    if nw == 1:
        fn(*args, m0, m1)
        return
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=nw) as ex:
        list(ex.map(lambda m: fn(*args, m, m + 1), range(m0, m1)))


def catalogue_positions(pos, vel=None, los=None, hz=None, z=None, box=1000.0, rsd_mode=1):
    """The catalogue step of IO.read_catalogues (pbi4.py:121-245) in numpy, with the
    reference's own operations and dtypes: pos, vel (N, 3) of the catalogue's dtype;
    RSD shift pos[:] += Vel[:] * los / Hz * (1 + z) (pbi4.py:158, 170, 214; rsd_mode 1)
    or pos[:] += Vel[:] * los (Minerva, pbi4.py:184; rsd_mode 0); then the wrap and the
    normalisation of pbi4.py:241-243.  Returns (3, N) float64."""
    pos = np.array(pos, copy=True)
    if vel is not None:
        if rsd_mode == 1:
            pos[:] += vel[:] * np.asarray(los) / hz * (1. + z)
        else:
            pos[:] += vel[:] * np.asarray(los)
    pos = pos.T
    pos = (pos + box) % box
    return np.minimum(1. - np.nextafter(0, 1), pos / box)
