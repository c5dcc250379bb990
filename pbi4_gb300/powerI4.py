"""Drop-in for the reference's f2py module ``powerI4`` (pbi4/F90_modules/powerI4.f90).

Same function names, argument order, argument kinds and return shapes/dtypes as
the f2py wrappers that ``pbi4/pbi4.py:12-13`` imports; the work runs on the GPU
through libpbi4gpu.so.  Grids are numpy arrays of shape (N, N, N) in Fortran
order (``a[ix-1, iy-1, iz-1]`` is Fortran ``a(ix, iy, iz)``), as f2py returns them.
"""
from __future__ import annotations

import numpy as np

from ._lib import check, lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _cgrid(a, n):
    a = np.asfortranarray(a, dtype=np.complex128)
    if a.shape != (n, n, n):
        raise ValueError(f"expected a ({n},{n},{n}) grid, got {a.shape}")
    return a


def _pos(pos, npart):
    pos = _f64(pos)
    if pos.ndim != 2 or pos.shape[0] != 3 or pos.shape[1] < npart:
        raise ValueError(f"pos must be (3, npart), got {pos.shape}")
    if pos.shape[1] != npart:
        pos = np.ascontiguousarray(pos[:, :npart])
    return pos


def assign_single_grid(grid, nintp, npart, pos, weight):
    """powerI4.f90:68-140 -> dtl float64 (N,N,N) Fortran order (bit-reproducible fixed-point sum)."""
    grid, nintp, npart = int(grid), int(nintp), int(npart)
    pos, weight = _pos(pos, npart), _f64(weight)[:npart]
    out = np.empty((grid, grid, grid), dtype=np.float64, order="F")
    check(lib().pbi4g_assign_single_grid(grid, nintp, npart, pos.ctypes.data, weight.ctypes.data, out.ctypes.data))
    return out


def assign_double_grid(grid, nintp, npart, pos, weight):
    """powerI4.f90:142-249 -> dcl complex128 (N,N,N): Re grid, Im interlaced grid."""
    grid, nintp, npart = int(grid), int(nintp), int(npart)
    pos, weight = _pos(pos, npart), _f64(weight)[:npart]
    out = np.empty((grid, grid, grid), dtype=np.complex128, order="F")
    check(lib().pbi4g_assign_double_grid(grid, nintp, npart, pos.ctypes.data, weight.ctypes.data, out.ctypes.data))
    return out


def fcomb(grid, nintp, interlacing, box, fdcl):
    """powerI4.f90:251-378 (interlacing combine + window deconvolution)."""
    grid = int(grid)
    a = _cgrid(fdcl, grid)
    out = np.empty_like(a, order="F")
    check(lib().pbi4g_fcomb(grid, int(nintp), int(bool(interlacing)), float(box), a.ctypes.data, out.ctypes.data))
    return out


def reduce_array(L, din, grid):
    """powerI4.f90:380-407 (down-sample an L^3 spectrum to grid^3)."""
    L, grid = int(L), int(grid)
    a = _cgrid(din, L)
    out = np.empty((grid, grid, grid), dtype=np.complex128, order="F")
    check(lib().pbi4g_reduce_array(L, a.ctypes.data, grid, out.ctypes.data))
    return out


def compute_q2k(grid, box, deltak, i, j):
    """powerI4.f90:409-458 (i, j 1-based)."""
    grid = int(grid)
    a = _cgrid(deltak, grid)
    out = np.empty_like(a, order="F")
    check(lib().pbi4g_compute_q2k(grid, float(box), a.ctypes.data, int(i), int(j), out.ctypes.data))
    return out


def compute_q4k(grid, box, deltak, i, j, l, k):
    """powerI4.f90:460-508 (indices 1-based)."""
    grid = int(grid)
    a = _cgrid(deltak, grid)
    out = np.empty_like(a, order="F")
    check(lib().pbi4g_compute_q4k(grid, float(box), a.ctypes.data, int(i), int(j), int(l), int(k), out.ctypes.data))
    return out


def measure_pk(grid, box, kbin, kcenter, nbins, dcl1, dcl2):
    """powerI4.f90:510-594 -> pout float64 (5, nbins): avgk, P, Nmodes, 0, 0."""
    grid, nbins = int(grid), int(nbins)
    a, b = _cgrid(dcl1, grid), _cgrid(dcl2, grid)
    pout = np.empty((5, nbins), dtype=np.float64, order="F")
    check(lib().pbi4g_measure_pk(grid, float(box), float(kbin), float(kcenter), nbins, a.ctypes.data, b.ctypes.data,
                                 pout.ctypes.data))
    return pout


def measure_pk_multipoles(grid, box, kbin, kcenter, nbins, dcl, dcl2, dcl4):
    """powerI4.f90:596-693 -> pout float64 (5, nbins): avgk, P0, P2, P4, Nmodes."""
    grid, nbins = int(grid), int(nbins)
    a, b, c = _cgrid(dcl, grid), _cgrid(dcl2, grid), _cgrid(dcl4, grid)
    pout = np.empty((5, nbins), dtype=np.float64, order="F")
    check(lib().pbi4g_measure_pk_multipoles(grid, float(box), float(kbin), float(kcenter), nbins, a.ctypes.data,
                                            b.ctypes.data, c.ctypes.data, pout.ctypes.data))
    return pout
