"""Drop-in for the reference's f2py module ``bispectrumI4``
(pbi4/F90_modules/bispectrumI4.f90), imported by ``pbi4/pbi4.py:14``.

Same names, arguments and return shapes/dtypes as the f2py wrappers.  The
``npool`` argument (FFTW threads) is accepted and ignored.  The arithmetic of
the shell maps and triangle sums is FP32 by default (``set_precision('fp64')``
switches to FP64); triangle counts are exact integers either way.
"""
from __future__ import annotations

import numpy as np

from ._lib import PRECISIONS, check, lib


def set_precision(name: str) -> None:
    """'fp32' (default), 'fp64', 'fp16split' or 'bf16' for the drop-in bispectrum routines."""
    check(lib().pbi4g_set_dropin_precision(PRECISIONS[name]))


def _cgrid(a, n):
    a = np.asfortranarray(a, dtype=np.complex128)
    if a.shape != (n, n, n):
        raise ValueError(f"expected a ({n},{n},{n}) grid, got {a.shape}")
    return a


def _counts(counts, itot):
    c = np.ascontiguousarray(counts, dtype=np.float32)  # f2py casts counts to real(4)
    if c.shape[0] < itot:
        raise ValueError(f"counts has {c.shape[0]} entries, itot={itot}")
    return c


def count_triangles(nbins, grid, kbin, kcenter, iopen, cross, npool, itot):
    """bispectrumI4.f90:763-915 -> counts float64 [itot] (grid^3 x exact integer count)."""
    itot = int(itot)
    out = np.empty(itot, dtype=np.float64)
    check(lib().pbi4g_count_triangles(int(nbins), int(grid), float(kbin), float(kcenter), int(bool(iopen)),
                                      int(bool(cross)), int(npool), itot, out.ctypes.data))
    return out


def measure_bk(nbins, grid, kbin, kcenter, iopen, kf, npool, itot, npart, counts, dcl):
    """bispectrumI4.f90:1-198 -> bout float64 (9, itot)."""
    grid, itot = int(grid), int(itot)
    a, c = _cgrid(dcl, grid), _counts(counts, itot)
    bout = np.empty((9, itot), dtype=np.float64, order="F")
    check(lib().pbi4g_measure_bk(int(nbins), grid, float(kbin), float(kcenter), int(bool(iopen)), float(kf),
                                 int(npool), itot, int(npart), c.ctypes.data, a.ctypes.data, bout.ctypes.data))
    return bout


def measure_bk_multipoles(nbins, grid, kbin, kcenter, iopen, kf, npool, itot, npart, counts, dcl, dcl2, dcl4):
    """bispectrumI4.f90:200-516 -> bout float64 (11, itot)."""
    grid, itot = int(grid), int(itot)
    a, b, d = _cgrid(dcl, grid), _cgrid(dcl2, grid), _cgrid(dcl4, grid)
    c = _counts(counts, itot)
    bout = np.empty((11, itot), dtype=np.float64, order="F")
    check(lib().pbi4g_measure_bk_multipoles(int(nbins), grid, float(kbin), float(kcenter), int(bool(iopen)),
                                            float(kf), int(npool), itot, int(npart), c.ctypes.data, a.ctypes.data,
                                            b.ctypes.data, d.ctypes.data, bout.ctypes.data))
    return bout


def measure_bk_cross(nbins, grid, kbin, kcenter, iopen, kf, npool, itot, npart, counts, dcl1, dcl2):
    """bispectrumI4.f90:518-761 -> bout float64 (5, itot)."""
    grid, itot = int(grid), int(itot)
    a, b = _cgrid(dcl1, grid), _cgrid(dcl2, grid)
    c = _counts(counts, itot)
    bout = np.empty((5, itot), dtype=np.float64, order="F")
    check(lib().pbi4g_measure_bk_cross(int(nbins), grid, float(kbin), float(kcenter), int(bool(iopen)), float(kf),
                                       int(npool), itot, int(npart), c.ctypes.data, a.ctypes.data, b.ctypes.data,
                                       bout.ctypes.data))
    return bout
