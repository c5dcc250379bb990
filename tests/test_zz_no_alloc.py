"""The allocation-free P(k) entry point (pbi4g_measure_pk_multipoles_noalloc).

Some callers may not allocate device memory: an application that hands out all
device memory through its own pool, or a pipeline that forbids allocation once
it runs.  They pass device inputs and outputs; the entry point keeps its scratch
in a fixed device array inside the library.  This file is collected last so a
run that stops at the first failure has run every other test first; it also
passes when run alone in a fresh process.

Checks: two calls in a row through the C ABI agree with the existing entry point
pbi4g_measure_pk_multipoles (host buffers) and with the FP64 oracle on the same
grids: mode counts bit-exact, the other rows within 1e-12 relative (the FP64
tolerance of tests/test_gpu_parity.py::test_measure_pk_dropin); the library's
count of device allocations does not move across the calls; a 256^3 grid with
512 bins (the scratch's largest bin count, and the binning kernel's tail over
the Nyquist plane) matches the existing entry point; sizes above the scratch
limit are rejected before any device work.
"""
import numpy as np
import pytest

from oracle import pbi4_oracle as O
from pbi4_gb300 import _lib
from pbi4_gb300 import powerI4 as P
from pbi4_gb300 import synthetic

from ._helpers import oracle_density, ref_params


def _half(torch, grid_full):
    n = grid_full.shape[0]
    # kx >= 0 half as [z][y][x] (x fastest): the Fortran-order grid transposed
    h = np.ascontiguousarray(np.asfortranarray(grid_full)[: n // 2 + 1].transpose(2, 1, 0))
    return torch.from_numpy(h.view(np.float64)).cuda()


def _call(torch, lib, grid, box, kbin, kc, nb, halves):
    pout = torch.full((nb, 5), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib.pbi4g_measure_pk_multipoles_noalloc(grid, box, kbin, kc, nb, halves[0].data_ptr(),
                                                 halves[1].data_ptr(), halves[2].data_ptr(), pout.data_ptr(), None)
    assert rc == 0, lib.pbi4g_last_error()
    torch.cuda.synchronize()
    return pout.cpu().numpy().T


def _close(got, ref, tol=1e-12):
    """Mode counts equal; bins without modes are NaN in both (powerI4.f90:590-592
    divide by the count); the others within tol relative to each row's largest value."""
    np.testing.assert_array_equal(got[4], ref[4])
    ok = ref[4] > 0
    np.testing.assert_array_equal(np.isnan(got[:4, ~ok]), np.isnan(ref[:4, ~ok]))
    g, r = got[:4, ok], ref[:4, ok]
    rel = np.abs(g - r) / np.abs(r).max(axis=1, keepdims=True)
    assert np.max(rel) < tol, np.max(rel)


@pytest.mark.gpu
def test_noalloc_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    lib = _lib.lib()
    grid, box, kbin, kc = 32, 1000.0, 1.0, 1.0
    pos = synthetic.zeldovich_box(24, box, seed=21)
    p = ref_params(grid, box, 4, True, True, kbin=kbin, kcenter=kc, los=(0.0, 0.0, 1.0))
    npart, d, d2, d4 = oracle_density(pos, p)
    nb = p["nbins_ps"]
    ref = P.measure_pk_multipoles(grid, box, kbin, kc, nb, d, d2, d4)
    oracle = O.measure_pk_multipoles(grid, box, kbin, kc, nb, d, d2, d4)
    halves = [_half(torch, g) for g in (d, d2, d4)]
    torch.cuda.synchronize()
    allocs = lib.pbi4g_device_allocs()
    for call in range(2):
        got = _call(torch, lib, grid, box, kbin, kc, nb, halves)
        _close(got, ref)
        _close(got, oracle)
    assert lib.pbi4g_device_allocs() == allocs, "the allocation-free entry point allocated device memory"


@pytest.mark.gpu
def test_noalloc_largest_binning():
    """grid 256 (the binning kernel's Nyquist-plane tail) and 512 bins (kbin = kcenter
    = 1/4: the scratch's largest bin count) against the host-buffer entry point."""
    torch = pytest.importorskip("torch")
    lib = _lib.lib()
    grid, box, kbin, kc = 256, 1000.0, 0.25, 0.25
    nb = int((grid / 2 + kbin - kc) // kbin)
    assert nb == 512
    rng = np.random.default_rng(8)
    shape = (grid, grid, grid)
    grids = [np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) for _ in range(3)]
    ref = P.measure_pk_multipoles(grid, box, kbin, kc, nb, *grids)
    halves = [_half(torch, g) for g in grids]
    del grids
    allocs = lib.pbi4g_device_allocs()
    for call in range(2):
        got = _call(torch, lib, grid, box, kbin, kc, nb, halves)
        _close(got, ref)
    assert lib.pbi4g_device_allocs() == allocs


def test_noalloc_rejects_sizes_beyond_scratch():
    """Host-side range checks: nothing reaches the device (no GPU needed)."""
    lib = _lib.lib()
    rc = lib.pbi4g_measure_pk_multipoles_noalloc(1024, 1000.0, 1.0, 1.0, 64, 1, 1, 1, 1, None)
    assert rc == 7  # PBI4G_ERR_RANGE
    assert b"scratch limit" in lib.pbi4g_last_error()
    rc = lib.pbi4g_measure_pk_multipoles_noalloc(64, 1000.0, 1.0, 1.0, 513, 1, 1, 1, 1, None)
    assert rc == 7
