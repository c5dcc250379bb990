"""The allocation-free P(k) entry point (pbi4g_measure_pk_multipoles_noalloc).

Some callers may not allocate device memory: an application that hands out all
device memory through its own pool, or a pipeline that forbids allocation once
it runs.  They pass device inputs and outputs; the entry point keeps its scratch
in a fixed device array inside the library.  This file is collected last so a
run that stops at the first failure has run every other test first; it also
passes when run alone in a fresh process.

Check: two calls in a row through the C ABI agree with the existing entry point
pbi4g_measure_pk_multipoles (host buffers) on the same grids: mode counts
bit-exact, the other rows within 1e-12 relative (the FP64 tolerance of
tests/test_gpu_parity.py::test_measure_pk_dropin); sizes above the scratch limit
are rejected.
"""
import ctypes

import numpy as np
import pytest

from oracle import pbi4_oracle as O
from pbi4_gb300 import _lib
from pbi4_gb300 import powerI4 as P
from pbi4_gb300 import synthetic

from ._helpers import oracle_density, ref_params

pytestmark = pytest.mark.gpu


def _half(torch, grid_full):
    n = grid_full.shape[0]
    # kx >= 0 half as [z][y][x] (x fastest): the Fortran-order grid transposed
    h = np.ascontiguousarray(np.asfortranarray(grid_full)[: n // 2 + 1].transpose(2, 1, 0))
    return torch.from_numpy(h.view(np.float64)).cuda()


def test_noalloc_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    lib = _lib.lib()
    grid, box, kbin, kc = 32, 1000.0, 1.0, 1.0
    pos = synthetic.zeldovich_box(24, box, seed=21)
    p = ref_params(grid, box, 4, True, True, kbin=kbin, kcenter=kc, los=(0.0, 0.0, 1.0))
    npart, d, d2, d4 = oracle_density(pos, p)
    nb = p["nbins_ps"]
    ref = P.measure_pk_multipoles(grid, box, kbin, kc, nb, d, d2, d4)
    h0, h2, h4 = _half(torch, d), _half(torch, d2), _half(torch, d4)
    for call in range(2):
        pout = torch.full((nb, 5), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.pbi4g_measure_pk_multipoles_noalloc(grid, box, kbin, kc, nb, h0.data_ptr(), h2.data_ptr(),
                                                     h4.data_ptr(), pout.data_ptr(), None)
        assert rc == 0, lib.pbi4g_last_error()
        torch.cuda.synchronize()
        got = pout.cpu().numpy().T
        np.testing.assert_array_equal(got[4], ref[4])
        rel = np.abs(got[:4] - ref[:4]) / np.abs(ref[:4]).max(axis=1, keepdims=True)
        assert np.max(rel) < 1e-12, (call, np.max(rel))


def test_noalloc_rejects_sizes_beyond_scratch():
    lib = _lib.lib()
    rc = lib.pbi4g_measure_pk_multipoles_noalloc(1024, 1000.0, 1.0, 1.0, 64, 1, 1, 1, 1, None)
    assert rc == _lib.PBI4G_OK + 7
    assert b"scratch limit" in lib.pbi4g_last_error()
    rc = lib.pbi4g_measure_pk_multipoles_noalloc(64, 1000.0, 1.0, 1.0, 513, 1, 1, 1, 1, None)
    assert rc == 7
