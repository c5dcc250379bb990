"""Tensor-core (tcgen05) triangle sums against the FP64 oracle.

Mixed-precision forms: FP16 hi+lo split and TF32 hi+lo split (3 products, FP32
accumulate; TF32 with the pair products in tensor memory) must stay within 1e-4
of FP64 under the B metric of tests/_helpers.b_errors; the single
BF16 product is checked against a looser 5e-2 bound (8-bit mantissas: its
per-element rounding is 2^-9, and the B2/B4 sums of these small, sparse boxes
cancel more than B0).  Triangle counts and the k columns are exact in both.
"""
import numpy as np
import pytest

from oracle import pbi4_oracle as O
from pbi4_gb300 import bispectrumI4 as B
from pbi4_gb300 import synthetic
from pbi4_gb300.estimator import Estimator, EstimatorConfig

from ._helpers import b_errors, oracle_density, ref_params

pytestmark = pytest.mark.gpu

TOL = {"fp16split": 1e-4, "tf32split": 1e-4, "bf16": 5e-2}


@pytest.fixture(scope="module")
def box_za():
    return synthetic.zeldovich_box(24, 1000.0, seed=12)


@pytest.mark.parametrize("precision", ["fp16split", "tf32split", "bf16"])
@pytest.mark.parametrize("grid,nb,kbin,multipoles", [(32, 8, 1.0, True), (32, 10, 1.0, False), (64, 10, 2.0, True),
                                                     (64, 24, 1.0, True)])
def test_plan_bispectrum_tensor_cores(box_za, precision, grid, nb, kbin, multipoles):
    p = ref_params(grid, 1000.0, 4, True, multipoles, kbin=kbin, kcenter=kbin)
    p["nbins_bisp"] = nb
    npart, d, d2, d4 = oracle_density(box_za, p)
    it = O.itot(nb, kbin, kbin, True)
    counts = O.count_triangles(nb, grid, kbin, kbin, True, False, 1, it)
    kf = 2 * np.pi / 1000.0
    if multipoles:
        ref = O.measure_bk_multipoles(nb, grid, kbin, kbin, True, kf, 1, it, npart, counts, d, d2, d4)
    else:
        ref = O.measure_bk(nb, grid, kbin, kbin, True, kf, 1, it, npart, counts, d)
    est = Estimator(EstimatorConfig.from_params(p, precision=precision))
    pout, bout = est.run_host(box_za)
    np.testing.assert_array_equal(bout[[0, 1, 2, 8]], ref[[0, 1, 2, 8]])
    errs, pw = b_errors(bout, ref)
    print(precision, grid, nb, multipoles, "B errors", errs, "pow", pw)
    assert max(errs) < TOL[precision] and pw < 1e-5, (errs, pw)


@pytest.mark.parametrize("precision", ["fp16split", "tf32split"])
def test_dropin_measure_bk_split(box_za, precision):
    p = ref_params(32, 1000.0, 4, True, True, kbin=1.0, kcenter=1.0)
    npart, d, d2, d4 = oracle_density(box_za, p)
    nb, it = 8, O.itot(8, 1.0, 1.0, True)
    counts = O.count_triangles(nb, 32, 1.0, 1.0, True, False, 1, it)
    kf = 2 * np.pi / 1000.0
    ref = O.measure_bk_multipoles(nb, 32, 1.0, 1.0, True, kf, 1, it, npart, counts, d, d2, d4)
    B.set_precision(precision)
    try:
        got = B.measure_bk_multipoles(nb, 32, 1.0, 1.0, True, kf, 1, it, npart, counts, d, d2, d4)
    finally:
        B.set_precision("fp32")
    errs, pw = b_errors(got, ref)
    assert max(errs) < 1e-4 and pw < 1e-5, (errs, pw)


@pytest.mark.parametrize("precision", ["fp16split", "tf32split"])
def test_tensor_core_forms_repeatable(box_za, precision):
    """Two runs of the same box agree: the triangle sums use a fixed reduction
    order; only the FP64 shell powers are summed with atomics (1e-15 level)."""
    p = ref_params(32, 1000.0, 4, True, True)
    p["nbins_bisp"] = 8
    est = Estimator(EstimatorConfig.from_params(p, precision=precision))
    _, b1 = est.run_host(box_za)
    _, b2 = est.run_host(box_za)
    np.testing.assert_array_equal(b1[[0, 1, 2, 8]], b2[[0, 1, 2, 8]])
    assert np.max(np.abs(b1 - b2) / np.maximum(np.abs(b1), 1e-300)) < 1e-12


@pytest.mark.parametrize("precision", ["fp32", "fp16split", "tf32split", "bf16"])
@pytest.mark.parametrize("grid,nb,multipoles", [(64, 10, True), (128, 16, False)])
def test_map_slabs_match_whole_grid(box_za, precision, grid, nb, multipoles):
    """A map budget below the whole grid's slab buffers streams the y pass, the
    x pass and the triangle sums over z-slabs (here with an uneven last slab;
    the 128^3 case has map grid 100, where a slab is a multiple of 4 z-planes
    so that it holds whole 64-point chunks); the results equal the one-slab run
    up to the order of the FP64 slab additions, and the counts and k columns
    are exact."""
    p = ref_params(grid, 1000.0, 4, True, multipoles, kbin=2.0, kcenter=2.0)
    p["nbins_bisp"] = nb
    whole = Estimator(EstimatorConfig.from_params(p, precision=precision))
    pw, bw = whole.run_host(box_za)
    nm_grid, nmaps = whole.map_grid, whole.nmaps
    assert whole.map_slabs() == (nm_grid, 1)
    q = 1
    while (q * nm_grid ** 2) % 64:
        q *= 2
    if grid == 128:
        assert nm_grid % 8 == 4 and q == 4, (nm_grid, q)
    # slab buffers per z-plane: the y pass's output (kxtot Nm complex) + the real maps
    kxtot = whole.map_work()[1] // nm_grid ** 2
    per_point = {"fp32": 4 * nmaps, "fp16split": 4 * nmaps + 4 * nb, "tf32split": 8 * nmaps + 4 * nb,
                 "bf16": 2 * nmaps + 4 * nb}[precision]
    per_plane = per_point * nm_grid ** 2 + 8 * kxtot * nm_grid

    def planes(m):
        return max(q, (m << 20) // per_plane // q * q)

    mb = next(m for m in range(1, 256) if 2 <= planes(m) < nm_grid and nm_grid % planes(m))
    zs = planes(mb)
    sl = Estimator(EstimatorConfig.from_params(p, precision=precision, map_budget_mb=mb))
    ps, bs = sl.run_host(box_za)
    assert sl.map_slabs() == (zs, -(-nm_grid // zs)), (sl.map_slabs(), zs)
    # P does not depend on the slabs; its FP32 per-block bin sums are added in
    # scheduling order, so two runs agree to ~1e-8 of P0, not bitwise
    np.testing.assert_allclose(ps[:2], pw[:2], rtol=1e-6, atol=0)
    np.testing.assert_array_equal(ps[4], pw[4])
    assert np.all(np.abs(ps[2:4] - pw[2:4]) <= 1e-6 * np.abs(pw[1]))  # P2, P4 against P0
    np.testing.assert_array_equal(bs[[0, 1, 2, 8]], bw[[0, 1, 2, 8]])
    errs, pow_err = b_errors(bs, bw)
    assert max(errs) < 1e-6 and pow_err < 1e-12, (errs, pow_err)
