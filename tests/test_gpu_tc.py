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
