"""GPU parity: every C-ABI entry point against the FP64 oracle on seeded inputs.

Tolerances (stated per test): integer outputs (mode counts, triangle counts)
bit-exact; FP64 GPU paths within 1e-9; FP32 paths within 1e-5 relative on P_l
and on B0 relative to max(|B|, P1P2+P1P3+P2P3), and within 3e-5 on B2 and B4
(see tests/_helpers.b_errors), whose l = 2, 4 bins on these small, sparse test
boxes are noise-dominated sums with more cancellation.
"""

TOL_FP32_B = (1e-5, 3e-5, 3e-5)  # B0, B2, B4
import numpy as np
import pytest

from oracle import pbi4_oracle as O
from pbi4_gb300 import bispectrumI4 as B
from pbi4_gb300 import powerI4 as P
from pbi4_gb300 import synthetic
from pbi4_gb300.estimator import Estimator, EstimatorConfig

from ._helpers import b_errors, oracle_density, p_errors, ref_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def box_uniform():
    return synthetic.uniform_box(20000, seed=11)


@pytest.fixture(scope="module")
def box_za():
    return synthetic.zeldovich_box(24, 1000.0, seed=12)


# ------------------------------------------------------------ assignment ---
@pytest.mark.parametrize("nintp", [1, 2, 3, 4])
@pytest.mark.parametrize("grid", [8, 16, 32])
def test_assign_single_grid(box_uniform, nintp, grid):
    pos = box_uniform
    w = np.ones(pos.shape[1])
    ref = O.assign_single_grid(grid, nintp, pos.shape[1], pos, w)
    got = P.assign_single_grid(grid, nintp, pos.shape[1], pos, w)
    assert got.shape == ref.shape and got.dtype == ref.dtype
    assert np.max(np.abs(got - ref)) <= 1e-11 * np.max(np.abs(ref))


@pytest.mark.parametrize("nintp", [1, 2, 3, 4])
@pytest.mark.parametrize("grid", [8, 16, 32])
def test_assign_double_grid(box_za, nintp, grid):
    pos = box_za
    w = np.random.default_rng(13).random(pos.shape[1]) + 0.5
    ref = O.assign_double_grid(grid, nintp, pos.shape[1], pos, w)
    got = P.assign_double_grid(grid, nintp, pos.shape[1], pos, w)
    assert got.dtype == np.complex128
    assert np.max(np.abs(got - ref)) <= 1e-11 * np.max(np.abs(ref))


def test_assign_bit_reproducible_under_permutation(box_uniform):
    pos = box_uniform
    w = np.ones(pos.shape[1])
    a = P.assign_double_grid(32, 4, pos.shape[1], pos, w)
    perm = np.random.default_rng(1).permutation(pos.shape[1])
    b = P.assign_double_grid(32, 4, pos.shape[1], np.ascontiguousarray(pos[:, perm]), w)
    c = P.assign_double_grid(32, 4, pos.shape[1], pos, w)
    assert a.tobytes() == b.tobytes()
    assert a.tobytes() == c.tobytes()


def test_assign_edge_positions():
    # positions at 0, just below 1 and exactly 1 (pbi4.py:243 can produce 1.0)
    pos = np.array([[0.0, 1.0 - 2 ** -53, 1.0, 0.5], [0.0, 0.999999, 1.0, 0.25], [1.0, 0.0, 0.5, 0.75]])
    w = np.ones(4)
    for nintp in (1, 2, 3, 4):
        ref = O.assign_double_grid(8, nintp, 4, pos, w)
        got = P.assign_double_grid(8, nintp, 4, pos, w)
        assert np.max(np.abs(got - ref)) <= 1e-12


# ------------------------------------------------------- fcomb and friends ---
@pytest.mark.parametrize("interlacing", [False, True])
@pytest.mark.parametrize("grid,nintp", [(8, 2), (16, 4), (16, 3), (32, 1)])
def test_fcomb_full(box_za, interlacing, grid, nintp):
    import scipy.fft
    p = ref_params(grid, 1000.0, nintp, interlacing, False)
    npart, dcl = O.assign_grid(box_za, p)
    f = scipy.fft.fftn(dcl / npart)
    ref = O.fcomb(grid, nintp, interlacing, 1000.0, f)
    got = P.fcomb(grid, nintp, interlacing, 1000.0, f)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_q2k_q4k_reduce(box_za):
    import scipy.fft
    rng = np.random.default_rng(3)
    d = scipy.fft.fftn(rng.standard_normal((16, 16, 16)))
    for ij in [(1, 1), (2, 1), (3, 2), (3, 3)]:
        ref = O.compute_q2k(16, 1000.0, d, *ij)
        got = P.compute_q2k(16, 1000.0, d, *ij)
        assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    for ijlk in [(1, 1, 1, 1), (3, 2, 2, 1), (3, 3, 1, 1)]:
        ref = O.compute_q4k(16, 1000.0, d, *ijlk)
        got = P.compute_q4k(16, 1000.0, d, *ijlk)
        assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    big = scipy.fft.fftn(rng.standard_normal((32, 32, 32)))
    assert np.array_equal(P.reduce_array(32, big, 16), O.reduce_array(32, big, 16))


# ------------------------------------------------------------------ P(k) ---
@pytest.mark.parametrize("kbin,kcenter", [(1.0, 1.0), (2.0, 2.0), (1.5, 0.5)])
def test_measure_pk_dropin(box_za, kbin, kcenter):
    p = ref_params(32, 1000.0, 4, True, True, kbin=kbin, kcenter=kcenter)
    npart, d, d2, d4 = oracle_density(box_za, p)
    nb = p["nbins_ps"]
    ref = O.measure_pk_multipoles(32, 1000.0, kbin, kcenter, nb, d, d2, d4)
    got = P.measure_pk_multipoles(32, 1000.0, kbin, kcenter, nb, d, d2, d4)
    np.testing.assert_array_equal(got[4], ref[4])
    assert np.max(np.abs(got[:4] - ref[:4]) / np.abs(ref[:4]).max(axis=1, keepdims=True)) < 1e-12
    ref1 = O.measure_pk(32, 1000.0, kbin, kcenter, nb, d, d2)
    got1 = P.measure_pk(32, 1000.0, kbin, kcenter, nb, d, d2)
    np.testing.assert_array_equal(got1[2], ref1[2])
    assert np.max(np.abs(got1[:2] - ref1[:2]) / np.abs(ref1[:2]).max(axis=1, keepdims=True)) < 1e-12


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("fp64", 1e-9)])
@pytest.mark.parametrize("grid,nintp,interlacing,multipoles",
                         [(32, 4, True, True), (32, 2, False, False), (64, 3, True, True), (16, 1, True, False)])
def test_plan_powerspectrum(box_za, precision, tol, grid, nintp, interlacing, multipoles):
    p = ref_params(grid, 1000.0, nintp, interlacing, multipoles, los=(0.0, 2.0, 1.0))
    npart, d, d2, d4 = oracle_density(box_za, p)
    nb = p["nbins_ps"]
    if multipoles:
        ref = O.measure_pk_multipoles(grid, 1000.0, 1.0, 1.0, nb, d, d2, d4)
    else:
        ref = O.measure_pk(grid, 1000.0, 1.0, 1.0, nb, d, d)
    est = Estimator(EstimatorConfig.from_params(p, precision=precision, do_bispectrum=False))
    pout, _ = est.run_host(box_za)
    rows = 4 if multipoles else 2
    np.testing.assert_array_equal(pout[rows], ref[rows])
    e0, e2, e4 = p_errors(pout, ref, multipoles)
    assert e0 < tol and e2 < tol and e4 < tol, (e0, e2, e4)
    assert np.max(np.abs(pout[0] / ref[0] - 1)) < 1e-12


# --------------------------------------------------------------- counts ---
def test_count_triangles_golden():
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                           "reference_testdata_cols.npz"))
    c = B.count_triangles(21, 64, 1.0, 1.0, True, False, 4, 1156)
    np.testing.assert_array_equal(np.round(c / 64.0 ** 3).astype(np.int64), g["bs_ntr"])
    assert np.array_equal(c, np.round(c / 64.0 ** 3) * 64.0 ** 3)


@pytest.mark.parametrize("grid,nb,kbin,kc,iopen,cross", [(16, 5, 1.0, 1.0, False, False), (32, 8, 2.0, 2.0, True, False),
                                                         (24, 6, 1.5, 1.5, True, True), (16, 4, 1.0, 1.0, True, True)])
def test_count_triangles(grid, nb, kbin, kc, iopen, cross):
    it = O.itot(nb, kbin, kc, iopen, cross)
    ref = O.count_triangles(nb, grid, kbin, kc, iopen, cross, 1, it)
    got = B.count_triangles(nb, grid, kbin, kc, iopen, cross, 1, it)
    np.testing.assert_array_equal(got / grid ** 3, np.round(ref / grid ** 3))


# ------------------------------------------------------------ bispectrum ---
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_measure_bk_dropin(box_za, precision, tol):
    p = ref_params(32, 1000.0, 4, True, True, kbin=1.0, kcenter=1.0)
    npart, d, d2, d4 = oracle_density(box_za, p)
    nb, it = 8, O.itot(8, 1.0, 1.0, True)
    counts = O.count_triangles(nb, 32, 1.0, 1.0, True, False, 1, it)
    kf = 2 * np.pi / 1000.0
    B.set_precision(precision)
    try:
        ref = O.measure_bk(nb, 32, 1.0, 1.0, True, kf, 1, it, npart, counts, d)
        got = B.measure_bk(nb, 32, 1.0, 1.0, True, kf, 1, it, npart, counts, d)
        np.testing.assert_array_equal(got[[0, 1, 2, 8]], ref[[0, 1, 2, 8]])
        lim = TOL_FP32_B if precision == "fp32" else (tol, tol, tol)
        errs, pw = b_errors(got, ref)
        assert all(e < t for e, t in zip(errs, lim)) and pw < tol, (errs, pw)
        refm = O.measure_bk_multipoles(nb, 32, 1.0, 1.0, True, kf, 1, it, npart, counts, d, d2, d4)
        gotm = B.measure_bk_multipoles(nb, 32, 1.0, 1.0, True, kf, 1, it, npart, counts, d, d2, d4)
        errs, pw = b_errors(gotm, refm)
        assert all(e < t for e, t in zip(errs, lim)) and pw < tol, (errs, pw)
    finally:
        B.set_precision("fp32")


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
@pytest.mark.parametrize("grid,nb,kbin,iopen", [(16, 4, 1.0, True), (32, 8, 1.0, True), (32, 6, 2.0, False)])
def test_measure_bk_cross_dropin(box_za, box_uniform, precision, tol, grid, nb, kbin, iopen):
    """measure_bk_cross (bispectrumI4.f90:518-761) in the drop-in's default FP32
    form and in FP64: the k columns and N_tr bit-exact, B0 within the stated
    relative tolerance of the larger of |B0| and the bin's |B0| scale (the cross
    bispectrum of two independent boxes is a noise sum and crosses zero)."""
    p = ref_params(grid, 1000.0, 3, True, False)
    n1, d1, _, _ = oracle_density(box_za, p)
    n2, d2, _, _ = oracle_density(box_uniform, p)
    it = O.itot(nb, kbin, kbin, iopen, True)
    counts = O.count_triangles(nb, grid, kbin, kbin, iopen, True, 1, it)
    kf = 2 * np.pi / 1000.0
    ref = O.measure_bk_cross(nb, grid, kbin, kbin, iopen, kf, 1, it, n1, counts, d1, d2)
    B.set_precision(precision)
    try:
        got = B.measure_bk_cross(nb, grid, kbin, kbin, iopen, kf, 1, it, n1, counts, d1, d2)
    finally:
        B.set_precision("fp32")
    np.testing.assert_array_equal(got[[0, 1, 2, 4]], ref[[0, 1, 2, 4]])
    # per triangle: |dB| / max(|B|, the rms of B over the triangles of its l shell)
    scale = np.zeros_like(ref[3])
    for kl in np.unique(ref[0]):
        sel = ref[0] == kl
        scale[sel] = np.sqrt(np.mean(ref[3][sel] ** 2))
    err = np.abs(got[3] - ref[3]) / np.maximum(np.abs(ref[3]), scale)
    assert err.max() <= tol, (precision, err.max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
@pytest.mark.parametrize("multipoles", [False, True])
def test_plan_bispectrum(box_za, precision, tol, multipoles):
    grid, nb = 32, 8
    p = ref_params(grid, 1000.0, 4, True, multipoles, kbin=1.0, kcenter=1.0)
    p["nbins_bisp"] = nb
    npart, d, d2, d4 = oracle_density(box_za, p)
    it = O.itot(nb, 1.0, 1.0, True)
    counts = O.count_triangles(nb, grid, 1.0, 1.0, True, False, 1, it)
    kf = 2 * np.pi / 1000.0
    if multipoles:
        ref = O.measure_bk_multipoles(nb, grid, 1.0, 1.0, True, kf, 1, it, npart, counts, d, d2, d4)
    else:
        ref = O.measure_bk(nb, grid, 1.0, 1.0, True, kf, 1, it, npart, counts, d)
    est = Estimator(EstimatorConfig.from_params(p, precision=precision))
    pout, bout = est.run_host(box_za)
    assert bout.shape == ref.shape
    np.testing.assert_array_equal(est.triangle_counts(), np.round(counts / grid ** 3).astype(np.int64))
    np.testing.assert_array_equal(bout[[0, 1, 2, 8]], ref[[0, 1, 2, 8]])
    errs, pw = b_errors(bout, ref)
    lim = TOL_FP32_B if precision == "fp32" else (tol, tol, tol)
    assert all(e < t for e, t in zip(errs, lim)) and pw < tol, (errs, pw)


@pytest.mark.parametrize("interlacing,nintp", [(True, 4), (False, 4), (False, 2), (True, 3)])
def test_plan_density_bit_reproducible(box_uniform, interlacing, nintp):
    """The plan's density (fixed-point tiles, then FFT) is bit-identical for any particle order."""
    p = ref_params(64, 1000.0, nintp, interlacing, False)
    est = Estimator(EstimatorConfig.from_params(p, precision="fp32", do_bispectrum=False))
    est.run_host(box_uniform)
    a = est.delta_half()
    perm = np.random.default_rng(2).permutation(box_uniform.shape[1])
    est.run_host(np.ascontiguousarray(box_uniform[:, perm]))
    b = est.delta_half()
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("nintp", [1, 2, 3, 4])
@pytest.mark.parametrize("interlacing", [False, True])
def test_plan_density_fp32_prep_matches_fp64(nintp, interlacing):
    """The FP32 forms find each particle's first cells and FP32 offsets from one
    FP64 product (integer fraction bits for the floor, the rounding and the
    half-cell shift); on positions at cell edges, half cells, 0, 1 - 2^-53 and
    1 the density equals the FP64 form's to FP32 rounding (a different cell for
    one particle would show as a 1e-4 error)."""
    n = 32
    rng = np.random.default_rng(5)
    k = np.arange(n + 1, dtype=np.float64)
    special = np.concatenate([k / n, (k + 0.5) / n, np.nextafter(k / n, 0), np.nextafter((k + 0.5) / n, 1),
                              [0.0, 1.0 - 2.0 ** -53, 1.0]])
    special = np.clip(special, 0.0, 1.0)
    m = special.size
    pos = np.concatenate([rng.random((3, 3000)),
                          np.stack([special, rng.permutation(special), special[::-1]])], axis=1)
    p = ref_params(n, 1000.0, nintp, interlacing, False)
    out = {}
    for prec in ("fp32", "fp64"):
        est = Estimator(EstimatorConfig.from_params(p, precision=prec, do_bispectrum=False))
        est.run_host(np.ascontiguousarray(pos))
        out[prec] = est.delta_half()
        est.close()
    assert m > 100
    err = np.max(np.abs(out["fp32"] - out["fp64"])) / np.max(np.abs(out["fp64"]))
    assert err < 2e-6, err


@pytest.mark.parametrize("interlacing,nintp", [(True, 4), (False, 4), (False, 2), (True, 3)])
def test_plan_density_weighted_fp32_matches_fp64(box_za, interlacing, nintp):
    """Per-particle weights through the FP32 owner tiles (the fixed-point scale
    set from the largest weight, one 32-bit value per contribution) against the
    FP64 form: the density equals it to FP32 rounding; zero weights and a wide
    weight range included."""
    rng = np.random.default_rng(21)
    n = box_za.shape[1]
    w = rng.uniform(0.5, 1.5, n)
    w[::7] = 0.0
    w[5] = 40.0
    p = ref_params(32, 1000.0, nintp, interlacing, False)
    out = {}
    for prec in ("fp32", "fp64"):
        est = Estimator(EstimatorConfig.from_params(p, precision=prec, do_bispectrum=False))
        est.run_host(box_za, w)
        out[prec] = est.delta_half()
        est.close()
    err = np.max(np.abs(out["fp32"] - out["fp64"])) / np.max(np.abs(out["fp64"]))
    assert err < 2e-6, err
