"""Self-consistency and analytic checks of the FP64 oracle (CPU only, small grids)."""
import itertools

import numpy as np
import pytest
import scipy.fft

from oracle import pbi4_oracle as O
from pbi4_gb300 import synthetic


@pytest.mark.parametrize("nintp", [1, 2, 3, 4])
@pytest.mark.parametrize("interlaced", [False, True])
def test_assign_conserves_weight(nintp, interlaced):
    pos = synthetic.uniform_box(500, seed=3)
    w = np.random.default_rng(4).random(500) + 0.5
    if interlaced:
        g = O.assign_double_grid(16, nintp, 500, pos, w)
        assert abs(g.real.sum() - w.sum()) < 1e-9 and abs(g.imag.sum() - w.sum()) < 1e-9
    else:
        g = O.assign_single_grid(16, nintp, 500, pos, w)
        assert abs(g.sum() - w.sum()) < 1e-9


def test_single_grid_cic_quirk_negative_weights():
    # single-grid CIC takes the cell from int() but the offset from nint(): at
    # vr = N*pos + 1 = 3.7 the weights are 1.3 and -0.3 (powerI4.f90:114-123)
    N = 8
    pos = np.array([[2.7 / N], [2.0 / N], [2.0 / N]])
    g = O.assign_single_grid(N, 2, 1, pos, np.ones(1))
    assert g.min() < 0 and abs(g.sum() - 1.0) < 1e-12


def test_fcomb_interlaced_output_is_hermitian():
    pos = synthetic.uniform_box(2000, seed=5)
    p = dict(grid=16, interpolation=3, interlacing=True, box=1000.0)
    _, dcl = O.assign_grid(pos, p)
    d = O.compute_density(2000, dcl, p)
    N = 16
    neg = (-np.arange(N)) % N
    mirror = np.conj(d[neg][:, neg][:, :, neg])
    diff = np.abs(d - mirror)
    # Hermitian everywhere except at the self-conjugate points (indices in {0, N/2}),
    # where the Nyquist phase of the interlacing combine leaves an imaginary part
    sc = np.zeros_like(diff, dtype=bool)
    for a, b, c in itertools.product((0, N // 2), repeat=3):
        sc[a, b, c] = True
    assert np.max(diff[~sc]) <= 1e-12 * np.max(np.abs(d))
    assert np.max(diff[sc]) > 0


def test_multipoles_pointwise_equals_literal():
    """delta_2 / delta_4 by the 22-FFT route of pbi4.py:343-388 equal the per-mode
    factors (-1/2 + 3/2 mu^2) and (3/8 - 30/8 mu^2 + 35/8 mu^4) on the kx >= 0 half."""
    N = 16
    pos = synthetic.zeldovich_box(12, 1000.0, seed=7)
    los = np.array([0.0, 2.0, 1.0])
    p = dict(grid=N, interpolation=4, interlacing=True, box=1000.0, los=los / (los @ los))
    npart, dcl = O.assign_grid(pos, p)
    d = O.compute_density(npart, dcl, p)
    d2, d4 = O.compute_density_multipoles(d, p)
    f = np.fft.fftfreq(N, 1.0 / N).astype(int)
    f[N // 2] = N // 2
    KX, KY, KZ = np.meshgrid(f, f, f, indexing="ij")
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    lk = p["los"][0] * KX + p["los"][1] * KY + p["los"][2] * KZ
    mu2 = np.where(k2 > 0, lk ** 2 / np.maximum(k2, 1), 0.0)
    L2 = -0.5 + 1.5 * mu2
    L4 = 0.375 - 3.75 * mu2 + 4.375 * mu2 ** 2
    half = slice(0, N // 2 + 1)
    scale = np.max(np.abs(d))
    assert np.max(np.abs(d2[half] - (L2 * d)[half])) < 1e-10 * scale
    assert np.max(np.abs(d4[half] - (L4 * d)[half])) < 1e-10 * scale


def test_triangle_counts_bruteforce():
    """N_tr = #{(q1,q2,q3) in shells i,j,l : q1+q2+q3 = 0 mod N} (FFT identity)."""
    N, nb, kbin, kc = 8, 3, 1.0, 1.0
    counts = O.count_triangles(nb, N, kbin, kc, True, False, 1, O.itot(nb, kbin, kc, True))
    shell = O.shell_index(N, kbin, kc)
    modes = {b: np.argwhere(shell == b) for b in range(1, nb + 1)}
    ishift = 2
    m = 0
    for l in range(1, nb + 1):
        for j in range(1, l + 1):
            for i in range(max(1, l - j + 1 - ishift), j + 1):
                cnt = 0
                Sl = {tuple(x) for x in modes[l]}
                for q1 in modes[i]:
                    for q2 in modes[j]:
                        q3 = tuple((-(q1 + q2)) % N)
                        cnt += q3 in Sl
                assert round(counts[m] / N ** 3) == cnt
                m += 1


def test_uniform_lattice_has_no_power():
    """A particle on every cell centre of a CIC grid: delta is a delta function at k=0."""
    N = 8
    q = (np.arange(N) + 0.0) / N
    pos = np.stack(np.meshgrid(q, q, q, indexing="ij")).reshape(3, -1)
    p = dict(grid=N, interpolation=2, interlacing=False, box=100.0)
    npart, dtl = O.assign_grid(pos, p)
    d = O.compute_density(npart, dtl, p)
    pk = O.measure_pk(N, 100.0, 1.0, 1.0, 4, d, d)
    assert np.all(np.abs(pk[1]) < 1e-20)


def test_catalogue_positions_oracle_wraps_and_clips():
    """The reference's catalogue normalisation (pbi4.py:241-243): periodic wrap into
    [0, box), division by box, and the clip that leaves an exact 1.0 when float
    rounding of (pos + box) % box returns box itself."""
    box = 1000.0
    pos = np.array([[0.0, box, -box], [2 * box, 250.0, -250.0]], dtype=np.float64)
    got = O.catalogue_positions(pos, box=box)
    np.testing.assert_array_equal(got, np.array([[0.0, 0.0], [0.0, 0.25], [0.0, 0.75]]))
    # a float32 position just below zero: (p + box) rounds to box, % box gives 0
    p32 = np.array([[-1e-6, 0.5, 999.9999]], dtype=np.float32)
    g32 = O.catalogue_positions(p32, box=box)
    assert g32.dtype == np.float64 and g32.min() >= 0.0 and g32.max() <= 1.0
    # the RSD shift is float64 arithmetic rounded once to the catalogue dtype
    vel = np.array([[0.0, 0.0, 100.0]], dtype=np.float32)
    shifted = O.catalogue_positions(np.array([[10.0, 10.0, 10.0]], dtype=np.float32), vel, [0.0, 0.0, 1.0], 100.0,
                                    0.0, box=box)
    np.testing.assert_allclose(shifted[:, 0], [0.01, 0.01, 0.011], rtol=1e-6)
