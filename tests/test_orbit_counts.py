"""The identity the triangle counts use: a sum over the grid of products of
shell indicator maps equals the sum over the cube group's orbit
representatives (a <= b <= c in [0, Nm/2]) weighted by the orbit sizes.
Checked on small grids with numpy FFTs (the counts themselves are checked on
the GPU against the oracle's counts)."""
import numpy as np
import pytest


def orbit_reps(nm):
    h = nm // 2
    reps, w = [], []
    for a in range(h + 1):
        for b in range(a, h + 1):
            for c in range(b, h + 1):
                sg = np.prod([1 if v in (0, h) else 2 for v in (a, b, c)])
                pm = 1 if a == b == c else (3 if (a == b or b == c) else 6)
                reps.append((a, b, c))
                w.append(sg * pm)
    return np.array(reps), np.array(w, dtype=np.float64)


def shell_maps(nm, edges):
    f = np.fft.fftfreq(nm, 1.0 / nm)
    k = np.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + f[None, None, :] ** 2)
    return [np.fft.ifftn(((k >= lo) & (k < hi)).astype(np.float64)).real * nm ** 3 for lo, hi in edges]


@pytest.mark.parametrize("nm", [12, 16, 20, 24])
def test_orbit_weights_cover_the_grid(nm):
    _, w = orbit_reps(nm)
    assert w.sum() == nm ** 3


@pytest.mark.parametrize("nm", [16, 20, 24])
def test_orbit_sum_equals_grid_sum(nm):
    kmax = (nm - 1) // 3
    edges = [(lo, lo + 1.5) for lo in np.arange(0.5, kmax - 1.0, 1.5)]
    maps = shell_maps(nm, edges)
    reps, w = orbit_reps(nm)
    for l in range(len(maps)):
        for j in range(l + 1):
            for i in range(j + 1):
                full = np.sum(maps[l] * maps[j] * maps[i])
                red = np.sum(w * maps[l][tuple(reps.T)] * maps[j][tuple(reps.T)] * maps[i][tuple(reps.T)])
                assert abs(full - red) / nm ** 3 < 1e-6  # in triangle counts
                # an exact triangle count times Nm^3
                assert abs(full / nm ** 3 - round(full / nm ** 3)) < 1e-6
