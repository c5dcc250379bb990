"""The catalogue step on the device (pbi4_gb300.catalog.positions) against the
reference's numpy operations (oracle.catalogue_positions, pbi4.py:121-245):
bit-identical float64 positions for float32 and float64 catalogues, with and
without the RSD shift, including positions on and beyond the box edges."""
import numpy as np
import pytest

from oracle import pbi4_oracle as O
from pbi4_gb300 import catalog

pytestmark = pytest.mark.gpu


def _catalogue(dtype, n=200_000, box=1000.0, seed=5):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-0.2 * box, 1.2 * box, (n, 3)).astype(dtype)
    # edges: 0, box, just below box, -box, 2 box, tiny negatives
    edge = np.array([0.0, box, np.nextafter(dtype(box), dtype(0)), -box, 2 * box, -1e-7, 1e-7, box / 2],
                    dtype=dtype)
    pos[: edge.size, 0] = edge
    pos[: edge.size, 1] = edge[::-1]
    vel = rng.normal(0.0, 600.0, (n, 3)).astype(dtype)
    return pos, vel


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("rsd", [None, 0, 1])
def test_catalogue_positions_match_reference(dtype, rsd):
    box = 1000.0
    pos, vel = _catalogue(dtype, box=box)
    los, hz, z = [0.0, 0.0, 1.0], 123.45, 0.57
    if rsd is None:
        ref = O.catalogue_positions(pos, box=box)
        got = catalog.positions(pos, box=box)
    else:
        ref = O.catalogue_positions(pos, vel, los, hz, z, box=box, rsd_mode=rsd)
        got = catalog.positions(pos, vel=vel, los=los, hz=hz, z=z, box=box, rsd_mode=rsd)
    got = got.cpu().numpy()
    assert got.shape == ref.shape == (3, pos.shape[0])
    assert ref.dtype == np.float64
    np.testing.assert_array_equal(got, ref)
    assert got.min() >= 0.0 and got.max() <= 1.0


def test_catalogue_positions_oblique_los():
    pos, vel = _catalogue(np.float32, n=50_000, seed=9)
    los = [0.3, -0.4, 0.866]
    ref = O.catalogue_positions(pos, vel, los, 100.0, 1.0, box=1000.0, rsd_mode=1)
    got = catalog.positions(pos, vel=vel, los=los, hz=100.0, z=1.0, box=1000.0).cpu().numpy()
    np.testing.assert_array_equal(got, ref)


def test_catalogue_positions_errors():
    with pytest.raises(ValueError):
        catalog.positions(np.zeros((4, 2)))
    with pytest.raises(ValueError):
        catalog.positions(np.zeros((4, 3)), vel=np.zeros((4, 3)))  # no los
