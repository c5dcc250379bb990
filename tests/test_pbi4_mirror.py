"""The reference's script flow (Tutorials/Script/test.py) on pbi4_gb300.pbi4.

IO -> DENSITIES.assign_grid -> compute_density -> compute_density_multipoles ->
MEASUREMENTS.powerspectrum / triangle_counts / bispectrum -> save_*, on a small
synthetic box, checked against the FP64 oracle run through the same sequence
(FP32 tolerances of tests/test_gpu_parity.py), plus the density round trip
through save_density / read_density.
"""
import json

import numpy as np
import pytest

from oracle import pbi4_oracle as O
from pbi4_gb300 import synthetic

from ._helpers import b_errors

pytestmark = pytest.mark.gpu


def _config(tmp_path, grid=32):
    cfg = {"cat": "npz", "box": 1000.0, "grid": grid, "interpolation": 4, "interlacing": True, "kbin": 1.0,
           "kcenter": 1.0, "iopen": True, "om": 0.3, "ol": 0.7, "z": 0.5, "multipoles": True,
           "los": [0.0, 0.0, 1.0], "cross": False, "cfile": str(tmp_path / "cfile.npz"), "npool": 4,
           "savedensity": False, "config_file": str(tmp_path / "config.json"), "ifile": str(tmp_path / "cat.npz"),
           "dfile": str(tmp_path / "dens.npz"), "ps_outfile": str(tmp_path / "ps.dat"),
           "bs_outfile": str(tmp_path / "bs.dat")}
    with open(cfg["config_file"], "w") as f:
        json.dump(cfg, f)
    return cfg


def test_script_flow_matches_oracle(tmp_path):
    import pbi4_gb300.pbi4 as pb
    cfg = _config(tmp_path)
    pos_norm = synthetic.zeldovich_box(20, 1000.0, seed=31)
    np.savez(cfg["ifile"], pos=(pos_norm * 1000.0).T)
    io = pb.IO(config_file=cfg["config_file"])
    params = io.read_params()
    params["nbins_bisp"] = 8
    params["itot"] = O.itot(8, 1.0, 1.0, True)
    pos = io.read_catalogues()
    density = pb.DENSITIES(params)
    npart, dcl = density.assign_grid(pos)
    dcl = density.compute_density(npart, dcl)
    dcl2, dcl4 = density.compute_density_multipoles(dcl)
    ms = pb.MEASUREMENTS(params)
    ps = ms.powerspectrum(npart, dcl, dcl2, dcl4)
    counts = ms.triangle_counts()
    bs = ms.bispectrum(npart, counts, dcl, dcl2, dcl4)
    ms.save_powerspectrum(ps)
    ms.save_bispectrum(bs)
    ms.save_triangle_counts(counts)

    # oracle, same sequence
    op = dict(params)
    n, d = O.assign_grid(pos, op)
    d = O.compute_density(n, d, op)
    d2, d4 = O.compute_density_multipoles(d, op)
    ref_ps = O.powerspectrum(n, d, op, d2, d4)
    ref_counts = O.count_triangles(8, 32, 1.0, 1.0, True, False, 1, params["itot"])
    ref_bs = O.bispectrum(n, ref_counts, d, op, d2, d4)
    np.testing.assert_array_equal(ps["Nmodes"], ref_ps["Nmodes"])
    assert np.max(np.abs(ps["P0+PSN"] / ref_ps["P0+PSN"] - 1)) < 1e-5
    assert np.max(np.abs(ps["P2"] - ref_ps["P2"]) / np.abs(ref_ps["P0+PSN"])) < 1e-5
    np.testing.assert_array_equal(np.round(counts / 32 ** 3), np.round(ref_counts / 32 ** 3))
    np.testing.assert_array_equal(bs["Ntr"], ref_bs["Ntr"])
    b = np.array([bs[c] for c in ("k1", "k2", "k3", "Pk1", "Pk2", "Pk3", "B0+BSN", "BSN", "Ntr", "B2", "B4")],
                 dtype=np.float64)
    r = np.array([ref_bs[c] for c in ("k1", "k2", "k3", "Pk1", "Pk2", "Pk3", "B0+BSN", "BSN", "Ntr", "B2", "B4")],
                 dtype=np.float64)
    errs, _ = b_errors(b, r)
    assert max(errs) < 2e-5  # float32 output records on top of the FP32 path
    assert (tmp_path / "ps.dat").exists() and (tmp_path / "bs.dat").exists()
    loaded = np.loadtxt(tmp_path / "ps.dat")
    assert loaded.shape == (params["nbins_ps"], 7)

    # density round trip: save at 32^3, read back reduced to 16^3 (reduce_array on the GPU)
    params["savedensity"] = True
    density.save_density(dcl, npart)
    p16 = dict(params)
    p16["grid"] = 16
    p16.update(io.derived_params(p16))
    npart2, dred = pb.DENSITIES(p16).read_density()
    assert npart2 == npart
    full32 = np.asarray(dcl)
    ref16 = O.reduce_array(32, full32, 16)
    got16 = np.asarray(dred)
    half = slice(0, 9)
    assert np.max(np.abs(got16[half] - ref16[half])) <= 1e-6 * np.max(np.abs(ref16))
