"""The reference's own pbi4/pbi4.py, unmodified, against this library's drop-ins.

tests/golden/reference_trace.npz was recorded by
tests/golden/make_reference_trace.py: it ran the reference's pbi4.py (its
Tutorials/Script/test.py sequence with a catalogue file, the notebook's
on-the-fly positions in real space, and a cross-spectrum session) with the FP64
oracle standing in for the compiled modules powerI4 / bispectrumI4, and kept
every call pbi4.py made into them (argument types, dtypes, shapes and memory
order, and the arrays), the records its MEASUREMENTS methods returned and the
text its save_* writers produced.

* not gpu: the oracle's driver (oracle/pbi4_oracle.py) reproduces the records of
  the real pbi4.py from the same inputs, and the writers of pbi4_gb300.pbi4
  reproduce the reference's text files byte for byte from its records;
* gpu: every recorded call, with its recorded argument types and layouts, goes
  through pbi4_gb300.powerI4 / bispectrumI4 and is compared with the oracle
  (the output's dtype, shape and Fortran order as f2py returns them), and the
  three sessions run through pbi4_gb300.pbi4 match the reference's records.
"""
import importlib
import json
import os

import numpy as np
import pytest

from oracle import pbi4_oracle as O

from ._helpers import b_errors

TRACE = os.path.join(os.path.dirname(__file__), "golden", "reference_trace.npz")


@pytest.fixture(scope="module")
def trace():
    z = np.load(TRACE)
    return z, json.loads(str(z["calls"]))


def _params(z, session):
    p = json.loads(str(z[f"input_{session}_params"]))
    p["los"] = np.asarray(p["los"], dtype=np.float64)
    p["kvec"] = np.asarray(p["kvec"])
    return p


def _arg(z, a):
    if a["kind"] == "array":
        v = z[a["key"]]
        order = "F" if a["f_contiguous"] and not a["c_contiguous"] else "C"
        v = np.array(v, dtype=np.dtype(a["dtype"]), order=order)
        assert list(v.shape) == a["shape"]
        return v
    t, val = a["type"], a["value"]
    return {"builtins.int": int, "builtins.float": float, "builtins.bool": bool,
            "numpy.float64": np.float64, "numpy.int64": np.int64, "numpy.float32": np.float32,
            "numpy.bool": np.bool_, "numpy.bool_": np.bool_}[t](val)


# ------------------------------------------------------------------ CPU ---
def test_trace_covers_the_call_sequence(trace):
    z, calls = trace
    names = {(c["session"], c["name"]) for c in calls}
    for s, n in [("script", "assign_double_grid"), ("script", "fcomb"), ("script", "compute_q2k"),
                 ("script", "compute_q4k"), ("script", "measure_pk_multipoles"), ("script", "count_triangles"),
                 ("script", "measure_bk_multipoles"), ("realspace", "assign_single_grid"),
                 ("realspace", "measure_pk"), ("realspace", "measure_bk"), ("cross", "measure_pk"),
                 ("cross", "measure_bk_cross")]:
        assert (s, n) in names, (s, n)
    # the reference's script config gives the grid as a float (Tutorials/Script/config.json)
    assert calls[0]["args"][0] == {"kind": "scalar", "type": "builtins.float", "value": 16.0}


def _oracle_session(z, session):
    p = _params(z, session)
    if session == "script":
        pos = O.catalogue_positions(z["input_script_catalogue"], box=p["box"])
        npart, dcl = O.assign_grid(pos, p)
        d = O.compute_density(npart, dcl, p)
        d2, d4 = O.compute_density_multipoles(d, p)
        ps = O.powerspectrum(npart, d, p, d2, d4)
        counts = O.count_triangles(p["nbins_bisp"], p["grid"], p["kbin"], p["kcenter"], p["iopen"], False, 1,
                                   p["itot"])
        bs = O.bispectrum(npart, counts, d, p, d2, d4)
    elif session == "realspace":
        npart, dcl = O.assign_grid(z["input_realspace_pos"], p)
        d = O.compute_density(npart, dcl, p)
        ps = O.powerspectrum(npart, d, p)
        counts = O.count_triangles(p["nbins_bisp"], p["grid"], p["kbin"], p["kcenter"], p["iopen"], False, 1,
                                   p["itot"])
        bs = O.bispectrum(npart, counts, d, p)
    else:
        na, da = O.assign_grid(z["input_cross_pos_a"], p)
        da = O.compute_density(na, da, p)
        nb, db = O.assign_grid(z["input_cross_pos_b"], p)
        db = O.compute_density(nb, db, p)
        ps = O.powerspectrum(na, da, p, dcl2=db)
        counts = O.count_triangles(p["nbins_bisp"], p["grid"], p["kbin"], p["kcenter"], p["iopen"], True, 1,
                                   p["itot"])
        bs = O.bispectrum(na, counts, da, p, dcl2=db)
    return ps, bs


# pbi4.py leaves P2 and P4 of a real-space record unset (np.ndarray, pbi4.py:419)
_UNSET = {"realspace": ("P2", "P4"), "cross": ("P2", "P4"), "script": ()}


@pytest.mark.parametrize("session", ["script", "realspace", "cross"])
def test_oracle_driver_reproduces_reference_records(trace, session):
    z, _ = trace
    ps, bs = _oracle_session(z, session)
    rps, rbs = z[f"record_{session}_ps"], z[f"record_{session}_bs"]
    assert ps.dtype.names == rps.dtype.names and bs.dtype.names == rbs.dtype.names
    for name in ps.dtype.names:
        if name not in _UNSET[session]:
            np.testing.assert_allclose(ps[name], rps[name], rtol=1e-6, err_msg=name)
    for name in bs.dtype.names:
        np.testing.assert_allclose(bs[name], rbs[name], rtol=1e-6, err_msg=name)


@pytest.mark.parametrize("session", ["script", "realspace", "cross"])
def test_writers_match_reference_text(trace, session, tmp_path):
    import pbi4_gb300.pbi4 as pb
    z, _ = trace
    p = _params(z, session)
    p["ps_outfile"], p["bs_outfile"] = str(tmp_path / "ps.dat"), str(tmp_path / "bs.dat")
    ms = pb.MEASUREMENTS(p)
    ms.save_powerspectrum(z[f"record_{session}_ps"])
    ms.save_bispectrum(z[f"record_{session}_bs"])
    assert open(p["ps_outfile"]).read() == str(z[f"text_{session}_ps"])
    assert open(p["bs_outfile"]).read() == str(z[f"text_{session}_bs"])


# ------------------------------------------------------------------ GPU ---
def _compare(name, got, ref, grid):
    if name.startswith("assign"):
        assert np.max(np.abs(got - ref)) <= 1e-11 * np.max(np.abs(ref))
    elif name in ("fcomb", "compute_q2k", "compute_q4k", "reduce_array"):
        assert np.max(np.abs(got - ref)) <= 1e-12 * max(np.max(np.abs(ref)), 1e-300)
    elif name == "measure_pk":
        np.testing.assert_array_equal(got[2], ref[2])
        assert np.max(np.abs(got[:2] - ref[:2]) / np.abs(ref[:2]).max(axis=1, keepdims=True)) < 1e-12
    elif name == "measure_pk_multipoles":
        np.testing.assert_array_equal(got[4], ref[4])
        assert np.max(np.abs(got[:4] - ref[:4]) / np.abs(ref[:4]).max(axis=1, keepdims=True)) < 1e-12
    elif name == "count_triangles":
        np.testing.assert_array_equal(got / float(grid) ** 3, np.round(ref / float(grid) ** 3))
    elif name == "measure_bk_cross":
        np.testing.assert_array_equal(got[[0, 1, 2, 4]], ref[[0, 1, 2, 4]])
        assert np.max(np.abs(got[3] - ref[3])) <= 1e-5 * np.max(np.abs(ref[3]))
    else:   # measure_bk, measure_bk_multipoles in the drop-in's default FP32 form
        np.testing.assert_array_equal(got[[0, 1, 2, 8]], ref[[0, 1, 2, 8]])
        errs, pw = b_errors(got, ref)
        assert max(errs) <= 1e-5 and pw <= 1e-5, (errs, pw)


@pytest.mark.gpu
def test_replay_reference_calls_through_dropins(trace):
    """Every call the unmodified pbi4.py made, replayed with its own argument
    types and layouts through the drop-in modules."""
    z, calls = trace
    mods = {"powerI4": importlib.import_module("pbi4_gb300.powerI4"),
            "bispectrumI4": importlib.import_module("pbi4_gb300.bispectrumI4")}
    for k, c in enumerate(calls):
        args = [_arg(z, a) for a in c["args"]]
        got = getattr(mods[c["module"]], c["name"])(*args)
        ref = getattr(O, c["name"])(*[_arg(z, a) for a in c["args"]])
        rec = c["out"]
        assert got.dtype.str == rec["dtype"] and list(got.shape) == rec["shape"], (k, c["name"])
        assert bool(got.flags.f_contiguous) == rec["f_contiguous"], (k, c["name"])
        grid = args[1] if c["module"] == "bispectrumI4" else args[0]
        _compare(c["name"], got, ref, grid)


@pytest.mark.gpu
@pytest.mark.parametrize("session", ["script", "realspace", "cross"])
def test_mirror_sessions_match_reference_records(trace, session, tmp_path):
    """The same three sessions through pbi4_gb300.pbi4 (the device plan) against
    the records the reference's pbi4.py returned: mode and triangle counts and
    the k columns exact, P and B within the FP32 form's 1e-5."""
    import pbi4_gb300.pbi4 as pb
    z, _ = trace
    p = _params(z, session)
    cfg = {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in p.items()}
    cfg.update(config_file=str(tmp_path / "config.json"), ifile=str(tmp_path / "cat.npz"),
               ps_outfile=str(tmp_path / "ps.dat"), bs_outfile=str(tmp_path / "bs.dat"),
               cfile=str(tmp_path / "absent.npz"))
    with open(cfg["config_file"], "w") as f:
        json.dump(cfg, f)
    io = pb.IO(config_file=cfg["config_file"])
    params = io.read_params()
    density, ms = pb.DENSITIES(params), pb.MEASUREMENTS(params)
    if session == "script":
        np.savez(cfg["ifile"], pos=z["input_script_catalogue"])
        pos = io.read_catalogues()
        npart, dcl = density.assign_grid(pos)
        dcl = density.compute_density(npart, dcl)
        dcl2, dcl4 = density.compute_density_multipoles(dcl)
        ps = ms.powerspectrum(npart, dcl, dcl2, dcl4)
        counts = ms.triangle_counts()
        bs = ms.bispectrum(npart, counts, dcl, dcl2, dcl4)
    elif session == "realspace":
        npart, dcl = density.assign_grid(z["input_realspace_pos"])
        dcl = density.compute_density(npart, dcl)
        ps = ms.powerspectrum(npart, dcl)
        counts = ms.triangle_counts()
        bs = ms.bispectrum(npart, counts, dcl)
    else:
        npart, da = density.assign_grid(z["input_cross_pos_a"])
        da = density.compute_density(npart, da)
        nb, db = density.assign_grid(z["input_cross_pos_b"])
        db = density.compute_density(nb, db)
        ps = ms.powerspectrum(npart, da, db)
        counts = ms.triangle_counts()
        bs = ms.bispectrum(npart, counts, da, db)
    ms.save_powerspectrum(ps)
    ms.save_bispectrum(bs)
    rps, rbs = z[f"record_{session}_ps"], z[f"record_{session}_bs"]
    assert ps.dtype.names == rps.dtype.names and bs.dtype.names == rbs.dtype.names
    np.testing.assert_array_equal(ps["Nmodes"], rps["Nmodes"])
    np.testing.assert_array_equal(ps["k"], rps["k"])
    for name in ("avgk", "P0+PSN", "PSN") + (("P2", "P4") if session == "script" else ()):
        ref = rps[name].astype(np.float64)
        rel = np.abs(ps[name] / ref - 1) if name != "P2" and name != "P4" else \
            np.abs(ps[name] - ref) / np.abs(rps["P0+PSN"])
        assert rel.max() <= 1e-5, (name, rel.max())
    for name in ("k1", "k2", "k3", "Ntr"):
        np.testing.assert_array_equal(bs[name], rbs[name])
    if session == "cross":
        err = np.abs(bs["B0"].astype(np.float64) - rbs["B0"]) / np.max(np.abs(rbs["B0"]))
        assert err.max() <= 1e-5, err.max()
    else:
        for name in ("Pk1", "Pk2", "Pk3", "BSN"):
            ref = rbs[name].astype(np.float64)
            assert np.max(np.abs(bs[name] / ref - 1)) <= 1e-5, name
        # B_l: relative error, or where B_l nearly cancels (|Q_l| < 1) relative to
        # (2l+1)(P1P2 + P1P3 + P2P3) (tests/test_gpu_configs.py states the rule)
        den = np.abs(rbs["Pk1"] * rbs["Pk2"]) + np.abs(rbs["Pk1"] * rbs["Pk3"]) + np.abs(rbs["Pk2"] * rbs["Pk3"])
        for name, f in (("B0+BSN", 1.0),) + ((("B2", 5.0), ("B4", 9.0)) if session == "script" else ()):
            ref = rbs[name].astype(np.float64)
            e = np.abs(bs[name] - ref) / np.maximum(np.abs(ref), f * den.astype(np.float64))
            assert e.max() <= 1e-5, (name, e.max())
