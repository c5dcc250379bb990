"""Run the reference's own, unmodified pbi4/pbi4.py and record every call it
makes into its compiled modules powerI4 / bispectrumI4, for the drop-in tests.

The reference's f2py modules cannot be built here (no Fortran compiler, no FFTW),
so the FP64 oracle (oracle/pbi4_oracle.py, a restatement of
pbi4/F90_modules/*.f90) stands in for them under the module names pbi4.py
imports (pbi4.py:12-14).  `pandas` and `h5py` are imported by pbi4.py:5 and by
its Gadget reader but not used on these paths; empty modules stand in for them.

Three sessions, each the reference's documented call sequence on a 16^3 grid:
  script     Tutorials/Script/test.py:3-15 literally: IO from a JSON config
             (grid given as a float, as in Tutorials/Script/config.json), a
             'sancho' catalogue (float32 positions, read and normalised by
             read_catalogues, pbi4.py:229-243), PCS with interlacing, multipoles,
             triangle counts computed (no cfile), save_powerspectrum/bispectrum;
  realspace  the notebook's on-the-fly positions (Tutorials/Notebook/test.ipynb
             cells 33-34): CIC single grid, no interlacing, real space, closed
             triangles (iopen False);
  cross      two boxes, TSC interlaced, real space, cross power spectrum and
             cross bispectrum (pbi4.py:445-449, 481-497) and the cross writer.

Recorded into tests/golden/reference_trace.npz:
  calls      for every module call: module, function, and for each argument its
             Python type and value (scalars) or dtype, shape and memory order
             with a key into the stored arrays (arrays, deduplicated);
  records    the structured arrays the reference's MEASUREMENTS methods return;
  text       the files its save_powerspectrum / save_bispectrum wrote.

Run from the repository root:
    python tests/golden/make_reference_trace.py REFERENCE_ROOT
(or with the reference's root in the environment variable PBI4_REFERENCE).
"""
import hashlib
import importlib.util
import json
import os
import sys
import tempfile
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pbi4_oracle as O  # noqa: E402

POWER = ["fcomb", "reduce_array", "assign_double_grid", "assign_single_grid", "compute_q2k", "compute_q4k",
         "measure_pk", "measure_pk_multipoles"]
BISPEC = ["measure_bk", "measure_bk_multipoles", "measure_bk_cross", "count_triangles"]


class Recorder:
    def __init__(self):
        self.calls, self.arrays, self.session = [], {}, None

    def _arg(self, a):
        if isinstance(a, np.ndarray):
            h = hashlib.sha1(a.tobytes(order="A") + str((a.dtype.str, a.shape, a.flags.f_contiguous)).encode())
            key = "arr_" + h.hexdigest()[:16]
            self.arrays[key] = np.array(a, copy=True, order="K")
            return {"kind": "array", "key": key, "dtype": a.dtype.str, "shape": list(a.shape),
                    "f_contiguous": bool(a.flags.f_contiguous), "c_contiguous": bool(a.flags.c_contiguous)}
        t = type(a)
        return {"kind": "scalar", "type": f"{t.__module__}.{t.__name__}",
                "value": a.item() if isinstance(a, np.generic) else a}

    def wrap(self, module, name, fn):
        def call(*args, **kwargs):
            if kwargs:
                raise TypeError(f"{name}: keyword arguments are not recorded")
            out = fn(*args)
            self.calls.append({"session": self.session, "module": module, "name": name,
                               "args": [self._arg(a) for a in args],
                               "out": {"dtype": out.dtype.str, "shape": list(out.shape),
                                       "f_contiguous": bool(out.flags.f_contiguous)}})
            return out
        return call


def install_modules(rec):
    for stub in ("pandas", "h5py"):
        sys.modules.setdefault(stub, types.ModuleType(stub))
    for mod, names in (("powerI4", POWER), ("bispectrumI4", BISPEC)):
        m = types.ModuleType(mod)
        for n in names:
            setattr(m, n, rec.wrap(mod, n, getattr(O, n)))
        sys.modules[mod] = m


def load_reference_pbi4(ref_root):
    pkg = os.path.join(ref_root, "pbi4")
    sys.path.insert(0, pkg)   # pbi4.py imports Utils.* relative to its own directory
    spec = importlib.util.spec_from_file_location("pbi4_reference", os.path.join(pkg, "pbi4.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def base_config(tmp, **over):
    cfg = {"cat": "sancho", "box": 1000, "grid": 16.0, "interpolation": 4, "interlacing": True, "kbin": 1.0,
           "kcenter": 1.0, "iopen": True, "om": 0.3, "ol": 0.7, "z": 0.5, "multipoles": True,
           "los": [0.0, 0.0, 1.0], "cross": False, "cfile": os.path.join(tmp, "cfile_absent.npz"), "npool": 4,
           "savedensity": False, "config_file": "config.json", "ifile": os.path.join(tmp, "catalogue.npz"),
           "ps_outfile": os.path.join(tmp, "ps.dat"), "bs_outfile": os.path.join(tmp, "bs.dat")}
    cfg.update(over)
    with open(os.path.join(tmp, "config.json"), "w") as f:
        json.dump(cfg, f, indent=4)
    return cfg


def positions(n, seed, zeldovich):
    from pbi4_gb300 import synthetic
    if zeldovich:
        return synthetic.zeldovich_box(n, 1000.0, n_s=-1.5, rms_disp=20.0, f_growth=0.7, seed=seed)
    return synthetic.uniform_box(n, 1000.0, seed=seed)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PBI4_REFERENCE")
    if not ref:
        sys.exit("usage: make_reference_trace.py REFERENCE_ROOT (or set PBI4_REFERENCE)")
    rec = Recorder()
    install_modules(rec)
    pb = load_reference_pbi4(os.path.abspath(ref))
    records, text, inputs = {}, {}, {}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            # -- script: Tutorials/Script/test.py:3-15 with a sancho catalogue
            rec.session = "script"
            cfg = base_config(tmp)
            cat = (positions(12, 41, True).T * 1000.0).astype(np.float32)   # (N, 3) float32 in Mpc/h
            np.savez(cfg["ifile"], pos=cat)
            inputs["script_catalogue"] = cat
            sys.argv = ["test.py"]
            io = pb.IO(config_file="config.json", verbose=True, scriptmode=True)
            params = io.read_params()
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
            records["script_ps"], records["script_bs"] = ps, bs
            text["script_ps"] = open(cfg["ps_outfile"]).read()
            text["script_bs"] = open(cfg["bs_outfile"]).read()
            inputs["script_params"] = json.dumps(json.load(open("config.json")))

            # -- realspace: on-the-fly positions (notebook cells 33-34), CIC, closed triangles
            rec.session = "realspace"
            base_config(tmp, cat="none", interpolation=2, interlacing=False, multipoles=False, iopen=False,
                        kbin=1.0, kcenter=1.0)
            io = pb.IO(config_file="config.json", verbose=False)
            params = io.read_params()
            p = positions(3000, 42, False)
            inputs["realspace_pos"] = p
            density = pb.DENSITIES(params)
            npart, dcl = density.assign_grid(p)
            dcl = density.compute_density(npart, dcl)
            ms = pb.MEASUREMENTS(params)
            ps = ms.powerspectrum(npart, dcl)
            counts = ms.triangle_counts()
            bs = ms.bispectrum(npart, counts, dcl)
            ms.save_powerspectrum(ps)
            ms.save_bispectrum(bs)
            records["realspace_ps"], records["realspace_bs"] = ps, bs
            text["realspace_ps"] = open(params["ps_outfile"]).read()
            text["realspace_bs"] = open(params["bs_outfile"]).read()
            inputs["realspace_params"] = json.dumps(json.load(open("config.json")))

            # -- cross: two boxes, real space, cross P and cross B
            rec.session = "cross"
            base_config(tmp, cat="none", interpolation=3, interlacing=True, multipoles=False, cross=True,
                        kbin=1.0, kcenter=1.0)
            io = pb.IO(config_file="config.json", verbose=False)
            params = io.read_params()
            pa, pbx = positions(12, 43, True), positions(2500, 44, False)
            inputs["cross_pos_a"], inputs["cross_pos_b"] = pa, pbx
            density = pb.DENSITIES(params)
            na, da = density.assign_grid(pa)
            da = density.compute_density(na, da)
            nbp, db = density.assign_grid(pbx)
            db = density.compute_density(nbp, db)
            ms = pb.MEASUREMENTS(params)
            ps = ms.powerspectrum(na, da, db)
            counts = ms.triangle_counts()
            bs = ms.bispectrum(na, counts, da, db)
            ms.save_powerspectrum(ps)
            ms.save_bispectrum(bs)
            records["cross_ps"], records["cross_bs"] = ps, bs
            text["cross_ps"] = open(params["ps_outfile"]).read()
            text["cross_bs"] = open(params["bs_outfile"]).read()
            inputs["cross_params"] = json.dumps(json.load(open("config.json")))
        finally:
            os.chdir(cwd)

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_trace.npz")
    payload = {"calls": np.array(json.dumps(rec.calls))}
    payload.update(rec.arrays)
    for k, v in records.items():
        payload["record_" + k] = v
    for k, v in text.items():
        payload["text_" + k] = np.array(v)
    for k, v in inputs.items():
        payload["input_" + k] = v if isinstance(v, np.ndarray) else np.array(v)
    np.savez_compressed(out, **payload)
    print("wrote", out, len(rec.calls), "calls,", len(rec.arrays), "arrays,", os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
