"""The reference's Python API (pbi4/pbi4.py) on the device-resident plan.

Same classes, method names, arguments and return values as ``IO``,
``DENSITIES`` and ``MEASUREMENTS`` of pbi4/pbi4.py, so a script such as the
reference's Tutorials/Script/test.py runs with ``import pbi4_gb300.pbi4 as pb``.
Between stages the density stays on the GPU: ``assign_grid`` returns a handle
holding the particles, ``compute_density`` leaves delta(k) resident in the
plan, and ``compute_density_multipoles`` returns handles for delta_2 / delta_4,
which the plan applies per mode (the constant line-of-sight identity stated in
csrc/spectrum.cu) instead of the 22 FFTs of pbi4.py:343-388.  ``np.asarray`` on
a handle materialises the reference-layout array when a caller needs it.

The arithmetic of the triangle sums follows ``params['precision']`` ('fp32'
default, 'fp64', 'fp16split', 'bf16').  Catalogue formats that need external
readers (Gadget, FoF, parquet) are not part of this module; positions from any
source enter through ``assign_grid`` as in the reference's notebook
(Tutorials/Notebook/test.ipynb, cells 33-34).
"""
from __future__ import annotations

import argparse
import json
import os
from json import JSONEncoder
from math import floor

import numpy as np

from .estimator import Estimator, EstimatorConfig

_PLANS: dict = {}


def _plan(params, do_bispectrum=True) -> Estimator:
    cfg = EstimatorConfig.from_params(params, precision=params.get("precision", "fp32"), do_bispectrum=do_bispectrum)
    key = cfg.key()
    if key not in _PLANS:
        _PLANS[key] = Estimator(cfg)
    return _PLANS[key]


class NumpyArrayEncoder(JSONEncoder):
    def default(self, obj):
        if isinstance(obj, np.ndarray):
            return obj.tolist()
        return JSONEncoder.default(self, obj)


class IO:
    """Configuration (pbi4.py:22-245): JSON file + command-line overrides + derived parameters."""

    def __init__(self, config_file=None, verbose=False, scriptmode=False):
        self.verbose = verbose
        self.args = vars(self.parse_arguments()) if scriptmode else {}
        self.config_file = config_file if config_file is not None else self.args["config_file"]
        with open(self.config_file) as f:
            self.params = json.load(f)
        if scriptmode:
            self.params.update({k: v for k, v in self.args.items() if v is not None})
        self.params.update(self.derived_params(self.params))
        if "config_file" in self.params:
            with open(self.params["config_file"], "w") as f:
                json.dump(self.params, f, indent=4, cls=NumpyArrayEncoder)

    def parse_arguments(self):
        p = argparse.ArgumentParser()
        for name, typ in (("config_file", str), ("ifile", str), ("dfile", str), ("ps_outfile", str),
                          ("bs_outfile", str), ("cat", str), ("box", float), ("grid", float),
                          ("interpolation", int), ("kbin", float), ("kcenter", float), ("om", float),
                          ("ol", float), ("z", float), ("cfile", str), ("npool", int), ("precision", str)):
            p.add_argument(f"--{name}", type=typ)
        for name in ("interlacing", "iopen", "multipoles", "cross", "savedensity"):
            p.add_argument(f"--{name}", action=argparse.BooleanOptionalAction)
        p.add_argument("--los", nargs="+", type=float)
        return p.parse_args()

    def read_params(self):
        if self.verbose:
            for k, v in self.params.items():
                print(k, " : ", v)
        return self.params

    def derived_params(self, params=None):
        """pbi4.py:86-119."""
        if params is None:
            params = self.params
        params["los"] = np.array(params["los"])
        d = {"dk": params["kbin"] * 2.0 * np.pi / params["box"],
             "nbins_ps": floor((params["grid"] / 2 + params["kbin"] - params["kcenter"]) / params["kbin"]),
             "nbins_bisp": floor((params["grid"] / 3 + params["kbin"] - params["kcenter"]) / params["kbin"]),
             "kf": 2.0 * np.pi / params["box"],
             "kN": 2 * np.pi / params["box"] * params["grid"] / 2.0,
             "Hz": 100.0 * np.sqrt(params["om"] * (1.0 + params["z"]) ** 3 + params["ol"]),
             "los": params["los"] / (params["los"] @ params["los"])}
        d["kvec"] = np.array([(i - 1) * d["dk"] + params["kcenter"] * 2.0 * np.pi / params["box"]
                              for i in range(1, d["nbins_ps"] + 1)])
        ishift = int(params["kcenter"] / params["kbin"]) + (1 if params["iopen"] else 0)
        itot = 0
        for l in range(1, d["nbins_bisp"] + 1):
            for j in range(1, l + 1):
                imax = min(d["nbins_bisp"], j + l - 1 + ishift) if params.get("cross") else j
                itot += max(0, imax - max(1, l - j + 1 - ishift) + 1)
        d.update({"itot": itot})
        return d

    def read_catalogues(self, params=None, device=False):
        """Positions of a numpy catalogue with a 'pos' field (N, 3) in Mpc/h (the
        npz layout of pbi4.py:235-240) and, optionally, a 'vel' field (N, 3) in km/s
        for the RSD shift along params['los'] when params['multipoles'] is set
        (pos += vel los / Hz (1 + z), pbi4.py:158-159).  The shift, the wrap and the
        normalisation of pbi4.py:241-243 run on the device (pbi4_gb300.catalog);
        returns (3, N) float64 positions, a CUDA tensor with device=True."""
        from .catalog import positions
        if params is None:
            params = self.params
        cat = np.load(params["ifile"])
        pos = np.asarray(cat["pos"])
        vel = None
        if params.get("multipoles") and "vel" in cat.files:
            vel = np.asarray(cat["vel"], dtype=pos.dtype)
        out = positions(pos, vel=vel, los=params.get("los"), hz=params.get("Hz"), z=params.get("z"),
                        box=params["box"], rsd_mode=1)
        return out if device else out.cpu().numpy()


class Density:
    """Device-resident density handle (a stage of DENSITIES).

    A handle made by compute_density refers to the density its plan holds; the
    plan is shared by every box of one configuration, so the handle records the
    plan's density generation and refuses to read a later box's density.  With
    params['cross'] set the handle keeps a host copy of its half spectrum
    instead, so two densities of one configuration can be measured together."""

    def __init__(self, params, npart, pos=None, weight=None, ell=0, plan=None, gen=0, half=None):
        self.params, self.npart, self.pos, self.weight, self.ell, self.plan = params, npart, pos, weight, ell, plan
        self.gen, self.half = gen, half

    def check_current(self):
        if self.half is None and self.plan is not None and getattr(self.plan, "density_gen", 0) != self.gen:
            raise RuntimeError("this density handle is stale: its plan has computed another box's density since "
                               "(set params['cross'] to keep several densities of one configuration)")

    def half_spectrum(self):
        """The kx >= 0 half spectrum [z][y][x] of this density (host array)."""
        if self.half is not None:
            return self.half
        self.check_current()
        return self.plan.delta_half()

    def __array__(self, dtype=None, copy=None):
        p = self.params
        if self.plan is None:  # assigned grid, not yet transformed (powerI4.assign_*)
            from . import powerI4
            w = np.ones(self.npart) if self.weight is None else self.weight
            f = powerI4.assign_double_grid if p["interlacing"] else powerI4.assign_single_grid
            return np.asarray(f(p["grid"], p["interpolation"], self.npart, self.pos, w), dtype=dtype)
        n = int(p["grid"])
        half = self.half_spectrum()                         # [z][y][x], x <= N/2
        full = np.zeros((n, n, n), dtype=np.complex128)      # [x][y][z] (Fortran index order)
        full[: n // 2 + 1] = half.transpose(2, 1, 0)
        neg = (-np.arange(n)) % n
        full[n // 2 + 1:] = np.conj(full[neg][:, neg][:, :, neg])[n // 2 + 1:]
        if self.ell:
            f = np.fft.fftfreq(n, 1.0 / n).astype(int)
            f[n // 2] = n // 2
            KX, KY, KZ = np.meshgrid(f, f, f, indexing="ij")
            k2 = KX ** 2 + KY ** 2 + KZ ** 2
            los = p["los"]
            lk = los[0] * KX + los[1] * KY + los[2] * KZ
            mu2 = np.where(k2 > 0, lk ** 2 / np.maximum(k2, 1), 0.0)
            L = -0.5 + 1.5 * mu2 if self.ell == 2 else 0.375 - 3.75 * mu2 + 4.375 * mu2 ** 2
            full = full * L
        return np.asfortranarray(full if dtype is None else full.astype(dtype))


class DENSITIES:
    """pbi4.py:248-396 on the GPU."""

    def __init__(self, params, verbose=False):
        self.params, self.verbose = params, verbose

    def assign_grid(self, pos, params=None, weight=None):
        """pbi4.py:290-302: returns (npart, handle); the scatter runs in compute_density."""
        params = params or self.params
        npart = len(pos.T)
        return npart, Density(params, npart, np.ascontiguousarray(pos, dtype=np.float64), weight)

    def compute_density(self, npart, dcl, params=None):
        """pbi4.py:304-341: assignment, FFT, interlacing combine and window correction on the GPU."""
        params = params or self.params
        cross = bool(params.get("cross", False))
        plan = _plan(params, do_bispectrum=not cross)
        if not isinstance(dcl, Density) or dcl.pos is None:
            raise TypeError("compute_density takes the handle returned by assign_grid")
        import torch
        dpos = torch.from_numpy(dcl.pos).cuda()
        dw = None if dcl.weight is None else torch.from_numpy(np.ascontiguousarray(dcl.weight, np.float64)).cuda()
        plan.density(npart, dpos, dw)
        torch.cuda.synchronize()
        plan.density_gen = getattr(plan, "density_gen", 0) + 1
        return Density(params, npart, plan=plan, gen=plan.density_gen, half=plan.delta_half() if cross else None)

    def compute_density_multipoles(self, dcl, params=None):
        """pbi4.py:343-388: delta_2, delta_4 as handles (factors applied per mode on the GPU)."""
        params = params or self.params
        return (Density(params, dcl.npart, ell=2, plan=dcl.plan, gen=dcl.gen, half=dcl.half),
                Density(params, dcl.npart, ell=4, plan=dcl.plan, gen=dcl.gen, half=dcl.half))

    def save_density(self, dcl, npart, params=None):
        """pbi4.py:390-396: npz with header [grid, npart, kf, kN] and the full grid."""
        params = params or self.params
        header = np.array([params["grid"], npart, params["kf"], params["kN"]])
        np.savez_compressed(params["dfile"], header=header, data=np.asarray(dcl))

    def read_density(self, params=None):
        """pbi4.py:257-288: load a saved density, reduce it on the GPU when the file's grid is larger."""
        params = params or self.params
        f = np.load(params["dfile"])
        header, data = f["header"], f["data"]
        if header[0] < params["grid"]:
            raise SystemExit("ERROR: Density file has smaller grid size than requested.")
        if header[0] > params["grid"]:
            from . import powerI4
            data = powerI4.reduce_array(int(header[0]), data, int(params["grid"]))
        npart = int(header[1])
        n = int(params["grid"])
        plan = _plan(params)
        half = np.ascontiguousarray(np.asarray(data)[: n // 2 + 1].transpose(2, 1, 0))
        plan.set_delta_half(npart, half)
        return npart, Density(params, npart, plan=plan)


class MEASUREMENTS:
    """pbi4.py:398-594 on the GPU."""

    PS_DTYPE = [("k", np.float32), ("avgk", np.float32), ("P0+PSN", np.float32), ("P2", np.float32),
                ("P4", np.float32), ("Nmodes", np.float32), ("PSN", np.float32)]
    BS_DTYPE = [("k1", np.float32), ("k2", np.float32), ("k3", np.float32), ("Pk1", np.float32),
                ("Pk2", np.float32), ("Pk3", np.float32), ("B0+BSN", np.float32), ("BSN", np.float32),
                ("Ntr", np.float32)]

    def __init__(self, params, verbose=False):
        self.params, self.verbose = params, verbose

    def powerspectrum(self, npart, dcl, dcl2=None, dcl4=None, params=None):
        """pbi4.py:405-461: auto spectra on the plan (which applies the multipole
        factors); with params['cross'] the real-space cross spectrum of dcl and
        dcl2 (pbi4.py:445-449) through powerI4.measure_pk."""
        import torch
        params = params or self.params
        if params.get("cross", False):
            if params["multipoles"]:
                print("ERROR: Cross power spectrum in redshift space not implemented yet!")
                raise SystemExit
            if dcl2 is None:
                print("ERROR: you did not include the second density field")
                raise SystemExit
            from . import powerI4
            pout = powerI4.measure_pk(params["grid"], params["box"], params["kbin"], params["kcenter"],
                                      params["nbins_ps"], np.asarray(dcl), np.asarray(dcl2))
        else:
            dcl.check_current()
            plan = dcl.plan
            pout_d, _ = plan.alloc_outputs()
            plan.powerspectrum(pout_d)
            torch.cuda.synchronize()
            pout = pout_d.cpu().numpy()
        out = np.zeros(len(params["kvec"]), dtype=self.PS_DTYPE)
        out["P0+PSN"] = pout[1]
        if params["multipoles"]:
            out["P2"], out["P4"], out["Nmodes"] = pout[2], pout[3], pout[4]
        else:
            out["Nmodes"] = pout[2]
        out["k"] = params["kvec"]
        out["avgk"] = pout[0]
        out["PSN"] = 1.0 / (npart * (2.0 * np.pi / params["box"]) ** 3)
        return out

    def triangle_counts(self, params=None):
        """pbi4.py:463-476: from the counts file when present, else exact counts on the GPU."""
        params = params or self.params
        cf = params.get("cfile")
        if cf and os.path.exists(cf) and os.path.getsize(cf) > 0:
            return np.load(cf)["counts"]
        if params.get("cross", False):
            from . import bispectrumI4
            return bispectrumI4.count_triangles(params["nbins_bisp"], params["grid"], params["kbin"],
                                                params["kcenter"], params["iopen"], True, params.get("npool", 1),
                                                params["itot"])
        plan = _plan(params)
        n = float(params["grid"])
        return plan.triangle_counts().astype(np.float64) * n ** 3

    CROSS_DTYPE = [("k1", np.float32), ("k2", np.float32), ("k3", np.float32), ("B0", np.float32),
                   ("Ntr", np.float32)]

    def bispectrum(self, npart, counts, dcl, dcl2=None, dcl4=None, params=None):
        """pbi4.py:478-553: auto spectra on the plan; with params['cross'] the cross
        bispectrum of dcl and dcl2 (pbi4.py:481-497) through bispectrumI4.measure_bk_cross."""
        import torch
        params = params or self.params
        if params.get("cross", False):
            from . import bispectrumI4
            bout = bispectrumI4.measure_bk_cross(params["nbins_bisp"], params["grid"], params["kbin"],
                                                 params["kcenter"], params["iopen"], params["kf"],
                                                 params.get("npool", 1), params["itot"], npart, counts,
                                                 np.asarray(dcl), np.asarray(dcl2))
            out = np.zeros(bout.shape[1], dtype=self.CROSS_DTYPE)
            for r, (name, _) in enumerate(self.CROSS_DTYPE):
                out[name] = bout[r]
            return out
        dcl.check_current()
        plan = dcl.plan
        plan.set_counts(np.asarray(counts, dtype=np.float64))
        _, bout_d = plan.alloc_outputs()
        plan.bispectrum(bout_d)
        torch.cuda.synchronize()
        bout = bout_d.cpu().numpy()
        dt = self.BS_DTYPE + ([("B2", np.float32), ("B4", np.float32)] if params["multipoles"] else [])
        out = np.zeros(bout.shape[1], dtype=dt)
        for r, (name, _) in enumerate(dt):
            out[name] = bout[r]
        return out

    def save_powerspectrum(self, pout, params=None):
        """pbi4.py:555-563 (same text format)."""
        params = params or self.params
        header = "k     avgk     P0+PSN      P2      P4     Nmodes    PSN\n"
        np.savetxt(params["ps_outfile"], np.array([pout["k"], pout["avgk"], pout["P0+PSN"], pout["P2"], pout["P4"],
                                                   pout["Nmodes"], pout["PSN"]]).T,
                   fmt=("%0.8e", "%0.8e", "%0.8e", "%0.8e", "%0.8e", "%d", "%0.8e"), header=header)

    def save_triangle_counts(self, counts, params=None):
        """pbi4.py:565-572."""
        params = params or self.params
        np.savez_compressed(params["cfile"], counts=counts)

    def save_bispectrum(self, bout, params=None):
        """pbi4.py:574-594 (same text formats)."""
        params = params or self.params
        if params.get("cross", False):
            header = "k1/kF k2/kF k3/kF      B0          N_tr\n"
            np.savetxt(params["bs_outfile"], np.array([bout["k1"], bout["k2"], bout["k3"], bout["B0"], bout["Ntr"]]).T,
                       fmt=("%d", "%d", "%d", "%0.8e", "%0.8e"), header=header)
            return
        if params["multipoles"]:
            header = "k1/kF k2/kF k3/kF P(k1) P(k2)       P(k3)       B0+BSN        BSN    N_tr    B2      B4\n"
            cols = ["k1", "k2", "k3", "Pk1", "Pk2", "Pk3", "B0+BSN", "BSN", "Ntr", "B2", "B4"]
        else:
            header = "k1/kF k2/kF k3/kF P(k1) P(k2)       P(k3)       B0+BSN        BSN    N_tr\n"
            cols = ["k1", "k2", "k3", "Pk1", "Pk2", "Pk3", "B0+BSN", "BSN", "Ntr"]
        fmt = ("%d", "%d", "%d") + ("%0.8e",) * (len(cols) - 3)
        np.savetxt(params["bs_outfile"], np.array([bout[c] for c in cols]).T, fmt=fmt, header=header)
