"""Shared helpers of the parity tests: oracle pipelines and error metrics."""
import numpy as np

from oracle import pbi4_oracle as O


def ref_params(grid, box, nintp, interlacing, multipoles, kbin=1.0, kcenter=1.0, iopen=True, los=(0.0, 0.0, 1.0),
               cross=False):
    p = dict(grid=grid, box=box, interpolation=nintp, interlacing=interlacing, multipoles=multipoles, kbin=kbin,
             kcenter=kcenter, iopen=iopen, los=list(los), cross=cross, om=0.3, ol=0.7, z=0.5, npool=1)
    p.update(O.derived_params(p))
    return p


def oracle_density(pos, p, multipoles_literal=True):
    """pbi4.py call sequence on the oracle: assign_grid -> compute_density (-> multipoles)."""
    npart, dcl = O.assign_grid(pos, p)
    d = O.compute_density(npart, dcl, p)
    d2 = d4 = None
    if p["multipoles"]:
        d2, d4 = O.compute_density_multipoles(d, p)
    return npart, d, d2, d4


def p_errors(pout, ref, multipoles):
    """Max relative error of P0 and, for l = 2, 4, the error relative to P0."""
    co = ref[4] if multipoles else ref[2]
    ok = co > 0
    e0 = np.max(np.abs(pout[1][ok] / ref[1][ok] - 1))
    if not multipoles:
        return e0, 0.0, 0.0
    e2 = np.max(np.abs(pout[2][ok] - ref[2][ok]) / np.abs(ref[1][ok]))
    e4 = np.max(np.abs(pout[3][ok] - ref[3][ok]) / np.abs(ref[1][ok]))
    return e0, e2, e4


def b_errors(bout, ref, rows=(6, 9, 10)):
    """Per-triangle error of B_l: |dB| / max(|B_ref|, (2l+1)(P1 P2 + P1 P3 + P2 P3)), i.e. the
    relative error of B, or, where B itself is near zero, the error of the reduced
    bispectrum Q = B / (P1 P2 + P1 P3 + P2 P3) (with the (2l+1) prefactor that
    measure_bk_multipoles puts on B2 and B4, bispectrumI4.f90:499-500).
    Also returns the plain relative error of the powers of the shells."""
    P1, P2, P3 = ref[3], ref[4], ref[5]
    den = np.abs(P1 * P2) + np.abs(P1 * P3) + np.abs(P2 * P3)
    out = []
    for r in rows:
        if r >= ref.shape[0]:
            continue
        ell_fac = {6: 1.0, 9: 5.0, 10: 9.0}[r]
        out.append(np.max(np.abs(bout[r] - ref[r]) / np.maximum(np.abs(ref[r]), ell_fac * den)))
    pw = np.max(np.abs(bout[3:6] / ref[3:6] - 1))
    return out, pw
