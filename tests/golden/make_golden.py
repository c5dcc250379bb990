"""Extract the input-independent columns of the reference's saved outputs into
a small fixture (tests/golden/reference_testdata_cols.npz).

Source: the reference's Tutorials/testdata/ps.dat and bs.dat (grid 64, box 1000,
kbin = kcenter = 1, iopen = True, multipoles; 32 P bins, 21 B shells, 1156
triangles).  Only columns that do not depend on the (missing) input catalogue
are kept: from ps.dat k, avgk, Nmodes and PSN; from bs.dat k1, k2, k3 and N_tr.

Run from the repository root:
    python tests/golden/make_golden.py REFERENCE_ROOT
(or with the reference's root in the environment variable PBI4_REFERENCE).
"""
import os
import sys

import numpy as np

ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PBI4_REFERENCE")
if not ref:
    sys.exit("usage: make_golden.py REFERENCE_ROOT (or set PBI4_REFERENCE)")
ps = np.loadtxt(os.path.join(ref, "Tutorials", "testdata", "ps.dat"))
bs = np.loadtxt(os.path.join(ref, "Tutorials", "testdata", "bs.dat"))
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_testdata_cols.npz")
np.savez(out,
         ps_k=ps[:, 0].astype(np.float32), ps_avgk=ps[:, 1].astype(np.float32),
         ps_nmodes=ps[:, 5].astype(np.int64), ps_psn=ps[:, 6].astype(np.float32),
         bs_k1=bs[:, 0].astype(np.int32), bs_k2=bs[:, 1].astype(np.int32), bs_k3=bs[:, 2].astype(np.int32),
         bs_ntr=bs[:, 8].astype(np.int64),
         meta=np.array([64, 1000, 1, 1, 32, 21, 1156], dtype=np.int64))
print("wrote", out, "ps rows", len(ps), "bs rows", len(bs))
