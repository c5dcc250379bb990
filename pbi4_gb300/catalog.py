"""Catalogue positions on the device: the RSD shift, wrap and normalisation of
IO.read_catalogues (pbi4.py:121-245) as one kernel, so a catalogue read into
device memory feeds the assignment without a host round trip.

``positions(pos, vel=None, los=None, hz=None, z=None, box=..., rsd_mode=1)``
takes (N, 3) catalogue positions in Mpc/h (float32 or float64; numpy arrays or
CUDA tensors) and optional velocities of the same shape and dtype, and returns
a CUDA tensor (3, N) float64 in [0, 1]: the same numbers numpy computes in the
reference (the shift in float64 rounded to the catalogue dtype, the wrap and
division in the catalogue dtype, the clip at 1.0).  rsd_mode 1 shifts by
vel * los / hz * (1 + z) (Gadget, Rockstar, Quijote), rsd_mode 0 by vel * los
(Minerva).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib


def positions(pos, vel=None, los=None, hz=None, z=None, box: float = 1000.0, rsd_mode: int = 1, stream=None):
    import torch
    tp = pos if isinstance(pos, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(pos))
    if tp.dim() != 2 or tp.shape[1] != 3 or tp.dtype not in (torch.float32, torch.float64):
        raise ValueError("positions: pos must be (N, 3) float32 or float64")
    tp = tp.cuda().contiguous()
    tv = None
    if vel is not None:
        if los is None or (rsd_mode == 1 and (hz is None or z is None)):
            raise ValueError("positions: an RSD shift needs los (and hz, z for rsd_mode 1)")
        tv = vel if isinstance(vel, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(vel))
        if tuple(tv.shape) != tuple(tp.shape) or tv.dtype != tp.dtype:
            raise ValueError("positions: vel must match pos in shape and dtype")
        tv = tv.cuda().contiguous()
    n = tp.shape[0]
    out = torch.empty((3, n), dtype=torch.float64, device=tp.device)
    l3 = (ctypes.c_double * 3)(*(los if los is not None else (0.0, 0.0, 0.0)))
    st = stream if stream is not None else torch.cuda.current_stream()
    check(lib().pbi4g_catalog_positions(n, ctypes.c_void_p(tp.data_ptr()),
                                        ctypes.c_void_p(tv.data_ptr()) if tv is not None else None,
                                        1 if tp.dtype == torch.float64 else 0, l3, int(rsd_mode),
                                        float(hz if hz is not None else 0.0), float(z if z is not None else 0.0),
                                        float(box), ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.cuda_stream)))
    return out
