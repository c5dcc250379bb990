"""Seeded synthetic particle boxes (stand-ins for the reference's catalogues).

Positions come out exactly as ``IO.read_catalogues`` leaves them
(pbi4.py:241-243): shape (3, npart) float64, wrapped into the box and divided
by its size, clipped below 1.
"""
from __future__ import annotations

import numpy as np


def normalise(pos_mpc: np.ndarray, box: float) -> np.ndarray:
    """pbi4.py:242-243 on a (3, npart) array in Mpc/h."""
    pos = (pos_mpc + box) % box
    return np.minimum(1.0 - np.nextafter(0, 1), pos / box)


def uniform_box(npart: int, box: float = 1000.0, seed: int = 1) -> np.ndarray:
    """npart positions uniform i.i.d. in float32 (then float64), as the 64^3 CIC workload."""
    rng = np.random.default_rng(seed)
    p = rng.random((3, npart), dtype=np.float32).astype(np.float64) * box
    return normalise(p, box)


def zeldovich_box(nside: int, box: float, n_s: float = -1.5, rms_disp: float = 5.0, f_growth: float = 0.7,
                  los: int = 2, seed: int = 2, rsd: bool = True) -> np.ndarray:
    """nside^3 particles on a lattice displaced by the Zel'dovich approximation.

    psi(k) = i k / k^2 delta(k) for a Gaussian field with P(k) ~ k^n_s, scaled
    so the rms displacement is rms_disp [Mpc/h].  Redshift space: the LOS
    component of the displacement is multiplied by (1 + f).
    """
    rng = np.random.default_rng(seed)
    n = nside
    kf = 2 * np.pi / box
    kx = np.fft.fftfreq(n, 1.0 / n) * kf
    kz = np.fft.rfftfreq(n, 1.0 / n) * kf
    KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    k2[0, 0, 0] = 1.0
    amp = np.sqrt(k2 ** (n_s / 2.0))
    amp[0, 0, 0] = 0.0
    white = np.fft.rfftn(rng.standard_normal((n, n, n)))
    dk = white * amp
    psi = []
    for K in (KX, KY, KZ):
        psi.append(np.fft.irfftn(1j * K / k2 * dk, s=(n, n, n)))
    psi = np.stack(psi)
    psi *= rms_disp / np.sqrt(np.mean(np.sum(psi ** 2, axis=0)))
    if rsd:
        psi[los] *= 1.0 + f_growth
    q = (np.arange(n) + 0.5) * (box / n)
    Q = np.stack(np.meshgrid(q, q, q, indexing="ij"))
    pos = (Q + psi).reshape(3, -1)
    return normalise(pos, box)


def zeldovich_box_device(nside: int, box: float, n_s: float = -1.5, rms_disp: float = 5.0, f_growth: float = 0.7,
                         los: int = 2, seed: int = 2, rsd: bool = True, device: str = "cuda"):
    """zeldovich_box generated with torch on `device` (for lattices whose numpy
    FFTs would take minutes): the same field statistics and construction from a
    torch random stream, so not the same particles as zeldovich_box(seed).
    Returns a (3, nside^3) float64 tensor on the device."""
    import torch

    n = nside
    f64 = torch.float64
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    kf = 2 * np.pi / box
    kx = torch.fft.fftfreq(n, 1.0 / n, dtype=f64, device=device) * kf
    kz = torch.fft.rfftfreq(n, 1.0 / n, dtype=f64, device=device) * kf
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    k2[0, 0, 0] = 1.0
    amp = k2 ** (n_s / 4.0)
    amp[0, 0, 0] = 0.0
    dk = torch.fft.rfftn(torch.randn((n, n, n), generator=g, dtype=f64, device=device)) * amp
    del amp
    dk /= k2
    del k2
    pos = torch.empty((3, n, n, n), dtype=f64, device=device)
    for a, K in enumerate((kx[:, None, None], kx[None, :, None], kz[None, None, :])):
        pos[a] = torch.fft.irfftn(1j * K * dk, s=(n, n, n))
    del dk
    pos *= rms_disp / torch.sqrt(torch.mean(torch.sum(pos ** 2, dim=0)))
    if rsd:
        pos[los] *= 1.0 + f_growth
    q = (torch.arange(n, dtype=f64, device=device) + 0.5) * (box / n)
    pos[0] += q[:, None, None]
    pos[1] += q[None, :, None]
    pos[2] += q[None, None, :]
    pos = pos.reshape(3, -1)
    # pbi4.py:242-243
    pos = torch.remainder(pos + box, box) / box
    return torch.clamp_max(pos, 1.0 - float(np.nextafter(0, 1)))
