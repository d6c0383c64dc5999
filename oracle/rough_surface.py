"""ORACLE — test infrastructure, not product code.

numpy restatement of the random-phase self-affine surface synthesis of
gfmd_rough_surface (include/gfmd_gb300.h, user-gfmd_gb300/csrc/gfmd_surface.cu).
The reference has no generator (it reads maps, src/extras/fix_wall_map.cpp:
1123-1190); this restates the published method: a power spectrum
C(q) ~ q^(-2-2H) between the cut-offs, random phases, and an inverse real
FFT (numpy.fft.irfft2, pocketfft), scaled to the spectral rms slope.
Only tests/ import this module.
"""
from __future__ import annotations

import numpy as np

_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def mix64(z):
    """SplitMix64 output function (Steele, Lea and Flood 2014) on uint64."""
    z = (z + np.uint64(0x9E3779B97F4A7C15)) & _M
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M
    return z ^ (z >> np.uint64(31))


def uniform(seed, i, j, nyc):
    key = i.astype(np.uint64) * np.uint64(nyc) + j.astype(np.uint64)
    z = mix64(np.uint64(seed) ^ mix64(key))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def spectrum(nx, ny, hurst, lambda_short, lambda_long, seed, lattice=1.0):
    """Half spectrum Z[nx, ny//2+1] (unscaled) and sum w |q|^2 |Z|^2."""
    nyc = ny // 2 + 1
    i, j = np.meshgrid(np.arange(nx), np.arange(nyc), indexing="ij")
    kx = np.where(i <= nx // 2, i, i - nx)
    qx = 2 * np.pi / (nx * lattice) * kx
    qy = 2 * np.pi / (ny * lattice) * j
    q2 = qx * qx + qy * qy
    ql2 = (2 * np.pi / lambda_long) ** 2
    qs2 = (2 * np.pi / lambda_short) ** 2
    ok = (q2 > 0) & (q2 >= ql2) & (q2 <= qs2)
    amp = np.zeros_like(q2)
    amp[ok] = np.sqrt((q2[ok] / ql2) ** (-(1.0 + hurst)))
    herm = (j == 0) | ((ny % 2 == 0) & (j == ny // 2))
    ii = np.where(i == 0, 0, np.minimum(i, nx - i))
    u = np.where(herm, uniform(seed, ii, j, nyc), uniform(seed, i, j, nyc))
    z = amp * np.exp(2j * np.pi * u)
    conj = herm & (i != ii)
    z = np.where(conj, np.conj(z), z)
    selfc = herm & ((i == 0) | (2 * i == nx))
    z = np.where(selfc, np.where(u < 0.5, amp, -amp) + 0j, z)
    w = np.where(herm, 1.0, 2.0)
    return z, float((w * q2 * amp * amp).sum())


def rough_surface(nx, ny, hurst, rms_slope, lambda_short, lambda_long, seed, lattice=1.0):
    z, s = spectrum(nx, ny, hurst, lambda_short, lambda_long, seed, lattice)
    h = np.fft.irfft2(z, s=(nx, ny)) * (nx * ny)
    return h.ravel() * (rms_slope / np.sqrt(s))
