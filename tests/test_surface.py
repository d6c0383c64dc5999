"""Self-affine rough surfaces: the oracle's properties (CPU) and the GPU
generator against the oracle."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import gfmd_pkg, rel_l2

_spec = importlib.util.spec_from_file_location(
    "rough_surface_oracle",
    os.path.join(os.path.dirname(__file__), "..", "oracle", "rough_surface.py"))
rs = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(rs)

CASES = [(64, 64, 0.8, 0.1, 4.0, 32.0, 7), (96, 75, 0.7, 0.2, 3.0, 48.0, 11),
         (75, 96, 0.5, 0.05, 2.5, 37.5, 3), (384, 384, 0.8, 0.1, 4.0, 192.0, 20261203)]


def _spectral_slope(h, nx, ny, lattice=1.0):
    z = np.fft.rfft2(h.reshape(nx, ny)) / (nx * ny)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny // 2 + 1), indexing="ij")
    kx = np.where(i <= nx // 2, i, i - nx)
    q2 = (2 * np.pi / (nx * lattice) * kx) ** 2 + (2 * np.pi / (ny * lattice) * j) ** 2
    w = np.where((j == 0) | ((ny % 2 == 0) & (j == ny // 2)), 1.0, 2.0)
    return np.sqrt((w * q2 * np.abs(z) ** 2).sum())


@pytest.mark.parametrize("case", CASES)
def test_oracle_surface_has_requested_slope_and_spectrum(case):
    nx, ny, H, slope, ls, ll, seed = case
    h = rs.rough_surface(nx, ny, H, slope, ls, ll, seed)
    assert abs(_spectral_slope(h, nx, ny) - slope) <= 1e-12 * slope
    assert abs(h.mean()) <= 1e-12 * np.abs(h).max()  # q = 0 excluded
    # the synthesised half spectrum is exactly that of the real field (the
    # ky = 0 and Nyquist columns are Hermitian)
    z, s = rs.spectrum(nx, ny, H, ls, ll, seed)
    back = np.fft.rfft2(h.reshape(nx, ny)) / (nx * ny) / (slope / np.sqrt(s))
    assert np.linalg.norm(back - z) <= 1e-12 * np.linalg.norm(z)


def test_oracle_surface_power_law():
    nx = ny = 512
    h = rs.rough_surface(nx, ny, 0.8, 0.1, 4.0, 256.0, 5)
    z = np.abs(np.fft.rfft2(h.reshape(nx, ny))) ** 2
    # |Z|^2 along the ky = 0 axis follows q^(-2-2H) inside the band
    k = np.arange(4, 100)
    slope = np.polyfit(np.log(k), np.log(z[k, 0]), 1)[0]
    assert abs(slope - (-2 - 2 * 0.8)) < 1e-9


def test_oracle_surface_seed_dependence():
    a = rs.rough_surface(64, 64, 0.8, 0.1, 4.0, 32.0, 1)
    b = rs.rough_surface(64, 64, 0.8, 0.1, 4.0, 32.0, 1)
    c = rs.rough_surface(64, 64, 0.8, 0.1, 4.0, 32.0, 2)
    assert np.array_equal(a, b)
    assert rel_l2(a, c) > 0.5


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES + [(2048, 2048, 0.8, 0.1, 4.0, 1024.0, 99)])
def test_gpu_surface_matches_oracle(case):
    torch = pytest.importorskip("torch")
    nx, ny, H, slope, ls, ll, seed = case
    g = gfmd_pkg()
    out = torch.empty(nx * ny, dtype=torch.float64, device="cuda")
    g.rough_surface(out, nx, ny, H, slope, ls, ll, seed)
    ref = rs.rough_surface(nx, ny, H, slope, ls, ll, seed)
    assert rel_l2(out.cpu().numpy(), ref) <= 1e-12


@pytest.mark.gpu
def test_gpu_surface_rejects_bad_parameters():
    torch = pytest.importorskip("torch")
    g = gfmd_pkg()
    out = torch.empty(64 * 64, dtype=torch.float64, device="cuda")
    with pytest.raises(g.GFMDError) as ei:
        g.rough_surface(out, 64, 64, 0.8, -0.1, 4.0, 32.0, 1)
    assert ei.value.code == 1
