"""The oracle restatement, pinned against the reference's own outputs.

The golden fixtures hold forces, energies and u(q=0) of the reference's
unmodified GFMDSolverStatic::post_force (see tests/golden/make_golden.py).
"""
import glob
import os

import numpy as np
import pytest

from conftest import (golden_cases, gfmd_pkg, kernel_for, half_to_full, load_golden, oracle,
                      oracle_post_force, oracle_post_force_half, rel_l2)


@pytest.mark.parametrize("nx,ny", [(8, 8), (12, 10), (37, 64), (64, 37), (30, 7), (1, 16), (16, 1)])
def test_oracle_fft_matches_numpy(nx, ny):
    rng = np.random.default_rng(nx * 1000 + ny)
    x = rng.normal(size=(nx, ny)) + 1j * rng.normal(size=(nx, ny))
    a = x.copy()
    assert oracle().orc_fft2d(a.ctypes.data, nx, ny, 1, 0) == 0
    b = x.copy()
    assert oracle().orc_fft2d(b.ctypes.data, nx, ny, -1, 0) == 0
    assert np.abs(a - np.fft.fft2(x)).max() <= 1e-12 * np.abs(x).sum() ** 0.5 * 10
    assert np.abs(b - np.fft.ifft2(x) * nx * ny).max() <= 1e-12 * np.abs(x).sum() ** 0.5 * 10


def test_oracle_fft_matches_direct_dft():
    nx, ny = 6, 10
    rng = np.random.default_rng(3)
    x = rng.normal(size=(nx, ny)) + 1j * rng.normal(size=(nx, ny))
    ix = np.arange(nx)[:, None]
    iy = np.arange(ny)[None, :]
    direct = np.zeros_like(x)
    for kx in range(nx):
        for ky in range(ny):
            direct[kx, ky] = np.sum(x * np.exp(-2j * np.pi * (kx * ix / nx + ky * iy / ny)))
    a = x.copy()
    oracle().orc_fft2d(a.ctypes.data, nx, ny, 1, 1)
    assert np.abs(a - direct).max() < 1e-12


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_fixture(path):
    c = load_golden(path)
    nx, ny = int(c["nx"]), int(c["ny"])
    if "phi" in c:
        phi = c["phi"]
    else:
        k = kernel_for(c)
        phi, _ = k.phi_table(nx, ny, "full")
    f, e, u0 = oracle_post_force(phi, c["linf"], c["u"], nx, ny)
    assert rel_l2(f, c["f"]) <= 1e-12
    assert abs(e - float(c["epot"])) <= 1e-12 * abs(float(c["epot"]))
    assert np.allclose(u0, c["u0"], rtol=1e-12, atol=1e-15)


def test_energy_identity_without_linf():
    # E = -1/2 sum u.f when the gamma-point force is zero (observed ~1e-16)
    c = load_golden(os.path.join(os.path.dirname(__file__), "golden", "fcc100x4_h64_8x8.npz"))
    e = float(c["epot"])
    assert abs(e + 0.5 * np.sum(c["u"] * c["f"])) <= 1e-13 * abs(e)


def test_half_table_expands_to_reference_table():
    c = load_golden(os.path.join(os.path.dirname(__file__), "golden", "fcc100x2_h64_12x10.npz"))
    nx, ny = int(c["nx"]), int(c["ny"])
    k = kernel_for(c)
    half, _ = k.phi_table(nx, ny, "half")
    full = half_to_full(half, nx, ny)
    assert np.abs(full - c["phi"]).max() <= 1e-13 * np.abs(c["phi"]).max()


def prec_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "prec", "*.npz")))


@pytest.mark.parametrize("path", prec_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_prec_gradient_matches_reference_fixture(path):
    # the fixtures hold the reference's own GFMDSolverStatic::prec_gradient
    # output (tests/golden/make_golden.py), including its ndof > 3 behaviour
    from solver_cases import osv

    c = load_golden(path)
    nx, ny = int(c["nx"]), int(c["ny"])
    full, _ = kernel_for(c).phi_table(nx, ny, "full")
    gP = osv.prec_gradient(full, c["cavg"], c["g"], nx, ny)
    assert rel_l2(gP, c["gP"]) <= 1e-12


def test_oracle_bicubic_map_matches_reference_table2d():
    # the reference's Table2D (as FixWallMap builds it) at random points of a
    # periodic 17 x 13 map, fixture from its own code (tests/golden/make_golden.py).
    # Its six-output eval never accumulates d2f/dy2 (table2d.cpp:229-262 leave
    # it at 0; only FixWallMap's curvature diagnostics read it), so the
    # restatement's d2f/dy2 is checked against a finite difference instead.
    from solver_cases import osv

    c = load_golden(os.path.join(os.path.dirname(__file__), "golden", "maps", "table2d_17x13.npz"))
    mine = np.stack(osv.map_bicubic(c["z"], c["x"], c["y"]), 1)
    for k in (0, 1, 2, 3, 5):
        assert np.abs(mine[:, k] - c["out"][:, k]).max() <= 1e-12
    assert np.all(c["out"][:, 4] == 0.0)
    h = 1e-4
    fp = osv.map_bicubic(c["z"], c["x"], c["y"] + h)[2]
    fm = osv.map_bicubic(c["z"], c["x"], c["y"] - h)[2]
    inside = np.abs(c["y"] - np.round(c["y"])) > 2 * h  # one cell on both sides
    assert np.abs((fp - fm)[inside] / (2 * h) - mine[inside, 4]).max() <= 1e-6
    # the table reproduces the map at the grid points
    assert np.abs(mine[:8, 0] - c["z"][c["x"][:8].astype(int), c["y"][:8].astype(int)]).max() <= 1e-14


@pytest.mark.parametrize("nx,ny", [(12, 10), (9, 7), (16, 5)])
def test_oracle_half_table_entry_equals_full_table_entry(nx, ny):
    # orc_post_force_half reads ky > ny/2 as conj Phi(-q); on the expanded
    # table orc_post_force must give the same forces, energy and u(q=0)
    k = gfmd_pkg().StiffnessKernel("ft fcc100 1.0 2 pair-potential 1 1.0 height 64")
    d = k.get_dimension()
    half, linf = k.phi_table(nx, ny, "half")
    u = np.random.default_rng(nx * ny).normal(0.0, 0.01, (d, nx * ny))
    fa, ea, ua = oracle_post_force(half_to_full(half, nx, ny), linf, u, nx, ny)
    fb, eb, ub = oracle_post_force_half(half, linf, u, nx, ny)
    assert rel_l2(fb, fa) <= 1e-14 and abs(ea - eb) <= 1e-14 * abs(ea)
    assert np.array_equal(ua, ub)


def test_oracle_synthetic_table_is_hermitian_and_mirror_conjugate():
    nx, ny, d = 6, 5, 6
    full = np.empty((nx * ny, d, d), np.complex128)
    oracle().orc_synthetic_phi_full(nx, ny, d, 99, 1e-3, full.ctypes.data, 0)
    again = np.empty_like(full)
    oracle().orc_synthetic_phi_full(nx, ny, d, 99, 1e-3, again.ctypes.data, 1)
    assert np.array_equal(full, again)  # independent of the thread count
    assert np.allclose(full, np.conj(np.transpose(full, (0, 2, 1))), rtol=0, atol=0)
    t = full.reshape(nx, ny, d, d)
    mirror = t[(-np.arange(nx)) % nx][:, (-np.arange(ny)) % ny]
    assert np.array_equal(t, np.conj(mirror))
    # the forces of a real field are real, as with a physical table
    u = np.random.default_rng(1).normal(0.0, 0.01, (d, nx * ny))
    f, e, _ = oracle_post_force(full, None, u, nx, ny)
    assert np.isfinite(f).all() and e > 0
