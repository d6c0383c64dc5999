"""The surface Green's function of the `nonperiodic` style (host producer,
StiffnessKernel::nonperiodic_green: displacement of an isotropic half-space
under a unit force spread over one grid cell, closed-form corner sums),
checked the way the reference's unit tests check its cell solution
(src/unittests/test_pohrt_li.cpp, test_li_berger.cpp: symmetry, rotational
and scale invariance, no NaNs, Boussinesq-Cerruti at large distances), plus
Betti reciprocity and mirror symmetry.  G[a][b] is displacement a under force
b.  A small C++ driver (tests/green_values.cpp) prints the values; no GPU."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
CSRC = os.path.join(ROOT, "user-gfmd_gb300", "csrc")
NU, MU = 0.3, 1.0
KERNEL = f"nonperiodic {NU} {MU}"


@pytest.fixture(scope="module")
def green(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("green") / "green_values")
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "green_values.cpp"),
                    os.path.join(CSRC, "stiffness.cpp"), "-lpthread", "-o", exe], check=True)

    def G(pairs, dx=1.0, dy=1.0):
        inp = "".join(f"{i} {j}\n" for i, j in pairs)
        out = subprocess.run([exe, KERNEL, repr(dx), repr(dy)], input=inp, check=True, capture_output=True,
                             text=True).stdout
        return np.array([ln.split() for ln in out.splitlines()], float).reshape(-1, 3, 3)
    return G


def _offsets(rng, n, span=12):
    return [tuple(int(v) for v in rng.integers(-span, span + 1, 2)) for _ in range(n)]


def test_finite_everywhere(green):
    pairs = [(i, j) for i in range(-6, 7) for j in range(-6, 7)]
    assert np.isfinite(green(pairs)).all()


def test_symmetry_of_the_cell_solution(green):
    # u_x under Q_y = u_y under Q_x; u_z under Q = -(u_Q under P) (the
    # reference's check_square_solution_symmetry)
    G = green(_offsets(np.random.default_rng(1), 100))
    assert np.allclose(G[:, 0, 1], G[:, 1, 0], rtol=0, atol=1e-15)
    assert np.allclose(G[:, 2, 0], -G[:, 0, 2], rtol=0, atol=1e-15)
    assert np.allclose(G[:, 2, 1], -G[:, 1, 2], rtol=0, atol=1e-15)


def test_rotation_by_quarter_turns(green):
    # a square cell: G(R r) = R G(r) R^T for rotations by 90 degrees about z
    pairs = _offsets(np.random.default_rng(2), 60)
    R = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    G0 = green(pairs)
    rot = pairs
    Rk = np.eye(3)
    for _ in range(3):
        rot = [(-j, i) for i, j in rot]
        Rk = R @ Rk
        G1 = green(rot)
        want = np.einsum("ab,nbc,dc->nad", Rk, G0, Rk)
        assert np.allclose(G1, want, rtol=1e-12, atol=1e-14 * np.abs(G0).max())


def test_mirror_and_reciprocity(green):
    pairs = _offsets(np.random.default_rng(3), 60)
    G0 = green(pairs, 1.0, 0.7)
    M = np.diag([-1.0, 1.0, 1.0])
    Gm = green([(-i, j) for i, j in pairs], 1.0, 0.7)
    assert np.allclose(Gm, M @ G0 @ M, rtol=1e-12, atol=1e-14 * np.abs(G0).max())
    # Betti: the displacement a at r under force b equals b at -r under a
    Gr = green([(-i, -j) for i, j in pairs], 1.0, 0.7)
    assert np.allclose(G0, np.transpose(Gr, (0, 2, 1)), rtol=1e-12, atol=1e-14 * np.abs(G0).max())


def test_scale_invariance(green):
    # unit total force: a cell and an offset scaled by f give G / f (the
    # reference's square_solution_is_scale_invariant, per unit force)
    pairs = _offsets(np.random.default_rng(4), 40)
    G0 = green(pairs, 1.0, 0.6)
    for f in (0.25, 3.0, 17.0):
        assert np.allclose(green(pairs, f, 0.6 * f), G0 / f, rtol=1e-12, atol=1e-14 * np.abs(G0).max() / f)


def test_far_field_is_boussinesq_cerruti(green):
    # at distances r >> cell size the cell solution is the point-force one:
    # normal force P (away from the solid): u_x = c x/r^2, u_y = c y/r^2,
    # u_z = (1 - nu)/(2 pi mu r); tangential force Q_x: u_x = ((1 - nu)/r +
    # nu x^2/r^3)/(2 pi mu), u_y = nu x y/(2 pi mu r^3), u_z = -c x/r^2,
    # c = (1 - 2 nu)/(4 pi mu); the difference is O((h/r)^2), h = 1
    pairs = [(40, 25), (-60, 10), (5, -70), (-35, -45)]
    G = green(pairs, 1.0, 1.0)
    c = (1 - 2 * NU) / (4 * np.pi * MU)
    k = 1.0 / (2 * np.pi * MU)
    for (i, j), g in zip(pairs, G):
        x, y = float(i), float(j)
        r = np.hypot(x, y)
        P = np.array([c * x / r**2, c * y / r**2, (1 - NU) * k / r])
        Qx = np.array([k * ((1 - NU) / r + NU * x * x / r**3), k * NU * x * y / r**3, -c * x / r**2])
        Qy = np.array([k * NU * x * y / r**3, k * ((1 - NU) / r + NU * y * y / r**3), -c * y / r**2])
        want = np.stack([Qx, Qy, P], axis=1)  # columns: force x, y, z
        # measured: 0.045-0.054 (h/r)^2 of the largest entry
        assert np.allclose(g, want, rtol=0, atol=0.1 / r**2 * np.abs(want).max())
