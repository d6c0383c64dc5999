"""The crystal surfaces behind the `ft` stiffness kernels (host producer,
csrc/stiffness.cpp), checked the way the reference's unit tests check its
CrystalSurface (src/unittests/test_crystal_surface.cpp: fcc100, fcc100_3nn,
fcc100_supercell, reverse_indices, fcc100_neighbor_shells):

* every neighbour entry points to an atom: r = r_i - r_j - cell.(x, y, ab);
* up to a cutoff of 1.8 nearest-neighbour distances, every atom sees exactly
  the lattice vectors of its crystal (fcc: 12 + 6 + 24 = 42, sc: 6 + 12 + 8
  = 26), generated here independently of the surface cells: the cubic fcc
  and sc lattices rotated into the surface frame;
* neighbour shells number the distinct distances in increasing order;
* a two-layer supercell (with the reference's reversed indices) gives every
  atom the same neighbours as the one-layer cell.

A small C++ driver (tests/surface_neighbors.cpp) is compiled with the
producer's sources and prints the surface; no GPU is needed."""
from __future__ import annotations

import itertools
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
CSRC = os.path.join(ROOT, "user-gfmd_gb300", "csrc")
RCUT = 1.8


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("surf") / "surface_neighbors")
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "surface_neighbors.cpp"),
                    os.path.join(CSRC, "stiffness.cpp"), "-lpthread", "-o", exe], check=True)
    return exe


def _surface(exe, surface, nu):
    args = f"ft {surface} 1.0 {nu} pair-potential 1 1.0 height 4"
    out = subprocess.run([exe, args, str(RCUT)], check=True, capture_output=True, text=True).stdout
    cell = pos = None
    neigh = []
    for ln in out.splitlines():
        w = ln.split()
        if w[0] == "cell":
            cell = np.array(w[1:], float).reshape(3, 3)
        elif w[0] == "pos":
            pos = np.array(w[1:], float).reshape(-1, 3)
        else:
            neigh.append((int(w[1]), int(w[2]), int(w[3]), int(w[4]), int(w[5]),
                          np.array(w[6:9], float), float(w[9]), int(w[10])))
    return cell, pos, neigh


def _cubic(fcc):
    """Lattice vectors with 0 < |r| < RCUT, nearest-neighbour distance 1, in
    the cube frame: sc (i, j, k); fcc (i, j, k) / sqrt 2 with i + j + k even."""
    out = []
    for i, j, k in itertools.product(range(-3, 4), repeat=3):
        if fcc and (i + j + k) % 2:
            continue
        v = np.array([i, j, k], float) / (np.sqrt(2.0) if fcc else 1.0)
        if 0.0 < np.linalg.norm(v) < RCUT:
            out.append(v)
    return np.array(out)


def _expected(surface):
    if surface == "sc100":
        return [_cubic(False)]
    if surface == "fcc100":  # (100) plane: in-plane nearest neighbours along x and y
        R = np.array([[1, 1, 0], [-1, 1, 0], [0, 0, np.sqrt(2.0)]]) / np.sqrt(2.0)
        return [_cubic(True) @ R.T]
    # (111) plane with a nearest neighbour along x, the layer above over the
    # hollow site at (1/2, sqrt(3)/6) (the other stacking is the y mirror)
    R = np.array([np.array([1, -1, 0]) / np.sqrt(2.0), np.array([-1, -1, 2]) / np.sqrt(6.0),
                  np.array([1, 1, 1]) / np.sqrt(3.0)])
    return [_cubic(True) @ R.T]


def _same_set(a, b, tol=1e-9):
    if len(a) != len(b):
        return False
    used = np.zeros(len(b), bool)
    for v in a:
        d = np.linalg.norm(b - v, axis=1)
        d[used] = np.inf
        k = int(np.argmin(d))
        if d[k] > tol:
            return False
        used[k] = True
    return True


CASES = [("sc100", 26, [6, 12, 8]), ("fcc100", 42, [12, 6, 24]), ("fcc111", 42, [12, 6, 24])]


@pytest.mark.parametrize("surface,count,shells", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("nu", [1, 2])
def test_neighbour_lists(driver, surface, count, shells, nu):
    cell, pos, neigh = _surface(driver, surface, nu)
    nat = len(pos)
    # every entry points to an atom of the (super)cell
    for i, j, x, y, ab, r, rn, sh in neigh:
        assert 0 <= i < nat and 0 <= j < nat
        assert np.allclose(r, pos[i] - pos[j] - cell @ np.array([x, y, ab], float), atol=1e-12)
        assert abs(rn - np.linalg.norm(r)) < 1e-12
    # each atom sees exactly the crystal's lattice vectors within the cutoff
    (expected,) = _expected(surface)
    for i in range(nat):
        rs = np.array([n[5] for n in neigh if n[0] == i])
        assert len(rs) == count
        assert _same_set(rs, expected), (surface, nu, i)
    # shells: distinct distances in increasing order, with the crystal's counts
    for i in range(nat):
        per = [n for n in neigh if n[0] == i]
        dist = sorted({round(n[6], 9) for n in per})
        assert [sum(1 for n in per if n[7] == k) for k in range(len(dist))] == shells
        for n in per:
            assert abs(n[6] - dist[n[7]]) < 1e-9


@pytest.mark.parametrize("surface", ["sc100", "fcc100", "fcc111"])
def test_supercell_sees_the_one_layer_neighbours(driver, surface):
    _, pos1, n1 = _surface(driver, surface, 1)
    _, pos2, n2 = _surface(driver, surface, 2)
    assert len(pos2) == 2 * len(pos1)
    ref = np.array([n[5] for n in n1 if n[0] == 0])
    for i in range(len(pos2)):
        assert _same_set(np.array([n[5] for n in n2 if n[0] == i]), ref)
