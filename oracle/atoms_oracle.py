"""ORACLE — test infrastructure, not product code.

numpy restatement of the atom list <-> grid mapping of fix gfmd for one rank
owning the grid: FixGFMD::pre_force, orthogonal box
(src/main/fix_gfmd.cpp:659-858; the minimum image by the reference's while
loops, :770-773) and FixGFMD::grid_to_list (fix_gfmd.cpp:952-1074).
Only tests/ import this module.
"""
from __future__ import annotations

import numpy as np


def _wrap(d, L):
    out = np.empty_like(d)
    for i, v in enumerate(d):
        while v > 0.5 * L:
            v -= L
        while v < -0.5 * L:
            v += L
        out[i] = v
    return out


def atoms_to_grid(x, xeq, gid, nx, ny, ndof, box, shift=(0, 0), v=None):
    N = nx * ny
    u = np.zeros((ndof, N))
    vg = np.zeros((ndof, N)) if v is not None else None
    ix = (gid[:, 0] - shift[0]) % nx
    iy = (gid[:, 1] - shift[1]) % ny
    s = ix * ny + iy
    iu = gid[:, 2]
    d = x - xeq
    comp = [_wrap(d[:, 0], box[0]), _wrap(d[:, 1], box[1]), d[:, 2]]
    for c in range(3):
        u[3 * iu + c, s] = comp[c]
        if v is not None:
            vg[3 * iu + c, s] = v[:, c]
    return u, vg


def grid_to_atoms(gid, f, nx, ny):
    s = gid[:, 0] * ny + gid[:, 1]
    iu = gid[:, 2]
    fa = np.stack([f[3 * iu + c, s] for c in range(3)], axis=1)
    return fa, fa.sum(axis=0)
