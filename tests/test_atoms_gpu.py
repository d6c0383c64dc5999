"""Atom list <-> grid kernels (gfmd_atoms_to_grid / gfmd_grid_to_atoms)
against the oracle's restatement of FixGFMD::pre_force and grid_to_list."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, gfmd_pkg

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import atoms_oracle as ao  # noqa: E402

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _layer(nx, ny, nu, seed, box):
    rng = np.random.default_rng(seed)
    ix, iy, iu = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nu), indexing="ij")
    gid = np.stack([ix.ravel(), iy.ravel(), iu.ravel()], axis=1).astype(np.int32)
    perm = rng.permutation(gid.shape[0])  # atoms in arbitrary order
    gid = gid[perm]
    xeq = np.stack([gid[:, 0] * box[0] / nx, gid[:, 1] * box[1] / ny, -gid[:, 2] * 0.7], axis=1)
    x = xeq + rng.normal(0, 0.3, xeq.shape)
    # some atoms moved across the periodic boundary
    x[:10, 0] += box[0]
    x[10:20, 1] -= box[1]
    v = rng.normal(0, 1, xeq.shape)
    return gid, xeq, x, v


@pytest.mark.parametrize("shift", [(0, 0), (3, -2)])
def test_atoms_to_grid_and_back_match_the_oracle(shift):
    g = gfmd_pkg()
    nx, ny, nu = 16, 12, 2
    box = (16.0, 12.0)
    gid, xeq, x, v = _layer(nx, ny, nu, 1, box)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    u = torch.zeros(3 * nu, nx * ny, dtype=torch.float64, device="cuda")
    vg = torch.zeros_like(u)
    st = g.atoms_to_grid(dev(x), dev(xeq), dev(gid), nx, ny, 3 * nu, box, u, dev(v), vg, shift)
    assert st == {"bad_ids": 0, "empty_slots": 0, "duplicate_slots": 0}
    u_ref, v_ref = ao.atoms_to_grid(x, xeq, gid, nx, ny, 3 * nu, box, shift, v)
    assert np.array_equal(u.cpu().numpy(), u_ref)
    assert np.array_equal(vg.cpu().numpy(), v_ref)
    f = np.random.default_rng(2).normal(0, 1, (3 * nu, nx * ny))
    fa = torch.zeros(gid.shape[0], 3, dtype=torch.float64, device="cuda")
    fsum = g.grid_to_atoms(dev(gid), dev(f), nx, ny, 3 * nu, fa)
    fa_ref, fsum_ref = ao.grid_to_atoms(gid, f, nx, ny)
    assert np.array_equal(fa.cpu().numpy(), fa_ref)
    assert np.allclose(fsum, fsum_ref, rtol=1e-12, atol=1e-12)
    fsum2 = g.grid_to_atoms(dev(gid), dev(f), nx, ny, 3 * nu, fa, accumulate=True)
    assert np.array_equal(fa.cpu().numpy(), 2 * fa_ref) and np.array_equal(fsum, fsum2)


def test_mapping_errors_are_reported_not_written():
    g = gfmd_pkg()
    nx, ny, nu = 8, 8, 1
    box = (8.0, 8.0)
    gid, xeq, x, v = _layer(nx, ny, nu, 3, box)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    u = torch.zeros(3 * nu, nx * ny, dtype=torch.float64, device="cuda")
    bad = gid.copy()
    bad[0, 2] = 5  # layer outside the grid
    with pytest.raises(g.GFMDError) as ei:
        g.atoms_to_grid(dev(x), dev(xeq), dev(bad), nx, ny, 3 * nu, box, u)
    assert ei.value.code == 1 and ei.value.status["bad_ids"] == 1
    dup = gid.copy()
    dup[1] = dup[0]  # two atoms on one slot, one slot empty
    with pytest.raises(g.GFMDError) as ei:
        g.atoms_to_grid(dev(x), dev(xeq), dev(dup), nx, ny, 3 * nu, box, u)
    assert ei.value.status["empty_slots"] == 1 and ei.value.status["duplicate_slots"] == 1
    fa = torch.zeros(gid.shape[0], 3, dtype=torch.float64, device="cuda")
    with pytest.raises(g.GFMDError):
        g.grid_to_atoms(dev(bad), torch.zeros_like(u), nx, ny, 3 * nu, fa)
