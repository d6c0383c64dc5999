"""Obstacle forces on the GPU against the oracle's restatements.

* GFMD_OBST_MAP_BICUBIC: FixWallMap's bicubic map table evaluated at each
  atom's displaced (x, y), exponential wall, lateral force -f_z dz/dx,
  -f_z dz/dy (src/extras/fix_wall_map.cpp:686-817, src/mathutils/table2d.cpp)
  against oracle_solvers.wall_map_bicubic, whose table matches the
  reference's own Table2D to 1e-14 (tests/test_oracle.py).
* The CG with the bicubic wall converges to a point where the oracle's
  elastic plus bicubic-wall force vanishes.
"""
import numpy as np
import pytest

from conftest import gfmd_pkg, half_to_full
from solver_cases import oracle_elastic, osv

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _rough(nx, ny, seed, amp=0.6):
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(nx)[:, None] ** 2 + np.fft.fftfreq(ny)[None, :] ** 2
    spec = (rng.normal(size=(nx, ny)) + 1j * rng.normal(size=(nx, ny))) / (1.0 + 200.0 * k)
    z = np.fft.ifft2(spec).real
    return amp * z / np.abs(z).max()


@pytest.mark.parametrize("lattice,nl", [((1.0, 1.0), 1), ((1.3, 0.8), 2)])
def test_bicubic_map_wall_matches_oracle(lattice, nl):
    g = gfmd_pkg()
    nx, ny = 32, 24
    zmap = _rough(nx, ny, 5)
    offs = [(0.0, 0.0, 0.0), (0.5 * lattice[0], 0.5 * lattice[1], -0.7)][:nl]
    rng = np.random.default_rng(7)
    u = np.zeros((3 * nl, nx * ny))
    u[0::3] = rng.uniform(-0.45, 0.45, (nl, nx * ny)) * lattice[0]  # lateral moves across pixel cells
    u[1::3] = rng.uniform(-0.45, 0.45, (nl, nx * ny)) * lattice[1]
    u[2::3] = rng.uniform(-0.2, 0.2, (nl, nx * ny))
    z0 = -1.2
    spec = osv.ObstacleSpec(4, epsilon=0.7, sigma=0.4, lattice=lattice, layer_offsets=offs, nlayer=nl,
                            zmap=zmap, map_z0=z0, norm=-1)
    e_ref, f_ref = osv.wall_map_bicubic(spec, u, nx, ny)
    d_map = torch.from_numpy(zmap.ravel()).cuda()
    ob = g.map_obstacle(d_map, 0.7, 0.4, z0=z0, norm=-1, nlayer=nl, bicubic=True, lattice=lattice,
                        layer_offsets=offs)
    ud = torch.from_numpy(u).cuda()
    fd = torch.empty_like(ud)
    e = g.obstacle_force(ob, ud, fd, nx, ny)
    f = fd.cpu().numpy()
    assert abs(e - e_ref) <= 1e-12 * abs(e_ref)
    assert np.abs(f - f_ref).max() <= 1e-12 * np.abs(f_ref).max()
    assert np.abs(f[0::3]).max() > 1e-3  # the lateral force is there


def test_site_map_wall_is_the_bicubic_wall_at_zero_lateral_displacement():
    # at u_x = u_y = 0 the bicubic table reproduces the map at the grid site
    g = gfmd_pkg()
    nx, ny = 16, 16
    zmap = _rough(nx, ny, 9)
    u = np.zeros((3, nx * ny))
    u[2] = np.random.default_rng(2).uniform(-0.3, 0.3, nx * ny)
    d_map = torch.from_numpy(zmap.ravel()).cuda()
    ud = torch.from_numpy(u).cuda()
    out = []
    for bic in (False, True):
        fd = torch.empty_like(ud)
        e = g.obstacle_force(g.map_obstacle(d_map, 1.0, 0.5, z0=-1.0, norm=-1, bicubic=bic), ud, fd, nx, ny)
        out.append((e, fd.cpu().numpy()))
    assert abs(out[0][0] - out[1][0]) <= 1e-12 * abs(out[0][0])
    assert np.abs(out[0][1][2] - out[1][1][2]).max() <= 1e-12 * np.abs(out[0][1][2]).max()


def test_cg_with_bicubic_wall_reaches_oracle_force_balance():
    g = gfmd_pkg()
    nx = ny = 32
    args = "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 16"
    k = g.StiffnessKernel(args)
    half, linf = k.phi_table(nx, ny, "half")
    zmap = _rough(nx, ny, 3, amp=0.8)
    z0 = -float(zmap.min()) + 0.3
    s = g.gfmd_solver_factory("static/gb300")
    s.set_grid_size(nx, ny, 3)
    s.set_phi(half, "half", linf)
    d_map = torch.from_numpy(zmap.ravel()).cuda()
    ob = g.map_obstacle(d_map, 1.0, 0.3, z0=z0, norm=-1, bicubic=True)
    ob.fz_ext = 0.02
    u = torch.zeros(3, nx * ny, dtype=torch.float64, device="cuda")
    rep = s.minimize(u, ob, "cg", ftol=1e-9, maxiter=100000, dmax=0.1)
    assert rep["status"] == 0
    uh = u.cpu().numpy()
    spec = osv.ObstacleSpec(4, epsilon=1.0, sigma=0.3, zmap=zmap, map_z0=z0, norm=-1, nlayer=1)
    _, fw = osv.wall_map_bicubic(spec, uh, nx, ny)
    fel, _ = oracle_elastic(half_to_full(half, nx, ny), linf, nx, ny)(uh, True)
    ftot = fel + fw
    ftot[2] += 0.02
    assert np.abs(ftot).max() <= 1e-8
    assert np.abs(fw[0]).max() > 1e-4  # lateral wall forces took part
