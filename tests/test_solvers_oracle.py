"""CPU checks of the solver-loop restatement in the oracle."""
import numpy as np
import pytest

from solver_cases import KERNEL_SC, oracle_elastic, osv, sphere_spec, tables


@pytest.mark.parametrize("kind", [osv.SPHERE_EXP, osv.SPHERE_LJ, osv.MAP_EXP])
def test_wall_force_and_curvature_are_derivatives_of_the_energy(kind):
    nx = ny = 8
    rng = np.random.default_rng(1)
    u = rng.normal(0, 0.05, (6, nx * ny))
    if kind == osv.MAP_EXP:
        ob = osv.ObstacleSpec(kind, epsilon=0.2, sigma=0.5, zmap=rng.normal(0, 0.1, nx * ny),
                              map_z0=-0.3, layer_offsets=[(0, 0, 0), (0.5, 0.5, -0.7)])
    else:
        ob = osv.ObstacleSpec(kind, center=(4.0, 4.0, 3.2), radius=3.0, epsilon=0.05,
                              sigma=0.3 if kind == osv.SPHERE_LJ else 0.5,
                              layer_offsets=[(0, 0, 0), (0.5, 0.5, -0.7)])
    d = rng.normal(0, 1, u.shape)
    E0, f, fd, cv = osv.wall(ob, u, nx, ny, d, 0.0)
    h = 1e-5
    Ep = osv.wall(ob, u + h * d, nx, ny)[0]
    Em = osv.wall(ob, u - h * d, nx, ny)[0]
    assert abs(-(Ep - Em) / (2 * h) - fd) <= 1e-6 * max(1.0, abs(fd))
    assert abs((Ep - 2 * E0 + Em) / h ** 2 - cv) <= 1e-4 * max(1.0, abs(cv))


def test_oracle_cg_and_fire_reach_the_same_minimum():
    # the box is large enough, with a gap cutoff, that no atom feels the
    # periodic-image boundary of the sphere (where the minimum-image force
    # jumps and no minimizer can converge)
    nx = ny = 32
    d, half, full, linf = tables(KERNEL_SC, nx, ny)
    el = oracle_elastic(full, linf, nx, ny)
    ob = sphere_spec(nx, ny, R=6.0, pen=0.3, cutoff=4.0)
    u0 = np.zeros((d, nx * ny))
    ucg, rcg = osv.cg(el, ob, u0, nx, ny, ftol=1e-8)
    assert rcg["fmax"] <= 1e-8
    ufi, rfi = osv.fire(el, ob, u0, nx, ny, ftol=1e-8, dtmax=0.2, dt=0.05, maxiter=20000)
    assert rfi["fmax"] <= 1e-8
    assert np.linalg.norm(ufi - ucg) <= 1e-6 * np.linalg.norm(ucg)
    assert abs(rfi["energy"] - rcg["energy"]) <= 1e-9 * abs(rcg["energy"])
    # the indenter pushes the surface down under its centre
    assert ucg[2].min() < -0.05


def test_oracle_nve_conserves_energy():
    nx = ny = 8
    d, half, full, linf = tables(KERNEL_SC, nx, ny)
    el = oracle_elastic(full, linf, nx, ny)
    u0 = np.random.default_rng(3).normal(0, 0.1, (d, nx * ny))
    _, _, e = osv.verlet(el, None, u0, np.zeros_like(u0), nx, ny, 0.01, 0.0, 2000)
    assert np.abs(e - e.mean()).max() / abs(e.mean()) < 1e-4


def test_oracle_trust_region_reaches_the_cg_minimum():
    # MinTRGFMD restated: with the (Phi + shift)^{-1} preconditioner and
    # without one (steepest descent in a trust region)
    from conftest import oracle_post_force

    nx = ny = 32
    d, half, full, linf = tables(KERNEL_SC, nx, ny)
    el = oracle_elastic(full, linf, nx, ny)
    ob = sphere_spec(nx, ny, R=6.0, pen=0.3, cutoff=4.0)
    u0 = np.zeros((d, nx * ny))
    ucg, rcg = osv.cg(el, ob, u0, nx, ny, ftol=1e-8)
    P = osv.preconditioner(full, nx, ny, 0.05, oracle_post_force)
    up, rp = osv.tr(el, P, ob, u0, nx, ny, ftol=1e-8)
    un, rn = osv.tr(el, None, ob, u0, nx, ny, ftol=1e-8, maxiter=20000)
    for u, r in ((up, rp), (un, rn)):
        assert r["fmax"] <= 1e-8
        assert np.linalg.norm(u - ucg) <= 1e-5 * np.linalg.norm(ucg)
        assert abs(r["energy"] - rcg["energy"]) <= 1e-9 * abs(rcg["energy"])
    assert rp["iterations"] < rn["iterations"] / 10


def test_bicubic_map_wall_forces_are_the_energy_gradient():
    # the restated FixWallMap force with the bicubic table: the lateral force
    # -f_z dz/dx is the exact gradient of the energy; at undisplaced sites the
    # table reproduces the map, so the normal force equals the site-sampled wall's
    nx, ny = 12, 10
    rng = np.random.default_rng(8)
    zmap = 0.2 * rng.normal(0, 1, nx * ny)
    ob = osv.ObstacleSpec(osv.MAP_EXP, epsilon=0.3, sigma=0.5, zmap=zmap, map_z0=-0.4, norm=1,
                          layer_offsets=[(0.0, 0.0, 0.0), (0.5, 0.5, 0.7)])
    u0 = np.zeros((6, nx * ny))
    E0, f0 = osv.wall_map_bicubic(ob, u0, nx, ny)
    Es, fs, _, _ = osv.wall(ob, u0, nx, ny)
    assert np.allclose(f0[2], fs[2], rtol=1e-13)  # layer 0 sits on the map's grid points
    u = rng.normal(0, 0.05, (6, nx * ny))
    E, fu = osv.wall_map_bicubic(ob, u, nx, ny)
    d = rng.normal(0, 1, u.shape)
    h = 1e-6
    Ep, _ = osv.wall_map_bicubic(ob, u + h * d, nx, ny)
    Em, _ = osv.wall_map_bicubic(ob, u - h * d, nx, ny)
    assert abs(-(Ep - Em) / (2 * h) - (fu * d).sum()) <= 1e-6 * np.abs(fu * d).sum()
    assert np.abs(fu[:2]).max() > 0.0  # lateral forces present


@pytest.mark.parametrize("args", [
    "fcc100 1.0 1",  # tests/TEST_energy_conservation_fcc100 (analytic kernel, no height)
    "ft fcc100 1.0 2 pair-potential 2 1.0 -0.1 height 10",  # ..._fcc100_pair_potential, ..._two_layers
])
def test_oracle_nve_energy_conservation_like_the_reference_tests(args):
    # 10 x 10, random displacements of 0.1 (seed 12472634), dt = 0.01,
    # |E - <E>| / <E| < 1e-4; 20 000 of the reference's 100 000 steps
    nx = ny = 10
    d, half, full, linf = tables(args, nx, ny)
    el = oracle_elastic(full, linf, nx, ny)
    u0 = np.random.default_rng(12472634).uniform(-0.1, 0.1, (d, nx * ny))
    _, _, e = osv.verlet(el, None, u0, np.zeros_like(u0), nx, ny, 0.01, 0.0, 20000)
    assert np.abs(e - e.mean()).max() / abs(e.mean()) < 1e-4
