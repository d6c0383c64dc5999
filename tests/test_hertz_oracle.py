"""The reference's Hertz contact tests on the lattice stiffness kernels,
restated on the CPU: this library's Phi tables, the oracle's CG with the
LAMMPS per-step displacement cap (min_modify dmax 0.1), the reference's
geometry and loading, and the residual of its eval.py against the Hertz
pressure with the contact modulus E* of each test.

Loading as in the reference's lammps.in: `fix gfmd` records the equilibrium
positions, then every atom is displaced 2.0 down, so the substrate's
finite-height q = 0 stiffness pushes the surface up into a Lennard-Jones
sphere (fix contact/sphere 0 0 99.5 100.0 1.38888888888889 0.890898718140339
1.0).  The solve stops at max|f_i| <= 1e-6.
"""
import numpy as np
import pytest

from conftest import gfmd_pkg, half_to_full
from solver_cases import oracle_elastic, osv

R, R3 = 100.0, 3.0 ** 0.5


def _sphere(lattice, offsets):
    return osv.ObstacleSpec(osv.SPHERE_LJ, center=(0.0, 0.0, 99.5), radius=R, epsilon=1.38888888888889,
                            sigma=0.890898718140339, cutoff=1.0, lattice=lattice, nlayer=len(offsets),
                            layer_offsets=offsets)


def _solve(args, nx, ny, ob):
    k = gfmd_pkg().StiffnessKernel(args)
    d = k.get_dimension()
    half, linf = k.phi_table(nx, ny, "half")
    el = oracle_elastic(half_to_full(half, nx, ny), linf, nx, ny)
    u0 = np.zeros((d, nx * ny))
    u0[2::3] = -2.0
    u, rep = osv.cg(el, ob, u0, nx, ny, ftol=1e-6, dmax=0.1)
    assert rep["fmax"] <= 1e-6
    return el(u, True)[0]


def _residual_area(f, r, estar, area):
    """eval.py: contact radius and peak pressure from the total load, then the
    summed squared deviation of the pressure f / area from p0 sqrt(1 - r^2/a^2)."""
    N = f.sum()
    a = R * (3.0 / 4 * (N / (estar * R ** 2))) ** (1.0 / 3)
    p0 = 3 * N / (2 * np.pi * a * a)
    pa = np.where(r < a, p0 * np.sqrt(np.clip(1.0 - (r / a) ** 2, 0.0, None)), 0.0)
    return float(((f / area - pa) ** 2).sum())


def _square_r(n, a0):
    x = np.arange(n) + 0.5
    x = np.where(x > n / 2, x - n, x) * a0
    return np.sqrt(x[:, None] ** 2 + x[None, :] ** 2).ravel()


@pytest.mark.parametrize(
    "name,args,estar,a0,zeq",
    [
        # tests/TEST_Hertz_sc100_128x128: E* = 8/3
        ("sc100", "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 128", 8.0 / 3, 1.0, 0.5),
        # tests/TEST_Hertz_sc100_128x128_a0_1.3: E* = 8/3 / 1.3, pressure per a0^2
        ("sc100_a0_1.3", "ft sc100 1.3 1 pair-potential 2 1.0 1.0 height 128", 8.0 / 3 / 1.3, 1.3, 0.5),
        # tests/TEST_Hertz_fcc100_128x128: E* = 1.39
        ("fcc100", "ft fcc100 1 1.0 pair-potential 1 1.0 height 128", 1.39, 1.0, 0.5),
        # tests/TEST_Hertz_fcc100_two_layers_128x128: top atoms at z = sqrt(2)/2 + 1/2
        ("fcc100_two_layers", "ft fcc100 1.0 2 pair-potential 1 1.0 height 64", 1.39, 1.0,
         0.5 * 2.0 ** 0.5 + 0.5),
    ],
)
def test_hertz_on_square_surfaces(name, args, estar, a0, zeq):
    n = 128
    # atoms at (a0 i + 1/2, a0 j + 1/2) of a sc lattice displaced by 0.5 box
    # units; the eval takes them at a0 (i + 1/2), as here
    ob = _sphere((a0, a0), [(0.5 * a0, 0.5 * a0, zeq)])
    f = _solve(args, n, n, ob)
    res = _residual_area(f[2], _square_r(n, a0), estar, a0 * a0)
    assert res < 1e-2


def test_hertz_on_fcc111():
    # tests/TEST_Hertz_fcc111_64x37_2: 64 x 37 cells of 1 x sqrt(3), two
    # atoms (0, 0) and (1/2, sqrt(3)/2), pressure per sqrt(3)/2, E* = 1.54,
    # residual < 2e-3
    nx, ny = 64, 37
    ob = _sphere((1.0, R3), [(0.0, 0.0, 0.0), (0.5, R3 / 2, 0.0)])
    f = _solve("ft fcc111 1 1.0 pair-potential 1 1.0 height 128", nx, ny, ob)
    ix, iy = np.divmod(np.arange(nx * ny), ny)

    def wrap(v, L):
        return np.where(v > L / 2, v - L, v)

    r1 = np.hypot(wrap(ix * 1.0, nx), wrap(iy * R3, ny * R3))
    r2 = np.hypot(wrap(ix + 0.5, nx), wrap((iy + 0.5) * R3, ny * R3))
    res = _residual_area(np.concatenate([f[2], f[5]]), np.concatenate([r1, r2]), 1.54, R3 / 2)
    assert res < 2e-3
