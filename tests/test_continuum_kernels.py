"""The continuum stiffness styles (isotropic, nonperiodic) on the CPU.

The reference's tests run the nonperiodic style in LAMMPS
(tests/TEST_Hertz_nonperiodic_{63x63,64x64}, TEST_flat_punch_nonperiodic_63x63,
TEST_energy_conservation_nonperiodic) and judge the result against continuum
contact mechanics.  Here the same problems are solved with the oracle's force
restatement on tables from this library's producer, and judged the same way
(same formulas, same residual bound).
"""
import numpy as np
import pytest

from conftest import gfmd_pkg, half_to_full
from solver_cases import oracle_elastic, osv


def _elastic(args, nx, ny):
    k = gfmd_pkg().StiffnessKernel(args)
    k.set_box(nx, ny)
    half, linf = k.phi_table(nx, ny, "half")
    return oracle_elastic(half_to_full(half, nx, ny), linf, nx, ny)


def hertz_residual(fz, nx, ny, R=100.0, G=1.0, nu=0.3):
    """The reference's Hertz check (tests/TEST_Hertz_nonperiodic_64x64/eval.py):
    contact radius and peak pressure from the total force, then the summed
    squared deviation from p0 sqrt(1 - r^2/a^2) around the corner (0, 0)."""
    E = 2 * G * (1 + nu) / (1 - nu * nu)
    x = np.arange(nx) + 0.5
    x = np.where(x > nx / 2, x - nx, x)
    y = np.arange(ny) + 0.5
    y = np.where(y > ny / 2, y - ny, y)
    r = np.sqrt(x[:, None] ** 2 + y[None, :] ** 2)
    N = fz.sum()
    a = R * (3.0 / 4 * (N / (E * R ** 2))) ** (1.0 / 3)
    p0 = 3 * N / (2 * np.pi * a * a)
    fa = np.where(r < a, p0 * np.sqrt(np.clip(1.0 - (r / a) ** 2, 0.0, None)), 0.0)
    return float(((fz - fa) ** 2).sum()), a


def hertz_sphere():
    """fix contact/sphere 0 0 99 100.0 1.38888888888889 0.890898718140339 1.0
    on sc atoms at (i + 1/2, j + 1/2, -3/2) (the reference's lammps.in)."""
    return osv.ObstacleSpec(osv.SPHERE_LJ, center=(0.0, 0.0, 99.0), radius=100.0,
                            epsilon=1.38888888888889, sigma=0.890898718140339, cutoff=1.0,
                            layer_offsets=[(0.5, 0.5, -1.5)])


@pytest.mark.parametrize("n", [63, 64])
def test_hertz_on_the_nonperiodic_kernel(n):
    el = _elastic("nonperiodic 0.3 1.0", n, n)
    u, rep = osv.cg(el, hertz_sphere(), np.zeros((3, n * n)), n, n, ftol=1e-6)
    assert rep["fmax"] <= 1e-6
    f, _ = el(u, True)
    res, a = hertz_residual(f[2].reshape(n, n), n, n)
    assert 4.0 < a < 12.0
    assert res < 1e-2


def test_flat_punch_on_the_nonperiodic_kernel():
    # tests/TEST_flat_punch_nonperiodic_63x63: sites within 13.7 of the centre
    # pushed 0.1 down and held; the rest relaxed; the pressure under the punch
    # follows N / sqrt(1 - r^2/a^2).  The free sites are solved exactly (the
    # problem is linear) with CG on the elastic operator.
    sla = pytest.importorskip("scipy.sparse.linalg")
    n = 63
    el = _elastic("nonperiodic 0.3 1.0", n, n)
    c = np.arange(n) - 31.0
    r = np.sqrt(c[:, None] ** 2 + c[None, :] ** 2)
    held = (r < 13.7).ravel()
    free = np.ones((3, n * n), bool)
    free[:, held] = False
    u_held = np.zeros((3, n * n))
    u_held[2, held] = -0.1

    def op(v):
        w = np.zeros((3, n * n))
        w[free] = v
        return -el(w, False)[0][free]

    A = sla.LinearOperator((free.sum(),) * 2, matvec=op, dtype=float)
    x, info = sla.cg(A, el(u_held, False)[0][free], rtol=1e-12, maxiter=5000)
    assert info == 0
    u = u_held.copy()
    u[free] = x
    f, _ = el(u, False)
    assert np.abs(f[free]).max() < 1e-10
    fz = f[2].reshape(n, n)
    a = 13.7
    N = fz[r < a / 2].min()
    fa = np.where(r < a, N / np.sqrt(np.clip(1.0 - (r / a) ** 2, 1e-300, None)), 0.0)
    assert ((fz - fa) ** 2).sum() < 1e-2


def test_nve_energy_conservation_on_the_nonperiodic_kernel():
    # tests/TEST_energy_conservation_nonperiodic: 15 x 15, random displacements
    # of 0.1, dt = 0.01, |E - <E>| / <E> < 1e-4 (here 5000 steps)
    n = 15
    el = _elastic("nonperiodic 0.3 1.0", n, n)
    u0 = np.random.default_rng(12472634).uniform(-0.1, 0.1, (3, n * n))
    _, _, e = osv.verlet(el, None, u0, np.zeros_like(u0), n, n, 0.01, 0.0, 5000)
    assert np.abs(e - e.mean()).max() / abs(e.mean()) < 1e-4


def test_nonperiodic_green_function_is_reciprocal_and_far_field_exact():
    # G_ab(r) = G_ba(-r) (Betti), so the transformed table is Hermitian up to
    # the rounding of the corner sums (5e-13 of the largest entry at 32 x 32);
    # far from the loaded cell the displacement is the point-force solution
    n = 32
    k = gfmd_pkg().StiffnessKernel("nonperiodic 0.3 1.0")
    k.set_box(n, n)
    phi, _ = k.phi_table(n, n, "full")
    assert np.abs(phi - np.conj(np.swapaxes(phi, 1, 2))).max() <= 1e-11 * np.abs(phi).max()
    # Phi(-q) = conj Phi(q): real-space G
    P = phi.reshape(n, n, 3, 3)
    Pm = P[(-np.arange(n)) % n][:, (-np.arange(n)) % n]
    assert np.abs(Pm - np.conj(P)).max() <= 1e-14 * np.abs(P).max()
    # compliance at q: inverse of the table (times nx*ny) transformed back
    G = np.fft.fft2(np.linalg.inv(P * n * n), axes=(0, 1)) / (n * n)
    nu, mu, x = 0.3, 1.0, 12
    assert abs(G[x, 0, 2, 2].real * 2 * np.pi * mu * x / (1 - nu) - 1) < 1e-3
    assert abs(G[x, 0, 0, 2].real * 4 * np.pi * mu * x / (1 - 2 * nu) - 1) < 1e-5
    assert abs(G[x, 0, 2, 0].real * 4 * np.pi * mu * x / (1 - 2 * nu) + 1) < 1e-5


def test_isotropic_kernel_arguments_and_square_box():
    g = gfmd_pkg()
    k = g.StiffnessKernel("isotropic 0.3 1.0 1.0")
    assert (k.get_dimension(), k.get_height()) == (3, 1)
    assert g.StiffnessKernel("isotropic 0.3 1.0 1e7").get_height() == 0
    # the reference allows square surfaces only (isotropic_stiffness.cpp:101-102)
    with pytest.raises(g.GFMDError):
        k.phi_table(8, 6, "half")
    k.set_box(5.0, 5.0)
    phi, _ = k.phi_table(8, 6, "half")
    assert np.isfinite(phi).all()
    for bad in ["isotropic", "isotropic 0.3", "isotropic 0.3 1.0", "nonperiodic 0.3",
                "nonperiodic x 1.0", "isotropic 0.3 1.0 1.0 extra"]:
        with pytest.raises(g.GFMDError):
            g.StiffnessKernel(bad)
    with pytest.raises(g.GFMDError):
        k.set_box(-1.0, 1.0)
