"""The reference's Hertz contact tests on the lattice stiffness kernels, run
through the GPU CG with the reference's own loading and LAMMPS' per-step
displacement cap (min_modify dmax 0.1), judged by the residual of the
reference's eval.py against the Hertz pressure with each test's E*.

Loading as in tests/TEST_Hertz_*/lammps.in: equilibrium positions recorded,
every atom displaced 2.0 down, so the substrate's finite-height q = 0
stiffness pushes the surface up into the Lennard-Jones sphere (fix
contact/sphere 0 0 99.5 100.0 1.38888888888889 0.890898718140339 1.0);
`minimize 0.0 1e-6` with min_style cg.  Without the cap the first Newton
step, which sees only the elastic energy, would carry the surface through the
sphere.  The plain FP64 CG and the FP32 CG with FP64 refinement both run.
"""
import numpy as np
import pytest

from conftest import gfmd_pkg
from solver_cases import gpu_obstacle, osv
from test_hertz_oracle import R, R3, _residual_area, _sphere, _square_r

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _solve_gpu(args, nx, ny, spec, mixed):
    g = gfmd_pkg()
    k = g.StiffnessKernel(args)
    d = k.get_dimension()
    half, linf = k.phi_table(nx, ny, "half")
    hs = {}
    for prec in ("f64", "f32"):
        s = g.gfmd_solver_factory("static/gb300" if prec == "f64" else "static/gb300/f32")
        s.set_grid_size(nx, ny, d)
        s.set_phi(half, "half", linf)
        hs[prec] = s
    u = torch.zeros(d, nx * ny, dtype=torch.float64, device="cuda")
    u[2::3] = -2.0
    ob = gpu_obstacle(spec)
    if mixed:
        rep = hs["f32"].minimize(u, ob, "cg", ftol=1e-6, maxiter=200000, refine=hs["f64"], dmax=0.1)
    else:
        rep = hs["f64"].minimize(u, ob, "cg", ftol=1e-6, maxiter=200000, dmax=0.1)
    assert rep["status"] == 0 and rep["fmax"] <= 1e-6, rep
    f = torch.empty_like(u)
    hs["f64"].post_force(u, f)
    return f.cpu().numpy(), rep


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize(
    "name,args,estar,a0,zeq",
    [
        ("sc100", "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 128", 8.0 / 3, 1.0, 0.5),
        ("fcc100", "ft fcc100 1 1.0 pair-potential 1 1.0 height 128", 1.39, 1.0, 0.5),
    ],
)
def test_hertz_square_surfaces_on_gpu(name, args, estar, a0, zeq, mixed):
    n = 128
    spec = _sphere((a0, a0), [(0.5 * a0, 0.5 * a0, zeq)])
    f, rep = _solve_gpu(args, n, n, spec, mixed)
    res = _residual_area(f[2], _square_r(n, a0), estar, a0 * a0)
    print(f"{name} {'mixed' if mixed else 'fp64'}: residual {res:.3e}, {rep['iterations']} iterations")
    assert res < 1e-2


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_hertz_fcc111_on_gpu(mixed):
    nx, ny = 64, 37
    spec = _sphere((1.0, R3), [(0.0, 0.0, 0.0), (0.5, R3 / 2, 0.0)])
    f, rep = _solve_gpu("ft fcc111 1 1.0 pair-potential 1 1.0 height 128", nx, ny, spec, mixed)
    ix, iy = np.divmod(np.arange(nx * ny), ny)

    def wrap(v, L):
        return np.where(v > L / 2, v - L, v)

    r1 = np.hypot(wrap(ix * 1.0, nx), wrap(iy * R3, ny * R3))
    r2 = np.hypot(wrap(ix + 0.5, nx), wrap((iy + 0.5) * R3, ny * R3))
    res = _residual_area(np.concatenate([f[2], f[5]]), np.concatenate([r1, r2]), 1.54, R3 / 2)
    print(f"fcc111 {'mixed' if mixed else 'fp64'}: residual {res:.3e}, {rep['iterations']} iterations")
    assert res < 2e-3


def test_dmax_caps_every_step_and_matches_the_oracle_minimum():
    # a small sc100 Hertz-like case: the GPU CG with the cap reaches the
    # oracle CG's minimum (same cap) from the same out-of-range start
    n = 32
    args = "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 16"
    spec = osv.ObstacleSpec(osv.SPHERE_LJ, center=(0.0, 0.0, 19.5), radius=20.0, epsilon=1.38888888888889,
                            sigma=0.890898718140339, cutoff=1.0, lattice=(1.0, 1.0), nlayer=1,
                            layer_offsets=[(0.5, 0.5, 0.5)])
    from conftest import half_to_full
    from solver_cases import oracle_elastic

    k = gfmd_pkg().StiffnessKernel(args)
    half, linf = k.phi_table(n, n, "half")
    el = oracle_elastic(half_to_full(half, n, n), linf, n, n)
    u0 = np.zeros((3, n * n))
    u0[2] = -2.0
    uo, rep_o = osv.cg(el, spec, u0, n, n, ftol=1e-8, dmax=0.1)
    f, rep = _solve_gpu(args, n, n, spec, False)
    s = gfmd_pkg().gfmd_solver_factory("static/gb300")
    s.set_grid_size(n, n, 3)
    s.set_phi(half, "half", linf)
    u = torch.from_numpy(u0).cuda()
    rep2 = s.minimize(u, gpu_obstacle(spec), "cg", ftol=1e-8, maxiter=200000, dmax=0.1)
    assert rep2["status"] == 0
    assert np.abs(u.cpu().numpy() - uo).max() <= 1e-6 * np.abs(uo).max()
    assert abs(rep2["energy"] - rep_o["energy"]) <= 1e-9 * abs(rep_o["energy"])
