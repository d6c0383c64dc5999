"""Batched CG (gfmd_minimize_batch): concurrent graph branches give the same
results as one-at-a-time solves, across grid sizes, obstacles and load
control, and load control agrees with the oracle."""
import numpy as np
import pytest

from conftest import gfmd_pkg, rel_l2
from solver_cases import KERNEL_SC, gpu_obstacle, oracle_elastic, osv, sphere_spec, tables

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _solver(nx, ny, d, half, linf, prec):
    s = gfmd_pkg().gfmd_solver_factory("static/gb300" if prec == "f64" else "static/gb300/f32")
    s.set_grid_size(nx, ny, d)
    s.set_phi(half, "half", linf)
    return s


def _map_problem(nx, ny, seed, fz):
    g = gfmd_pkg()
    zmap = torch.empty(nx * ny, dtype=torch.float64, device="cuda")
    g.rough_surface(zmap, nx, ny, 0.8, 0.1, 4.0, nx / 2.0, seed)
    z0 = -float(zmap.min())  # indenter just touching at its lowest point
    o = g.map_obstacle(zmap, 0.05, 0.5, z0=z0, norm=-1, nlayer=1)
    o.fz_ext = fz
    return o, zmap


def _problems(prec):
    out = []
    for k, (nx, ny) in enumerate([(32, 32), (64, 48), (48, 64), (96, 96)]):
        d, half, full, linf = tables(KERNEL_SC, nx, ny)
        s = _solver(nx, ny, d, half, linf, prec)
        ref = _solver(nx, ny, d, half, linf, "f64") if prec == "f32" else None
        if k % 2 == 0:
            ob = gpu_obstacle(sphere_spec(nx, ny, R=8.0, pen=0.3, cutoff=4.0))
            keep = None
        else:
            ob, keep = _map_problem(nx, ny, 100 + k, 2e-3)
        out.append((s, ob, ref, keep, d, nx, ny))
    return out


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_batch_matches_individual_solves(prec):
    probs = _problems(prec)
    singles = []
    for s, ob, ref, keep, d, nx, ny in probs:
        u = torch.zeros(d, nx * ny, dtype=torch.float64, device="cuda")
        rep = s.minimize(u, ob, "cg", ftol=1e-8, refine=ref)
        singles.append((u, rep))
    us = [torch.zeros(d, nx * ny, dtype=torch.float64, device="cuda") for _, _, _, _, d, nx, ny in probs]
    reps = gfmd_pkg().minimize_batch([(p[0], u, p[1], p[2]) for p, u in zip(probs, us)], ftol=1e-8)
    for (u1, r1), u2, r2 in zip(singles, us, reps):
        assert r2["status"] == 0 and r2["fmax"] <= 1e-8
        assert torch.equal(u1, u2)
        assert r1["iterations"] == r2["iterations"]


def test_load_control_matches_oracle():
    nx = ny = 32
    d, half, full, linf = tables(KERNEL_SC, nx, ny)
    ob, zmap = _map_problem(nx, ny, 5, 2e-3)
    s = _solver(nx, ny, d, half, linf, "f64")
    u = torch.zeros(d, nx * ny, dtype=torch.float64, device="cuda")
    rep = s.minimize(u, ob, "cg", ftol=1e-9)
    spec = osv.ObstacleSpec(osv.MAP_EXP, epsilon=0.05, sigma=0.5, zmap=zmap.cpu().numpy(),
                            map_z0=ob.map_z0, norm=-1, nlayer=1, fz_ext=2e-3)
    el = oracle_elastic(full, linf, nx, ny)
    u_ref, r_ref = osv.cg(el, spec, np.zeros((d, nx * ny)), nx, ny, ftol=1e-9)
    assert rel_l2(u.cpu().numpy(), u_ref) <= 1e-6
    assert abs(rep["energy"] - r_ref["energy"]) <= 1e-8 * abs(r_ref["energy"])
    # equilibrium: elastic + wall + external forces balance on every atom
    f_el, _ = el(u_ref, True)
    _, f_w, _, _ = osv.wall(spec, u_ref, nx, ny)  # includes the external force
    assert np.abs(f_el + f_w).max() <= 1e-9
    assert abs((f_el + f_w)[2].sum()) <= 1e-9 * nx * ny


def test_batch_rejects_mixed_precisions():
    g = gfmd_pkg()
    nx = ny = 16
    d, half, full, linf = tables(KERNEL_SC, nx, ny)
    a = _solver(nx, ny, d, half, linf, "f64")
    b = _solver(nx, ny, d, half, linf, "f32")
    u1 = torch.zeros(d, nx * ny, dtype=torch.float64, device="cuda")
    u2 = torch.zeros_like(u1)
    with pytest.raises(g.GFMDError) as ei:
        g.minimize_batch([(a, u1, None, None), (b, u2, None, None)])
    assert ei.value.code == 1


def test_batch_rejects_a_handle_in_two_items():
    g = gfmd_pkg()
    nx = ny = 16
    d, half, full, linf = tables(KERNEL_SC, nx, ny)
    a = _solver(nx, ny, d, half, linf, "f64")
    u1 = torch.zeros(d, nx * ny, dtype=torch.float64, device="cuda")
    u2 = torch.zeros_like(u1)
    with pytest.raises(g.GFMDError) as ei:
        g.minimize_batch([(a, u1, None, None), (a, u2, None, None)])
    assert ei.value.code == 1


_DIRECT = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from solver_cases import KERNEL_SC, gpu_obstacle, sphere_spec, tables
from conftest import gfmd_pkg
nx = ny = 32
d, half, full, linf = tables(KERNEL_SC, nx, ny)
outs = []
for prec in ("f64", "f32"):
    s = gfmd_pkg().gfmd_solver_factory("static/gb300" if prec == "f64" else "static/gb300/f32")
    s.set_grid_size(nx, ny, d); s.set_phi(half, "half", linf)
    r = None
    if prec == "f32":
        r = gfmd_pkg().gfmd_solver_factory("static/gb300"); r.set_grid_size(nx, ny, d); r.set_phi(half, "half", linf)
    u = torch.zeros(d, nx * ny, dtype=torch.float64, device="cuda")
    rep = s.minimize(u, gpu_obstacle(sphere_spec(nx, ny, R=8.0, pen=0.3, cutoff=4.0)), "cg", ftol=1e-8, refine=r)
    outs.append(u.cpu().numpy())
np.save(sys.argv[2], np.stack(outs))
"""


def test_direct_launch_mode_matches_graphs(tmp_path):
    import os
    import subprocess
    import sys
    here = os.path.dirname(__file__)
    script = tmp_path / "direct.py"
    script.write_text(_DIRECT)
    res = {}
    for mode in ("0", "1"):
        out = tmp_path / f"u{mode}.npy"
        env = dict(os.environ, GFMD_NO_GRAPHS=mode)
        subprocess.run([sys.executable, str(script), here, str(out)], check=True, env=env, timeout=300)
        res[mode] = np.load(out)
    assert np.array_equal(res["0"], res["1"])
