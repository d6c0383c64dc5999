"""Warm-start network: the oracle's backward (finite differences, CPU), and
the GPU kernels against the oracle (initial weights exactly; forward, loss
and gradients with the oracle emulating the BF16 operand rounding)."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import gfmd_pkg, rel_l2

_spec = importlib.util.spec_from_file_location(
    "warmstart_oracle", os.path.join(os.path.dirname(__file__), "..", "oracle", "warmstart_oracle.py"))
wo = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(wo)


def test_oracle_backward_matches_finite_differences():
    net = wo.Net(2, 3, 8, bf16=False)
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.2, net.nparam)
    x = rng.normal(0, 1, (1, 16, 16, 2))
    t = rng.normal(0, 1, (1, 16, 16, 3))
    _, g, _ = net.loss_grad(w, x, t)
    for i in rng.choice(net.nparam, 40, replace=False):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (net.loss_grad(wp, x, t)[0] - net.loss_grad(wm, x, t)[0]) / (2 * h)
        assert abs(g[i] - fd) <= 1e-6 * max(1.0, abs(fd))


def test_bf16_rounding_is_nearest_even():
    a = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159], np.float32)
    r = wo.to_bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == 1.0078125
    assert abs(r[4] + 3.140625) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(1, 16, 16), (2, 32, 24)])
def test_gpu_network_matches_oracle(shape):
    torch = pytest.importorskip("torch")
    g = gfmd_pkg()
    from importlib import import_module
    W = import_module(g.__name__ + ".warmstart")
    b, H, Wd = shape
    net = W.WarmStartNet(2, 3, 8, seed=7)
    ref = wo.Net(2, 3, 8, bf16=True)
    w0 = net.params()
    assert np.array_equal(w0, wo.he_init(ref, 7))
    rng = np.random.default_rng(3)
    x = rng.normal(0, 1, (b, H, Wd, 2)).astype(np.float32)
    t = rng.normal(0, 1, (b, H, Wd, 3)).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(t).cuda()
    y = torch.empty(b, H, Wd, 3, dtype=torch.float32, device="cuda")
    net.forward(xd, y)
    loss = net.loss_grad(xd, td)
    gg = net.grad()
    lref, gref, yref = ref.loss_grad(w0.astype(np.float64), x, t)
    assert rel_l2(y.cpu().numpy(), yref) <= 2e-3
    assert abs(loss - lref) <= 2e-3 * abs(lref)
    for i in range(9):
        a, bb = ref.offs[i]
        ci, co = ref.io[i]
        assert rel_l2(gg[a:bb], gref[a:bb]) <= 1e-2, f"layer {i} weights"
        assert rel_l2(gg[bb:bb + co], gref[bb:bb + co]) <= 1e-2, f"layer {i} bias"


@pytest.mark.gpu
def test_gpu_training_reduces_loss():
    torch = pytest.importorskip("torch")
    from importlib import import_module
    W = import_module(gfmd_pkg().__name__ + ".warmstart")
    net = W.WarmStartNet(2, 3, 8, seed=3)
    rng = np.random.default_rng(1)
    x = torch.from_numpy(rng.normal(0, 1, (16, 32, 32, 2)).astype(np.float32)).cuda()
    # a smooth target: local averages of the first channel
    k = torch.nn.functional.avg_pool2d(x[..., :1].permute(0, 3, 1, 2), 3, 1, 1).permute(0, 2, 3, 1)
    t = torch.cat([k, -k, 2 * k], dim=3).contiguous()
    first = net.loss_grad(x, t)
    for _ in range(150):
        net.loss_grad(x, t)
        net.adam_step(3e-3)
    assert net.loss_grad(x, t) < 0.2 * first


@pytest.mark.gpu
def test_warm_started_solve_converges_to_the_cold_solution(capsys):
    """Pairs from the solver, training on the GPU, and the solver as judge:
    from the network's guess it converges to the same minimum as from u = 0
    (the iteration counts of both are reported)."""
    torch = pytest.importorskip("torch")
    from importlib import import_module
    g = gfmd_pkg()
    W = import_module(g.__name__ + ".warmstart")
    rc = W.RoughContact("ft sc100 1.0 1 pair-potential 2 1.0 1.0 height 16", 0.7, 0.2, 4.0, 32.0, 8.0 / 3.0)
    n = 64
    rng = np.random.default_rng(2)
    loads = 10 ** rng.uniform(-3, -2, 32)
    zs, us, reps = rc.solve_many(g, torch, n, loads, list(range(100, 132)))
    assert all(r["status"] == 0 for r in reps)
    hs = float(torch.stack([z - z.min() for z in zs]).std())
    usc = float(torch.stack([u[2] for u in us]).std())
    ws = W.WarmStart(3, 8, 1, h_scale=hs, u_scale=usc)
    X = ws.features(torch, zs, loads, n, n)
    T = ws.targets(torch, us, n, n)
    losses = ws.train(torch, X, T, epochs=8, batch=4, lr=3e-3)
    assert losses[-1] < 0.5 * losses[0]
    tl, ts = [3e-3, 8e-3], [900, 901]
    _, ucold, cold = rc.solve_many(g, torch, n, tl, ts)
    guesses = []
    for p, sd in zip(tl, ts):
        z, _ = rc.problem(g, torch, n, p, sd)
        u = torch.zeros(3, n * n, dtype=torch.float64, device="cuda")
        guesses.append(ws.initial_guess(torch, z, p, n, n, u).clone())
    _, uwarm, warm = rc.solve_many(g, torch, n, tl, ts, guesses=guesses)
    for a, b, r in zip(ucold, uwarm, warm):
        assert r["status"] == 0 and r["fmax"] <= 1e-6
        assert float((a - b).norm() / a.norm()) <= 1e-4
    with capsys.disabled():
        print(f"\nwarm start: cold iterations {[r['iterations'] for r in cold]}, "
              f"warm {[r['iterations'] for r in warm]}")
