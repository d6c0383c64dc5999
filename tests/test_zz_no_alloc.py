"""gfmd_post_force_noalloc: the force evaluation for callers that cannot
allocate device memory (their own pooling allocator owns the GPU, or an
allocation's implicit synchronization is not acceptable where they call).

It is checked against gfmd_post_force, the handle-based entry point, on two
calls in a row (the fixed scratch array keeps the previous call's contents),
with the FP64 parity tolerance of the other GPU tests.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import gfmd_pkg, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

F64_TOL = 1e-10


def _call(L, nx, ny, d, phi, linf, u, f, ep):
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gfmd_post_force_noalloc(nx, ny, d, phi.data_ptr(),
                                   None if linf is None else linf.data_ptr(),
                                   u.data_ptr(), f.data_ptr(), ep.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize(
    "args,nx,ny,linf_vals",
    [
        ("ft fcc100 1.0 2 pair-potential 1 1.0 height 64", 96, 80, (0.05, -0.05)),
        ("ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 128", 64, 37, None),
    ],
)
def test_noalloc_matches_post_force_on_two_calls(args, nx, ny, linf_vals):
    g = gfmd_pkg()
    L = g.lib()
    k = g.StiffnessKernel(args)
    d = k.get_dimension()
    half, _ = k.phi_table(nx, ny, "half")
    linf = None if linf_vals is None else np.array(linf_vals)

    s = g.gfmd_solver_factory("static")
    s.set_grid_size(nx, ny, d)
    s.set_phi(half, "half", linf)

    d_phi = torch.from_numpy(np.ascontiguousarray(half).view(np.float64)).cuda()
    d_linf = None if linf is None else torch.from_numpy(linf).cuda()
    rng = np.random.default_rng(11)
    for call in range(2):
        u = torch.from_numpy(rng.normal(0.0, 0.01, (d, nx * ny))).cuda()
        f_ref = torch.empty_like(u)
        e_ref = s.post_force(u, f_ref)
        f = torch.full_like(u, float("nan"))
        ep = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        rc = _call(L, nx, ny, d, d_phi, d_linf, u, f, ep)
        assert rc == 0, L.gfmd_last_error().decode()
        assert rel_l2(f.cpu().numpy(), f_ref.cpu().numpy()) <= F64_TOL, f"call {call}"
        assert abs(float(ep.item()) - e_ref) <= F64_TOL * abs(e_ref), f"call {call}"


def test_noalloc_rejects_grids_beyond_its_scratch():
    L = gfmd_pkg().lib()
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = _call(L, 2048, 2048, 12, small, None, small, small[8:], small[4:5])
    assert rc == 1
    msg = L.gfmd_last_error().decode()
    assert "scratch" in msg and "16 MiB" in msg


def test_noalloc_refuses_host_memory():
    # a plain host array handed as u is refused before any launch
    L = gfmd_pkg().lib()
    nx = ny = 16
    d = 3
    phi = torch.zeros(nx * (ny // 2 + 1) * d * d * 2, dtype=torch.float64, device="cuda")
    u_host = np.zeros(d * nx * ny)
    f = torch.zeros(d * nx * ny, dtype=torch.float64, device="cuda")
    ep = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.gfmd_post_force_noalloc(nx, ny, d, phi.data_ptr(), None, u_host.ctypes.data, f.data_ptr(),
                                   ep.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 1
    assert "device-accessible" in L.gfmd_last_error().decode()
