"""Learned warm start for the static solve.

``WarmStartNet`` wraps the library's BF16 encoder-decoder (gfmd_ws_* in
include/gfmd_gb300.h): forward, loss and gradient, Adam, all on the GPU
with the library's own tensor-core kernels.  ``WarmStart`` adds what the
solver needs around it: features from a rigid height map and a load,
training pairs generated by the solver itself (batched CG), training, and
``initial_guess`` to seed ``GFMDSolverGB300.minimize``.  The solver then
converges from the guess to the same tolerance, so the network only changes
where the iteration starts; a bad guess costs iterations, never accuracy.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import GFMDError, check, lib


class WarmStartNet:
    """The network: NHWC FP32 device tensors, H and W multiples of 8."""

    def __init__(self, in_ch=2, out_ch=3, base=32, seed=1):
        h = ctypes.c_void_p()
        check(lib().gfmd_ws_create(in_ch, out_ch, base, seed, ctypes.byref(h)))
        self._h = h
        self.in_ch, self.out_ch, self.base = in_ch, out_ch, base
        n = ctypes.c_longlong()
        check(lib().gfmd_ws_num_params(h, ctypes.byref(n)))
        self.nparam = n.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().gfmd_ws_destroy(h)
            self._h = ctypes.c_void_p()

    def set_stream(self, stream):
        addr = stream if isinstance(stream, int) else int(getattr(stream, "cuda_stream", 0))
        check(lib().gfmd_ws_set_stream(self._h, addr))

    def params(self):
        w = np.empty(self.nparam, np.float32)
        check(lib().gfmd_ws_get_params(self._h, w.ctypes.data, None))
        return w

    def grad(self):
        g = np.empty(self.nparam, np.float32)
        check(lib().gfmd_ws_get_params(self._h, None, g.ctypes.data))
        return g

    def set_params(self, w):
        w = np.ascontiguousarray(w, np.float32)
        if w.size != self.nparam:
            raise GFMDError(_lib.GFMD_EINVAL, "parameter count mismatch")
        check(lib().gfmd_ws_set_params(self._h, w.ctypes.data))

    def forward(self, x, out):
        b, H, W, _ = x.shape
        check(lib().gfmd_ws_forward(self._h, b, H, W, x.data_ptr(), out.data_ptr()))
        return out

    def loss_grad(self, x, target):
        b, H, W, _ = x.shape
        loss = ctypes.c_double()
        check(lib().gfmd_ws_loss_grad(self._h, b, H, W, x.data_ptr(), target.data_ptr(), ctypes.byref(loss)))
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        check(lib().gfmd_ws_adam_step(self._h, lr, beta1, beta2, eps))


class WarmStart:
    """Height map + load -> displacement guess for a load-controlled
    rough contact (exponential map wall above the surface, ``fz_ext`` per
    atom).  Inputs: (z_map - min z_map) / h_scale and log10(load / load_ref)
    as a constant channel; outputs: the ndof displacement components divided
    by u_scale."""

    def __init__(self, ndof=3, base=32, seed=1, h_scale=1.0, u_scale=1.0, load_ref=1e-3):
        self.net = WarmStartNet(2, ndof, base, seed)
        self.ndof = ndof
        self.h_scale, self.u_scale, self.load_ref = h_scale, u_scale, load_ref

    def features(self, torch, zmaps, loads, nx, ny):
        """[batch, nx, ny, 2] FP32 features from FP64 height maps."""
        b = len(zmaps)
        x = torch.empty(b, nx, ny, 2, dtype=torch.float32, device=zmaps[0].device)
        for i, (z, p) in enumerate(zip(zmaps, loads)):
            h = (z - z.min()).view(nx, ny) / self.h_scale
            x[i, :, :, 0] = h.float()
            x[i, :, :, 1] = math.log10(p / self.load_ref)
        return x

    def targets(self, torch, us, nx, ny):
        b = len(us)
        t = torch.empty(b, nx, ny, self.ndof, dtype=torch.float32, device=us[0].device)
        for i, u in enumerate(us):
            t[i] = (u.view(self.ndof, nx, ny).permute(1, 2, 0) / self.u_scale).float()
        return t

    def initial_guess(self, torch, zmap, load, nx, ny, u_out):
        """Writes the network's guess into u_out ([ndof][nx*ny] FP64)."""
        x = self.features(torch, [zmap], [load], nx, ny)
        y = torch.empty(1, nx, ny, self.ndof, dtype=torch.float32, device=x.device)
        self.net.forward(x, y)
        u_out.copy_((y[0].permute(2, 0, 1).reshape(self.ndof, nx * ny).double()) * self.u_scale)
        return u_out

    def train(self, torch, x, t, epochs=10, batch=8, lr=2e-3, seed=0, log=None):
        """Adam on mean-squared error over the pairs (x, t); returns losses."""
        n = x.shape[0]
        rng = np.random.default_rng(seed)
        losses = []
        for ep in range(epochs):
            order = rng.permutation(n)
            tot = 0.0
            for k in range(0, n - batch + 1, batch):
                idx = torch.from_numpy(order[k:k + batch]).to(x.device)
                xb, tb = x.index_select(0, idx).contiguous(), t.index_select(0, idx).contiguous()
                tot += self.net.loss_grad(xb, tb)
                self.net.adam_step(lr * (0.5 ** (ep // max(1, epochs // 3))))
            losses.append(tot / max(1, n // batch))
            if log:
                log(ep, losses[-1])
        return losses


# ---------------------------------------------------------------------------
# Rough-contact problems and solver-generated training pairs

class RoughContact:
    """Load-controlled contact of a rigid self-affine indenter (exponential
    map wall of strength ``eps`` and range ``sigma`` above the surface, its
    lowest point touching the undeformed surface) with an elastic surface
    under the external pressure ``load * e_star`` (per site area ``area``)."""

    def __init__(self, kernel_args, hurst, rms_slope, lambda_short, lambda_long, e_star,
                 eps=1.0, sigma=0.5, area=1.0, nlayer=1):
        self.kernel_args = kernel_args
        self.hurst, self.rms_slope = hurst, rms_slope
        self.lambda_short, self.lambda_long = lambda_short, lambda_long
        self.e_star, self.eps, self.sigma, self.area, self.nlayer = e_star, eps, sigma, area, nlayer
        self._tables = {}

    def solvers(self, g, n, shift=0.0):
        """(FP32, FP64, ndof[, FP32 preconditioner]) for an n x n grid
        (tables generated once per n)."""
        if n not in self._tables:
            k = g.StiffnessKernel(self.kernel_args)
            self._tables[n] = (k.get_dimension(),) + k.phi_table(n, n, "half")
        d, half, linf = self._tables[n]
        out = []
        for name in ("static/gb300/f32", "static/gb300"):
            s = g.gfmd_solver_factory(name)
            s.set_grid_size(n, n, d)
            s.set_phi(half, "half", linf)
            out.append(s)
        if shift > 0.0:
            return out[0], out[1], d, out[0].make_preconditioner(shift)
        return out[0], out[1], d

    def problem(self, g, torch, n, load, seed, device="cuda"):
        """(height map, obstacle) for an n x n grid."""
        z = torch.empty(n * n, dtype=torch.float64, device=device)
        g.rough_surface(z, n, n, self.hurst, self.rms_slope, self.lambda_short, self.lambda_long, seed)
        ob = g.map_obstacle(z, self.eps, self.sigma, z0=-float(z.min()), norm=-1, nlayer=self.nlayer)
        ob.fz_ext = float(load) * self.e_star * self.area / self.nlayer
        return z, ob

    def solve_many(self, g, torch, n, loads, seeds, ftol=1e-6, chunk=32, guesses=None, shift=0.0):
        """Solves the problems (batched, mixed precision; preconditioned CG
        when shift > 0); returns (height maps, displacements, reports)."""
        zs, us, reps = [], [], []
        for c0 in range(0, len(loads), chunk):
            items, keep = [], []
            for i in range(c0, min(len(loads), c0 + chunk)):
                hs = self.solvers(g, n, shift)
                s32, s64, d = hs[:3]
                z, ob = self.problem(g, torch, n, loads[i], seeds[i])
                u = torch.zeros(d, n * n, dtype=torch.float64, device="cuda")
                if guesses is not None:
                    u.copy_(guesses[i])
                items.append((s32, u, ob, s64) + tuple(hs[3:]))
                keep.append(z)
            reps += g.minimize_batch(items, ftol=ftol, maxiter=50000)
            zs += keep
            us += [it[1] for it in items]
        return zs, us, reps
