"""ORACLE — test infrastructure, not product code.

FP64 numpy restatement of the solver loops and obstacles the GPU library runs
(user-gfmd_gb300/csrc/gfmd_solvers.cu), with elastic forces from the C
oracle's restatement of GFMDSolverStatic::post_force (oracle/gfmd_oracle.c).
Only tests/ import this module.

Reference behaviour restated:
  obstacles  exponential wall e = eps exp(-g/sigma) - offset
             (FixWallMap::eval_exp, src/extras/fix_wall_map.cpp:575-582) on a
             sphere gap g = |r - c| - R; Lennard-Jones 12-6 sphere
             (FixContactSphere::post_force, src/extras/fix_contact_sphere.cpp:207-264);
             exponential map wall, normal force (FixWallMap::pre_force,
             src/extras/fix_wall_map.cpp:686-817);
  FIRE       FixFIRE::initial_integrate / final_integrate
             (src/cuda/fix_fire.cpp:117-297);
  TR         MinTRGFMD::iterate (src/extras/min_tr_gfmd.cpp:95-241);
  CG         Polak-Ribiere conjugate gradients (LAMMPS min_style cg, which
             the reference's Hertz tests run on fix gfmd) with a Newton line
             search along the direction;
  dynamics   velocity Verlet (fix nve) with linear damping.
"""
from __future__ import annotations

import numpy as np

SPHERE_EXP, SPHERE_LJ, MAP_EXP = 1, 2, 3


class ObstacleSpec:
    def __init__(self, kind, center=(0, 0, 0), radius=0.0, epsilon=1.0, sigma=1.0, cutoff=0.0,
                 lattice=(1.0, 1.0), layer_offsets=(), nlayer=0, zmap=None, map_z0=0.0, norm=1,
                 fz_ext=0.0):
        self.kind, self.c, self.R = kind, np.asarray(center, float), radius
        self.eps, self.sigma, self.cutoff = epsilon, sigma, cutoff
        self.ax, self.ay = lattice
        self.offsets = list(layer_offsets)
        self.nlayer = nlayer
        self.zmap, self.map_z0, self.norm = zmap, map_z0, norm
        self.fz_ext = fz_ext  # constant +z force per obstacle atom (load control)
        if kind == SPHERE_LJ:
            self.c1 = 48.0 * epsilon * sigma ** 12
            self.c2 = 24.0 * epsilon * sigma ** 6
            self.c3 = 4.0 * epsilon * sigma ** 12
            self.c4 = 4.0 * epsilon * sigma ** 6
            r6 = cutoff ** -6 if cutoff > 0 else 0.0
            self.offset = r6 * (self.c3 * r6 - self.c4) if cutoff > 0 else 0.0
        else:
            self.offset = epsilon * np.exp(-cutoff / sigma) if cutoff > 0 else 0.0


def map_bicubic(zmap, x, y):
    """The reference's bicubic map table (Table2D with interpolated
    derivatives, src/mathutils/table2d.cpp, as FixWallMap builds it,
    src/extras/fix_wall_map.cpp:267), restated in the cubic Hermite basis:
    on the periodic cell [i, i+1] x [j, j+1] (pixel units) the bicubic that
    takes the corner values, the central-difference slopes
    (z[i+1] - z[i-1]) / 2 along each axis and zero cross derivatives
    (the reference's 16 conditions, solved there by a 16 x 16 inverse).
    Returns f, df/dx, df/dy, d2f/dx2, d2f/dy2, d2f/dxdy at the points."""
    z = np.asarray(zmap, float)
    nx, ny = z.shape
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    i0 = np.floor(x).astype(int)
    j0 = np.floor(y).astype(int)
    t, s = x - i0, y - j0

    def zz(di, dj):
        return z[(i0 + di) % nx, (j0 + dj) % ny]

    # Hermite basis in t (value at 0, value at 1, slope at 0, slope at 1) and
    # its first and second derivatives
    def basis(t):
        h = [2 * t**3 - 3 * t**2 + 1, -2 * t**3 + 3 * t**2, t**3 - 2 * t**2 + t, t**3 - t**2]
        d1 = [6 * t**2 - 6 * t, -6 * t**2 + 6 * t, 3 * t**2 - 4 * t + 1, 3 * t**2 - 2 * t]
        d2 = [12 * t - 6, -12 * t + 6, 6 * t - 4, 6 * t - 2]
        return h, d1, d2

    hx, dx1, dx2 = basis(t)
    hy, dy1, dy2 = basis(s)
    out = [np.zeros_like(t) for _ in range(6)]
    for a in (0, 1):
        for b in (0, 1):
            f = zz(a, b)
            fx = 0.5 * (zz(a + 1, b) - zz(a - 1, b))
            fy = 0.5 * (zz(a, b + 1) - zz(a, b - 1))
            # value term H_a(t) H_b(s), slope terms G_a(t) H_b(s) and H_a(t) G_b(s)
            terms = ((f, hx[a], hy[b], dx1[a], dy1[b], dx2[a], dy2[b]),
                     (fx, hx[2 + a], hy[b], dx1[2 + a], dy1[b], dx2[2 + a], dy2[b]),
                     (fy, hx[a], hy[2 + b], dx1[a], dy1[2 + b], dx2[a], dy2[2 + b]))
            for c, X, Y, Xd, Yd, Xdd, Ydd in terms:
                out[0] += c * X * Y
                out[1] += c * Xd * Y
                out[2] += c * X * Yd
                out[3] += c * Xdd * Y
                out[4] += c * X * Ydd
                out[5] += c * Xd * Yd
    return out


def wall_map_bicubic(ob: ObstacleSpec, u, nx, ny):
    """FixWallMap::pre_force (src/extras/fix_wall_map.cpp:686-817) with the
    bicubic map table and the exponential wall (eval_exp, :575-582): at each
    site's displaced position r the map height z(r_x, r_y) and slopes (map
    pixel = one lattice spacing), dz = norm (r_z - z - map_z0), e = eps
    exp(-dz/sigma) - offset, f_z = norm eps exp(-dz/sigma)/sigma and the
    lateral force (f_x, f_y) = -f_z (dz/dx, dz/dy).  Returns (E, f)."""
    ndof = u.shape[0]
    f = np.zeros_like(u)
    nl = ndof // 3
    nlo = min(nl, ob.nlayer if ob.nlayer > 0 else nl)
    ix, iy = np.divmod(np.arange(nx * ny), ny)
    zmap = np.asarray(ob.zmap, float).reshape(nx, ny)
    E = 0.0
    for l in range(nlo):
        off = ob.offsets[l] if l < len(ob.offsets) else (0.0, 0.0, 0.0)
        rx = ix * ob.ax + off[0] + u[3 * l]
        ry = iy * ob.ay + off[1] + u[3 * l + 1]
        rz = off[2] + u[3 * l + 2]
        z, zx, zy, _, _, _ = map_bicubic(zmap, rx / ob.ax, ry / ob.ay)
        zx, zy = zx / ob.ax, zy / ob.ay
        dz = ob.norm * (rz - (z + ob.map_z0))
        m = np.ones_like(dz, bool) if ob.cutoff <= 0 else dz < ob.cutoff
        ex = ob.eps * np.exp(-dz / ob.sigma)
        fz = ob.norm * ex / ob.sigma
        f[3 * l] = np.where(m, -fz * zx, 0.0)
        f[3 * l + 1] = np.where(m, -fz * zy, 0.0)
        f[3 * l + 2] = np.where(m, fz, 0.0)
        E += np.where(m, ex - ob.offset, 0.0).sum()
    return E, f


def wall(ob: ObstacleSpec | None, u, nx, ny, direction=None, a=0.0):
    """Obstacle energy E, force f [ndof, N], and along `direction`:
    sum f.dir and sum dir^T H dir at u + a*dir."""
    ndof = u.shape[0]
    f = np.zeros_like(u)
    if ob is None:
        return 0.0, f, 0.0, 0.0
    nl = ndof // 3
    nlo = min(nl, ob.nlayer if ob.nlayer > 0 else nl)
    ix, iy = np.divmod(np.arange(nx * ny), ny)
    E = fdir = curv = 0.0
    for l in range(nlo):
        off = ob.offsets[l] if l < len(ob.offsets) else (0.0, 0.0, 0.0)
        d = direction[3 * l:3 * l + 3] if direction is not None else np.zeros((3, nx * ny))
        r = u[3 * l:3 * l + 3] + a * d
        r = r + np.asarray(off, float)[:, None]
        r[0] += ix * ob.ax
        r[1] += iy * ob.ay
        if ob.kind in (SPHERE_EXP, SPHERE_LJ):
            dv = r - ob.c[:, None]
            lx, ly = ob.ax * nx, ob.ay * ny
            dv[0] -= lx * np.rint(dv[0] / lx)
            dv[1] -= ly * np.rint(dv[1] / ly)
            rho = np.sqrt((dv ** 2).sum(0))
            g = rho - ob.R
            m = np.ones_like(g, bool) if ob.cutoff <= 0 else g < ob.cutoff
            if ob.kind == SPHERE_EXP:
                ex = ob.eps * np.exp(-g / ob.sigma)
                e = ex - ob.offset
                F = ex / ob.sigma
                E2 = F / ob.sigma
            else:
                gi = 1.0 / g
                g6 = gi ** 6
                e = g6 * (ob.c3 * g6 - ob.c4) - ob.offset
                F = g6 * (ob.c1 * g6 - ob.c2) * gi
                E2 = g6 * gi * gi * (13.0 * ob.c1 * g6 - 7.0 * ob.c2)
            n = dv / rho
            fl = F * n
            dn = (d * n).sum(0)
            dd = (d * d).sum(0)
            cv = E2 * dn * dn - F / rho * (dd - dn * dn)
            f[3 * l:3 * l + 3] = np.where(m, fl, 0.0)
            E += np.where(m, e, 0.0).sum()
            fdir += np.where(m, (fl * d).sum(0), 0.0).sum()
            curv += np.where(m, cv, 0.0).sum()
        if ob.kind == MAP_EXP:
            dz = ob.norm * (r[2] - (ob.zmap + ob.map_z0))
            m = np.ones_like(dz, bool) if ob.cutoff <= 0 else dz < ob.cutoff
            ex = ob.eps * np.exp(-dz / ob.sigma)
            fz = ob.norm * ex / ob.sigma
            f[3 * l + 2] = np.where(m, fz, 0.0)
            E += np.where(m, ex - ob.offset, 0.0).sum()
            fdir += np.where(m, fz * d[2], 0.0).sum()
            curv += np.where(m, ex / ob.sigma ** 2 * d[2] ** 2, 0.0).sum()
        if ob.fz_ext != 0.0:
            f[3 * l + 2] += ob.fz_ext
            E -= ob.fz_ext * (u[3 * l + 2] + a * d[2]).sum()
            fdir += ob.fz_ext * d[2].sum()
    return E, f, fdir, curv


def cg(elastic, ob, u, nx, ny, ftol=1e-6, maxiter=100000, recompute=50, dmax=None):
    """Polak-Ribiere CG with a Newton line search; elastic(v, with_linf)
    returns (force, energy).  dmax: largest displacement of any component in
    one line search (LAMMPS min_modify dmax, default 0.1 there; None: no
    cap).  Returns (u, report)."""
    u = u.copy()
    it = evals = 0

    def restart():
        nonlocal evals
        fel, _ = elastic(u, True)
        evals += 1
        _, fw, _, _ = wall(ob, u, nx, ny)
        g = fel + fw
        return fel, g, g.copy()

    fel, g, h = restart()
    since = 0
    while True:
        fmax = np.abs(g).max()
        if fmax <= ftol or it >= maxiter:
            break
        fKh, _ = elastic(h, False)
        evals += 1
        Kh = -fKh
        hKh = (h * Kh).sum()
        felh = (fel * h).sum()
        a, lo, hi = 0.0, 0.0, -1.0
        if dmax is not None:
            hi = dmax / np.abs(h).max()  # the step's upper bracket
        for _ in range(16):
            fwh = cw = 0.0
            if ob is not None:
                _, _, fwh, cw = wall(ob, u, nx, ny, h, a)
            gdir = felh - a * hKh + fwh
            curv = hKh + cw
            if gdir > 0:
                lo = a
            else:
                hi = a
            an = a + gdir / curv if curv > 0 else -1.0
            if hi >= 0 and (an <= lo or an >= hi or an < 0):
                an = 0.5 * (lo + hi)
            elif an < 0:
                an = 2 * lo if lo > 0 else 1e-3
            step = abs(an - a)
            a = an
            if step <= 1e-6 * abs(a) or ob is None:
                break
        u += a * h
        fel -= a * Kh
        _, fw, _, _ = wall(ob, u, nx, ny)
        gn = fel + fw
        it += 1
        since += 1
        if since >= recompute:
            fel, g, h = restart()
            since = 0
            continue
        beta = max(0.0, ((gn * gn).sum() - (gn * g).sum()) / (g * g).sum())
        h = gn + beta * h
        if (h * gn).sum() <= 0:
            h = gn.copy()
        g = gn
    fel, E_el = elastic(u, True)
    E_w, fw, _, _ = wall(ob, u, nx, ny)
    f = fel + fw
    return u, {"iterations": it, "force_evals": evals + 1, "energy": E_el + E_w,
               "fmax": np.abs(f).max(), "fnorm": np.sqrt((f * f).sum())}


def pcg(elastic, precond, ob, u, nx, ny, ftol=1e-6, maxiter=100000, recompute=50):
    """Preconditioned Polak-Ribiere CG of the reference's min_style cg/gfmd
    (src/extras/min_cg_gfmd.cpp:96-207): z = precond(g) = (Phi + c)^{-1} g,
    beta = max(0, z.(g - g_old) / (g_old.z_old)), h = z + beta h, reset to
    h = z when h.g <= 0; the line search and the restarts every `recompute`
    iterations are those of ``cg``.  Returns (u, report)."""
    u = u.copy()
    it = evals = 0

    def restart():
        nonlocal evals
        fel, _ = elastic(u, True)
        evals += 1
        _, fw, _, _ = wall(ob, u, nx, ny)
        g = fel + fw
        z = precond(g)
        return fel, g, z, z.copy(), (g * z).sum()

    fel, g, z, h, gz = restart()
    since = 0
    while True:
        if np.abs(g).max() <= ftol or it >= maxiter:
            break
        fKh, _ = elastic(h, False)
        evals += 1
        Kh = -fKh
        hKh = (h * Kh).sum()
        felh = (fel * h).sum()
        a, lo, hi = 0.0, 0.0, -1.0
        for _ in range(16):
            fwh = cw = 0.0
            if ob is not None:
                _, _, fwh, cw = wall(ob, u, nx, ny, h, a)
            gdir = felh - a * hKh + fwh
            curv = hKh + cw
            if gdir > 0:
                lo = a
            else:
                hi = a
            an = a + gdir / curv if curv > 0 else -1.0
            if hi >= 0 and (an <= lo or an >= hi or an < 0):
                an = 0.5 * (lo + hi)
            elif an < 0:
                an = 2 * lo if lo > 0 else 1e-3
            step = abs(an - a)
            a = an
            if step <= 1e-6 * abs(a) or ob is None:
                break
        u += a * h
        fel -= a * Kh
        _, fw, _, _ = wall(ob, u, nx, ny)
        gn = fel + fw
        it += 1
        since += 1
        if since >= recompute:
            fel, g, z, h, gz = restart()
            since = 0
            continue
        zn = precond(gn)
        zg = (zn * gn).sum()
        beta = max(0.0, (zg - (zn * g).sum()) / gz)
        hg = (h * gn).sum()
        if not zg + beta * hg > 0:
            beta = 0.0
        h = zn + beta * h
        g, gz = gn, zg
    fel, E_el = elastic(u, True)
    E_w, fw, _, _ = wall(ob, u, nx, ny)
    f = fel + fw
    return u, {"iterations": it, "force_evals": evals + 1, "energy": E_el + E_w,
               "fmax": np.abs(f).max(), "fnorm": np.sqrt((f * f).sum())}


def preconditioner(full, nx, ny, shift, post_force):
    """z = (Phi(q) + shift I)^{-1} g(q) with the oracle's force routine on the
    inverted full table (restates precondition_gradient, gfmd_misc.h:40-133)."""
    N = nx * ny
    d = full.shape[-1]
    inv = np.linalg.inv(full * N + shift * np.eye(d)[None]) / N
    zero = np.zeros(d // 3)

    def apply(g):
        f, _, _ = post_force(inv, zero, g, nx, ny)
        return -f
    return apply


def prec_gradient(full, cavg, g, nx, ny):
    """GFMDSolverStatic::prec_gradient (src/solvers/gfmd_solver_static.cpp:253-269):
    gP = IFFT((Phi(q) + Cavg)^{-1} FFT(g)), table `full` [nx*ny, d, d] as
    fill_phi_buffer leaves it (divided by nx*ny), both transforms unscaled
    (forward exp(-i), backward exp(+i)).  For d > 3 precondition_gradient<DEF_G>
    writes back three components only (src/main/gfmd_misc.h:121-124): the other
    components leave the transform pair as nx*ny*g."""
    d = g.shape[0]
    gq = np.fft.fft2(g.reshape(d, nx, ny), axes=(1, 2)).reshape(d, -1)
    M = np.linalg.inv(full + np.asarray(cavg, float)[None])
    out = np.einsum("qij,jq->iq", M, gq)
    if d > 3:
        out[3:] = gq[3:]
    return (np.fft.ifft2(out.reshape(d, nx, ny), axes=(1, 2)) * (nx * ny)).real.reshape(d, -1)


def tr(elastic, precond, ob, u, nx, ny, ftol=1e-6, maxiter=100000, dmax=0.1, rho_tol=0.01):
    """Trust region on the preconditioned force (MinTRGFMD::iterate,
    src/extras/min_tr_gfmd.cpp:95-241): step a h, h = P f, a = min(1,
    delta/sqrt(g.h)); accepted when (E_prev - E) >= rho_tol (a - a^2/2) g.h,
    else undone with delta = a sqrt(g.h)/2; after acceptance delta =
    min(2 delta, max(delta/2, 2|dE| / (min(1/2, 1 - delta/(2 sqrt(g.h))) sqrt(g.h)))).
    P: callable (preconditioned force) or None (identity).  Converged when
    max|f_i| <= ftol."""
    u = u.copy()

    def total(v):
        fe, ee = elastic(v, True)
        ew, fw, _, _ = wall(ob, v, nx, ny)
        return fe + fw, ee + ew

    f, E = total(u)
    evals, it = 1, 0
    P = precond if precond is not None else (lambda x: x.copy())
    if np.abs(f).max() > ftol:
        h = P(f)
        g = f.copy()
        gg = float((g * h).sum())
        delta = min(dmax, np.sqrt(gg))
        Eprev = E
    while np.abs(f).max() > ftol and it < maxiter:
        sg = np.sqrt(gg)
        a = min(1.0, delta / sg)
        u += a * h
        f, E = total(u)
        evals += 1
        it += 1
        if np.abs(f).max() <= ftol:
            break
        rho = (Eprev - E) / ((a - 0.5 * a * a) * gg)
        if not rho >= rho_tol:
            delta = 0.5 * a * sg
            u -= a * h
            f = g.copy()
            E = Eprev
        else:
            fac = 2.0 * abs(E - Eprev) / (min(0.5, 1.0 - delta / (2.0 * sg)) * sg)
            delta = min(2.0 * delta, max(0.5 * delta, fac))
            Eprev = E
            h = P(f)
            g = f.copy()
            gg = float((g * h).sum())
    f, E = total(u)
    return u, {"iterations": it, "force_evals": evals, "energy": E, "fmax": np.abs(f).max(),
               "fnorm": np.sqrt((f * f).sum())}


def fire(elastic, ob, u, nx, ny, ftol=1e-6, maxiter=100000, minsteps=10, incfac=1.2,
         decfac=0.5, mix_in=0.1, mixdec=0.99, dtmax=0.001, dt=None, xlimit=0.0):
    """FixFIRE (src/cuda/fix_fire.cpp:117-297) with unit masses."""
    u = u.copy()
    v = np.zeros_like(u)
    dt = dtmax if dt is None else dt
    nl = u.shape[0] // 3

    def total():
        fel, E = elastic(u, True)
        Ew, fw, _, _ = wall(ob, u, nx, ny)
        return fel + fw, E + Ew

    def limit(vv, vlimsq):
        if vlimsq <= 0:
            return vv
        vv = vv.reshape(nl, 3, -1)
        vsq = (vv ** 2).sum(1, keepdims=True)
        sc = np.where(vsq > vlimsq, np.sqrt(vlimsq / np.maximum(vsq, 1e-300)), 1.0)
        return (vv * sc).reshape(3 * nl, -1)

    f, E = total()
    evals, it, cut, mix = 1, 0, minsteps, mix_in
    while np.abs(f).max() > ftol and it < maxiter:
        dtf = 0.5 * dt
        vlimsq = (xlimit / dt) ** 2 if xlimit > 0 else 0.0
        v = limit(v + dtf * f, vlimsq)
        u += dt * v
        f, E = total()
        evals += 1
        v = limit(v + dtf * f, vlimsq)
        vf, vv, ff = (v * f).sum(), (v * v).sum(), (f * f).sum()
        help_ = mix * np.sqrt(vv / ff) if ff > 0 else 0.0
        if vf < 0:
            v[:] = 0.0
            cut, dt, mix = minsteps, dt * decfac, mix_in
        else:
            v = (1 - mix) * v + help_ * f
            if cut < 0:
                dt, mix = min(dt * incfac, dtmax), mix * mixdec
            else:
                cut -= 1
        it += 1
    return u, {"iterations": it, "force_evals": evals, "energy": E, "fmax": np.abs(f).max()}


def verlet(elastic, ob, u, v, nx, ny, dt, gamma, nsteps):
    """Damped velocity Verlet; returns (u, v, energies[nsteps+1])."""
    u, v = u.copy(), v.copy()

    def total():
        fel, E = elastic(u, True)
        Ew, fw, _, _ = wall(ob, u, nx, ny)
        return fel + fw, E + Ew

    f, E = total()
    out = [E + 0.5 * (v * v).sum()]
    for _ in range(nsteps):
        v = v + 0.5 * dt * (f - gamma * v)
        u += dt * v
        f, E = total()
        v = (v + 0.5 * dt * f) / (1.0 + 0.5 * dt * gamma)
        out.append(E + 0.5 * (v * v).sum())
    return u, v, np.array(out)
