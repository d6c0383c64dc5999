"""File formats of the reference that sit either side of the hot path.

* Height maps (FixWallMap::read_map / write_map,
  src/extras/fix_wall_map.cpp:1121-1213): whitespace-separated text, one
  line per x, ny values per line; the reader counts the columns of the
  first line (a token starts with an alphanumeric character, '-' or 'e'
  after a blank), assumes a square map and reads nx*nx values with x
  slow; the writer prints "%f " per value and a newline per x.
* Real-space grid dumps (FixGFMD::dump, src/main/fix_gfmd.cpp:1948-2009):
  for dump prefix P and step s, files P.s.r.u<i>.out and P.s.r.f<i>.out per
  degree of freedom and P.s.r.uP.out, .fP.out, .e.out (|u|^2, |f|^2, u.f per
  site); each line is one y (iy), each value " %20.10e " over x.
* Reciprocal-space dumps written by the solver when post_force gets a dump
  prefix (GFMDSolverFFT::dump, src/solvers/gfmd_solver_fft.cpp:209-285):
  P.q.u<i>.real.out / .imag.out with u(q) (forward transform, unscaled),
  P.q.f<i>.real.out / .imag.out with F(q) = Phi(q) u(q) (the table scaled by
  1/(nx ny)), and P.q.uP.out, .fP.out, .e.out with sum |u|^2, sum |F|^2 and
  Re sum u conj(F) per wavevector; same line layout.
* Map preprocessing (FixWallMap::filter_map / displace_map,
  src/extras/fix_wall_map.cpp:1220-1366): a low-pass filter that zeroes every
  Fourier mode with |q| = sqrt((kx/xprd)^2 + (ky/yprd)^2) > 1/lambda (k the
  folded mode index, q in cycles per length), and a shift that puts the
  map's bottom, top or average at z0, reporting min, max, rms height and mean.
* Stiffness and Green's function dumps (GFMDSolverFFT::dump_stiffness,
  dump_greens_function, src/solvers/gfmd_solver_fft.cpp:294-420): files
  phi<i><j>.real.out / .imag.out (g<i><j>... for the Green's function, the
  inverse of each block of the table scaled by 1/(nx ny)) with " %e " per
  value; the table's blocks are read in storage order, ny lines of nx values
  (line j holds blocks j*nx .. j*nx + nx - 1); phitr/gtr .real/.imag.out
  hold one empty line per line of the other files (the reference computes a
  trace there but writes nothing else).

Grids here are [ndof][nx*ny] arrays with index ix*ny + iy, as on the solver.
"""
from __future__ import annotations

import numpy as np


def _count_columns(line: str) -> int:
    n, last = 0, " "
    for c in line:
        if (c.isalnum() or c in "-e") and last == " ":
            n += 1
        last = c
    return n


def read_map(path: str) -> np.ndarray:
    """Height map as FixWallMap::read_map reads it: [nx, nx], x slow."""
    with open(path) as fh:
        first = fh.readline()
        if not first.endswith("\n"):
            raise ValueError(f"{path}: could not read map file")
        nx = _count_columns(first.rstrip("\n"))
        if nx <= 0:
            raise ValueError(f"{path}: no columns in the first line")
        values = np.array((first + fh.read()).split(), dtype=np.float64)
    if values.size < nx * nx:
        raise ValueError(f"{path}: error reading map file ({values.size} values for {nx} x {nx})")
    return values[:nx * nx].reshape(nx, nx)


def write_map(path: str, zmap) -> None:
    """FixWallMap::write_map: "%f " per value, one line per x."""
    z = np.asarray(zmap, np.float64)
    with open(path, "w") as fh:
        for row in z:
            fh.write("".join("%f " % v for v in row))
            fh.write("\n")


def _write_grid(path: str, values, nx: int, ny: int) -> None:
    g = np.asarray(values, np.float64).reshape(nx, ny)
    with open(path, "w") as fh:
        for iy in range(ny):
            fh.write("".join(" %20.10e " % v for v in g[:, iy]))
            fh.write("\n")


def read_grid(path: str, nx: int, ny: int) -> np.ndarray:
    """One dump file back as [nx*ny] (index ix*ny + iy)."""
    a = np.loadtxt(path, ndmin=2)
    if a.shape != (ny, nx):
        raise ValueError(f"{path}: expected {ny} lines of {nx} values, got {a.shape}")
    return a.T.reshape(nx * ny).copy()


def write_real_space_dump(prefix: str, step: int, u, f, nx: int, ny: int) -> str:
    """FixGFMD::dump; returns the file prefix P.s."""
    u = np.asarray(u, np.float64)
    f = np.asarray(f, np.float64)
    base = f"{prefix}.{step}"
    for i in range(u.shape[0]):
        _write_grid(f"{base}.r.u{i}.out", u[i], nx, ny)
        _write_grid(f"{base}.r.f{i}.out", f[i], nx, ny)
    _write_grid(f"{base}.r.uP.out", (u * u).sum(0), nx, ny)
    _write_grid(f"{base}.r.fP.out", (f * f).sum(0), nx, ny)
    _write_grid(f"{base}.r.e.out", (u * f).sum(0), nx, ny)
    return base


def write_q_space_dump(dump_prefix: str, u, phi_full, nx: int, ny: int) -> None:
    """GFMDSolverFFT::dump for displacements u [ndof][nx*ny] and the full
    Phi table [nx*ny][ndof][ndof] scaled by 1/(nx ny)."""
    u = np.asarray(u, np.float64)
    d = u.shape[0]
    uq = np.fft.fft2(u.reshape(d, nx, ny)).reshape(d, nx * ny)   # exp(-i q.r), unscaled
    Fq = np.einsum("qij,jq->iq", np.asarray(phi_full), uq)
    for i in range(d):
        _write_grid(f"{dump_prefix}.q.u{i}.real.out", uq[i].real, nx, ny)
        _write_grid(f"{dump_prefix}.q.u{i}.imag.out", uq[i].imag, nx, ny)
        _write_grid(f"{dump_prefix}.q.f{i}.real.out", Fq[i].real, nx, ny)
        _write_grid(f"{dump_prefix}.q.f{i}.imag.out", Fq[i].imag, nx, ny)
    _write_grid(f"{dump_prefix}.q.uP.out", (np.abs(uq) ** 2).sum(0), nx, ny)
    _write_grid(f"{dump_prefix}.q.fP.out", (np.abs(Fq) ** 2).sum(0), nx, ny)
    _write_grid(f"{dump_prefix}.q.e.out", (uq * np.conj(Fq)).sum(0).real, nx, ny)


def filter_map(zmap, lam: float, xprd: float | None = None, yprd: float | None = None) -> np.ndarray:
    """FixWallMap::filter_map: remove wavelengths shorter than lam from an
    nx x ny map (box xprd x yprd, default one length unit per pixel)."""
    z = np.asarray(zmap, np.float64)
    nx, ny = z.shape
    xprd = float(nx if xprd is None else xprd)
    yprd = float(ny if yprd is None else yprd)
    if not lam > 0.0:
        raise ValueError("the cut-off wavelength must be positive")
    zq = np.fft.fft2(z)  # exp(-i), as FFT3d::compute(+1)
    kx = np.minimum(np.arange(nx), nx - np.arange(nx)) / xprd
    ky = np.minimum(np.arange(ny), ny - np.arange(ny)) / yprd
    r = np.sqrt(kx[:, None] ** 2 + ky[None, :] ** 2)
    zq[r > 1.0 / lam] = 0.0
    return np.fft.ifft2(zq).real  # exp(+i) / (nx ny)


def displace_map(zmap, z0: float, align: str = "average"):
    """FixWallMap::displace_map: shift the map so that its bottom, top or
    average ("bottom", "top", "average") lies at z0.  Returns the shifted map
    and {"min", "max", "rms", "mean"} of it (rms: the standard deviation)."""
    z = np.asarray(zmap, np.float64)
    n = z.size
    mean = z.sum() / n
    rms = np.sqrt((z * z).sum() / n - mean * mean)
    if align == "bottom":
        shift = z0 - z.min()
    elif align == "top":
        shift = z0 - z.max()
    elif align == "average":
        shift = z0 - mean
    else:
        raise ValueError(f"unknown alignment {align!r}")
    out = z + shift
    return out, {"min": float(z.min() + shift), "max": float(z.max() + shift), "rms": float(rms),
                 "mean": float(mean + shift)}


def write_stiffness_dump(directory: str, phi_full, nx: int, ny: int, greens: bool = False) -> None:
    """dump_stiffness (greens False) or dump_greens_function (greens True)
    of a full table [nx*ny, d, d] (scaled by 1/(nx ny)) into `directory`.
    A singular block raises numpy.linalg.LinAlgError (the reference aborts)."""
    import os

    tab = np.asarray(phi_full, np.complex128).reshape(nx * ny, *np.shape(phi_full)[-2:])
    d = tab.shape[-1]
    if greens:
        tab = np.linalg.inv(tab)
    stem = "g" if greens else "phi"
    blocks = tab.reshape(ny, nx, d, d)
    for i in range(d):
        for j in range(d):
            for part, vals in (("real", blocks[:, :, i, j].real), ("imag", blocks[:, :, i, j].imag)):
                with open(os.path.join(directory, f"{stem}{i}{j}.{part}.out"), "w") as fh:
                    for row in vals:
                        fh.write("".join(" %e " % v for v in row) + "\n")
    for part in ("real", "imag"):
        with open(os.path.join(directory, f"{stem}tr.{part}.out"), "w") as fh:
            fh.write("\n" * ny)


def half_to_full(half, nx: int, ny: int) -> np.ndarray:
    """[nx, ny//2+1, d, d] half-spectrum table -> [nx*ny, d, d] full table,
    Phi(-q) = conj Phi(q) for the wavevectors the half spectrum omits."""
    half = np.asarray(half)
    d = half.shape[-1]
    full = np.empty((nx, ny, d, d), dtype=np.complex128)
    nyc = ny // 2 + 1
    full[:, :nyc] = half
    kx = (-np.arange(nx)) % nx
    for ky in range(nyc, ny):
        full[:, ky] = np.conj(half[kx, ny - ky])
    return full.reshape(nx * ny, d, d)
