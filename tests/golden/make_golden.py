"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own, unmodified ``fill_phi_buffer``,
``GFMDSolverStatic::post_force``, ``GFMDSolverStatic::prec_gradient``, the
``GFMDSolverFFT`` stiffness / Green's function dumps and the ``Table2D`` bicubic
map table through oracle/_ref/libgfmdref.so (built
from the reference sources by oracle/ref/Makefile; needs the reference tree,
so this script runs only where it is present).  Each fixture stores the
kernel arguments, the grid, seeded displacements, the reference's forces,
energy and u(q=0), and — for grids small enough to commit — the reference's
full Phi table and linear forces.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libgfmdref.so")

# (name, kernel arguments, nx, ny, store phi?)
CASES = [
    ("sc100_nnn_h128_16x16", "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 128", 16, 16, True),
    ("fcc100x2_h64_12x10", "ft fcc100 1.0 2 pair-potential 1 1.0 height 64", 12, 10, True),
    ("fcc111_h128_8x6", "ft fcc111 1 1.0 pair-potential 1 1.0 height 128", 8, 6, True),
    ("fcc100x4_h64_8x8", "ft fcc100 1.0 4 pair-potential 1 1.0 height 64", 8, 8, True),
    ("fcc100x2_nn2_h10_10x10", "ft fcc100 1.0 2 pair-potential 2 1.0 -0.1 height 10", 10, 10, True),
    ("sc100_a13_9x7", "ft sc100 1.3 1 pair-potential 2 1.0 1.0 height 128", 9, 7, True),
    ("fcc100_analytic_linf_8x8", "fcc100 2 1.0 0.0 0.0 height 10 linf 0.05 -0.05", 8, 8, True),
    ("fcc111_h128_64x37", "ft fcc111 1 1.0 pair-potential 1 1.0 height 128", 64, 37, False),
    ("sc100_nnn_h128_32x32", "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 128", 32, 32, False),
    ("fcc100x2_h64_36x36", "ft fcc100 1.0 2 pair-potential 1 1.0 height 64", 36, 36, False),
    # the analytic styles (SC100StiffnessKernel, FCC100StiffnessKernel)
    ("sc100_analytic_h16_9x7", "sc100 height 16", 9, 7, True),
    ("fcc100x4_analytic_h10_6x8", "fcc100 4 1.0 0.3 0.1 height 10", 6, 8, True),
    ("fcc100x2_kappa_normal_8x8", "fcc100 x 2 1.0 0.2 0.3 0.1 0.1 0.05 normal -1 height 10", 8, 8, True),
    # the continuum styles, with the box of the reference's tests (one length
    # unit per grid point: xprd = nx, yprd = ny)
    ("isotropic_nu03_12x12", "isotropic 0.3 1.0 1.0", 12, 12, True),
    ("nonperiodic_nu03_9x7", "nonperiodic 0.3 1.0", 9, 7, True),
    ("nonperiodic_nu025_16x12", "nonperiodic 0.25 2.0", 16, 12, True),
    ("nonperiodic_nu03_63x63", "nonperiodic 0.3 1.0", 63, 63, False),
    # prime grid sizes: the host transform's generic radix
    ("nonperiodic_nu03_31x29", "nonperiodic 0.3 1.0", 31, 29, True),
]

# kernels that read the box lengths; the fixtures store them as xprd, yprd
BOX_STYLES = ("isotropic", "nonperiodic")

SEED = 20261203

# GFMDSolverStatic::prec_gradient fixtures (tests/golden/prec/): kernel, grid
PREC_CASES = [
    ("prec_sc100_nnn_h16_8x6", "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 16", 8, 6),
    ("prec_fcc100x2_h8_6x8", "ft fcc100 1.0 2 pair-potential 1 1.0 height 8", 6, 8),
]


def load_ref() -> ctypes.CDLL:
    if not os.path.exists(REF_LIB):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle", "ref"), "-j8"])
    L = ctypes.CDLL(REF_LIB)
    L.gref_last_error.restype = ctypes.c_char_p
    return L


def run_case(L, args: str, nx: int, ny: int, seed: int):
    box = (float(nx), float(ny)) if args.split()[0] in BOX_STYLES else (1.0, 1.0)
    L.gref_set_box(ctypes.c_double(box[0]), ctypes.c_double(box[1]))
    nd, ht = ctypes.c_int(), ctypes.c_int()
    if L.gref_kernel_info(args.encode(), ctypes.byref(nd), ctypes.byref(ht)):
        raise RuntimeError(L.gref_last_error().decode())
    d = nd.value
    phi = np.zeros((nx * ny, d, d), np.complex128)
    linf = np.zeros(d // 3)
    if L.gref_phi_full(args.encode(), nx, ny, 1, phi.ctypes.data_as(ctypes.c_void_p),
                       linf.ctypes.data_as(ctypes.c_void_p)):
        raise RuntimeError(L.gref_last_error().decode())
    rng = np.random.default_rng(seed)
    u = rng.normal(0.0, 0.01, (d, nx * ny))
    f = np.zeros_like(u)
    u0 = np.zeros(d)
    e = ctypes.c_double()
    if L.gref_post_force(args.encode(), nx, ny, u.ctypes.data_as(ctypes.c_void_p),
                         f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(e),
                         u0.ctypes.data_as(ctypes.c_void_p)):
        raise RuntimeError(L.gref_last_error().decode())
    return d, ht.value, phi, linf, u, f, e.value, u0


def run_prec_case(L, args: str, nx: int, ny: int, seed: int):
    L.gref_set_box(ctypes.c_double(1.0), ctypes.c_double(1.0))
    nd, ht = ctypes.c_int(), ctypes.c_int()
    if L.gref_kernel_info(args.encode(), ctypes.byref(nd), ctypes.byref(ht)):
        raise RuntimeError(L.gref_last_error().decode())
    d = nd.value
    rng = np.random.default_rng(seed)
    g = rng.normal(0.0, 1.0, (d, nx * ny))
    c = rng.normal(0.0, 0.1, (d, d))
    cavg = c + c.T + 0.5 * np.eye(d)
    gP = np.zeros_like(g)
    if L.gref_prec_gradient(args.encode(), nx, ny, cavg.ctypes.data_as(ctypes.c_void_p),
                            g.ctypes.data_as(ctypes.c_void_p), gP.ctypes.data_as(ctypes.c_void_p)):
        raise RuntimeError(L.gref_last_error().decode())
    return dict(args=np.array(args), nx=nx, ny=ny, ndof=d, cavg=cavg, g=g, gP=gP)


# GFMDSolverFFT::dump_stiffness / dump_greens_function fixtures
# (tests/golden/dumps/): the reference's files as text, kernel and grid
DUMP_CASES = [
    ("dump_fcc100x2_h8_5x3", "ft fcc100 1.0 2 pair-potential 1 1.0 height 8", 5, 3),
]


# Table2D (bicubic map) fixture (tests/golden/maps/): map, points, reference output
MAP_CASES = [("table2d_17x13", 17, 13, 400)]


def run_map_case(L, nx: int, ny: int, npts: int, seed: int):
    rng = np.random.default_rng(seed)
    z = rng.normal(0.0, 1.0, (nx, ny))
    x = rng.uniform(-2 * nx, 3 * nx, npts)
    y = rng.uniform(-2 * ny, 3 * ny, npts)
    x[:8] = np.arange(8) % nx  # grid points
    y[:8] = (3 * np.arange(8)) % ny
    out = np.zeros((npts, 6))
    if L.gref_table2d(nx, ny, z.ctypes.data_as(ctypes.c_void_p), npts, x.ctypes.data_as(ctypes.c_void_p),
                      y.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p)):
        raise RuntimeError(L.gref_last_error().decode())
    return dict(z=z, x=x, y=y, out=out)


def run_dump_case(L, args: str, nx: int, ny: int):
    import tempfile
    L.gref_set_box(ctypes.c_double(1.0), ctypes.c_double(1.0))
    out = dict(args=np.array(args), nx=nx, ny=ny)
    cwd = os.getcwd()
    for greens in (0, 1):
        with tempfile.TemporaryDirectory() as d:
            os.chdir(d)
            try:
                if L.gref_dump(args.encode(), nx, ny, greens):
                    raise RuntimeError(L.gref_last_error().decode())
                for fn in sorted(os.listdir(d)):
                    with open(fn) as fh:
                        out["file:" + fn] = np.array(fh.read())
            finally:
                os.chdir(cwd)
    return out


def main() -> int:
    L = load_ref()
    os.makedirs(os.path.join(HERE, "maps"), exist_ok=True)
    for i, (name, nx, ny, npts) in enumerate(MAP_CASES):
        path = os.path.join(HERE, "maps", f"{name}.npz")
        np.savez_compressed(path, **run_map_case(L, nx, ny, npts, SEED + 200 + i))
        print(f"{name} -> {os.path.getsize(path)} bytes")
    os.makedirs(os.path.join(HERE, "dumps"), exist_ok=True)
    for name, args, nx, ny in DUMP_CASES:
        path = os.path.join(HERE, "dumps", f"{name}.npz")
        np.savez_compressed(path, **run_dump_case(L, args, nx, ny))
        print(f"{name} -> {os.path.getsize(path)} bytes")
    os.makedirs(os.path.join(HERE, "prec"), exist_ok=True)
    for i, (name, args, nx, ny) in enumerate(PREC_CASES):
        path = os.path.join(HERE, "prec", f"{name}.npz")
        np.savez_compressed(path, **run_prec_case(L, args, nx, ny, SEED + 100 + i))
        print(f"{name} -> {os.path.getsize(path)} bytes")
    for i, (name, args, nx, ny, keep_phi) in enumerate(CASES):
        d, h, phi, linf, u, f, e, u0 = run_case(L, args, nx, ny, SEED + i)
        out = dict(args=np.array(args), nx=nx, ny=ny, ndof=d, height=h, u=u, f=f,
                   epot=np.array(e), u0=u0, linf=linf)
        if args.split()[0] in BOX_STYLES:
            out["xprd"], out["yprd"] = np.array(float(nx)), np.array(float(ny))
        if keep_phi:
            out["phi"] = phi
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{name}: ndof={d} E={e:.16e} -> {os.path.getsize(path)} bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
