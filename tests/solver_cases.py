"""Shared small solver problems for the CPU and GPU solver tests."""
import os
import sys

import numpy as np

from conftest import ROOT, gfmd_pkg, half_to_full, oracle_post_force

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle_solvers as osv  # noqa: E402

KERNEL_SC = "ft sc100 1 1.0 pair-potential 2 1.0 1.0 height 16"
KERNEL_FCC2 = "ft fcc100 1.0 2 pair-potential 2 1.0 -0.1 height 10"


def tables(args, nx, ny):
    k = gfmd_pkg().StiffnessKernel(args)
    half, linf = k.phi_table(nx, ny, "half")
    return k.get_dimension(), half, half_to_full(half, nx, ny), linf


def oracle_elastic(full, linf, nx, ny):
    def el(v, with_linf):
        f, e, _ = oracle_post_force(full, linf if with_linf else np.zeros_like(linf), v, nx, ny)
        return f, e
    return el


def sphere_spec(nx, ny, R=10.0, pen=0.5, eps=0.1, sigma=0.5, kind=osv.SPHERE_EXP, cutoff=0.0):
    c = (nx / 2.0, ny / 2.0, R - pen)
    return osv.ObstacleSpec(kind, center=c, radius=R, epsilon=eps, sigma=sigma, cutoff=cutoff)


def gpu_obstacle(spec):
    g = gfmd_pkg()
    o = g.Obstacle()
    o.kind = spec.kind
    o.center[:] = [float(x) for x in spec.c]
    o.radius, o.epsilon, o.sigma, o.cutoff = spec.R, spec.eps, spec.sigma, spec.cutoff
    o.lattice[:] = [spec.ax, spec.ay]
    o.nlayer = spec.nlayer
    o.norm = spec.norm
    o.map_z0 = spec.map_z0
    o.fz_ext = spec.fz_ext
    for l, off in enumerate(spec.offsets):
        o.layer_offset[l][:] = list(off)
    return o
