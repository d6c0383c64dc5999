"""gfmd_gb300: GB300-native GFMD elastic force evaluation and solver loop.

The package is a thin host layer over the C ABI of ``libgfmd_gb300.so``
(include/gfmd_gb300.h).  Import it with
``importlib.import_module("user-gfmd_gb300")``.
"""
from ._lib import GFMDError, MinParams, MinReport, Obstacle, SurfaceParams, check, lib  # noqa: F401
from ._lib import (GFMD_OBST_MAP_EXP, GFMD_OBST_MAP_BICUBIC, GFMD_OBST_NONE, GFMD_OBST_SPHERE_EXP,  # noqa: F401
                   GFMD_OBST_SPHERE_LJ)
from .solver import (  # noqa: F401
    GFMDSolverGB300,
    PhiTableFile,
    atoms_to_grid,
    grid_to_atoms,
    StiffnessKernel,
    gfmd_solver_factory,
    minimize_batch,
    stiffness_kernel_factory,
)

from .warmstart import WarmStart, WarmStartNet  # noqa: F401

__all__ = [
    "WarmStart",
    "WarmStartNet",
    "GFMDError",
    "Obstacle",
    "sphere_obstacle",
    "rough_surface",
    "map_obstacle",
    "GFMDSolverGB300",
    "StiffnessKernel",
    "PhiTableFile",
    "atoms_to_grid",
    "grid_to_atoms",
    "gfmd_solver_factory",
    "minimize_batch",
    "stiffness_kernel_factory",
    "lib",
]


def sphere_obstacle(center, radius, epsilon, sigma, cutoff=0.0, kind="exp", lattice=(1.0, 1.0),
                    layer_offsets=None, nlayer=0) -> Obstacle:
    """A rigid sphere: exponential wall (kind "exp") or Lennard-Jones 12-6
    (kind "lj") on the gap |r - c| - R."""
    o = Obstacle()
    o.kind = GFMD_OBST_SPHERE_EXP if kind == "exp" else GFMD_OBST_SPHERE_LJ
    o.center[:] = list(center)
    o.radius, o.epsilon, o.sigma, o.cutoff = radius, epsilon, sigma, cutoff
    o.lattice[:] = list(lattice)
    o.nlayer = nlayer
    for l, off in enumerate(layer_offsets or []):
        o.layer_offset[l][:] = list(off)
    return o


def rough_surface(out, nx, ny, hurst, rms_slope, lambda_short, lambda_long, seed, lattice=1.0,
                  stream=0):
    """Self-affine random-phase height map into the CUDA float64 tensor
    ``out`` (nx*ny elements, x slow); see gfmd_rough_surface."""
    p = SurfaceParams(lattice, hurst, rms_slope, lambda_short, lambda_long, seed)
    check(lib().gfmd_rough_surface(nx, ny, p, out.data_ptr(), stream))
    return out


def map_obstacle(d_map, epsilon, sigma, z0=0.0, norm=-1, cutoff=0.0, nlayer=1, bicubic=False,
                 lattice=(1.0, 1.0), layer_offsets=None) -> Obstacle:
    """Rigid height map z_map (CUDA float64 tensor, nx*ny) with an
    exponential wall on dz = norm (r_z - z_map - z0); norm = -1 for an
    indenter above the surface.  ``bicubic`` evaluates FixWallMap's bicubic
    map table at each atom's displaced (x, y) and adds the lateral force
    (GFMD_OBST_MAP_BICUBIC); otherwise the map height at the grid site and
    the normal force only (GFMD_OBST_MAP_EXP)."""
    o = Obstacle()
    o.kind = GFMD_OBST_MAP_BICUBIC if bicubic else GFMD_OBST_MAP_EXP
    o.d_map = d_map.data_ptr()
    o.map_z0, o.norm = z0, norm
    o.epsilon, o.sigma, o.cutoff = epsilon, sigma, cutoff
    o.nlayer = nlayer
    o.lattice[:] = list(lattice)
    for l, off in enumerate(layer_offsets or []):
        o.layer_offset[l][:] = list(off)
    return o


def obstacle_force(obstacle, u, f, nx, ny, stream=0) -> float:
    """Force of the obstacle on the grid's atoms at displacements u (CUDA
    float64 tensors [ndof, nx*ny]) into f; returns the obstacle energy
    (gfmd_obstacle_force)."""
    import ctypes

    e = torch_scalar(u)
    check(lib().gfmd_obstacle_force(nx, ny, u.shape[0], ctypes.byref(obstacle), u.data_ptr(), f.data_ptr(),
                                    e.data_ptr(), stream))
    return float(e.item())


def torch_scalar(like):
    """One float64 device scalar on the device of ``like``."""
    import torch

    return torch.zeros(1, dtype=torch.float64, device=like.device)
