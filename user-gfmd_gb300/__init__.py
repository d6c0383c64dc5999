"""gfmd_gb300: GB300-native GFMD elastic force evaluation and solver loop.

The package is a thin host layer over the C ABI of ``libgfmd_gb300.so``
(include/gfmd_gb300.h).  Import it with
``importlib.import_module("user-gfmd_gb300")``.
"""
from ._lib import GFMDError, MinParams, MinReport, Obstacle, lib  # noqa: F401
from ._lib import (GFMD_OBST_MAP_EXP, GFMD_OBST_NONE, GFMD_OBST_SPHERE_EXP,  # noqa: F401
                   GFMD_OBST_SPHERE_LJ)
from .solver import (  # noqa: F401
    GFMDSolverGB300,
    StiffnessKernel,
    gfmd_solver_factory,
    stiffness_kernel_factory,
)

__all__ = [
    "GFMDError",
    "Obstacle",
    "sphere_obstacle",
    "GFMDSolverGB300",
    "StiffnessKernel",
    "gfmd_solver_factory",
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
