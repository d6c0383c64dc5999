"""gfmd_gb300: GB300-native GFMD elastic force evaluation and solver loop.

The package is a thin host layer over the C ABI of ``libgfmd_gb300.so``
(include/gfmd_gb300.h).  Import it with
``importlib.import_module("user-gfmd_gb300")``.
"""
from ._lib import GFMDError, lib  # noqa: F401
from .solver import (  # noqa: F401
    GFMDSolverGB300,
    StiffnessKernel,
    gfmd_solver_factory,
    stiffness_kernel_factory,
)

__all__ = [
    "GFMDError",
    "GFMDSolverGB300",
    "StiffnessKernel",
    "gfmd_solver_factory",
    "stiffness_kernel_factory",
    "lib",
]
