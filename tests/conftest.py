"""Shared test setup: markers, package and oracle loaders, golden fixtures."""
from __future__ import annotations

import ctypes
import glob
import importlib
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gfmd_pkg():
    """The product package (directory user-gfmd_gb300/)."""
    return importlib.import_module("user-gfmd_gb300")


_oracle = None


def oracle() -> ctypes.CDLL:
    """The oracle restatement (oracle/liboracle.so), built on first use."""
    global _oracle
    if _oracle is None:
        path = os.path.join(ROOT, "oracle", "liboracle.so")
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
        L = ctypes.CDLL(path)
        L.orc_post_force.restype = ctypes.c_double
        L.orc_post_force.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 5 + [ctypes.c_int]
        L.orc_fft2d.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_fft2d.restype = ctypes.c_int
        L.orc_post_force_half.restype = ctypes.c_double
        L.orc_post_force_half.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 5 + [ctypes.c_int]
        L.orc_synthetic_phi_full.restype = None
        L.orc_synthetic_phi_full.argtypes = [ctypes.c_int] * 3 + [ctypes.c_ulonglong, ctypes.c_double,
                                                                  ctypes.c_void_p, ctypes.c_int]
        _oracle = L
    return _oracle


def oracle_post_force(phi_full, linf, u, nx, ny, nthreads=0):
    """Oracle force evaluation: returns (f, E, u0)."""
    d = u.shape[0]
    phi_full = np.ascontiguousarray(phi_full, np.complex128)
    u = np.ascontiguousarray(u, np.float64)
    lf = np.ascontiguousarray(linf if linf is not None else np.zeros(d // 3), np.float64)
    f = np.zeros_like(u)
    u0 = np.zeros(d)
    e = oracle().orc_post_force(nx, ny, d, phi_full.ctypes.data, lf.ctypes.data, u.ctypes.data,
                                f.ctypes.data, u0.ctypes.data, nthreads)
    return f, e, u0


def oracle_post_force_half(phi_half, linf, u, nx, ny, nthreads=0):
    """Oracle force evaluation from the half-spectrum table
    [nx, ny//2+1, d, d] (entries with ky > ny/2 read as conj Phi(-q)):
    returns (f, E, u0)."""
    d = u.shape[0]
    phi_half = np.ascontiguousarray(phi_half, np.complex128)
    u = np.ascontiguousarray(u, np.float64)
    lf = np.ascontiguousarray(linf if linf is not None else np.zeros(d // 3), np.float64)
    f = np.zeros_like(u)
    u0 = np.zeros(d)
    e = oracle().orc_post_force_half(nx, ny, d, phi_half.ctypes.data, lf.ctypes.data, u.ctypes.data,
                                     f.ctypes.data, u0.ctypes.data, nthreads)
    return f, e, u0


def golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def kernel_for(c):
    """The stiffness kernel of a fixture, with the box lengths the reference
    ran it in when the fixture stores them (isotropic, nonperiodic)."""
    k = gfmd_pkg().StiffnessKernel(str(c["args"]))
    if "xprd" in c:
        k.set_box(float(c["xprd"]), float(c["yprd"]))
    return k


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def half_to_full(phi_half, nx, ny):
    """Expand a half-spectrum table [nx, ny//2+1, d, d] to the full grid using
    Phi(-q) = conj Phi(q)."""
    d = phi_half.shape[-1]
    full = np.zeros((nx, ny, d, d), np.complex128)
    nyc = ny // 2 + 1
    full[:, :nyc] = phi_half
    for ky in range(nyc, ny):
        my = ny - ky
        mx = (-np.arange(nx)) % nx
        full[:, ky] = np.conj(phi_half[mx, my])
    return full.reshape(nx * ny, d, d)


def needs_gpu():
    try:
        import torch

        return not torch.cuda.is_available()
    except Exception:
        return True
