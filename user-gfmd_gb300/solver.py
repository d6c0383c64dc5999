"""Host-side mirror of the reference's solver and stiffness-kernel interface.

Names, argument meaning and error behaviour follow the USER-GFMD classes they
stand in for, so a caller of the reference's API finds the same calls:

* ``StiffnessKernel`` / ``stiffness_kernel_factory`` —
  ``StiffnessKernel`` (src/main/surface_stiffness.h:36-180) and
  ``stiffness_kernel_factory`` (src/main/surface_stiffness.cpp:440-481);
* ``GFMDSolverGB300`` / ``gfmd_solver_factory`` —
  ``GFMDSolver`` (src/main/gfmd_solver.h:34-123), ``GFMDSolverStatic``
  (src/solvers/gfmd_solver_static.cpp) and ``gfmd_solver_factory``
  (src/main/gfmd_solver.cpp:209-256).

Everything runs through the C ABI of ``libgfmd_gb300.so``; errors surface as
``GFMDError`` carrying the C status code.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import struct

import numpy as np

from . import _lib
from ._lib import GFMDError, check, lib


def _ptr(a) -> int:
    """Device or host address of a torch tensor or numpy array."""
    if hasattr(a, "data_ptr"):
        return int(a.data_ptr())
    if isinstance(a, np.ndarray):
        return int(a.ctypes.data)
    if hasattr(a, "__cuda_array_interface__"):
        return int(a.__cuda_array_interface__["data"][0])
    raise TypeError(f"cannot take the address of {type(a)!r}")


def _check_device_array(a, dtype: str, count: int, what: str) -> None:
    """A device buffer passed by address must hold `count` contiguous
    elements of `dtype` ("float64" or "float32"); anything else would be
    read as the wrong numbers by the C ABI, so it is refused here."""
    if hasattr(a, "dtype") and hasattr(a, "is_contiguous"):  # torch tensor
        got = str(a.dtype).replace("torch.", "")
        if got != dtype:
            raise TypeError(f"{what} must be {dtype}, got {got}")
        if not a.is_contiguous():
            raise TypeError(f"{what} must be contiguous")
        if a.numel() < count:
            raise ValueError(f"{what} holds {a.numel()} elements, needs {count}")
    elif hasattr(a, "__cuda_array_interface__"):
        ai = a.__cuda_array_interface__
        want = {"float64": "<f8", "float32": "<f4"}[dtype]
        if ai.get("typestr") != want:
            raise TypeError(f"{what} must be {dtype}, got {ai.get('typestr')}")
        if ai.get("strides") is not None:
            raise TypeError(f"{what} must be contiguous")
        if int(np.prod(ai["shape"])) < count:
            raise ValueError(f"{what} holds fewer than {count} elements")


def _is_device(a) -> bool:
    if hasattr(a, "is_cuda"):
        return bool(a.is_cuda)
    return hasattr(a, "__cuda_array_interface__")


class StiffnessKernel:
    """A stiffness kernel parsed from the kernel part of a ``fix gfmd`` line,
    e.g. ``"ft fcc100 1.0 2 pair-potential 1 1.0 height 64"``."""

    def __init__(self, args: str):
        h = ctypes.c_void_p()
        check(lib().gfmd_kernel_create(args.encode(), ctypes.byref(h)))
        self._h = h
        self.args = args
        nd, ht = ctypes.c_int(), ctypes.c_int()
        check(lib().gfmd_kernel_info(self._h, ctypes.byref(nd), ctypes.byref(ht)))
        self._ndof, self._height = nd.value, ht.value
        self._name = args.split()[0]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            lib().gfmd_kernel_destroy(h)
            self._h = ctypes.c_void_p()

    def set_box(self, xprd: float, yprd: float) -> None:
        """Lateral box lengths (LAMMPS ``domain->xprd``, ``yprd``) for the
        isotropic and nonperiodic styles; 0 means one unit per grid point."""
        check(lib().gfmd_kernel_set_box(self._h, float(xprd), float(yprd)))
        self._box = (float(xprd), float(yprd))

    def _cache_key(self) -> str:
        box = getattr(self, "_box", (0.0, 0.0))
        return self.args if box == (0.0, 0.0) else f"{self.args} box {box[0]!r} {box[1]!r}"

    def get_dimension(self) -> int:
        return self._ndof

    def get_number_of_atoms(self) -> int:
        return self._ndof // 3

    def get_height(self) -> int:
        return self._height

    def get_name(self) -> str:
        return self._name

    def phi_table(self, nx: int, ny: int, layout: str = "half", nthreads: int = 0):
        """Phi(q) / (nx*ny) on the grid; returns (phi, linf).  ``layout``
        "full" gives [nx*ny, ndof, ndof] (fill_phi_buffer's output), "half"
        gives [nx, ny//2+1, ndof, ndof]."""
        d = self._ndof
        if layout == "full":
            phi = np.empty((nx * ny, d, d), dtype=np.complex128)
            lay = _lib.GFMD_PHI_FULL
        elif layout == "half":
            phi = np.empty((nx, ny // 2 + 1, d, d), dtype=np.complex128)
            lay = _lib.GFMD_PHI_HALF
        else:
            raise ValueError(f"unknown layout {layout!r}")
        linf = np.zeros(d // 3)
        check(lib().gfmd_kernel_phi(self._h, nx, ny, lay, _ptr(phi), _ptr(linf), nthreads))
        return phi, linf

    def phi_table_cached(self, nx: int, ny: int, cache_dir: str, layout: str = "half", nthreads: int = 0):
        """``phi_table`` through an on-disk cache (``PhiTableFile``): the file
        for (kernel arguments, nx, ny, layout) is read if present and valid,
        else the table is generated and written."""
        key = self._cache_key()
        path = PhiTableFile.path(cache_dir, key, nx, ny, layout)
        got = PhiTableFile.read(path, key, nx, ny, layout)
        if got is not None:
            return got
        phi, linf = self.phi_table(nx, ny, layout, nthreads)
        PhiTableFile.write(path, key, nx, ny, layout, phi, linf)
        return phi, linf

    def get_force_at_gamma_point(self) -> np.ndarray:
        _, linf = self.phi_table(1, 1, "full")
        return linf


class PhiTableFile:
    """Versioned binary Phi(q) table: a 64-byte little-endian header
    (magic b"GFMDPHI\\0", format version, nx, ny, ndof, layout 0 = half /
    1 = full, payload bytes, SHA-256 prefix of the kernel arguments), the
    complex128 table as ``phi_table`` returns it, then linf (float64).
    Files are written to a temporary name and renamed, so a reader never
    sees a partial table; a header that does not match is a cache miss."""

    MAGIC = b"GFMDPHI\0"
    VERSION = 1
    _HDR = struct.Struct("<8sIiiiiQ24s")

    @staticmethod
    def key(args: str, nx: int, ny: int, layout: str) -> bytes:
        canon = " ".join(args.split())
        return hashlib.sha256(f"{canon}|{nx}|{ny}|{layout}".encode()).digest()[:24]

    @classmethod
    def path(cls, cache_dir: str, args: str, nx: int, ny: int, layout: str) -> str:
        return os.path.join(cache_dir, f"phi_{cls.key(args, nx, ny, layout).hex()[:32]}_{nx}x{ny}_{layout}.bin")

    @classmethod
    def write(cls, path: str, args: str, nx: int, ny: int, layout: str, phi, linf) -> None:
        phi = np.ascontiguousarray(phi, np.complex128)
        linf = np.ascontiguousarray(linf, np.float64)
        hdr = cls._HDR.pack(cls.MAGIC, cls.VERSION, nx, ny, phi.shape[-1], 0 if layout == "half" else 1,
                            phi.nbytes + linf.nbytes, cls.key(args, nx, ny, layout))
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "wb") as fh:
            fh.write(hdr.ljust(64, b"\0"))
            fh.write(phi.tobytes())
            fh.write(linf.tobytes())
        os.replace(tmp, path)

    @classmethod
    def read(cls, path: str, args: str, nx: int, ny: int, layout: str):
        if not os.path.exists(path):
            return None
        with open(path, "rb") as fh:
            raw = fh.read(64)
            if len(raw) < 64:
                return None
            magic, ver, fx, fy, nd, lay, nb, key = cls._HDR.unpack(raw[:cls._HDR.size])
            if (magic != cls.MAGIC or ver != cls.VERSION or (fx, fy) != (nx, ny)
                    or lay != (0 if layout == "half" else 1) or key != cls.key(args, nx, ny, layout)):
                return None
            body = fh.read()
        shape = (nx, ny // 2 + 1, nd, nd) if layout == "half" else (nx * ny, nd, nd)
        nphi = int(np.prod(shape)) * 16
        if len(body) != nb or nb != nphi + (nd // 3) * 8:
            return None
        phi = np.frombuffer(body[:nphi], np.complex128).reshape(shape).copy()
        linf = np.frombuffer(body[nphi:], np.float64).copy()
        return phi, linf


def stiffness_kernel_factory(keyword: str, *args: str) -> StiffnessKernel:
    """``stiffness_kernel_factory(keyword, narg, carg, arg, ...)`` for string
    arguments: ``stiffness_kernel_factory("ft", "sc100", "1.0", "1", ...)``."""
    return StiffnessKernel(" ".join((keyword,) + tuple(args)))


class GFMDSolverGB300:
    """GB300 force evaluation behind the ``GFMDSolver`` interface.

    ``post_force(u, f)`` takes [ndof, nx*ny] arrays: numpy (host, copied in
    and out inside the call) or CUDA tensors (device, no host copies), and
    returns the elastic energy like ``GFMDSolverStatic::post_force``.
    """

    def __init__(self, precision: str = "f64", name: str = "static/gb300"):
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        self.precision = precision
        self.name = name
        self._h = ctypes.c_void_p()
        self.nx = self.ny = self.ndof = 0
        self.u0 = None

    # -- GFMDSolver API ------------------------------------------------------
    def get_name(self) -> str:
        return self.name

    def set_grid_size(self, nx: int, ny: int, ndof: int) -> None:
        self._free()
        prec = _lib.GFMD_PREC_F64 if self.precision == "f64" else _lib.GFMD_PREC_F32
        check(lib().gfmd_create(nx, ny, ndof, prec, ctypes.byref(self._h)))
        self.nx, self.ny, self.ndof = nx, ny, ndof

    def set_kernel(self, kernel: StiffnessKernel, normalize: bool = True) -> None:
        if kernel.get_dimension() != self.ndof:
            raise GFMDError(_lib.GFMD_EINVAL, "kernel dimension does not match ndof")
        phi, linf = kernel.phi_table(self.nx, self.ny, "half")
        if not normalize:
            phi = phi * float(self.nx * self.ny)
        self.set_phi(phi, "half", linf)

    # host copy of the table kept for q-space dumps up to this size
    DUMP_TABLE_BYTES = 256 << 20

    def set_phi(self, phi: np.ndarray, layout: str = "full", linf=None) -> None:
        """Upload a table already scaled by 1/(nx*ny)."""
        phi = np.ascontiguousarray(phi, dtype=np.complex128)
        self._dump_table = (phi, layout) if phi.nbytes <= self.DUMP_TABLE_BYTES else None
        lay = _lib.GFMD_PHI_FULL if layout == "full" else _lib.GFMD_PHI_HALF
        lf = None if linf is None else np.ascontiguousarray(linf, dtype=np.float64)
        check(lib().gfmd_set_phi(self._handle(), _ptr(phi), lay, None if lf is None else _ptr(lf)))

    def _host_table(self, who: str):
        tab = getattr(self, "_dump_table", None)
        if tab is None:
            raise GFMDError(_lib.GFMD_EINVAL, f"{who} needs a table of at most "
                            f"{self.DUMP_TABLE_BYTES >> 20} MiB kept by set_phi")
        from . import formats
        phi, layout = tab
        return formats.half_to_full(phi, self.nx, self.ny) if layout == "half" else phi

    def dump_stiffness(self, directory: str = ".") -> None:
        """phi<i><j>.{real,imag}.out of the uploaded table (GFMDSolverFFT::dump_stiffness)."""
        from . import formats
        formats.write_stiffness_dump(directory, self._host_table("dump_stiffness"), self.nx, self.ny)

    def dump_greens_function(self, directory: str = ".") -> None:
        """g<i><j>.{real,imag}.out, the inverse of every block of the table
        (GFMDSolverFFT::dump_greens_function)."""
        from . import formats
        try:
            formats.write_stiffness_dump(directory, self._host_table("dump_greens_function"),
                                         self.nx, self.ny, greens=True)
        except np.linalg.LinAlgError as ex:
            raise GFMDError(_lib.GFMD_ENONFINITE, f"dump_greens_function: singular block ({ex})")

    def set_stream(self, stream) -> None:
        addr = stream if isinstance(stream, int) else int(getattr(stream, "cuda_stream", 0))
        check(lib().gfmd_set_stream(self._handle(), addr))

    def post_force(self, u, f, dump_prefix=None) -> float:
        """Elastic forces of u into f, energy returned.  With ``dump_prefix``
        the reciprocal-space dump of GFMDSolverFFT::dump is written as well
        (formats.write_q_space_dump; needs the table on the host)."""
        if dump_prefix is not None:
            tab = getattr(self, "_dump_table", None)
            if tab is None:
                raise GFMDError(_lib.GFMD_EINVAL, "q-space dumps need a table of at most "
                                f"{self.DUMP_TABLE_BYTES >> 20} MiB kept by set_phi")
            from . import formats
            phi, layout = tab
            full = formats.half_to_full(phi, self.nx, self.ny) if layout == "half" else phi
            uh = u.detach().cpu().numpy() if hasattr(u, "detach") else np.asarray(u)
            formats.write_q_space_dump(dump_prefix, uh, full, self.nx, self.ny)
        e = ctypes.c_double()
        if _is_device(u) and _is_device(f):
            # the reference's GPU post_force takes double buffers whatever the
            # arithmetic of the handle (the FP32 handle converts on the fly)
            n = self.ndof * self.nx * self.ny
            _check_device_array(u, "float64", n, "u")
            _check_device_array(f, "float64", n, "f")
            check(lib().gfmd_post_force(self._handle(), _ptr(u), _ptr(f), ctypes.byref(e)))
        elif not _is_device(u) and not _is_device(f):
            uh = np.ascontiguousarray(u, dtype=np.float64)
            if not (isinstance(f, np.ndarray) and f.dtype == np.float64 and f.flags.c_contiguous):
                raise TypeError("f must be a C-contiguous float64 numpy array")
            check(lib().gfmd_post_force_host(self._handle(), _ptr(uh), _ptr(f), ctypes.byref(e)))
        else:
            raise TypeError("u and f must both be host arrays or both be device tensors")
        return e.value

    def force_async(self, u, f, epot) -> None:
        """Device-resident evaluation without a host sync; epot is a device
        float64 scalar tensor."""
        fn = lib().gfmd_force_f64 if self.precision == "f64" else lib().gfmd_force_f32
        n = self.ndof * self.nx * self.ny
        dt = "float64" if self.precision == "f64" else "float32"
        _check_device_array(u, dt, n, "u")
        _check_device_array(f, dt, n, "f")
        _check_device_array(epot, "float64", 1, "epot")
        check(fn(self._handle(), _ptr(u), _ptr(f), _ptr(epot)))

    def make_preconditioner(self, shift: float) -> "GFMDSolverGB300":
        """A handle applying -(Phi + shift)^{-1} (gfmd_make_preconditioner),
        for ``minimize(..., precond=...)``."""
        out = GFMDSolverGB300(self.precision, name=self.name + "/precond")
        h = ctypes.c_void_p()
        check(lib().gfmd_make_preconditioner(self._handle(), shift, ctypes.byref(h)))
        out._h = h
        out.nx, out.ny, out.ndof = self.nx, self.ny, self.ndof
        return out

    def prec_gradient(self, cavg, g, gP) -> None:
        """gP = IFFT((Phi(q) + Cavg)^{-1} FFT(g)), [ndof, nx*ny] float64 CUDA
        tensors (gfmd_prec_gradient) or contiguous host arrays
        (gfmd_prec_gradient_host); Cavg is a symmetric ndof x ndof matrix
        (GFMDSolverStatic::prec_gradient)."""
        c = np.ascontiguousarray(np.broadcast_to(np.asarray(cavg, np.float64), (self.ndof, self.ndof)))
        if _is_device(g) != _is_device(gP):
            raise GFMDError(_lib.GFMD_EINVAL, "prec_gradient: g and gP must both be on the device or both on the host")
        if _is_device(g):
            check(lib().gfmd_prec_gradient(self._handle(), _ptr(c), _ptr(g), _ptr(gP)))
        else:
            check(lib().gfmd_prec_gradient_host(self._handle(), _ptr(c), _ptr(g), _ptr(gP)))

    def minimize(self, u, obstacle=None, method: str = "cg", ftol: float = 1e-6,
                 maxiter: int = 0, refine: "GFMDSolverGB300 | None" = None,
                 precond: "GFMDSolverGB300 | None" = None, dmax: float = 0.0, **fire) -> dict:
        """Static minimization from the displacements in u (CUDA float64
        tensor [ndof, nx*ny], updated in place); returns the report.  ``dmax``
        caps the CG's move of any component per line-search step (LAMMPS
        min_modify dmax; 0: no cap).  Raises GFMDError on failure (e.g.
        ENOTCONVERGED)."""
        p = _lib.MinParams()
        methods = {"cg": _lib.GFMD_MIN_CG, "fire": _lib.GFMD_MIN_FIRE, "tr": _lib.GFMD_MIN_TR}
        if method not in methods:
            raise ValueError(f"unknown method {method!r}")
        p.method = methods[method]
        p.ftol = ftol
        p.maxiter = maxiter
        p.refine = refine._handle().value if refine is not None else None
        p.precond = precond._handle().value if precond is not None else None
        p.dmax = dmax
        for k, v in fire.items():  # FIRE parameters by name; TR ones as tr_dmax, tr_rho_tol
            setattr(p, k if k.startswith("tr_") else "fire_" + k, v)
        rep = _lib.MinReport()
        ob = ctypes.byref(obstacle) if obstacle is not None else None
        rc = lib().gfmd_minimize(self._handle(), ob, ctypes.byref(p), _ptr(u), ctypes.byref(rep))
        if rc != _lib.GFMD_OK:
            err = GFMDError(rc, lib().gfmd_last_error().decode(errors="replace"))
            err.report = rep.as_dict()
            raise err
        return rep.as_dict()

    def run_dynamics(self, u, v, dt: float, gamma: float, nsteps: int, obstacle=None):
        """Damped velocity Verlet on CUDA float64 tensors u, v (in place);
        returns (energies[nsteps+1], report)."""
        e = np.zeros(nsteps + 1)
        rep = _lib.MinReport()
        ob = ctypes.byref(obstacle) if obstacle is not None else None
        check(lib().gfmd_run_dynamics(self._handle(), ob, dt, gamma, nsteps, _ptr(u), _ptr(v),
                                      _ptr(e), ctypes.byref(rep)))
        return e, rep.as_dict()

    def get_u0(self) -> np.ndarray:
        u0 = np.zeros(self.ndof)
        check(lib().gfmd_get_u0(self._handle(), _ptr(u0)))
        return u0

    def memory_usage(self) -> float:
        b = ctypes.c_double()
        check(lib().gfmd_memory_usage(self._handle(), ctypes.byref(b)))
        return b.value

    def info(self) -> dict:
        """Launches per force evaluation and whether the fused path runs."""
        n, f = ctypes.c_int(), ctypes.c_int()
        check(lib().gfmd_solver_info(self._handle(), ctypes.byref(n), ctypes.byref(f)))
        rb, pf = ctypes.c_int(), ctypes.c_int()
        check(lib().gfmd_plan_info(self._handle(), ctypes.byref(rb), ctypes.byref(pf)))
        rw, cl, pv = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().gfmd_kernel_plan(self._handle(), ctypes.byref(rw), ctypes.byref(cl), ctypes.byref(pv)))
        pat, npq = ctypes.c_int(), ctypes.c_int()
        check(lib().gfmd_phi_pattern(self._handle(), ctypes.byref(pat), ctypes.byref(npq)))
        return {"launches_per_eval": n.value, "fused": bool(f.value),
                "rows_per_block": rb.value, "phi_prefetch": pf.value,
                "row_warp_tma": bool(rw.value), "col_cluster": cl.value, "phi_vector": pv.value,
                "phi_pattern": pat.value, "phi_reals_per_wavevector": npq.value}

    def kernel_times(self, u, f, epot) -> list:
        """Device milliseconds of each launch of one evaluation of u (device
        buffers of the handle's arithmetic type), from CUDA events on the
        handle's stream."""
        n = self.ndof * self.nx * self.ny
        dt = "float64" if self.precision == "f64" else "float32"
        _check_device_array(u, dt, n, "u")
        _check_device_array(f, dt, n, "f")
        _check_device_array(epot, "float64", 1, "epot")
        ms = (ctypes.c_float * 16)()
        nk = ctypes.c_int()
        check(lib().gfmd_force_kernel_times(self._handle(), _ptr(u), _ptr(f), _ptr(epot), ms, 16,
                                            ctypes.byref(nk)))
        return [float(ms[i]) for i in range(nk.value)]

    def get_nxy_loc(self) -> int:
        return self.nx * self.ny

    def get_xlo_loc(self) -> int:
        return 0

    def get_xhi_loc(self) -> int:
        return self.nx - 1

    def get_ylo_loc(self) -> int:
        return 0

    def get_yhi_loc(self) -> int:
        return self.ny - 1

    # -- internals -----------------------------------------------------------
    def _handle(self) -> ctypes.c_void_p:
        if not self._h.value:
            raise GFMDError(_lib.GFMD_EINVAL, "set_grid_size has not been called")
        return self._h

    def _free(self) -> None:
        if self._h.value:
            lib().gfmd_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self._free()
        except Exception:
            pass


def minimize_batch(problems, ftol: float = 1e-6, maxiter: int = 0, recompute: int = 0):
    """Batched CG (gfmd_minimize_batch): ``problems`` is a list of
    (solver, u, obstacle_or_None, refine_solver_or_None[, precond]) with u a CUDA
    float64 tensor updated in place.  Returns the list of reports; raises
    GFMDError (with ``.reports``) if any item failed."""
    n = len(problems)
    items = (_lib.BatchItem * n)()
    keep = []
    for i, prob in enumerate(problems):
        s, u, ob, ref = prob[:4]
        pre = prob[4] if len(prob) > 4 else None
        items[i].handle = s._handle().value
        items[i].refine = ref._handle().value if ref is not None else None
        items[i].precond = pre._handle().value if pre is not None else None
        if ob is not None:
            items[i].obstacle = ctypes.pointer(ob)
            keep.append(ob)
        items[i].d_u = _ptr(u)
    p = _lib.MinParams()
    p.method = _lib.GFMD_MIN_CG
    p.ftol = ftol
    p.maxiter = maxiter
    p.recompute = recompute
    rc = lib().gfmd_minimize_batch(n, items, ctypes.byref(p))
    reports = [items[i].report.as_dict() for i in range(n)]
    if rc != _lib.GFMD_OK:
        err = GFMDError(rc, lib().gfmd_last_error().decode(errors="replace"))
        err.reports = reports
        raise err
    return reports


def atoms_to_grid(x, xeq, gid, nx, ny, ndof, box, u, v=None, vgrid=None, shift=(0, 0), check=True,
                  stream=0):
    """gfmd_atoms_to_grid on CUDA tensors: x, xeq, v [natoms, 3] float64, gid
    [natoms, 3] int32, u (and vgrid) [ndof, nx*ny] float64.  With ``check``
    the atoms must fill the grid slots one to one.  Returns the status."""
    import torch
    st = (ctypes.c_int * 3)()
    slots = torch.empty((ndof // 3) * nx * ny, dtype=torch.int32, device=u.device) if check else None
    rc = lib().gfmd_atoms_to_grid(x.shape[0], _ptr(x), _ptr(xeq), _ptr(v) if v is not None else None, _ptr(gid),
                                  nx, ny, ndof, float(box[0]), float(box[1]), int(shift[0]), int(shift[1]),
                                  _ptr(u), _ptr(vgrid) if vgrid is not None else None,
                                  _ptr(slots) if slots is not None else None, st, stream)
    status = {"bad_ids": st[0], "empty_slots": st[1], "duplicate_slots": st[2]}
    if rc != _lib.GFMD_OK:
        err = GFMDError(rc, lib().gfmd_last_error().decode(errors="replace"))
        err.status = status
        raise err
    return status


def grid_to_atoms(gid, f, nx, ny, ndof, fatoms, accumulate=False, stream=0):
    """gfmd_grid_to_atoms on CUDA tensors; returns the summed force (3,)."""
    s = (ctypes.c_double * 3)()
    check(lib().gfmd_grid_to_atoms(gid.shape[0], _ptr(gid), _ptr(f), nx, ny, ndof, _ptr(fatoms),
                                   1 if accumulate else 0, s, stream))
    return np.array(list(s))


_SOLVERS = {"static": "f64", "static/gb300": "f64", "static/gb300/f32": "f32"}


def gfmd_solver_factory(keyword: str | None = None, suffix: str | None = "gb300") -> GFMDSolverGB300:
    """Solver by name.  Like the reference, ``<name>/<suffix>`` is looked up
    when a suffix is active (src/main/gfmd_solver.cpp:215-221); the default
    style is ``static``."""
    name = keyword or "static"
    if suffix and not name.endswith("/" + suffix) and "/" not in name:
        name = f"{name}/{suffix}"
    if name not in _SOLVERS:
        raise GFMDError(_lib.GFMD_EINVAL, f"Unknown solver name encountered: '{name}'")
    return GFMDSolverGB300(precision=_SOLVERS[name], name=name)
