"""The C-ABI library: loads, exports every declared entry point, rejects bad
arguments before touching a GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, gfmd_pkg


def _declared():
    src = open(os.path.join(ROOT, "include", "gfmd_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gfmd_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = gfmd_pkg().lib()
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n


def test_python_binding_covers_the_header():
    from importlib import import_module

    sig = import_module("user-gfmd_gb300._lib").SIGNATURES
    assert sorted(sig) == _declared()


def test_argument_errors_return_status_without_gpu():
    L = gfmd_pkg().lib()
    h = ctypes.c_void_p()
    assert L.gfmd_create(0, 8, 3, 0, ctypes.byref(h)) == 1
    assert L.gfmd_create(8, 8, 4, 0, ctypes.byref(h)) == 1
    assert L.gfmd_create(8, 8, 27, 0, ctypes.byref(h)) == 1
    assert L.gfmd_create(8, 8, 3, 7, ctypes.byref(h)) == 1
    assert L.gfmd_create(8, 8, 3, 0, None) == 1
    assert L.gfmd_destroy(None) == 1
    assert L.gfmd_post_force(None, None, None, None) == 1
    assert L.gfmd_set_phi(None, None, 0, None) == 1
    assert b"NULL" in L.gfmd_last_error()
    c = (ctypes.c_double * 9)()
    assert L.gfmd_prec_gradient(None, c, None, None) == 1
    assert L.gfmd_prec_gradient_host(None, c, None, None) == 1
    assert L.gfmd_kernel_set_box(None, 1.0, 1.0) == 1
    assert L.gfmd_minimize(None, None, None, None, None) == 1


# Every entry point that takes a handle, or sizes and pointers, rejects NULL
# handles, NULL outputs and impossible sizes with GFMD_EINVAL and a message,
# before any CUDA call (this host has no GPU): nothing aborts or exits.
_BAD_CALLS = {
    "gfmd_set_stream": (None, None),
    "gfmd_post_force_host": (None, None, None, None),
    "gfmd_force_f64": (None, None, None, None),
    "gfmd_force_f32": (None, None, None, None),
    "gfmd_get_u0": (None, None),
    "gfmd_plan_info": (None, None, None),
    "gfmd_memory_usage": (None, None),
    "gfmd_solver_info": (None, None, None),
    "gfmd_phi_pattern": (None, None, None),
    "gfmd_make_preconditioner": (None, 0.0, None),
    "gfmd_minimize_batch": (0, None, None),
    "gfmd_run_dynamics": (None, None, 0.01, 0.0, 10, None, None, None, None),
    "gfmd_obstacle_force": (0, 8, 3, None, None, None, None, None),
    "gfmd_post_force_noalloc": (0, 8, 3, None, None, None, None, None, None),
    "gfmd_kernel_create": (None, None),
    "gfmd_kernel_destroy": (None,),
    "gfmd_kernel_info": (None, None, None),
    "gfmd_kernel_phi": (None, 8, 8, 0, None, None, 0),
    "gfmd_atoms_to_grid": (-1, None, None, None, None, 8, 8, 3, 8.0, 8.0, 0, 0, None, None, None, None, None),
    "gfmd_grid_to_atoms": (-1, None, None, 8, 8, 3, None, 0, None, None),
    "gfmd_rough_surface": (0, 8, None, None, None),
    "gfmd_ws_create": (0, 0, 0, 0, None),
    "gfmd_ws_destroy": (None,),
    "gfmd_ws_set_stream": (None, None),
    "gfmd_ws_num_params": (None, None),
    "gfmd_ws_get_params": (None, None, None),
    "gfmd_ws_set_params": (None, None),
    "gfmd_ws_forward": (None, 1, 8, 8, None, None),
    "gfmd_ws_adam_step": (None, 1e-3, 0.9, 0.999, 1e-8),
}


@pytest.mark.parametrize("name", sorted(_BAD_CALLS))
def test_every_entry_point_rejects_bad_arguments_without_gpu(name):
    L = gfmd_pkg().lib()
    assert getattr(L, name)(*_BAD_CALLS[name]) == 1  # GFMD_EINVAL
    assert L.gfmd_last_error().startswith(name.encode() + b":")


def test_solver_factory_names():
    g = gfmd_pkg()
    assert g.gfmd_solver_factory().get_name() == "static/gb300"
    assert g.gfmd_solver_factory("static").get_name() == "static/gb300"
    assert g.gfmd_solver_factory("static/gb300/f32").precision == "f32"
    with pytest.raises(g.GFMDError):
        g.gfmd_solver_factory("nosuch")


# ctypes mirror -> C typedef of include/gfmd_gb300.h
_STRUCTS = {"Obstacle": "gfmd_obstacle_t", "MinParams": "gfmd_min_params_t",
            "MinReport": "gfmd_min_report_t", "BatchItem": "gfmd_batch_item_t",
            "SurfaceParams": "gfmd_surface_params_t"}


def test_ctypes_structs_match_the_c_layout(tmp_path):
    # sizeof and every field's offset, from the C compiler on the header
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from importlib import import_module

    lib = import_module("user-gfmd_gb300._lib")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gfmd_gb300.h"', "int main(void) {"]
    for py, c in _STRUCTS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in getattr(lib, py)._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        py, name, v = line.split()
        got[(py, name)] = int(v)
    for py in _STRUCTS:
        S = getattr(lib, py)
        assert got[(py, "size")] == ctypes.sizeof(S), py
        for name, _ in S._fields_:
            assert got[(py, name)] == getattr(S, name).offset, (py, name)


def test_device_buffer_dtype_is_checked_before_the_c_abi():
    # a float32 tensor handed to an entry that reads doubles would be read as
    # the wrong numbers; the Python mirror refuses it (CPU tensors suffice)
    torch = pytest.importorskip("torch")
    from importlib import import_module

    chk = import_module("user-gfmd_gb300.solver")._check_device_array
    chk(torch.zeros(12, dtype=torch.float64), "float64", 12, "u")
    with pytest.raises(TypeError):
        chk(torch.zeros(12, dtype=torch.float32), "float64", 12, "u")
    with pytest.raises(TypeError):
        chk(torch.zeros(4, 6, dtype=torch.float64).t(), "float64", 12, "u")
    with pytest.raises(ValueError):
        chk(torch.zeros(11, dtype=torch.float64), "float64", 12, "u")


def test_timing_and_plan_entries_reject_bad_arguments_without_gpu():
    L = gfmd_pkg().lib()
    nk = ctypes.c_int()
    ms = (ctypes.c_float * 4)()
    assert L.gfmd_force_kernel_times(None, None, None, None, ms, 4, ctypes.byref(nk)) == 1
    assert L.gfmd_kernel_plan(None, None, None, None) == 1
