"""Reference file formats: height maps (FixWallMap::read_map/write_map) and
the real- and reciprocal-space grid dumps (FixGFMD::dump,
GFMDSolverFFT::dump)."""
import importlib

import numpy as np
import pytest

from conftest import gfmd_pkg, half_to_full, oracle_post_force

fmt = importlib.import_module("user-gfmd_gb300.formats")


def test_map_round_trip_and_reference_column_rule(tmp_path):
    rng = np.random.default_rng(1)
    z = rng.normal(0, 1, (12, 12))
    p = tmp_path / "map.matrix"
    fmt.write_map(str(p), z)
    lines = p.read_text().splitlines()
    assert len(lines) == 12 and lines[0].endswith(" ") and "%f " % z[0, 0] in lines[0]
    back = fmt.read_map(str(p))
    assert back.shape == (12, 12)
    assert np.allclose(back, z, atol=5e-7)  # "%f" keeps six decimals
    # the reader counts columns in the first line and assumes a square map
    p.write_text("1 2 3\n4 5 6\n7 8 9\n10 11\n")
    assert np.array_equal(fmt.read_map(str(p)), np.arange(1, 10, dtype=float).reshape(3, 3))
    p.write_text("1 2 3")
    with pytest.raises(ValueError):
        fmt.read_map(str(p))


def test_real_space_dump_layout(tmp_path):
    nx, ny, d = 4, 3, 3
    rng = np.random.default_rng(2)
    u = rng.normal(0, 1, (d, nx * ny))
    f = rng.normal(0, 1, (d, nx * ny))
    base = fmt.write_real_space_dump(str(tmp_path / "gfmd"), 100, u, f, nx, ny)
    assert base.endswith("gfmd.100")
    first = (tmp_path / "gfmd.100.r.u0.out").read_text().splitlines()
    assert len(first) == ny  # one line per iy, nx values
    assert first[0] == "".join(" %20.10e " % u[0, ix * ny] for ix in range(nx))
    for i in range(d):
        assert np.allclose(fmt.read_grid(f"{base}.r.u{i}.out", nx, ny), u[i], rtol=1e-9)
        assert np.allclose(fmt.read_grid(f"{base}.r.f{i}.out", nx, ny), f[i], rtol=1e-9)
    assert np.allclose(fmt.read_grid(f"{base}.r.e.out", nx, ny), (u * f).sum(0), rtol=1e-9)


def test_q_space_dump_matches_the_force_evaluation(tmp_path):
    nx, ny = 8, 6
    k = gfmd_pkg().StiffnessKernel("ft fcc100 1.0 2 pair-potential 1 1.0 height 16")
    d = k.get_dimension()
    half, linf = k.phi_table(nx, ny, "half")
    full = half_to_full(half, nx, ny)
    assert np.allclose(fmt.half_to_full(half, nx, ny), full)
    rng = np.random.default_rng(3)
    u = rng.normal(0, 0.1, (d, nx * ny))
    fmt.write_q_space_dump(str(tmp_path / "dq"), u, full, nx, ny)
    Fr = np.stack([fmt.read_grid(str(tmp_path / f"dq.q.f{i}.real.out"), nx, ny) for i in range(d)])
    Fi = np.stack([fmt.read_grid(str(tmp_path / f"dq.q.f{i}.imag.out"), nx, ny) for i in range(d)])
    # f(r) = -sum_q F(q) exp(+i q.r) is the oracle force (no gamma-point term)
    fq = -np.fft.ifft2((Fr + 1j * Fi).reshape(d, nx, ny)).real.reshape(d, nx * ny) * nx * ny
    f_ref, _, _ = oracle_post_force(full, np.zeros(d // 3), u, nx, ny)
    assert np.allclose(fq, f_ref, rtol=1e-8, atol=1e-9 * np.abs(f_ref).max())  # 11 digits in the file
    e = fmt.read_grid(str(tmp_path / "dq.q.e.out"), nx, ny).sum()
    _, E, _ = oracle_post_force(full, np.zeros(d // 3), u, nx, ny)
    assert abs(0.5 * e - E) <= 1e-8 * abs(E)  # E = 1/2 sum Re(u conj F) with no linf


@pytest.mark.gpu
def test_post_force_writes_the_q_space_dump(tmp_path):
    nx, ny = 16, 12
    g = gfmd_pkg()
    k = g.StiffnessKernel("ft fcc100 1.0 2 pair-potential 1 1.0 height 16")
    s = g.gfmd_solver_factory("static")
    s.set_grid_size(nx, ny, k.get_dimension())
    s.set_kernel(k)
    u = np.random.default_rng(4).normal(0, 0.1, (k.get_dimension(), nx * ny))
    f = np.empty_like(u)
    s.post_force(u, f, dump_prefix=str(tmp_path / "step"))
    assert (tmp_path / "step.q.u0.real.out").exists() and (tmp_path / "step.q.e.out").exists()


def _dump_fixtures():
    import glob
    import os
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "dumps", "*.npz")))


def _check_dump_dir(directory, c):
    # same files, same line and column layout, values within the "%e" digits
    # (noise-level entries of a table, ~1e-18, differ between any two
    # computations of it, hence a floor at 1e-12 of the dump's largest value)
    import os
    want = {k[5:]: str(c[k]) for k in c if k.startswith("file:")}
    stem = "g" if any(k.startswith("g") for k in os.listdir(directory)) else "phi"
    mine = {fn: open(os.path.join(directory, fn)).read() for fn in os.listdir(directory)}
    assert set(mine) == {k for k in want if k.startswith(stem)}
    scale = max(np.abs(np.array(want[fn].split(), float)).max(initial=0.0) for fn in mine)
    for fn, text in mine.items():
        ref = want[fn]
        assert [len(l.split()) for l in text.split("\n")] == [len(l.split()) for l in ref.split("\n")]
        assert all(l == "" or (l.startswith(" ") and l.endswith(" ")) for l in text.split("\n"))
        a = np.array(text.split(), float)
        b = np.array(ref.split(), float)
        if b.size:
            assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max() + 1e-12 * scale


@pytest.mark.parametrize("path", _dump_fixtures(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_stiffness_and_greens_dumps_match_the_reference(path, tmp_path):
    from conftest import kernel_for, load_golden
    c = load_golden(path)
    nx, ny = int(c["nx"]), int(c["ny"])
    full, _ = kernel_for(c).phi_table(nx, ny, "full")
    for greens in (False, True):
        d = tmp_path / ("g" if greens else "phi")
        d.mkdir()
        fmt.write_stiffness_dump(str(d), full, nx, ny, greens=greens)
        _check_dump_dir(str(d), c)


@pytest.mark.gpu
def test_solver_dump_stiffness_and_greens_function(tmp_path):
    from conftest import kernel_for, load_golden
    path = _dump_fixtures()[0]
    c = load_golden(path)
    nx, ny = int(c["nx"]), int(c["ny"])
    k = kernel_for(c)
    s = gfmd_pkg().gfmd_solver_factory("static/gb300")
    s.set_grid_size(nx, ny, k.get_dimension())
    s.set_kernel(k)
    for greens in (False, True):
        d = tmp_path / ("g" if greens else "phi")
        d.mkdir()
        (s.dump_greens_function if greens else s.dump_stiffness)(str(d))
        _check_dump_dir(str(d), c)


def test_filter_map_keeps_long_and_removes_short_wavelengths():
    nx, ny = 48, 40
    x = np.arange(nx)[:, None]
    y = np.arange(ny)[None, :]
    long_ = 0.3 * np.cos(2 * np.pi * 2 * x / nx) + 0.2 * np.sin(2 * np.pi * 3 * y / ny)
    short = 0.1 * np.cos(2 * np.pi * (9 * x / nx + 7 * y / ny))
    z = 1.5 + long_ + short
    # box 2 length units per pixel: mode (2, 0) has |q| = 2/96, mode (9, 7)
    # sqrt((9/96)^2 + (7/80)^2) = 0.128; cut at wavelength 10 (|q| = 0.1)
    out = fmt.filter_map(z, 10.0, xprd=2.0 * nx, yprd=2.0 * ny)
    assert np.abs(out - (1.5 + long_)).max() < 1e-13
    assert np.abs(fmt.filter_map(z, 1.0, 2.0 * nx, 2.0 * ny) - z).max() < 1e-13  # cut above every mode
    with pytest.raises(ValueError):
        fmt.filter_map(z, 0.0)


def test_displace_map_alignment_and_statistics():
    z = np.random.default_rng(5).normal(0.3, 0.2, (16, 16))
    for align, key in (("bottom", "min"), ("top", "max"), ("average", "mean")):
        out, info = fmt.displace_map(z, -1.25, align)
        assert abs(info[key] + 1.25) < 1e-14
        assert abs(info["rms"] - z.std()) < 1e-14
        assert np.allclose(out - z, out[0, 0] - z[0, 0])
    assert abs(fmt.displace_map(z, 0.0, "bottom")[0].min()) < 1e-15
    with pytest.raises(ValueError):
        fmt.displace_map(z, 0.0, "middle")
