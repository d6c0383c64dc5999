"""Host-side Phi(q) table producer against the reference's fill_phi_buffer."""
import os

import numpy as np
import pytest

from conftest import golden_cases, gfmd_pkg, kernel_for, load_golden


def _table_cases():
    """Fixtures that carry the reference's full Phi table: the `ft` style and
    the analytic sc100 and fcc100 styles."""
    out = []
    for p in golden_cases():
        c = load_golden(p)
        if "phi" in c:
            out.append(p)
    return out


@pytest.mark.parametrize("path", _table_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_phi_table_matches_reference(path):
    c = load_golden(path)
    nx, ny = int(c["nx"]), int(c["ny"])
    k = kernel_for(c)
    assert k.get_dimension() == int(c["ndof"])
    assert k.get_height() == int(c["height"])
    phi, linf = k.phi_table(nx, ny, "full")
    ref = c["phi"]
    # per wavevector, relative to that wavevector's matrix norm
    num = np.linalg.norm((phi - ref).reshape(nx * ny, -1), axis=1)
    den = np.linalg.norm(ref.reshape(nx * ny, -1), axis=1)
    assert (num / den).max() <= 1e-12
    assert np.array_equal(linf, c["linf"])


def test_phi_half_layout_is_a_slice_of_full():
    k = gfmd_pkg().StiffnessKernel("ft fcc111 1 1.0 pair-potential 1 1.0 height 16")
    full, _ = k.phi_table(6, 8, "full")
    half, _ = k.phi_table(6, 8, "half")
    assert np.array_equal(full.reshape(6, 8, 6, 6)[:, :5], half)


def test_pair_potential_linf_keyword_gives_zero_gamma_force():
    # FCPairPotential::linear does not override ForceConstants::linear in the
    # reference, so the gamma-point force of `ft ... pair-potential ... linf`
    # is zero; the values must still sum to zero.
    k = gfmd_pkg().StiffnessKernel("ft fcc100 1.0 2 pair-potential 1 1.0 linf 2 0.1 -0.1 height 4")
    assert np.array_equal(k.get_force_at_gamma_point(), np.zeros(2))
    g = gfmd_pkg()
    with pytest.raises(g.GFMDError):
        g.StiffnessKernel("ft fcc100 1.0 2 pair-potential 1 1.0 linf 2 0.1 0.1 height 4")


@pytest.mark.parametrize(
    "args",
    [
        "",
        "nosuchkernel 1 2",
        "ft",
        "ft sc100",
        "ft nosuchsurface 1.0 1 pair-potential 1 1.0",
        "ft sc100 1.0 1",
        "ft sc100 1.0 1 lj/cut 1",
        "ft sc100 abc 1 pair-potential 1 1.0",
        "ft sc100 1.0 1 pair-potential 1 1.0 height 8 extra",
        "ft sc100 1.0 1 pair-potential 4 1 1 1 1",
        "fcc100",
        "fcc100 5 1.0",
        "fcc100 2 1.0 0.3",
        "fcc100 x 1 1.0",
        "fcc100 1 abc",
        "fcc100 2 1.0 0 0 normal 0",
        "fcc100 1 1.0 height 4 extra",
        "sc100 extra",
    ],
)
def test_malformed_kernel_arguments_raise(args):
    g = gfmd_pkg()
    with pytest.raises(g.GFMDError) as ei:
        g.StiffnessKernel(args)
    assert ei.value.code == 1


def test_analytic_fcc100_linf_is_the_gamma_point_force():
    # FCC100StiffnessKernel::get_force_at_gamma_point returns the `linf`
    # values (fcc100_stiffness.cpp:482-487); they must sum to zero
    g = gfmd_pkg()
    k = g.StiffnessKernel("fcc100 2 1.0 0.0 0.0 linf 0.05 -0.05 height 4")
    assert np.array_equal(k.get_force_at_gamma_point(), np.array([0.05, -0.05]))
    assert k.get_dimension() == 6
    with pytest.raises(g.GFMDError):
        g.StiffnessKernel("fcc100 2 1.0 0.0 0.0 linf 0.1 0.1")


def test_singular_nn_only_simple_cubic_is_reported():
    # central nearest-neighbour springs on sc carry no shear: the reference
    # aborts with "Singular matrix in complex GaussJordan"
    g = gfmd_pkg()
    k = g.StiffnessKernel("ft sc100 1.0 1 pair-potential 1 1.0 height 16")
    with pytest.raises(g.GFMDError):
        k.phi_table(4, 4, "half")


def test_phi_is_hermitian_and_inversion_symmetric():
    k = gfmd_pkg().StiffnessKernel("ft fcc100 1.0 4 pair-potential 1 1.0 height 8")
    nx, ny = 6, 10
    phi, _ = k.phi_table(nx, ny, "full")
    assert np.abs(phi - np.conj(np.swapaxes(phi, 1, 2))).max() < 1e-15
    P = phi.reshape(nx, ny, 12, 12)
    Pm = P[(-np.arange(nx)) % nx][:, (-np.arange(ny)) % ny]
    assert np.abs(Pm - np.conj(P)).max() < 1e-15


def test_phi_table_cache_round_trip(tmp_path):
    g = gfmd_pkg()
    k = g.StiffnessKernel("ft fcc100 1.0 2 pair-potential 1 1.0 height 16")
    phi, linf = k.phi_table_cached(16, 12, str(tmp_path))
    files = list(tmp_path.iterdir())
    assert len(files) == 1
    phi2, linf2 = k.phi_table_cached(16, 12, str(tmp_path))  # from the file
    assert np.array_equal(phi, phi2) and np.array_equal(linf, linf2)
    ref, _ = k.phi_table(16, 12, "half")
    assert np.array_equal(phi, ref)
    # a different kernel, grid or layout is a different key; a corrupt file is a miss
    assert g.PhiTableFile.read(str(files[0]), "ft fcc100 1.0 2 pair-potential 1 1.0 height 17", 16, 12, "half") is None
    assert g.PhiTableFile.read(str(files[0]), k.args, 16, 14, "half") is None
    files[0].write_bytes(files[0].read_bytes()[:100])
    assert g.PhiTableFile.read(str(files[0]), k.args, 16, 12, "half") is None
    phi3, _ = k.phi_table_cached(16, 12, str(tmp_path))
    assert np.array_equal(phi3, ref)


def test_phi_table_cache_keys_on_the_box(tmp_path):
    # the continuum styles read the box lengths; tables for different boxes
    # are different cache entries
    g = gfmd_pkg()
    a = g.StiffnessKernel("nonperiodic 0.3 1.0")
    b = g.StiffnessKernel("nonperiodic 0.3 1.0")
    b.set_box(24.0, 20.0)
    pa, _ = a.phi_table_cached(12, 10, str(tmp_path))
    pb, _ = b.phi_table_cached(12, 10, str(tmp_path))
    assert len(list(tmp_path.iterdir())) == 2
    assert not np.allclose(pa, pb)
    ref, _ = b.phi_table(12, 10, "half")
    assert np.array_equal(b.phi_table_cached(12, 10, str(tmp_path))[0], ref)
