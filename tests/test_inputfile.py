"""Input-format reader/writer (InputT.cpp semantics) and the mesh generators."""
import numpy as np
import pytest

from conftest import load_golden
from tdbem import inputfile, meshes


def test_reference_bar1_parses():
    z, m = load_golden("ref_bar1")
    assert (m.nnd, m.nel, m.etype, m.numstep) == (24, 22, 1, 10)
    assert m.dt == 1e-3 and m.E == 1e6 and m.nu == 0 and m.rho == 1
    assert list(m.ubc_dofs[:6]) == [0, 1, 2, 3, 4, 5]
    assert list(m.fbc_dofs) == [6, 21, 39, 54]
    assert m.ien[0].tolist() == [1, 0, 6, 8]


def test_roundtrip_is_exact():
    m = meshes.bar(1, 1, 4, per_unit=2)
    m2 = inputfile.parse(inputfile.dumps(m))
    assert np.array_equal(m.coords, m2.coords) and np.array_equal(m.ien, m2.ien)
    assert np.array_equal(m.fbc_vals, m2.fbc_vals) and m.dt == m2.dt and m.E == m2.E


def test_unknown_keyword_is_an_error():
    with pytest.raises(inputfile.InputError):
        inputfile.parse("numstep=3;\nbogus=1;\n")


def test_c_number_parsing():
    assert inputfile.c_atoi("12abc") == 12 and inputfile.c_atoi("1e6") == 1
    assert inputfile.c_atof("2.5e-3;") == 2.5e-3 and inputfile.c_atof("x") == 0.0


def test_bar_mesh_counts_and_bcs():
    m = meshes.bar(1, 1, 4, per_unit=2)
    assert (m.nel, m.nnd, m.ndof, m.max_step()) == (72, 74, 222, 26)
    assert len(m.ubc_dofs) == 27 and len(m.fbc_dofs) == 9
    for q in m.ien:  # outward normals
        p = m.coords[q]
        n = np.cross(p[1] - p[0], p[3] - p[0])
        assert np.dot(n, p.mean(0) - np.array([0.5, 0.5, 2.0])) > 0


def test_cubed_sphere_counts_and_orientation():
    m = meshes.cubed_sphere(16)
    assert (m.nel, m.nnd, m.ndof, m.if_ext) == (1536, 1538, 4614, 1)
    assert np.allclose(np.linalg.norm(m.coords, axis=1), 1.0)
    p = m.coords[m.ien]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 3] - p[:, 0])
    assert (np.einsum("ij,ij->i", n, p.mean(1)) < 0).all()  # into the cavity
    assert abs(m.dt - 0.6 * (np.pi / 32) / np.sqrt(3)) < 1e-15


def test_closed_form_static_limit():
    u = meshes.sphere_cavity_closed_form(np.array([0.0, 1e-9, 60.0]))
    assert u[0] == 0 and abs(u[-1] - 0.25) < 1e-6
