"""Host-side logic with no GPU: file formats, link lists, parameter transform,
the seeded workloads."""
import os

import numpy as np
import pytest

from tests.conftest import REFERENCE, has_reference
from toastpp_gb300 import capi, meshio, workloads


def test_mesh_file_round_trip(tmp_path):
    for P in [workloads.disc(6, 1, 0.0, 4), workloads.cylinder(rings=3, layers=4, seed=2)]:
        f = tmp_path / "m.msh"
        meshio.write_mesh(str(f), P.coords, P.elems)
        c, e = meshio.read_mesh(str(f))
        assert np.allclose(c, P.coords, rtol=0, atol=1e-12 * np.abs(P.coords).max())
        assert np.array_equal(e, P.elems)


def test_qm_file_round_trip(tmp_path):
    P = workloads.disc(6, 1, 0.0, 4)
    f = tmp_path / "a.qm"
    meshio.write_qm(str(f), P.qm)
    qm = meshio.read_qm(str(f))
    assert np.allclose(qm.Q, P.qm.Q) and np.allclose(qm.M, P.qm.M)
    assert np.array_equal(qm.link_ofs, P.qm.link_ofs) and np.array_equal(qm.link_m, P.qm.link_m)


def test_qm_list_flags_and_normals(tmp_path):
    """The list flags and normals of a QM file (qmmesh.cc:338-347, 399-408):
    "fixed" / "external" as the second header token, "default" normals as
    the third; a normal read with a position where one is given, 0
    elsewhere."""
    f = tmp_path / "e.qm"
    f.write_text("QM file 2D\nDimension 2\n\nSourceList 2 External default\n1 2 0.5 -0.5\n3 4\n\n"
                 "MeasurementList 2 external\n5 6 0 1\n7 8 1 0\n\nLinkList\n1: 0\n2: 0 1\n")
    qm = meshio.read_qm(str(f))
    assert qm.q_external and qm.q_default_normals and not qm.q_fixed
    assert qm.m_external and not qm.m_default_normals
    assert np.array_equal(qm.Q, [[1, 2], [3, 4]]) and np.array_equal(qm.QN, [[0.5, -0.5], [0, 0]])
    assert np.array_equal(qm.MN, [[0, 1], [1, 0]])
    assert list(qm.link_ofs) == [0, 1, 3] and list(qm.link_m) == [0, 0, 1]
    f.write_text("QM file 2D\nDimension 2\n\nSourceList 1 fixed\n1 2\n\nMeasurementList 1\n5 6\n\n"
                 "LinkList\n1: 0\n")
    qm = meshio.read_qm(str(f))
    assert qm.q_fixed and not qm.q_external and not qm.m_fixed and not qm.m_external


@pytest.mark.skipif(not has_reference(), reason="reference tree not available")
def test_reads_reference_meshes():
    c, e = meshio.read_mesh(os.path.join(REFERENCE, "test", "2D", "meshes", "circle25_32.msh"))
    assert c.shape == (3511, 2) and e.shape == (6840, 3)
    c, e = meshio.read_mesh(os.path.join(REFERENCE, "test", "3D", "meshes", "cyl2.msh"))
    assert c.shape == (9043, 3) and e.shape == (45438, 4)
    qm = meshio.read_qm(os.path.join(REFERENCE, "test", "2D", "meshes", "circle25_32x32.qm"))
    assert qm.nQ == 32 and qm.nM == 32 and qm.nQM == 1024


def test_links_all_to_all():
    L = capi.Links.all_to_all(3, 4)
    assert L.nqm == 12 and list(L.ofs) == [0, 4, 8, 12] and list(L.m[:5]) == [0, 1, 2, 3, 0]
    qm = meshio.QMSpec.all_to_all(np.zeros((3, 2)), np.zeros((4, 2)))
    assert np.array_equal(qm.link_ofs, L.ofs) and np.array_equal(qm.link_m, L.m)


def test_parameter_transform_matches_oracle(oracle_mod):
    rng = np.random.default_rng(0)
    mua = rng.uniform(0.005, 0.05, 50)
    mus = rng.uniform(0.5, 3.0, 50)
    nref = rng.uniform(1.3, 1.5, 50)
    a = capi.optical_coefficients(mua, mus, nref)
    b = oracle_mod.optical_coefficients(mua, mus, nref)
    for x, y in zip(a, b):
        assert np.allclose(x, y, rtol=1e-14, atol=0)
    assert capi.omega_of(100.0) == pytest.approx(6.283185307179586e-4, rel=1e-15)


def test_workloads_are_seeded_and_sized():
    a = workloads.disc(32, 0, 0.0, 16)
    b = workloads.disc(32, 0, 0.0, 16)
    assert np.array_equal(a.coords, b.coords) and np.array_equal(a.mua, b.mua)
    assert a.n == 3169 and a.qm.nQ == 16 and a.qm.nQM == 256
    c = workloads.cylinder(seed=0)
    assert c.n == 30810 and c.elems.shape == (169128, 4) and c.qm.nQ == 80 and c.qm.nM == 80


def test_elements_positively_oriented():
    for P in [workloads.disc(8, 3, 0.0, 4), workloads.cylinder(rings=4, layers=5, seed=1)]:
        x = P.coords[P.elems]
        if P.dim == 2:
            v = (x[:, 1, 0] - x[:, 0, 0]) * (x[:, 2, 1] - x[:, 0, 1]) - (x[:, 2, 0] - x[:, 0, 0]) * (x[:, 1, 1] - x[:, 0, 1])
        else:
            v = np.einsum("ij,ij->i", np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]), x[:, 3] - x[:, 0])
        assert np.all(v > 0)
