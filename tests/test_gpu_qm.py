"""tg_qm_load (QMMesh::LoadQM with InitM's detector placement and the
"external" lists' boundary projection) against what the compiled reference's
LoadQM made of the same files (tests/golden/qm_*.npz), its error paths, and
its positions and links driving a forward request."""
import numpy as np
import pytest

from tests.golden_util import load_qm, qm_names
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", qm_names())
def test_qm_load_matches_reference(name, tmp_path):
    g, path = load_qm(name, tmp_path)
    qm = capi.QM(capi.Mesh(g["coords"], g["elems"]), path)
    assert np.array_equal(qm.Q, g["qpos"])
    assert np.array_equal(qm.M, g["mpos"])
    assert np.array_equal(qm.links.ofs, g["link_ofs"])
    assert np.array_equal(qm.links.m, g["link_m"])


def _edit(text, old, new):
    assert old in text
    return text.replace(old, new, 1)


@pytest.mark.parametrize("change,code", [
    (lambda t: _edit(t, "QM file", "XX file"), capi.ERR_ARG),
    (lambda t: _edit(t, "Dimension 2", "Dimension 3"), capi.ERR_ARG),
    (lambda t: _edit(t, "MeasurementList 6", "MeasurementList 6 external"), capi.ERR_ARG),
    (lambda t: _edit(t, "SourceList 6", "SourceList 6 external"), capi.ERR_ARG),
    (lambda t: t[:t.index("LinkList")], capi.ERR_ARG),
    (lambda t: t.rstrip() + " 9\n", None),
    (lambda t: _edit(t, "LinkList\n6:", "LinkList\n6: 7"), capi.ERR_ARG),
], ids=["header", "dimension", "external_detector_without_normal", "external_source_without_normal",
        "no_linklist", "trailing", "detector_range"])
def test_qm_load_errors(change, code, tmp_path):
    g, path = load_qm("qm_disc_pull", tmp_path)
    mesh = capi.Mesh(g["coords"], g["elems"])
    bad = tmp_path / "bad.qm"
    bad.write_text(change(g["qm_text"]))
    if code is None:  # text after the last source's links is not read
        capi.QM(mesh, str(bad))
        return
    with pytest.raises(capi.ToastGPUError) as e:
        capi.QM(mesh, str(bad))
    assert e.value.code == code
    with pytest.raises(capi.ToastGPUError):
        capi.QM(mesh, str(tmp_path / "missing.qm"))


def test_qm_drives_a_request(tmp_path):
    """Loaded positions and links give the same request result as the same
    positions and links passed directly."""
    g, path = load_qm("qm_cyl_pull", tmp_path)
    mesh = capi.Mesh(g["coords"], g["elems"])
    qm = capi.QM(mesh, path)
    n = mesh.n
    cm, ck, ca = capi.optical_coefficients(np.full(n, 0.01), np.full(n, 1.0), np.full(n, 1.4))
    s = capi.FwdSolver(mesh, "BICGSTAB", 1e-12, "ICH", True, precision="fp64")
    q = mesh.qvec_gaussian(qm.Q, 2.0)
    m = mesh.qvec_gaussian(qm.M, 2.0) * ca[None, :]
    r1 = s.forward_path(cm, ck, ca, capi.omega_of(100.0), q, m, qm.links)
    q2 = mesh.qvec_gaussian(g["qpos"], 2.0)
    m2 = mesh.qvec_gaussian(g["mpos"], 2.0) * ca[None, :]
    r2 = s.forward_path(cm, ck, ca, capi.omega_of(100.0), q2, m2, capi.Links(g["link_ofs"], g["link_m"]))
    assert len(r1["logproj"]) == int(g["link_ofs"][-1])
    assert np.array_equal(r1["logproj"], r2["logproj"])
