"""Element basis on the GPU: Reset with one coefficient per element and the
element-basis Jacobian, against the compiled reference's own outputs
(tests/golden/*_el.npz) and the oracle."""
import numpy as np
import pytest

from tests.golden_util import load, names, sparse_links
from tests.gpu_util import rel2, relmax
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu

ELEM = [n for n in names() if n.endswith("_el")]


def setup(name, precision="fp64"):
    g = load(name)
    gm = capi.Mesh(g["coords"], g["elems"])
    cplx = np.iscomplexobj(g["proj"])
    s = capi.FwdSolver(gm, g["solver"], 1e-15, g["precon"], cplx, precision=precision)
    cm, ck, ca = capi.optical_coefficients(g["elmua"], g["elmus"], g["elnref"])
    s.reset_elbasis(cm, ck, ca, capi.omega_of(g["freq_mhz"]))
    return g, gm, s, capi.Links(g["link_ofs"], g["link_m"])


@pytest.mark.parametrize("name", ELEM)
def test_element_basis_assembly(name):
    """Entries agree to 1e-14 of the largest; off-diagonal entries where the
    mass and stiffness terms nearly cancel agree to 1e-11 relative (the
    device sums round with fused multiply-adds)."""
    g, gm, s, L = setup(name)
    A = s.system_matrix()
    assert np.abs(A - g["sysval"]).max() <= 1e-14 * np.abs(g["sysval"]).max()
    assert relmax(A, g["sysval"]) < 1e-11


@pytest.mark.parametrize("name", ELEM)
def test_element_jacobian_on_reference_fields(name):
    g, gm, s, L = setup(name)
    J = s.jacobian_el(g["dphi"], g["aphi"], g["proj"], L)
    assert J.shape == g["Jel"].shape
    assert rel2(J, g["Jel"]) < 1e-13
    J32 = s.jacobian_el(g["dphi"], g["aphi"], g["proj"], L, fp32=True)
    assert rel2(J32.astype(np.float64), g["Jel"]) < 1e-5


@pytest.mark.parametrize("name", ELEM)
def test_element_jacobian_linear_data_against_oracle(name, oracle_mod):
    g, gm, s, L = setup(name)
    J = s.jacobian_el(g["dphi"], g["aphi"], None, L, scale=capi.DATA_LIN)
    om = oracle_mod.Mesh(g["coords"], g["elems"])
    ref = oracle_mod.jacobian_el(om, g["dphi"], g["aphi"], g["proj"], g["link_ofs"], g["link_m"], logscale=False)
    assert rel2(J, ref) < 1e-13


@pytest.mark.parametrize("name", ELEM)
def test_element_jacobian_sparse_links_against_oracle(name, oracle_mod):
    """Links missing for some (source, detector) pairs and a source without
    any, with a source count that leaves a partial group of sources."""
    g, gm, s, L = setup(name)
    ofs, lm, keep = sparse_links(g)
    J = s.jacobian_el(g["dphi"], g["aphi"], g["proj"][keep], capi.Links(ofs, lm))
    om = oracle_mod.Mesh(g["coords"], g["elems"])
    ref = oracle_mod.jacobian_el(om, g["dphi"], g["aphi"], g["proj"][keep], ofs, lm)
    assert J.shape == ref.shape == (2 * len(keep), g["Jel"].shape[1])
    assert rel2(J, ref) < 1e-13


@pytest.mark.parametrize("name", ELEM)
def test_element_basis_end_to_end(name):
    """Element-basis reset, GPU FP64 fields, projections and element-basis
    Jacobian against the reference's."""
    g, gm, s, L = setup(name)
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    q = gm.qvec_gaussian(g["Q"], g["qwidth"])
    m = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    dphi, _ = s.calc_fields(q)
    aphi, _ = s.calc_fields(m)
    proj = s.project_all(m, dphi, L, capi.DATA_LIN)
    assert relmax(proj, g["proj"]) < 1e-8
    J = s.jacobian_el(dphi, aphi, proj, L)
    assert rel2(J, g["Jel"]) < 1e-9
