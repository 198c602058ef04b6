"""A solver keeps the last link list it was given, validated and copied to
the device, and reuses both while the same list comes back.  Calls that
alternate between lists, edit a list in place, or move the solver to
another stream give the results of a fresh solver."""
import numpy as np
import pytest

from tests.golden_util import load, sparse_links
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu


def _setup(name="disc_fd_grid"):
    g = load(name)
    gm = capi.Mesh(g["coords"], g["elems"])
    cplx = np.iscomplexobj(g["proj"])
    s = capi.FwdSolver(gm, g["solver"], 1e-15, g["precon"], cplx, precision="fp64")
    return g, gm, s


def test_alternating_link_lists():
    g, gm, s = _setup()
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    m = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    A = capi.Links(g["link_ofs"], g["link_m"])
    ofs, lm, keep = sparse_links(g)
    B = capi.Links(ofs, lm)
    r = capi.Raster(gm, g["bdim"])

    def run(solver, L, proj):
        return (solver.project_all(m, g["dphi"], L, capi.DATA_LIN),
                solver.jacobian(g["dphi"], g["aphi"], proj, L),
                solver.jacobian_grid(r, g["dphi"], g["aphi"], proj, L))

    ref = {}
    for key, L, proj in (("A", A, g["proj"]), ("B", B, g["proj"][keep])):
        ref[key] = run(capi.FwdSolver(gm, g["solver"], 1e-15, g["precon"], True, precision="fp64"), L, proj)
    for key, L, proj in (("A", A, g["proj"]), ("A", A, g["proj"]), ("B", B, g["proj"][keep]),
                         ("A", A, g["proj"]), ("B", B, g["proj"][keep])):
        for got, want in zip(run(s, L, proj), ref[key]):
            assert np.array_equal(got, want), key


def test_list_edited_in_place_and_new_stream():
    g, gm, s = _setup()
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    m = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    ofs = np.array(g["link_ofs"], np.int32)
    lm = np.array(g["link_m"], np.int32)
    L = capi.Links(ofs, lm)
    y0 = s.project_all(m, g["dphi"], L, capi.DATA_LIN)
    # the same arrays, edited: the detectors of source 0 reversed
    L.m[ofs[0]:ofs[1]] = L.m[ofs[0]:ofs[1]][::-1].copy()
    y1 = s.project_all(m, g["dphi"], L, capi.DATA_LIN)
    fresh = capi.FwdSolver(gm, g["solver"], 1e-15, g["precon"], True, precision="fp64")
    assert np.array_equal(y1, fresh.project_all(m, g["dphi"], L, capi.DATA_LIN))
    n0 = ofs[1] - ofs[0]
    assert np.array_equal(y1[:n0], y0[:n0][::-1])
    # a caller's stream: the device copies are made again on it
    torch = pytest.importorskip("torch")
    st = torch.cuda.Stream()
    s.set_stream(st.cuda_stream)
    y2 = s.project_all(m, g["dphi"], L, capi.DATA_LIN)
    s.set_stream(0)
    assert np.array_equal(y2, y1)


def test_invalid_list_keeps_the_cached_one():
    g, gm, s = _setup()
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    m = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    L = capi.Links(g["link_ofs"], g["link_m"])
    y0 = s.project_all(m, g["dphi"], L, capi.DATA_LIN)
    bad = np.array(g["link_m"], np.int32)
    bad[0] = len(g["M"])  # detector out of range
    with pytest.raises(capi.ToastGPUError):
        s.project_all(m, g["dphi"], capi.Links(g["link_ofs"], bad), capi.DATA_LIN)
    assert np.array_equal(s.project_all(m, g["dphi"], L, capi.DATA_LIN), y0)
