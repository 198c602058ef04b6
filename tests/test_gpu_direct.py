"""LSOLVER_DIRECT on the GPU (tg_solver_create with TG_SOLVER_DIRECT: a
complete L L^T factor in a nested-dissection ordering, applied by the two
level-scheduled sweeps) against the oracle's restatement of the reference's
direct path (symbolic Cholesky fill, left-looking factor, substitution) and
against the reference's own direct solves (tests/golden/*_direct.npz:
Cholesky for CW, SuperLU for 100 MHz, written by the compiled reference)."""
import numpy as np
import pytest

from tests.golden_util import load, names
from tests.gpu_util import gpu_problem_inputs, rel2, relmax, small_cyl, small_disc
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu

CASES = [("disc_cw", lambda: small_disc(0.0)), ("disc_fd", lambda: small_disc(100.0)),
         ("cyl_cw", lambda: small_cyl(0.0)), ("cyl_fd", lambda: small_cyl(100.0))]


def logdiff(a, b):
    """max |a - b| over the entries finite in both (log of a negative CW
    projection is NaN, in the reference too); NaNs must sit at the same places"""
    a, b = np.asarray(a), np.asarray(b)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = np.isfinite(a) & np.isfinite(b)
    return float(np.max(np.abs(a - b)[ok])) if ok.any() else 0.0


@pytest.mark.parametrize("name,factory", CASES, ids=[c[0] for c in CASES])
def test_direct_fields_match_oracle(oracle_mod, name, factory):
    P = factory()
    om = oracle_mod.Mesh(P.coords, P.elems)
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    s = capi.FwdSolver(gm, "DIRECT", 1e-10, "NONE", P.complex)
    s.reset(cm, ck, ca, omega)
    B = np.concatenate([qvec, mvec])
    phi, res = s.calc_fields(B)
    val = om.assemble(cm, ck, ca, omega, P.complex)
    X = oracle_mod.solve_direct(om.rowptr, om.colidx, val, B.astype(phi.dtype), "nd", om.coords)
    # two exact FP64 solves in different orderings: round-off apart
    assert rel2(phi, X) < 1e-13
    assert relmax(phi, X) < 1e-10
    assert all(r[0] == 0 and r[1] == 0 and r[2] < 1e-13 for r in res), res


@pytest.mark.parametrize("name", [n for n in names(nodal_only=True) if n.endswith("_direct")])
def test_direct_matches_reference_direct(name):
    """The reference's own direct solve (Cholesky / SuperLU in its natural
    ordering) and ours agree to round-off: boundary data elementwise and the
    nodal Jacobian."""
    g = load(name)
    gm = capi.Mesh(g["coords"], g["elems"])
    cplx = g["freq_mhz"] != 0.0
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    qvec = gm.qvec_gaussian(g["Q"], g["qwidth"])
    mvec = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    s = capi.FwdSolver(gm, "DIRECT", 1e-10, "NONE", cplx)
    L = capi.Links(g["link_ofs"], g["link_m"])
    out = s.forward_path(cm, ck, ca, capi.omega_of(g["freq_mhz"]), qvec, mvec, L, want_fields=False)
    assert relmax(out["proj"], g["proj"]) < 1e-11
    assert logdiff(out["logproj"], g["logproj"]) < 1e-11
    assert rel2(out["J"].reshape(g["J"].shape), g["J"]) < 1e-12


def test_direct_solver_settings_and_refactor(oracle_mod):
    """A second reset with other parameters refactors (the result follows the
    new matrix); the solver reports 0 iterations per right-hand side."""
    P = small_disc(100.0)
    om = oracle_mod.Mesh(P.coords, P.elems)
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    s = capi.FwdSolver(gm, "DIRECT", 1e-10, "ICH", True, precision="mixed")
    for f in (1.0, 1.7):
        s.reset(cm * f, ck, ca, capi.omega_of(P.freq_mhz))
        phi, res = s.calc_fields(qvec)
        val = om.assemble(cm * f, ck, ca, capi.omega_of(P.freq_mhz), True)
        X = oracle_mod.solve_direct(om.rowptr, om.colidx, val, qvec.astype(phi.dtype), "rcm")
        assert rel2(phi, X) < 1e-13
        assert all(r[0] == 0 for r in res)
