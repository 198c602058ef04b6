"""The GPU path against the reference's own outputs (tests/golden: fixtures
written by the compiled reference, tests/golden/make_golden.py), through the
C ABI: projections (ProjectAll LIN and LOG) and the nodal Jacobian, FP64 and
mixed precision, for every solver / preconditioner the fixtures hold."""
import numpy as np
import pytest

from tests.golden_util import load, names
from tests.gpu_util import rel2, relmax
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu


def run(g, precision):
    gm = capi.Mesh(g["coords"], g["elems"])
    cplx = g["freq_mhz"] != 0.0
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    qvec = gm.qvec_gaussian(g["Q"], g["qwidth"])
    mvec = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    # same solver, preconditioner and tolerance as the reference run
    s = capi.FwdSolver(gm, g["solver"], g["tol"], g["precon"], cplx, precision=precision)
    L = capi.Links(g["link_ofs"], g["link_m"])
    return s.forward_path(cm, ck, ca, capi.omega_of(g["freq_mhz"]), qvec, mvec, L, want_fields=False,
                          want_jac="J" in g)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", names(nodal_only=True))
def test_gpu_matches_reference_fixture(name, precision):
    g = load(name)
    out = run(g, precision)
    # Elementwise bounds on ln|y| and arg y.  The FP64 path runs the
    # reference's recursion and must agree to 1e-8 / 1e-7.  The mixed path
    # converges the true residual by refinement instead; the far detectors
    # (|y| ~ e^-25 of the near ones) then see the reference's own solve error:
    # the reference's BiCGSTAB+DIAG, BiCGSTAB+NONE and GMRES runs at tol 1e-15
    # differ from its BiCGSTAB+ICH run by up to 2.5e-8 (ln|y|) and 4.8e-7
    # (arg y) on this disc, so the mixed bound is the reference's own 2D
    # complex golden tolerance (test/2D/fwdfem/Makefile: cmpvec -r=1e-7 / 1e-6).
    tol_mod, tol_arg = (1e-8, 1e-7) if precision == "fp64" else (1e-7, 1e-6)
    assert relmax(out["logproj"].real, g["logproj"].real) < tol_mod
    if np.iscomplexobj(g["logproj"]):
        assert relmax(out["logproj"].imag, g["logproj"].imag) < tol_arg
    assert rel2(out["proj"], g["proj"]) < 1e-10
    if "J" in g:
        # The log-data Jacobian amplifies field differences far from the
        # optodes: the reference itself run at tol 1e-16 instead of 1e-15
        # moves J by up to 6e-8 (L2) on these meshes, so that is the scale of
        # agreement two correct solvers can reach.
        J = out["J"].reshape(g["J"].shape)
        err = rel2(J, g["J"])
        assert err < (1e-7 if precision == "fp64" else 1e-6), err
