"""The GPU path on the reference's own forward-model regression data.

The reference's tests (test/2D/fwdfem/Makefile:24-174, test/3D/fwdfem/
Makefile:9-77) run fwdfem on circle25_32.msh (3511 nodes, 32 x 32 links) and
cyl2.msh (9043 nodes, 80 x 80 links) at tol 1e-15 and hold ln|y| and arg y
to their golden vectors with cmpvec -r=<tol> (elementwise relative).  The
meshes, optodes and golden vectors travel in tests/golden/ref_*.npz
(tests/golden/make_refdata.py).  Each case runs here through the C ABI:

- the FP64 path with the golden run's own solver and preconditioner;
- the mixed path (FP32 inner process, FP64 refinement to the componentwise
  backward-error bound);
- the direct solver;

each against the golden vector with the Makefile's tolerance."""
import os

import numpy as np
import pytest

from tests.golden_util import GOLDEN
from tests.gpu_util import relmax
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu

# (mesh, kind, method, precon, tag, tol_fmod, tol_farg): the Makefile targets
CASES = [
    ("circle25_32", "real", "CG", "NONE", "cg", 1e-8, None),
    ("circle25_32", "real", "CG", "DIAG", "cg_diag", 1e-8, None),
    ("circle25_32", "real", "CG", "ICH", "cg_ich", 1e-8, None),
    ("circle25_32", "cplx", "BICGSTAB", "NONE", "bicgstab", 1e-7, 1e-6),
    ("circle25_32", "cplx", "BICGSTAB", "DIAG", "bicgstab_diag", 1e-7, 1e-6),
    ("circle25_32", "cplx", "BICGSTAB", "ICH", "bicgstab_ich", 1e-7, 1e-7),
    ("circle25_32", "cplx", "BICGSTAB", "DILU", "bicgstab_dilu", 1e-7, 1e-6),
    ("circle25_32", "cplx", "GMRES", "NONE", "gmres", 1e-7, 1e-7),
    ("circle25_32", "cplx", "GMRES", "DIAG", "gmres_diag", 1e-7, 1e-7),
    ("circle25_32", "cplx", "GMRES", "ICH", "gmres_ich", 1e-7, 1e-7),
    ("circle25_32", "cplx", "GMRES", "DILU", "gmres_dilu", 1e-7, 1e-7),
    ("cyl2", "real", "CG", "NONE", "cg", 1e-8, None),
    ("cyl2", "real", "CG", "ICH", "cg_ich", 1e-8, None),
    ("cyl2", "cplx", "BICGSTAB", "NONE", "bicgstab", 1e-8, 1e-8),
    ("cyl2", "cplx", "BICGSTAB", "ICH", "bicgstab_ich", 1e-8, 1e-8),
]
_data = {}


def data(mesh):
    if mesh not in _data:
        z = np.load(os.path.join(GOLDEN, f"ref_{mesh}.npz"))
        d = {k: z[k] for k in z.files}
        gm = capi.Mesh(d["coords"], d["elems"])
        _data[mesh] = (d, gm)
    return _data[mesh]


def run(mesh, kind, method, precon, precision):
    d, gm = data(mesh)
    cplx = kind == "cplx"
    cm, ck, ca = capi.optical_coefficients(d["mua"], d["mus"], d["nref"])
    # fwdfem's scripts: Gaussian source and detector profiles of width 2 mm
    # (Neumann), 100 MHz for the complex runs, tol 1e-15, maxit 10000
    qvec = gm.qvec_gaussian(d["Q"], 2.0)
    mvec = gm.qvec_gaussian(d["M"], 2.0) * ca[None, :]
    s = capi.FwdSolver(gm, method, 1e-15 if method != "DIRECT" else 1e-10, precon, cplx, maxit=10000,
                       precision=precision)
    L = capi.Links(d["link_ofs"], d["link_m"])
    out = s.forward_path(cm, ck, ca, capi.omega_of(100.0 if cplx else 0.0), qvec, mvec, L, want_fields=False,
                         want_jac=False)
    return d, out


def check(d, out, kind, tag, tol_mod, tol_arg):
    lp = np.asarray(out["logproj"])
    assert relmax(lp.real, d[f"fmod_{kind}_{tag}"]) <= tol_mod
    if kind == "cplx":
        assert relmax(lp.imag, d[f"farg_{kind}_{tag}"]) <= tol_arg


@pytest.mark.parametrize("mesh,kind,method,precon,tag,tol_mod,tol_arg", CASES,
                         ids=[f"{c[0]}-{c[1]}_{c[4]}" for c in CASES])
def test_fp64_matches_reference_golden(mesh, kind, method, precon, tag, tol_mod, tol_arg):
    d, out = run(mesh, kind, method, precon, "fp64")
    check(d, out, kind, tag, tol_mod, tol_arg)


# The mixed path and the direct solver converge to the exact FP64 solution.
# On circle25_32 the iterative goldens themselves sit up to 1.5e-8 (CW
# ln|y|) and 3.2e-7 (arg y) from it (the oracle's direct solve measures
# that), above the Makefile's 1e-8 / 1e-7 for the ICH runs; so the exact
# solvers are held to the oracle's exact solve at 1e-8 and to the goldens at
# 5e-8 / 5e-7 there, and at the Makefile's tolerance on cyl2.
EXACT_TOL = {"circle25_32": (5e-8, 5e-7)}


@pytest.mark.parametrize("mesh,kind,method,precon,tag,tol_mod,tol_arg",
                         [c for c in CASES if c[3] == "ICH"], ids=[f"{c[0]}-{c[1]}_{c[4]}" for c in CASES
                                                                  if c[3] == "ICH"])
def test_mixed_and_direct_match_reference_golden(oracle_mod, mesh, kind, method, precon, tag, tol_mod, tol_arg):
    d, gm = data(mesh)
    om = oracle_mod.Mesh(d["coords"], d["elems"])
    ex = oracle_mod.forward_path(om, d["Q"], d["M"], d["link_ofs"], d["link_m"], d["mua"], d["mus"], d["nref"],
                                 100.0 if kind == "cplx" else 0.0, 2.0, 2.0, "DIRECT", jac=False, nthreads=8)
    tm, ta = EXACT_TOL.get(mesh, (tol_mod, tol_arg))
    for meth, prec, pre in ((method, "mixed", "ICH"), ("DIRECT", "fp64", "NONE")):
        d, out = run(mesh, kind, meth, pre, prec)
        lp = np.asarray(out["logproj"])
        assert relmax(lp.real, np.real(ex.logproj)) < 1e-8
        if kind == "cplx":
            assert relmax(lp.imag, np.imag(ex.logproj)) < 1e-8
        check(d, out, kind, tag, tm, ta)
