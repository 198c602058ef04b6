"""The GPU path on the full-size benchmark configurations that the oracle
finishes in seconds: the 2D 3.2k-node CW disc (CG + ICH, tol 1e-10) and the
2D 12.5k-node 100 MHz disc (BiCGSTAB + ICH), 16 + 16 and 32 + 32 optodes.

- FP64 path against the oracle running the same algorithm at the same
  tolerance: fields, boundary data and Jacobian within 1e-10.
- Mixed path against the oracle's exact FP64 solve (direct factorisation):
  boundary data entry by entry and the Jacobian within 1e-8.
- Direct solver against the same: within 1e-10."""
import numpy as np
import pytest

from tests.gpu_util import gpu_problem_inputs, rel2, relmax
from toastpp_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

CONFIGS = ["c0_disc3k_cw", "c1_disc13k_fd"]
_cache = {}


def problem(cfg, oracle_mod):
    if cfg not in _cache:
        P = workloads.CONFIGS[cfg]()
        om = oracle_mod.Mesh(P.coords, P.elems)
        gm = capi.Mesh(P.coords, P.elems)
        exact = oracle_mod.forward_path(om, P.qm.Q, P.qm.M, P.qm.link_ofs, P.qm.link_m, P.mua, P.mus, P.nref,
                                        P.freq_mhz, P.qwidth, P.mwidth, "DIRECT", jac=True, nthreads=8)
        _cache[cfg] = (P, om, gm, exact)
    return _cache[cfg]


def run_gpu(P, gm, method, precision, tol, precon="ICH"):
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    s = capi.FwdSolver(gm, method, tol, precon, P.complex, precision=precision)
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    return s.forward_path(cm, ck, ca, capi.omega_of(P.freq_mhz), qvec, mvec, L)


def logdiff(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = np.isfinite(a) & np.isfinite(b)
    return float(np.max(np.abs(a - b)[ok]))


@pytest.mark.parametrize("cfg,tol", [("c0_disc3k_cw", 1e-10), ("c1_disc13k_fd", 1e-12)])
def test_fp64_matches_oracle_same_algorithm(oracle_mod, cfg, tol):
    """Same recursion on both sides; at tol 1e-10 two such runs of the 12.5k
    complex system part by 2.5e-10 (the solutions themselves are only that
    accurate), so that one is compared at 1e-12."""
    P, om, gm, exact = problem(cfg, oracle_mod)
    method = "BICGSTAB" if P.complex else "CG"
    out = run_gpu(P, gm, method, "fp64", tol)
    ref = oracle_mod.forward_path(om, P.qm.Q, P.qm.M, P.qm.link_ofs, P.qm.link_m, P.mua, P.mus, P.nref,
                                  P.freq_mhz, P.qwidth, P.mwidth, method, "ICH", tol, jac=True, nthreads=8)
    assert rel2(out["dphi"], ref.dphi) < 1e-10 and rel2(out["aphi"], ref.aphi) < 1e-10
    assert rel2(out["proj"], ref.proj) < 1e-10
    if not P.complex:
        assert rel2(out["J"], ref.J) < 1e-10
    # The log-data Jacobian rows of far links are quotients of field values
    # e^-20 below their peaks, which two runs stopped on the normwise test
    # carry with 1e-4 relative error each (against the exact solve, too), so
    # on the complex disc the kernel is checked on the GPU's own fields
    Jk = oracle_mod.jacobian(om, out["dphi"], out["aphi"], out["proj"], P.qm.link_ofs, P.qm.link_m, True, 8)
    assert rel2(out["J"], Jk) < 1e-12
    # iteration counts: the same recursion with different summation orders;
    # near tol 1e-12 BiCGSTAB's last digits of the residual wander, so a
    # column may stop a few iterations apart (up to 15 %)
    gits = np.array([r[0] for r in out["results"]])
    rits = np.concatenate([ref.its_fwd, ref.its_adj])
    assert np.all(np.abs(gits - rits) <= np.maximum(2, 0.15 * rits))


@pytest.mark.parametrize("cfg", CONFIGS)
def test_mixed_matches_exact_fp64(oracle_mod, cfg):
    P, om, gm, exact = problem(cfg, oracle_mod)
    out = run_gpu(P, gm, "BICGSTAB" if P.complex else "CG", "mixed", 1e-10)
    assert all(r[1] == 0 for r in out["results"])
    assert relmax(out["proj"], exact.proj) < 1e-8
    assert logdiff(out["logproj"], exact.logproj) < 1e-8
    assert rel2(out["J"], exact.J) < 1e-8


@pytest.mark.parametrize("cfg", CONFIGS)
def test_direct_matches_exact_fp64(oracle_mod, cfg):
    P, om, gm, exact = problem(cfg, oracle_mod)
    out = run_gpu(P, gm, "DIRECT", "fp64", 1e-10, "NONE")
    assert relmax(out["proj"], exact.proj) < 1e-10
    assert logdiff(out["logproj"], exact.logproj) < 1e-10
    assert rel2(out["J"], exact.J) < 1e-10
