"""Shared helpers for the GPU parity tests: small seeded problems and the
oracle reference results for them."""
import numpy as np

from toastpp_gb300 import capi, workloads


def small_disc(freq=0.0, rings=8, nopt=6, seed=3):
    return workloads.disc(rings, seed, freq, nopt)


def small_cyl(freq=100.0, rings=4, layers=6, seed=5):
    P = workloads.cylinder(rings=rings, layers=layers, seed=seed, freq_mhz=freq)
    # fewer optodes for a small case: one ring of sources and detectors
    idx = np.arange(0, 80, 10)
    P.qm = type(P.qm).all_to_all(P.qm.Q[idx] * 1.0, P.qm.M[idx] * 1.0)
    return P


def relmax(a, b):
    """cmpvec-style elementwise relative difference |a-b|/max(|a|,|b|)
    (src/bintools/cmpvec.cc:101-112); NaNs must sit at the same positions
    (log of a negative CW projection is NaN in the reference too)."""
    a = np.asarray(a)
    b = np.asarray(b)
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return float("inf")
    a, b = a[~na], b[~nb]
    if a.size == 0:
        return 0.0
    den = np.maximum(np.abs(a), np.abs(b))
    den[den == 0] = 1.0
    return float(np.max(np.abs(a - b) / den))


def rel2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def gpu_problem_inputs(P, gmesh):
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    qvec = gmesh.qvec_gaussian(P.qm.Q, P.qwidth)
    mvec = gmesh.qvec_gaussian(P.qm.M, P.mwidth) * ca[None, :]
    return cm, ck, ca, qvec, mvec
