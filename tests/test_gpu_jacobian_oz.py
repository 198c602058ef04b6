"""The complex FP64 Jacobian on the tensor cores on the shapes its tiling has
to pad: a source count that is not a multiple of 8, a detector count that is
not a multiple of 4, a sparse link list, nodes of degree above 16 (three
K-steps), and both data scalings (log data divides each link by its
projection, linear data does not).  Held to the oracle's FP64 Jacobian of the
same GPU fields."""
import numpy as np
import pytest

from toastpp_gb300 import capi, workloads
from toastpp_gb300.meshio import QMSpec
from tests.gpu_util import gpu_problem_inputs, rel2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem(oracle_mod):
    P = workloads.cylinder(rings=8, layers=10, seed=2)   # 2170 nodes, 152 of degree 17
    Q, M = P.qm.Q[:11] * 1.0, P.qm.M[::11][:7] * 1.0     # 11 sources, 7 detectors
    ofs, lm = [0], []
    for q in range(len(Q)):
        lm += [m for m in range(len(M)) if (q + m) % 3]  # a sparse link list
        ofs.append(len(lm))
    P.qm = QMSpec(Q, M, np.array(ofs, np.int32), np.array(lm, np.int32), True, True)
    om = oracle_mod.Mesh(P.coords, P.elems)
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    s = capi.FwdSolver(gm, "BICGSTAB", 1e-13, "ICH", True)
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    out = s.forward_path(cm, ck, ca, capi.omega_of(P.freq_mhz), qvec, mvec, L)
    return P, om, s, L, out


@pytest.mark.parametrize("log", [True, False], ids=["log", "lin"])
def test_tensor_core_jacobian_padded_shapes(problem, oracle_mod, log):
    P, om, s, L, out = problem
    dphi, aphi, proj = (np.asarray(out[k]) for k in ("dphi", "aphi", "proj"))
    J = np.asarray(s.jacobian(dphi, aphi, proj, L, scale=capi.DATA_LOG if log else capi.DATA_LIN))
    Jor = oracle_mod.jacobian(om, dphi, aphi, proj, P.qm.link_ofs, P.qm.link_m, logscale=log)
    assert J.shape == Jor.shape == (2 * P.qm.nQM, 2 * P.n)
    assert rel2(J, Jor) < 2e-14
    assert np.max(np.abs(J - Jor)) < 5e-14 * np.max(np.abs(Jor))
    # FP32 storage of the same sums: one FP32 rounding per entry
    J32 = np.asarray(s.jacobian(dphi, aphi, proj, L, scale=capi.DATA_LOG if log else capi.DATA_LIN,
                                fp32=2)).astype(np.float64)
    assert np.all(np.abs(J32 - J) <= 6.0e-8 * np.abs(J) + 1e-300)
