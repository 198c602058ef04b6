"""The two ways of running an IC(0) apply (a launch per level, one persistent
cooperative launch with a grid barrier per level) compute every row with the
same sums in the same order: whole requests come out bit-identical whichever
the autotuner picks."""
import numpy as np
import pytest

from toastpp_gb300 import capi, workloads
from tests.gpu_util import gpu_problem_inputs

pytestmark = pytest.mark.gpu

CASES = [("cyl_fd", lambda: workloads.cylinder(rings=6, layers=8, seed=3)),   # 80 + 80 optodes: k = 160
         ("disc_cw", lambda: workloads.disc(24, 2, 0.0, 16))]                  # 16 + 16: k = 32


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("name,factory", CASES, ids=[c[0] for c in CASES])
def test_ic_apply_variants_bit_identical(name, factory, precision, monkeypatch):
    P = factory()
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    method = "BICGSTAB" if P.complex else "CG"
    outs = []
    for v in ("0", "1"):
        monkeypatch.setenv("TOASTGPU_IC_PERSISTENT", v)
        s = capi.FwdSolver(gm, method, 1e-12, "ICH", P.complex, precision=precision)
        out = s.forward_path(cm, ck, ca, capi.omega_of(P.freq_mhz), qvec, mvec, L)
        outs.append(out)
    for v, out in zip((1,), outs[1:]):
        for key in ("dphi", "aphi", "proj", "J"):
            assert np.array_equal(np.asarray(out[key]), np.asarray(outs[0][key])), (v, key)
