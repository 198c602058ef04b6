"""ProjectAll through tg_project_all_noalloc, the entry point for callers that
cannot call cudaMalloc (a device memory pool owned by another runtime,
real-time loops that must not allocate after start-up, plug-ins whose host
forbids allocation).  It keeps its scratch in a fixed device array instead of
allocating; its results must match tg_project_all's, call after call, because
every call reuses (and overwrites) the same scratch.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

from tests.gpu_util import gpu_problem_inputs, relmax, small_cyl, small_disc
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu


def _device(a):
    import torch
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        a = a.view(np.float64)
    return torch.from_numpy(a.copy()).cuda()


@pytest.mark.parametrize("make", [lambda: small_disc(100.0), lambda: small_cyl(100.0), lambda: small_disc(0.0)],
                         ids=["disc_fd", "cyl_fd", "disc_cw"])
def test_noalloc_projection_matches_project_all(make, oracle_mod):
    import torch
    P = make()
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    method = "BICGSTAB" if P.complex else "CG"
    s = capi.FwdSolver(gm, method, 1e-12, "ICH", P.complex)
    s.reset(cm, ck, ca, capi.omega_of(P.freq_mhz))
    phi, _ = s.calc_fields(qvec)
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    ref_log = s.project_all(mvec, phi, L, capi.DATA_LOG)
    ref_lin = s.project_all(mvec, phi, L, capi.DATA_LIN)
    dt = np.complex128 if P.complex else np.float64
    d_phi = _device(phi.astype(dt))
    d_m = _device(mvec.astype(dt))
    width = 2 if P.complex else 1
    # two calls in a row (log, then linear, then log again) reuse the same scratch
    for scale, ref in ((capi.DATA_LOG, ref_log), (capi.DATA_LIN, ref_lin), (capi.DATA_LOG, ref_log)):
        d_out = torch.full((L.nqm * width,), float("nan"), dtype=torch.float64, device="cuda")
        s.project_all_noalloc(d_phi, P.qm.nQ, d_m, P.qm.nM, L, scale, d_out)
        got = d_out.cpu().numpy().view(dt)
        assert relmax(got, ref) < 1e-12
        # and the oracle's ProjectAll of the same fields
        want = oracle_mod.project(phi.astype(dt), mvec.astype(dt), P.qm.link_ofs, P.qm.link_m,
                                  logscale=scale == capi.DATA_LOG)
        assert relmax(got, want) < 1e-12


def test_noalloc_checks_its_buffers():
    """Host tensors, float32 tensors and short buffers are refused before any
    kernel could read past them."""
    import torch
    P = small_disc(100.0)
    gm = capi.Mesh(P.coords, P.elems)
    s = capi.FwdSolver(gm, "BICGSTAB", 1e-10, "ICH", True)
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    nq, nm = P.qm.nQ, P.qm.nM
    ok_phi = torch.zeros(2 * nq * gm.n, dtype=torch.float64, device="cuda")
    ok_m = torch.zeros(2 * nm * gm.n, dtype=torch.float64, device="cuda")
    ok_out = torch.zeros(2 * L.nqm, dtype=torch.float64, device="cuda")
    for bad in (ok_phi.cpu(), ok_phi.float(), ok_phi[:-1]):
        with pytest.raises(ValueError):
            s.project_all_noalloc(bad, nq, ok_m, nm, L, capi.DATA_LIN, ok_out)
    with pytest.raises(ValueError):
        s.project_all_noalloc(ok_phi, nq, ok_m, nm, L, capi.DATA_LIN, ok_out[:-1])


def test_noalloc_rejects_problems_beyond_the_fixed_scratch():
    import torch
    from toastpp_gb300 import workloads
    P = workloads.disc(64, 2, 100.0, 4)          # 12481 nodes
    gm = capi.Mesh(P.coords, P.elems)
    s = capi.FwdSolver(gm, "BICGSTAB", 1e-10, "ICH", True)
    nm = 48                                        # dense detector vectors: 12481 x 48 complex > 8 MiB
    d_phi = torch.ones(2 * 4 * P.n, dtype=torch.float64, device="cuda")
    d_m = torch.ones(2 * nm * P.n, dtype=torch.float64, device="cuda")
    L = capi.Links.all_to_all(4, nm)
    d_out = torch.zeros(2 * L.nqm, dtype=torch.float64, device="cuda")
    with pytest.raises(capi.ToastGPUError) as ei:
        s.project_all_noalloc(d_phi, 4, d_m, nm, L, capi.DATA_LIN, d_out)
    assert ei.value.code == 5 and "fixed scratch" in str(ei.value)
