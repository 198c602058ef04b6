"""The request server: admission, concurrency on per-slot streams, and the
invariance of every result to the other requests on the device."""
import numpy as np
import pytest

from tests.gpu_util import small_cyl, small_disc
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu


def make_problems():
    return [small_disc(0.0), small_disc(100.0), small_cyl(100.0), small_cyl(0.0)]


def make_request(P, gm, precision="mixed", solver=None):
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    q = gm.qvec_gaussian(P.qm.Q, P.qwidth)
    m = gm.qvec_gaussian(P.qm.M, P.mwidth) * ca[None, :]
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    return capi.Request(gm, cm, ck, ca, capi.omega_of(P.freq_mhz), q, m, L, solver=solver, tol=1e-12,
                        precision=precision, want_jac=True, j_fp32=True)


def outputs(r):
    return r.proj.copy(), r.logproj.copy(), r.J.copy()


def test_alone_equals_mix():
    probs = make_problems()
    meshes = [capi.Mesh(P.coords, P.elems) for P in probs]
    # alone: one slot, one request at a time
    alone = []
    srv = capi.Server(slots=1, hbm_budget_gb=8.0)
    for P, gm in zip(probs, meshes):
        t = srv.submit(make_request(P, gm))
        alone.append(outputs(srv.wait(t)))
    srv.close()
    # mix: every request three times, all submitted at once to four slots
    srv = capi.Server(slots=4, hbm_budget_gb=8.0)
    tickets = []
    for rep in range(3):
        for i, (P, gm) in enumerate(zip(probs, meshes)):
            tickets.append((i, srv.submit(make_request(P, gm))))
    for i, t in tickets:
        got = outputs(srv.wait(t))
        for a, b in zip(alone[i], got):
            assert np.array_equal(a, b, equal_nan=True), f"request {i} differs in the mix"
    st = srv.stats()
    assert st["completed"] == len(tickets) and st["failed"] == 0
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    srv.close()


def test_server_matches_direct_call():
    P = small_cyl(100.0)
    gm = capi.Mesh(P.coords, P.elems)
    srv = capi.Server(slots=2, hbm_budget_gb=8.0)
    r = srv.wait(srv.submit(make_request(P, gm, precision="fp64")))
    srv.close()
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    q = gm.qvec_gaussian(P.qm.Q, P.qwidth)
    m = gm.qvec_gaussian(P.qm.M, P.mwidth) * ca[None, :]
    s = capi.FwdSolver(gm, "BICGSTAB", 1e-12, "ICH", True, precision="fp64")
    out = s.forward_path(cm, ck, ca, capi.omega_of(P.freq_mhz), q, m, capi.Links(P.qm.link_ofs, P.qm.link_m),
                         want_fields=False, want_jac=True, j_fp32=True)
    assert np.array_equal(out["proj"], r.proj) and np.array_equal(out["logproj"], r.logproj, equal_nan=True)
    assert np.array_equal(out["J"], r.J)


def test_budget_admission_serialises_but_completes():
    probs = make_problems()
    meshes = [capi.Mesh(P.coords, P.elems) for P in probs]
    # a budget below any request: each runs alone, in arrival order
    srv = capi.Server(slots=4, hbm_budget_gb=1e-6)
    ts = [srv.submit(make_request(P, gm)) for P, gm in zip(probs, meshes)]
    lat = [srv.wait(t).latency_ms for t in ts]
    assert all(x > 0 for x in lat)
    # arrival order is kept: each later request finished no earlier
    assert srv.stats()["completed"] == len(ts)
    srv.close()


def test_failed_request_reports_error():
    P = small_disc(100.0)
    gm = capi.Mesh(P.coords, P.elems)
    srv = capi.Server(slots=2, hbm_budget_gb=8.0)
    bad = make_request(P, gm, solver="CG")  # CG is not defined for complex systems
    t = srv.submit(bad)
    with pytest.raises(capi.ToastGPUError):
        srv.wait(t)
    ok = srv.wait(srv.submit(make_request(P, gm)))
    assert np.all(np.isfinite(ok.proj))
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1
    srv.close()


def pinned_outputs(P, gm):
    """(proj, logproj, J) in page-locked memory (deferred Jacobian copies)."""
    torch = pytest.importorskip("torch")
    nqm, n = len(P.qm.link_m), gm.n
    dt = torch.complex128 if P.complex else torch.float64
    cols = 2 * n if P.complex else n
    return (torch.zeros(nqm, dtype=dt).pin_memory().numpy(), torch.zeros(nqm, dtype=dt).pin_memory().numpy(),
            torch.zeros((2 * nqm, cols), dtype=torch.float32).pin_memory().numpy())


def make_pinned_request(P, gm):
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    q = gm.qvec_gaussian(P.qm.Q, P.qwidth)
    m = gm.qvec_gaussian(P.qm.M, P.mwidth) * ca[None, :]
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    return capi.Request(gm, cm, ck, ca, capi.omega_of(P.freq_mhz), q, m, L, tol=1e-12, precision="mixed",
                        want_jac=True, j_fp32=True, outputs=pinned_outputs(P, gm))


def test_pipelined_requests_keep_their_jacobians():
    """One slot, requests back to back with page-locked outputs: each
    Jacobian's device-to-host copy overlaps the next request's compute (two
    device J buffers per solver), and every request still receives its own
    complete J, equal to the one of a request run alone."""
    probs = [small_cyl(100.0), small_cyl(100.0, seed=9)]
    meshes = [capi.Mesh(P.coords, P.elems) for P in probs]
    ref = []
    for P, gm in zip(probs, meshes):
        srv = capi.Server(slots=1, hbm_budget_gb=8.0)
        ref.append(outputs(srv.wait(srv.submit(make_request(P, gm)))))
        srv.close()
    assert not np.array_equal(ref[0][2], ref[1][2])
    srv = capi.Server(slots=1, hbm_budget_gb=8.0)
    order = [0, 1, 0, 0, 1, 1, 0, 1]
    ts = [srv.submit(make_pinned_request(probs[i], meshes[i])) for i in order]
    got = [outputs(srv.wait(t)) for t in ts]
    srv.close()
    for i, g in zip(order, got):
        assert np.array_equal(g[0], ref[i][0])
        assert np.array_equal(g[2], ref[i][2])


def test_deferred_output_stream_on_the_solver():
    """tg_solver_set_output_stream: a page-locked Jacobian lands in host memory
    once the copy stream's work is done (tg_solver_sync), equal to the direct
    result, also when calls follow one another without a sync."""
    torch = pytest.importorskip("torch")
    P = small_cyl(100.0)
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    q = gm.qvec_gaussian(P.qm.Q, P.qwidth)
    m = gm.qvec_gaussian(P.qm.M, P.mwidth) * ca[None, :]
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    s = capi.FwdSolver(gm, "BICGSTAB", 1e-12, "ICH", True, precision="mixed")
    om = capi.omega_of(P.freq_mhz)
    direct = s.forward_path(cm, ck, ca, om, q, m, L, want_fields=False, j_fp32=True)
    cs = torch.cuda.Stream()
    s.set_output_stream(cs.cuda_stream)
    outs = [pinned_outputs(P, gm) for _ in range(3)]
    qc, mc = np.ascontiguousarray(q, np.complex128), np.ascontiguousarray(m, np.complex128)
    for o in outs:
        s.forward_path_raw(np.ascontiguousarray(cm), np.ascontiguousarray(ck), np.ascontiguousarray(ca), om,
                           q.shape[0], qc, m.shape[0], mc, L, None, None, o[0], o[1], o[2], 1, capi.MEM_HOST)
    s.sync()
    for o in outs:
        assert np.array_equal(o[2], direct["J"])
        assert np.array_equal(o[0], direct["proj"])
    s.set_output_stream(None)
