"""GPU path vs the CPU oracle on small seeded meshes, through the C ABI."""
import numpy as np
import pytest

from toastpp_gb300 import capi
from tests.gpu_util import gpu_problem_inputs, rel2, relmax, small_cyl, small_disc

pytestmark = pytest.mark.gpu

CASES = [("disc_cw", lambda: small_disc(0.0)), ("disc_fd", lambda: small_disc(100.0)),
         ("cyl_cw", lambda: small_cyl(0.0)), ("cyl_fd", lambda: small_cyl(100.0))]


@pytest.fixture(scope="module", params=CASES, ids=[c[0] for c in CASES])
def case(request, oracle_mod):
    P = request.param[1]()
    om = oracle_mod.Mesh(P.coords, P.elems)
    gm = capi.Mesh(P.coords, P.elems)
    return P, om, gm


def test_mesh_structure(case):
    P, om, gm = case
    rp, ci = gm.csr()
    assert np.array_equal(rp, om.rowptr) and np.array_equal(ci, om.colidx)
    assert np.array_equal(gm.boundary(), om.bnd)


def test_source_vectors(case):
    P, om, gm = case
    q_gpu = gm.qvec_gaussian(P.qm.Q, P.qwidth)
    q_ref = np.stack([om.qvec_gaussian(q, P.qwidth) for q in P.qm.Q])
    assert relmax(q_gpu, q_ref) < 1e-14


def test_assembly(case):
    P, om, gm = case
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    omega = capi.omega_of(P.freq_mhz)
    s = capi.FwdSolver(gm, "BICGSTAB" if P.complex else "CG", 1e-10, "ICH", P.complex)
    s.reset(cm, ck, ca, omega)
    F = s.system_matrix()
    Fr = om.assemble(cm, ck, ca, omega, P.complex)
    assert relmax(F, Fr) < 1e-13


@pytest.mark.parametrize("precon", ["ICH", "DIAG", "NONE"])
def test_solve_fp64(case, oracle_mod, precon):
    P, om, gm = case
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    method = "BICGSTAB" if P.complex else "CG"
    s = capi.FwdSolver(gm, method, 1e-14, precon, P.complex)
    s.reset(cm, ck, ca, omega)
    phi, res = s.calc_fields(qvec)
    val = om.assemble(cm, ck, ca, omega, P.complex)
    Xr, its, errs = oracle_mod.solve(om.rowptr, om.colidx, val, qvec.astype(phi.dtype), method, precon, 1e-14)
    assert rel2(phi, Xr) < 1e-10
    assert all(r[1] == 0 for r in res), res
    gits = np.array([r[0] for r in res])
    assert np.all(np.abs(gits - its) <= 2), (gits, its)


@pytest.mark.parametrize("precon", ["ICH", "DIAG", "NONE"])
def test_solve_gmres(case, oracle_mod, precon):
    """GMRES(20) (gmres_imp.hpp:39-230) per right-hand side against the oracle:
    same fields and the same number of restart cycles."""
    P, om, gm = case
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    s = capi.FwdSolver(gm, "GMRES", 1e-12, precon, P.complex)
    s.reset(cm, ck, ca, omega)
    phi, res = s.calc_fields(qvec)
    val = om.assemble(cm, ck, ca, omega, P.complex)
    Xr, its, errs = oracle_mod.solve(om.rowptr, om.colidx, val, qvec.astype(phi.dtype), "GMRES", precon, 1e-12)
    assert rel2(phi, Xr) < 1e-9
    assert all(r[1] == 0 for r in res), res
    gits = np.array([r[0] for r in res])
    assert np.all(np.abs(gits - its) <= 1), (gits, its)
    gerr = np.array([r[2] for r in res])
    assert np.all(gerr <= 1e-12) and np.all(errs <= 1e-12)


@pytest.mark.parametrize("freq", [0.0, 100.0])
@pytest.mark.parametrize("precon", ["ICH", "DIAG", "NONE"])
def test_solve_gmres_restarts(oracle_mod, freq, precon):
    """A 1801-node disc on which GMRES(20) needs several restart cycles."""
    from toastpp_gb300 import workloads
    P = workloads.disc(24, 7, freq, 8)
    om = oracle_mod.Mesh(P.coords, P.elems)
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    s = capi.FwdSolver(gm, "GMRES", 1e-12, precon, P.complex)
    s.reset(cm, ck, ca, omega)
    phi, res = s.calc_fields(qvec)
    val = om.assemble(cm, ck, ca, omega, P.complex)
    Xr, its, errs = oracle_mod.solve(om.rowptr, om.colidx, val, qvec.astype(phi.dtype), "GMRES", precon, 1e-12)
    assert rel2(phi, Xr) < 1e-9
    gits = np.array([r[0] for r in res])
    assert np.all(np.abs(gits - its) <= 1), (gits, its)
    assert np.mean(gits == its) >= 0.75, (gits, its)


@pytest.mark.parametrize("method", ["BICGSTAB", "GMRES"])
def test_calc_fields_mixed(case, oracle_mod, method):
    """FP32 inner solves inside FP64 refinement reach the FP64 oracle's fields."""
    P, om, gm = case
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    s = capi.FwdSolver(gm, method, 1e-12, "ICH", P.complex, precision="mixed")
    s.reset(cm, ck, ca, omega)
    phi, res = s.calc_fields(qvec)
    val = om.assemble(cm, ck, ca, omega, P.complex)
    Xr, its, errs = oracle_mod.solve(om.rowptr, om.colidx, val, qvec.astype(phi.dtype), method, "ICH", 1e-13)
    assert rel2(phi, Xr) < 1e-10
    assert all(r[1] == 0 for r in res), res


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["restart", "reliable_bicgstab", "reliable_cocg"])
def test_mixed_inner_modes(case, oracle_mod, mode):
    """Every FP32 inner scheme of the mixed path (restarted refinement, reliable
    updates of BiCGSTAB or of COCG) reaches the FP64 oracle's fields."""
    P, om, gm = case
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    s = capi.FwdSolver(gm, "BICGSTAB", 1e-12, "ICH", P.complex, precision="mixed")
    s.set_reliable_updates(mode)
    s.reset(cm, ck, ca, omega)
    B = np.concatenate([qvec, mvec])
    phi, res = s.calc_fields(B)
    val = om.assemble(cm, ck, ca, omega, P.complex)
    Xr, its, errs = oracle_mod.solve(om.rowptr, om.colidx, val, B.astype(phi.dtype), "BICGSTAB", "ICH", 1e-13)
    assert rel2(phi, Xr) < 1e-10
    assert all(r[1] == 0 for r in res), res
    assert all(r[2] <= 1e-12 for r in res), res


def test_project_and_jacobian(case, oracle_mod):
    P, om, gm = case
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    method = "BICGSTAB" if P.complex else "CG"
    s = capi.FwdSolver(gm, method, 1e-13, "ICH", P.complex)
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    out = s.forward_path(cm, ck, ca, omega, qvec, mvec, L)
    ref = oracle_mod.forward_path(om, P.qm.Q, P.qm.M, P.qm.link_ofs, P.qm.link_m, P.mua, P.mus, P.nref,
                                  P.freq_mhz, P.qwidth, P.mwidth, method, "ICH", 1e-13)
    assert rel2(out["dphi"], ref.dphi) < 1e-10
    assert rel2(out["aphi"], ref.aphi) < 1e-10
    assert relmax(out["proj"], ref.proj) < 1e-9
    assert relmax(out["logproj"], ref.logproj) < 1e-9
    assert rel2(out["J"], ref.J) < 1e-10
    # the stand-alone entry points agree with the fused path
    lp = s.project_all(mvec, out["dphi"], L, capi.DATA_LOG)
    assert relmax(lp, out["logproj"]) < 1e-13
    J2 = s.jacobian(out["dphi"], out["aphi"], out["proj"], L)
    assert rel2(J2, out["J"]) < 1e-13


def test_mixed_precision_boundary_data(case, oracle_mod):
    """The mixed path (FP32 inner process, FP64 refinement until the
    componentwise backward error is 1e-10) against the oracle's exact FP64
    solve (the direct factorisation): fields, boundary data entry by entry,
    and the Jacobian, each within 1e-8; the FP32 Jacobian of the same fields
    within 1e-6 (FP32 products and storage)."""
    P, om, gm = case
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    method = "BICGSTAB" if P.complex else "CG"
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    s = capi.FwdSolver(gm, method, 1e-12, "ICH", P.complex, precision="mixed")
    out = s.forward_path(cm, ck, ca, omega, qvec, mvec, L)
    ref = oracle_mod.forward_path(om, P.qm.Q, P.qm.M, P.qm.link_ofs, P.qm.link_m, P.mua, P.mus, P.nref,
                                  P.freq_mhz, P.qwidth, P.mwidth, "DIRECT", jac=True)
    assert rel2(out["dphi"], ref.dphi) < 1e-10 and rel2(out["aphi"], ref.aphi) < 1e-10
    assert relmax(out["proj"], ref.proj) < 1e-8
    lp, lr = np.asarray(out["logproj"]), np.asarray(ref.logproj)
    assert np.array_equal(np.isnan(lp), np.isnan(lr))
    ok = np.isfinite(lp) & np.isfinite(lr)
    assert np.max(np.abs(lp - lr)[ok]) < 1e-8
    assert rel2(out["J"], ref.J) < 1e-8
    J32 = s.jacobian(out["dphi"], out["aphi"], out["proj"], L, fp32=True)
    assert rel2(J32, ref.J) < 1e-6
    # FP32 storage of the FP64-accurate sums: each entry is the FP64 J
    # rounded once to float
    J32a = s.jacobian(out["dphi"], out["aphi"], out["proj"], L, fp32=2).astype(np.float64)
    J64 = np.asarray(out["J"])
    assert np.all(np.abs(J32a - J64) <= 6.0e-8 * np.abs(J64) + 1e-300)


def test_tensor_core_jacobian_matches_float_float(case, oracle_mod, monkeypatch):
    """The complex FP64 Jacobian on the tensor cores (exact bf16 digit
    products) and the float-float kernel, on the same GPU fields, against the
    oracle's FP64 Jacobian of those fields: both at the FP64 rounding level."""
    P, om, gm = case
    if not P.complex:
        pytest.skip("the tensor-core Jacobian is the complex path")
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    s = capi.FwdSolver(gm, "BICGSTAB", 1e-12, "ICH", True)
    L = capi.Links(P.qm.link_ofs, P.qm.link_m)
    out = s.forward_path(cm, ck, ca, capi.omega_of(P.freq_mhz), qvec, mvec, L)
    Joz = np.asarray(s.jacobian(out["dphi"], out["aphi"], out["proj"], L))
    monkeypatch.setenv("TOASTGPU_JAC_OZ", "0")
    Jff = np.asarray(s.jacobian(out["dphi"], out["aphi"], out["proj"], L))
    Jor = oracle_mod.jacobian(om, np.asarray(out["dphi"]), np.asarray(out["aphi"]), np.asarray(out["proj"]),
                              P.qm.link_ofs, P.qm.link_m)
    assert rel2(Joz, Jor) < 2e-14
    assert rel2(Jff, Jor) < 5e-14
    assert np.max(np.abs(Joz - Jor)) < 5e-14 * np.max(np.abs(Jor))
    assert rel2(Joz, np.asarray(out["J"])) == 0.0  # the fused path uses the same kernel


def test_componentwise_bound_off_is_normwise(case):
    """With the componentwise bound off the mixed path stops on the normwise
    test alone (fewer iterations); both results meet the normwise tolerance."""
    P, om, gm = case
    cm, ck, ca, qvec, mvec = gpu_problem_inputs(P, gm)
    omega = capi.omega_of(P.freq_mhz)
    method = "BICGSTAB" if P.complex else "CG"
    its = {}
    for cw in (0.0, 1e-10):
        s = capi.FwdSolver(gm, method, 1e-12, "ICH", P.complex, precision="mixed")
        s.set_backward_error(cw)
        s.reset(cm, ck, ca, omega)
        phi, res = s.calc_fields(np.concatenate([qvec, mvec]))
        assert all(r[1] == 0 and r[2] <= 1e-12 for r in res), res
        its[cw] = sum(r[0] for r in res)
    assert its[0.0] <= its[1e-10]
    with pytest.raises(capi.ToastGPUError):
        s.set_backward_error(-1.0)


@pytest.mark.parametrize("neumann", [True, False], ids=["neumann", "isotropic"])
def test_source_vectors_on_device(case, neumann):
    """tg_qvec_gaussian_ex (device) against the host QVec_Gaussian: the same
    sums in the same order; the device's rounding of exp(-d^2 / 2w^2) and of
    its argument shows in the far tail (values near e^-300, where one unit of
    the argument's last place is 3e-14 of the value), so the elementwise
    bound is 1e-12 and the L2 one 1e-15; detector vectors times c2a."""
    P, om, gm = case
    q_host = gm.qvec_gaussian(P.qm.Q, P.qwidth, neumann)
    q_dev = gm.qvec_gaussian_device(P.qm.Q, P.qwidth, neumann)
    assert relmax(q_dev, q_host) < 1e-12
    assert rel2(q_dev, q_host) < 1e-15
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    m_dev = gm.qvec_gaussian_device(P.qm.M, P.mwidth, neumann, scale=ca)
    m_host = gm.qvec_gaussian(P.qm.M, P.mwidth, neumann) * ca[None, :]
    assert relmax(m_dev, m_host) < 1e-12
    assert rel2(m_dev, m_host) < 1e-15
    torch = pytest.importorskip("torch")
    d_out = torch.zeros((len(P.qm.Q), gm.n), dtype=torch.float64, device="cuda")
    gm.qvec_gaussian_device(P.qm.Q, P.qwidth, neumann, out=d_out)
    assert relmax(d_out.cpu().numpy(), q_host) < 1e-12


def test_mesh_file_load(case, tmp_path):
    """tg_mesh_load on a file in the reference's format equals the mesh built
    from the arrays (geometry, CSR, boundary), trailing sections ignored."""
    from toastpp_gb300 import meshio
    P, om, gm = case
    path = str(tmp_path / "m.msh")
    meshio.write_mesh(path, P.coords, P.elems)
    with open(path, "a") as f:
        f.write("\n[ParameterList]\nSize 1\nParam1 MUA\n")
    lm = capi.Mesh.load(path)
    coords, el = lm.geometry()
    assert np.array_equal(el, P.elems) and np.allclose(coords, P.coords, rtol=0, atol=1e-15 * np.abs(P.coords).max())
    rp, ci = lm.csr()
    rp0, ci0 = gm.csr()
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0)
    assert np.array_equal(lm.boundary(), gm.boundary())


def test_inner_tolerance_bound(case):
    """The mixed path refuses inner tolerances below 1e-5, where its FP32
    process stagnates or diverges, and accepts the bound itself."""
    P, om, gm = case
    s = capi.FwdSolver(gm, "BICGSTAB" if P.complex else "CG", 1e-12, "ICH", P.complex, precision="mixed")
    with pytest.raises(capi.ToastGPUError):
        s.set_refinement(1e-6)
    s.set_refinement(1e-5)
