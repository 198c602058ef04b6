"""The C++ face (include/toastgpu.hpp) driven by a compiled caller in the
reference's call sequence gives the C ABI's results bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from tests.cpp_shim import build, write_input
from tests.gpu_util import small_cyl, small_disc
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make", [lambda: small_disc(0.0), lambda: small_cyl(100.0)], ids=["disc_cw", "cyl_fd"])
def test_cpp_caller_matches_c_abi(tmp_path, make):
    P = make()
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, P, cm, ck, ca)
    exe = build(str(tmp_path))
    subprocess.run([exe, inp, out], check=True)
    gm = capi.Mesh(P.coords, P.elems)
    q = gm.qvec_gaussian(P.qm.Q, P.qwidth)
    m = gm.qvec_gaussian(P.qm.M, P.mwidth) * ca[None, :]
    s = capi.FwdSolver(gm, "BICGSTAB" if P.complex else "CG", 1e-12, "ICH", P.complex)
    r = s.forward_path(cm, ck, ca, capi.omega_of(P.freq_mhz), q, m, capi.Links(P.qm.link_ofs, P.qm.link_m))
    raw = np.fromfile(out, np.float64)
    nqm = P.qm.nQM
    nl = 2 * nqm if P.complex else nqm
    lp = raw[:nl].view(np.complex128) if P.complex else raw[:nl]
    J = raw[nl:nl + r["J"].size].reshape(r["J"].shape)
    assert np.array_equal(lp, r["logproj"])
    assert np.array_equal(J, r["J"])
    # grid basis: Raster_Pixel of 12 points per axis
    rast = capi.Raster(gm, [12] * P.dim)
    Jg = s.jacobian_grid(rast, r["dphi"], r["aphi"], r["proj"], capi.Links(P.qm.link_ofs, P.qm.link_m))
    assert np.array_equal(raw[nl + r["J"].size:].reshape(Jg.shape), Jg)


def test_cpp_load_qm(tmp_path):
    """Mesh(path) and LoadQM through the C++ face give the reference's QM
    positions and links (tests/golden/qm_cyl_pull.npz) bit for bit."""
    from tests.golden_util import load_qm
    from toastpp_gb300 import meshio
    g, qpath = load_qm("qm_cyl_pull", tmp_path)
    mpath, out = str(tmp_path / "m.msh"), str(tmp_path / "qm.bin")
    meshio.write_mesh(mpath, g["coords"], g["elems"])
    exe = build(str(tmp_path))
    subprocess.run([exe, "qm", mpath, qpath, out], check=True)
    raw = open(out, "rb").read()
    dim, nq, nm, nqm = np.frombuffer(raw[:16], np.int32)
    o = 16
    Q = np.frombuffer(raw[o:o + 8 * nq * dim], np.float64).reshape(nq, dim)
    o += 8 * nq * dim
    M = np.frombuffer(raw[o:o + 8 * nm * dim], np.float64).reshape(nm, dim)
    o += 8 * nm * dim
    ofs = np.frombuffer(raw[o:o + 4 * (nq + 1)], np.int32)
    o += 4 * (nq + 1)
    lm = np.frombuffer(raw[o:o + 4 * nqm], np.int32)
    assert np.array_equal(Q, g["qpos"]) and np.array_equal(M, g["mpos"])
    assert np.array_equal(ofs, g["link_ofs"]) and np.array_equal(lm, g["link_m"])
