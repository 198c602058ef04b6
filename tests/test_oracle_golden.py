"""The oracle against the reference's own forward-model golden vectors.

The reference's regression tests (test/2D/fwdfem/Makefile:24-174,
test/3D/fwdfem/Makefile:9-77) run fwdfem / fwdfem_cw on circle25_32.msh
(3511 nodes, 32 x 32 links) and cyl2.msh (9043 nodes, 80 x 80 links) and
compare ln|y| (fmod) and arg y (farg) with cmpvec -r=<tol>.  These tests run
the oracle on the same meshes, optodes and parameters and apply the same
element-wise relative tolerance.  They read the reference tree and skip
where it is absent.
"""
import os
import zipfile

import numpy as np
import pytest

from tests.conftest import REFERENCE, has_reference
from tests.gpu_util import relmax
from toastpp_gb300 import meshio

pytestmark = pytest.mark.skipif(not has_reference(), reason="reference tree not available")

T = os.path.join(REFERENCE, "test")

# (dim, kind, method, precon, tag, tol_fmod, tol_farg): the Makefile targets
CASES_2D = [
    ("real", "CG", "NONE", "cg", 1e-8, None),
    ("real", "CG", "DIAG", "cg_diag", 1e-8, None),
    ("real", "CG", "ICH", "cg_ich", 1e-8, None),
    ("cplx", "BICGSTAB", "NONE", "bicgstab", 1e-7, 1e-6),
    ("cplx", "BICGSTAB", "DIAG", "bicgstab_diag", 1e-7, 1e-6),
    ("cplx", "BICGSTAB", "ICH", "bicgstab_ich", 1e-7, 1e-7),
    ("cplx", "BICGSTAB", "DILU", "bicgstab_dilu", 1e-7, 1e-6),
    ("cplx", "GMRES", "NONE", "gmres", 1e-7, 1e-7),
    ("cplx", "GMRES", "DIAG", "gmres_diag", 1e-7, 1e-7),
    ("cplx", "GMRES", "ICH", "gmres_ich", 1e-7, 1e-7),
    ("cplx", "GMRES", "DILU", "gmres_dilu", 1e-7, 1e-7),
]
CASES_3D = [
    ("real", "CG", "NONE", "cg", 1e-8, None),
    ("real", "CG", "ICH", "cg_ich", 1e-8, None),
    ("cplx", "BICGSTAB", "NONE", "bicgstab", 1e-8, 1e-8),
    ("cplx", "BICGSTAB", "ICH", "bicgstab_ich", 1e-8, 1e-8),
]
SETUP = {
    2: ("circle25_32.msh", "circle25_32x32.qm", "2D/fwdfem/testdata.zip", 0.025, 2.0),
    3: ("cyl2.msh", "cyl_5ring.qm", "3D/fwdfem/testdata.zip", 0.01, 1.0),
}


def golden(zpath, name):
    with zipfile.ZipFile(zpath) as z:
        txt = z.read(name).decode()
    return np.array(txt.replace("[", " ").replace("]", " ").split(), float)


_problems = {}


def problem(dim, oracle_mod):
    if dim not in _problems:
        msh, qmf, _, _, _ = SETUP[dim]
        coords, els = meshio.read_mesh(os.path.join(T, f"{dim}D", "meshes", msh))
        qm = meshio.read_qm(os.path.join(T, f"{dim}D", "meshes", qmf))
        mesh = oracle_mod.Mesh(coords, els)
        M = mesh.place_detectors(qm.M, qm.m_fixed)
        _problems[dim] = (mesh, qm, M)
    return _problems[dim]


def run_case(oracle_mod, dim, kind, method, precon):
    mesh, qm, M = problem(dim, oracle_mod)
    _, _, _, mua, mus = SETUP[dim]
    n = mesh.n
    # fwdfem: 100 MHz for the complex runs, Gaussian source/detector width 2,
    # tol 1e-15, maxit 10000 (the Makefile's stdin scripts)
    return oracle_mod.forward_path(mesh, qm.Q, M, qm.link_ofs, qm.link_m, np.full(n, mua), np.full(n, mus),
                                   np.full(n, 1.4), freq_mhz=100.0 if kind == "cplx" else 0.0, method=method,
                                   precon=precon, tol=1e-15, maxit=10000, jac=False, nthreads=8)


@pytest.mark.parametrize("kind,method,precon,tag,tol_mod,tol_arg", CASES_2D, ids=[c[3] for c in CASES_2D])
def test_golden_2d(oracle_mod, kind, method, precon, tag, tol_mod, tol_arg):
    res = run_case(oracle_mod, 2, kind, method, precon)
    z = os.path.join(T, SETUP[2][2])
    if kind == "cplx":
        assert relmax(res.logproj.real, golden(z, f"fmod_cplx_{tag}.fem")) <= tol_mod
        assert relmax(res.logproj.imag, golden(z, f"farg_cplx_{tag}.fem")) <= tol_arg
    else:
        assert relmax(res.logproj, golden(z, f"fmod_real_{tag}.fem")) <= tol_mod


@pytest.mark.parametrize("kind,method,precon,tag,tol_mod,tol_arg", CASES_3D, ids=[c[3] for c in CASES_3D])
def test_golden_3d(oracle_mod, kind, method, precon, tag, tol_mod, tol_arg):
    res = run_case(oracle_mod, 3, kind, method, precon)
    z = os.path.join(T, SETUP[3][2])
    if kind == "cplx":
        assert relmax(res.logproj.real, golden(z, f"fmod_cplx_{tag}.fem")) <= tol_mod
        assert relmax(res.logproj.imag, golden(z, f"farg_cplx_{tag}.fem")) <= tol_arg
    else:
        assert relmax(res.logproj, golden(z, f"fmod_real_{tag}.fem")) <= tol_mod
