"""The reference-typed shim (toastpp_gb300/shim): the reference's own callers
of the forward path relink unedited against libtoastgpu.so.

toastpp_gb300/shim/Makefile compiles src/supertoast/fwdfem.cc and
fwdfem_cw.cc from the reference tree as they are, and the reference-sequence
driver oracle/ref_driver.cc, and links them against the reference's objects
with its fwdsolver object replaced by fwdsolver_gpu.cc and its five public
GenerateJacobian functions by jacobian_gpu.cc.  These tests need the
reference tree and the compiled reference (oracle/Makefile.ref) and skip
without them.  Where no GPU is present the scripted fwdfem_cw run must get
through the reference's own parameter prompts to the GPU library (which then
reports that it has no device)."""
import os
import subprocess

import pytest

from tests.conftest import REFERENCE, has_reference

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "toastpp_gb300", "_build", "shim")
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libtoastref.a")

pytestmark = pytest.mark.skipif(not (has_reference() and os.path.exists(REFLIB)),
                                reason="reference tree or compiled reference not available")


@pytest.fixture(scope="module")
def built():
    from toastpp_gb300 import build as B
    B.build()
    r = subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "toastpp_gb300", "shim", "Makefile"),
                        f"REF={REFERENCE}", "-j8"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return OUT


def symbols(path):
    return subprocess.run(["nm", "-C", path], capture_output=True, text=True, check=True).stdout


def test_reference_callers_link_against_the_gpu_library(built):
    for prog in ("fwdfem_gpu", "fwdfem_cw_gpu", "ref_driver_gpu"):
        path = os.path.join(built, prog)
        assert os.path.exists(path), prog
        syms = symbols(path)
        # TFwdSolver members and the Jacobian come from the shim, which calls the C ABI
        assert "U tg_solver_create" in syms and "U tg_calc_fields" in syms
    shim = symbols(os.path.join(built, "fwdsolver_gpu.o"))
    for member in ("TFwdSolver<std::complex<double> >::CalcFields", "TFwdSolver<double>::Reset",
                   "TFwdSolver<std::complex<double> >::ProjectAll_real", "TFwdSolver<double>::Allocate"):
        assert member in shim, member
    jac = symbols(os.path.join(built, "jacobian_gpu.o"))
    assert jac.count(" T GenerateJacobian") >= 5


def test_fwdfem_cw_runs_its_script_to_the_gpu(built, tmp_path):
    """fwdfem_cw with the reference's own stdin script (test/2D/fwdfem/Makefile:35-43,
    CG, tol 1e-15) in a scratch directory laid out like the test directory."""
    torch = pytest.importorskip("torch")
    meshes = tmp_path / "meshes"
    run = tmp_path / "fwdfem"
    meshes.mkdir()
    run.mkdir()
    for f in ("circle25_32.msh", "circle25_32x32.qm"):
        os.symlink(os.path.join(REFERENCE, "test", "2D", "meshes", f), meshes / f)
    script = "../meshes/circle25_32.msh ../meshes/circle25_32x32.qm 2 2 1e-15 10000 0 1 2 2 2 2 2 0.025 2 2 2 1.4 0 1\n"
    r = subprocess.run([os.path.join(built, "fwdfem_cw_gpu")], input=script, cwd=str(run), capture_output=True,
                       text=True, timeout=300)
    if not torch.cuda.is_available():
        assert r.returncode != 0
        assert "tg_mesh_create" in (r.stdout + r.stderr)
    else:
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        assert os.path.exists(run / "fmod.fem")
