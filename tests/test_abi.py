"""The C-ABI library: it builds for sm_103a, loads, and exports every entry
point that include/toastgpu.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

from toastpp_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "toastgpu.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\s*\*)\s*(tg_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    return ctypes.CDLL(build.build(verbose=False))


def test_header_declares_the_boundary():
    names = declared()
    for required in ["tg_mesh_create", "tg_solver_create", "tg_solver_reset", "tg_calc_fields", "tg_project_all",
                     "tg_jacobian", "tg_forward_path", "tg_project_all_noalloc", "tg_last_error"]:
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    assert set(declared()) <= set(capi.EXPORTS), sorted(set(declared()) - set(capi.EXPORTS))


def test_library_has_no_cpu_fallback_symbols(lib):
    # the product library carries no CPU solver: the oracle's entry points are
    # not linked into it
    for n in ["tor_solve", "tor_assemble", "tor_jacobian", "tor_project"]:
        assert not hasattr(lib, n)


def test_error_path_without_gpu(lib):
    # argument checks run before any device call
    lib.tg_last_error.restype = ctypes.c_char_p
    h = ctypes.c_void_p()
    rc = lib.tg_mesh_create(4, 0, None, 0, None, ctypes.byref(h))
    assert rc == 1  # TG_ERR_ARG
    assert lib.tg_last_error()


def test_server_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    lib.tg_server_create.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]
    assert lib.tg_server_create(2, 1.0, ctypes.byref(h)) == 3  # TG_ERR_CUDA
    assert lib.tg_server_create(0, 1.0, ctypes.byref(h)) == 1  # TG_ERR_ARG


def test_cpp_face_compiles_and_links(tmp_path):
    """include/toastgpu.hpp builds into a caller and links against the library."""
    from tests.cpp_shim import build
    assert os.path.exists(build(str(tmp_path)))


@pytest.mark.parametrize("text,code", [
    ("not a mesh\n", 1),                                                      # no MeshData 5.0 header
    ("MeshData 5.0\n\nNodeList 3 1\nN[0 0]R0\nN[1 0]R0\n", 1),                # truncated node list
    ("MeshData 5.0\n\nNodeList 3 1\nN[0 0]R0\nN[1 0]R0\nN[0 1]R0\n\nElementList 1\nq 1 2 3 4\n", 5),  # 4-noded quad
    ("MeshData 5.0\n\nNodeList 3 1\nN[0 0]R0\nN[1 0]R0\nN[0 1]R0\n\nElementList 1\no 1 2 9\n", 1),    # index out of range
])
def test_mesh_file_errors_without_gpu(lib, tmp_path, text, code):
    """tg_mesh_load parses on the host and rejects bad files before any
    device call: missing header, truncated lists, element types other than
    P1 triangles / tetrahedra, out-of-range node indices."""
    p = tmp_path / "m.msh"
    p.write_text(text)
    h = ctypes.c_void_p()
    lib.tg_mesh_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
    assert lib.tg_mesh_load(str(p).encode(), ctypes.byref(h)) == code
    assert not h.value

