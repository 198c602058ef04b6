"""Build and input helpers for the C++ caller tests/cpp/fwd_shim.cc."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build(outdir):
    from toastpp_gb300 import build as B
    lib = B.build(verbose=False)
    exe = os.path.join(outdir, "fwd_shim")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "fwd_shim.cc"), "-o", exe, lib,
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def write_input(path, P, cmua, ckap, c2a):
    with open(path, "wb") as f:
        np.array([P.dim, P.n, len(P.elems), P.qm.nQ, P.qm.nM, int(P.complex)], np.int32).tofile(f)
        np.array([P.freq_mhz, P.qwidth], np.float64).tofile(f)
        np.ascontiguousarray(P.coords, np.float64).tofile(f)
        np.ascontiguousarray(P.elems, np.int32).tofile(f)
        np.concatenate([cmua, ckap, c2a]).astype(np.float64).tofile(f)
        np.ascontiguousarray(P.qm.Q, np.float64).tofile(f)
        np.ascontiguousarray(P.qm.M, np.float64).tofile(f)
