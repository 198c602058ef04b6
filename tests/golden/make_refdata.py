"""Packs the reference's own forward-model regression data into fixtures the
GPU tests can read on a machine without the reference tree.

The reference's direct-solver goldens (fmod/farg_*_direct) are computed on
ellips_tri10.msh, a mesh of 10-noded triangles, outside this P1 path; they
are not packed.

The reference's regression tests (test/2D/fwdfem/Makefile:24-174,
test/3D/fwdfem/Makefile:9-77) run fwdfem / fwdfem_cw on its test meshes and
compare ln|y| (fmod) and arg y (farg) with cmpvec -r=<tol> against the
golden vectors in testdata.zip.  For each mesh this script stores, in
tests/golden/ref_<mesh>.npz:

- the mesh (node coordinates, elements) as the reference reads it;
- the source positions and the detector positions after QMMesh::InitM's
  placement (done by the oracle, which equals the reference's placement bit
  for bit, tests/test_oracle_fixtures.py) and the link list;
- the nodal mua / mus' of the runs (constants here; the NIM reader serves
  image-valued runs);
- every golden vector of the mesh (fmod_*, farg_*).

Usage:  python tests/golden/make_refdata.py [reference tree]
        (default: $TOASTPP_REFERENCE)
"""
import os
import sys
import zipfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from toastpp_gb300 import meshio  # noqa: E402

# name -> (dim, mesh, qm, testdata, {"mua": value or NIM file, "mus": ...}, golden names)
SETS = {
    "circle25_32": (2, "circle25_32.msh", "circle25_32x32.qm", "2D/fwdfem/testdata.zip", 0.025, 2.0,
                    ["real_cg", "real_cg_diag", "real_cg_ich", "cplx_bicgstab", "cplx_bicgstab_diag",
                     "cplx_bicgstab_ich", "cplx_bicgstab_dilu", "cplx_gmres", "cplx_gmres_diag", "cplx_gmres_ich",
                     "cplx_gmres_dilu"]),
    "cyl2": (3, "cyl2.msh", "cyl_5ring.qm", "3D/fwdfem/testdata.zip", 0.01, 1.0,
             ["real_cg", "real_cg_ich", "cplx_bicgstab", "cplx_bicgstab_ich"]),
}


def read_nim(path):
    """A nodal image file (fwdfem.cc ReadNim): header up to EndHeader with
    ImageSize, then the values after the first line starting with Image."""
    with open(path) as f:
        lines = f.read().splitlines()
    assert lines[0].strip() == "NIM"
    size = 0
    i = 1
    while lines[i].strip().lower() != "endheader":
        if lines[i].lower().startswith("imagesize"):
            size = int(lines[i].split("=")[1])
        i += 1
    while not lines[i].lower().startswith("image"):
        i += 1
    vals = np.array(" ".join(lines[i + 1:]).split(), float)
    return vals[:size]


def golden(z, name):
    txt = z.read(name).decode()
    return np.array(txt.replace("[", " ").replace("]", " ").split(), float)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TOASTPP_REFERENCE", "")
    T = os.path.join(ref, "test")
    for name, (dim, msh, qmf, tz, mua, mus, gold) in SETS.items():
        md = os.path.join(T, f"{dim}D", "meshes")
        coords, els = meshio.read_mesh(os.path.join(md, msh))
        qm = meshio.read_qm(os.path.join(md, qmf))
        mesh = oracle.Mesh(coords, els)
        M = mesh.place_detectors(qm.M, qm.m_fixed)
        n = len(coords)
        mua_v = read_nim(os.path.join(md, mua)) if isinstance(mua, str) else np.full(n, mua)
        mus_v = read_nim(os.path.join(md, mus)) if isinstance(mus, str) else np.full(n, mus)
        out = dict(coords=coords, elems=els.astype(np.int32), Q=qm.Q, M=M, link_ofs=qm.link_ofs.astype(np.int32),
                   link_m=qm.link_m.astype(np.int32), mua=mua_v, mus=mus_v, nref=np.full(n, 1.4))
        with zipfile.ZipFile(os.path.join(T, tz)) as z:
            for g in gold:
                out["fmod_" + g] = golden(z, f"fmod_{g}.fem")
                if g.startswith("cplx"):
                    out["farg_" + g] = golden(z, f"farg_{g}.fem")
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **out)
        print(name, n, len(els), os.path.getsize(path))


if __name__ == "__main__":
    main()
