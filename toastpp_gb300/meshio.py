"""Mesh and QM file I/O in the reference's text formats.

Mesh files ("MeshData 5.0") follow the reader in src/libfe/mesh.cc:1787-1836,
src/libfe/ndlist.cc:146 and src/libfe/ellist.cc:154-195: a NodeList of
``N[x y]R0`` / ``B[x y z]R0`` lines and an ElementList whose lines start with a
one-letter type code ('o' = 3-noded triangle, 'c' = 4-noded tetrahedron,
src/libfe/element.h:30-49) followed by 1-based node indices.

QM files follow QMMesh::LoadQM (src/libfe/qmmesh.cc:319-460): SourceList,
MeasurementList and LinkList sections.
"""
from __future__ import annotations

import re
from dataclasses import dataclass

import numpy as np

_TYPE_NN = {"o": 3, "c": 4}
_NN_TYPE = {3: "o", 4: "c"}


@dataclass
class QMSpec:
    """Source/detector positions and the measurement link list."""

    Q: np.ndarray            # nQ x dim
    M: np.ndarray            # nM x dim
    link_ofs: np.ndarray     # nQ+1 int32, offsets into link_m (Qofs)
    link_m: np.ndarray       # nQM int32, detector index per measurement (QMref)
    q_fixed: bool = False
    m_fixed: bool = False
    # "external" lists (qmmesh.cc:343-344, 404-405): sources are moved to the
    # boundary along their normals when the mesh is attached, detectors stay
    # where they were read.  QN / MN hold the normals read with the positions
    # (zero where a line has none); *_default_normals is the "default" flag
    # (the direction -q instead of the normal read)
    q_external: bool = False
    m_external: bool = False
    QN: np.ndarray | None = None
    MN: np.ndarray | None = None
    q_default_normals: bool = False
    m_default_normals: bool = False

    @property
    def nQ(self) -> int:
        return int(self.Q.shape[0])

    @property
    def nM(self) -> int:
        return int(self.M.shape[0])

    @property
    def nQM(self) -> int:
        return int(self.link_ofs[-1])

    @staticmethod
    def all_to_all(Q: np.ndarray, M: np.ndarray) -> "QMSpec":
        nq, nm = len(Q), len(M)
        ofs = np.arange(nq + 1, dtype=np.int32) * nm
        lm = np.tile(np.arange(nm, dtype=np.int32), nq)
        return QMSpec(np.asarray(Q, float), np.asarray(M, float), ofs, lm, True, True)


def read_mesh(path: str):
    """Return (coords[n,dim] float64, elems[ne,nn] int32 0-based)."""
    with open(path) as f:
        text = f.read()
    pos = text.find("NodeList")
    if pos < 0:
        raise ValueError(f"{path}: NodeList not found")
    lines = text[pos:].splitlines()
    n = int(lines[0].split()[1])
    coords = []
    for ln in lines[1:1 + n]:
        inner = ln[ln.index("[") + 1: ln.index("]")]
        coords.append([float(v) for v in inner.split()])
    coords = np.asarray(coords, dtype=np.float64)
    epos = text.find("ElementList")
    elines = text[epos:].splitlines()
    ne = int(elines[0].split()[1])
    els = []
    for ln in elines[1:1 + ne]:
        tok = ln.split()
        if tok[0] not in _TYPE_NN:
            raise ValueError(f"unsupported element type '{tok[0]}' (only P1 triangles and tetrahedra)")
        nn = _TYPE_NN[tok[0]]
        els.append([int(v) - 1 for v in tok[1:1 + nn]])
    return coords, np.asarray(els, dtype=np.int32)


def write_mesh(path: str, coords: np.ndarray, elems: np.ndarray) -> None:
    """Write a mesh the reference can read (node boundary flags are recomputed
    by the reader's Mesh::Setup, so every node is written as 'N')."""
    coords = np.asarray(coords, float)
    elems = np.asarray(elems)
    code = _NN_TYPE[elems.shape[1]]
    with open(path, "w") as f:
        f.write("MeshData 5.0\n\n")
        f.write(f"NodeList {len(coords)} 1\n")
        for p in coords:
            f.write("N[" + " ".join(repr(float(v)) for v in p) + "]R0\n")
        f.write(f"\nElementList {len(elems)}\n")
        for e in elems:
            f.write(code + " " + " ".join(str(int(v) + 1) for v in e) + "\n")


def read_qm(path: str) -> QMSpec:
    """Parse a QM file (QMMesh::LoadQM, src/libfe/qmmesh.cc:319-460)."""
    with open(path) as f:
        lines = f.read().splitlines()
    if not lines[0].startswith("QM file"):
        raise ValueError("QM file not found or invalid format")
    dim = int(lines[1].split()[1])
    i = 2

    def section(tag):
        nonlocal i
        while not lines[i].startswith(tag):
            i += 1
        hdr = lines[i][len(tag):].split()
        cnt = int(hdr[0])
        flag = hdr[1].lower() if len(hdr) > 1 else ""
        # normals are "specified" unless a third token says "default"
        default_normals = len(hdr) > 2 and hdr[2].lower() == "default"
        pts, nrm = [], []
        for k in range(cnt):
            vals = [float(v) for v in lines[i + 1 + k].split()[:2 * dim]]
            pts.append(vals[:dim])
            nrm.append((vals[dim:] + [0.0] * dim)[:dim])
        i += 1 + cnt
        return (np.asarray(pts, float).reshape(-1, dim), np.asarray(nrm, float).reshape(-1, dim), flag,
                default_normals)

    Q, QN, qflag, qdef = section("SourceList")
    M, MN, mflag, mdef = section("MeasurementList")
    while not lines[i].startswith("LinkList"):
        i += 1
    rest = " ".join(lines[i + 1:])
    ofs = [0]
    lm = []
    for q in range(len(Q)):
        m = re.match(r"\s*(\d+)\s*:", rest)
        cnt = int(m.group(1))
        rest = rest[m.end():]
        toks = rest.split(None, cnt)
        lm.extend(int(t) for t in toks[:cnt])
        rest = toks[cnt] if len(toks) > cnt else ""
        ofs.append(ofs[-1] + cnt)
    return QMSpec(Q, M, np.asarray(ofs, np.int32), np.asarray(lm, np.int32), qflag == "fixed", mflag == "fixed",
                  qflag == "external", mflag == "external", QN, MN, qdef, mdef)


def write_qm(path: str, qm: QMSpec) -> None:
    dim = qm.Q.shape[1]
    with open(path, "w") as f:
        f.write(f"QM file {dim}D\nDimension {dim}\n\n")
        f.write(f"SourceList {qm.nQ} fixed\n")
        for p in qm.Q:
            f.write(" ".join(repr(float(v)) for v in p) + "\n")
        f.write(f"\nMeasurementList {qm.nM} fixed\n")
        for p in qm.M:
            f.write(" ".join(repr(float(v)) for v in p) + "\n")
        f.write("\nLinkList\n")
        for q in range(qm.nQ):
            ms = qm.link_m[qm.link_ofs[q]:qm.link_ofs[q + 1]]
            f.write(f"{len(ms)}: " + " ".join(str(int(m)) for m in ms) + "\n")
