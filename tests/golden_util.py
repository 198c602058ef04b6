"""Loading of the golden fixtures in tests/golden (outputs of the reference
itself; see tests/golden/make_golden.py)."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(nodal_only=False):
    """Forward-path fixture names (not the QM-file ones); nodal_only drops the
    element-basis fixtures (*_el), whose solves use one coefficient per
    element."""
    out = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    out = [n for n in out if not n.startswith("qm_") and not n.startswith("ref_")]
    return [n for n in out if not n.endswith("_el")] if nodal_only else out


def qm_names():
    """The QM-file fixtures: a QM text, its mesh and what the reference's
    LoadQM made of them (positions after InitM, link list)."""
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "qm_*.npz")))


def load_qm(name, tmp_path):
    """(fixture dict, path of its QM text written under tmp_path)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    d["qm_text"] = str(d["qm_text"])
    path = os.path.join(str(tmp_path), name + ".qm")
    with open(path, "w") as f:
        f.write(d["qm_text"])
    return d, path


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    for k in ("solver", "precon"):
        d[k] = str(d[k])
    for k in ("freq_mhz", "qwidth", "mwidth", "tol"):
        d[k] = float(d[k])
    return d


def sparse_links(g):
    """A subset of the fixture's links: source 1 keeps none, source 0 keeps
    all, the others every second detector.  Returns (link_ofs, link_m,
    indices of the kept links)."""
    ofs, lm = g["link_ofs"], g["link_m"]
    new_ofs, new_m, keep = [0], [], []
    for q in range(len(ofs) - 1):
        for i in range(ofs[q], ofs[q + 1]):
            if q != 1 and (q == 0 or (q + int(lm[i])) % 2 == 0):
                new_m.append(int(lm[i]))
                keep.append(i)
        new_ofs.append(len(new_m))
    return np.array(new_ofs, np.int32), np.array(new_m, np.int32), np.array(keep)
