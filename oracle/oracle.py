"""ctypes wrapper of the CPU oracle (oracle/toast_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of bench.py, as the checker.  The product path
never imports it.

``forward_path`` restates the reference's caller sequence for one problem:
source/measurement vectors (src/supertoast/fwdfem.cc:127-176,
src/python/toastmodule.cc:1189-1220), assembly and preconditioner reset
(src/libstoast/fwdsolver.cc:493-505), forward and adjoint CalcFields (653-750),
ProjectAll (1415-1447) and the nodal Jacobian (src/libstoast/jacobian.cc:441-497,
738-802).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "toast_oracle.c")
LIB = os.path.join(HERE, "libtoast_oracle.so")

_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the oracle shared library in place (gcc, a second or two)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, SRC, "-lm", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.tor_mesh_create.restype = C.c_void_p
        L.tor_mesh_create.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip]
        L.tor_mesh_free.argtypes = [C.c_void_p]
        L.tor_mesh_nnz.restype = C.c_int
        L.tor_mesh_nnz.argtypes = [C.c_void_p]
        L.tor_mesh_csr.argtypes = [C.c_void_p, _ip, _ip]
        L.tor_mesh_bndnodes.argtypes = [C.c_void_p, _up]
        L.tor_mesh_elsize.argtypes = [C.c_void_p, _dp]
        L.tor_pull_to_boundary.restype = C.c_int
        L.tor_pull_to_boundary.argtypes = [C.c_void_p, _dp, _dp]
        L.tor_rcm.argtypes = [C.c_int, _ip, _ip, _ip]
        L.tor_nd_order.argtypes = [C.c_int, _ip, _ip, _dp, C.c_int, _ip]
        L.tor_direct_factor.restype = C.c_void_p
        L.tor_direct_factor.argtypes = [C.c_int, _ip, _ip, _dp, C.c_int, C.c_void_p]
        L.tor_direct_nnz.restype = C.c_int
        L.tor_direct_nnz.argtypes = [C.c_void_p]
        L.tor_direct_free.argtypes = [C.c_void_p]
        L.tor_direct_solve.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.tor_el_found.restype = C.c_int
        L.tor_el_found.argtypes = [C.c_void_p, _dp]
        L.tor_bnd_intersect.restype = C.c_int
        L.tor_bnd_intersect.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.tor_external_source.restype = C.c_int
        L.tor_external_source.argtypes = [C.c_void_p, _dp, C.c_void_p, _dp]
        L.tor_qvec_gaussian.argtypes = [C.c_void_p, _dp, C.c_double, C.c_int, _dp]
        L.tor_assemble.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_double, C.c_int, _dp]
        L.tor_solve.restype = C.c_int
        L.tor_solve.argtypes = [C.c_int, _ip, _ip, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                C.c_int, _dp, _dp, _ip, _dp, C.c_int]
        L.tor_ic_factor.restype = C.c_int
        L.tor_ic_factor.argtypes = [C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp, _dp]
        L.tor_project.argtypes = [C.c_int, C.c_int, _dp, _dp, _ip, _ip, C.c_int, C.c_int, _dp]
        L.tor_jacobian.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _ip, _ip, C.c_int, C.c_int,
                                   _dp, C.c_int]
        L.tor_a_keijzer.restype = C.c_double
        L.tor_a_keijzer.argtypes = [C.c_double]
        L.tor_assemble_el.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_double, C.c_int, _dp]
        L.tor_jacobian_el.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _ip, _ip, C.c_int, C.c_int, _dp]
        L.tor_gradient_weights.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _dp]
        L.tor_gradient_grid.argtypes = [C.c_void_p, C.c_int, _ip, _ip, C.c_int, _dp, _dp, _dp]
        L.tor_blob_create.restype = C.c_void_p
        L.tor_blob_create.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, _ip]
        L.tor_blob_info.argtypes = [C.c_void_p, _ip, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                    _dp, _dp]
        L.tor_blob_arrays.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip, _dp]
        L.tor_blob_free.argtypes = [C.c_void_p]
        L.tor_jacobian_blob.restype = C.c_int
        L.tor_jacobian_blob.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _ip, _ip, C.c_int,
                                        C.c_int, _dp]
        L.tor_gradient_blob.argtypes = [C.c_void_p, C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.tor_cubic_map.restype = C.c_int
        L.tor_cubic_map.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _ip, C.c_int, _ip, C.c_void_p, C.c_void_p]
        L.tor_linpix_map.restype = C.c_int
        L.tor_linpix_map.argtypes = [C.c_int, _ip, _ip, _ip, C.c_int, _ip, C.c_void_p, C.c_void_p]
        L.tor_basis_support.restype = C.c_int
        L.tor_basis_support.argtypes = [C.c_int, _ip, _ip, _ip, _ip]
        L.tor_csr_ab.restype = C.c_int
        L.tor_csr_ab.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, _ip, C.c_void_p, C.c_void_p]
        L.tor_node_map.argtypes = [C.c_void_p, _ip, _dp, _dp, _ip, _ip, _ip, _dp]
        L.tor_raster_pixel.restype = C.c_int
        L.tor_raster_pixel.argtypes = [C.c_void_p, _ip, _dp, _dp, _ip, _ip, _ip, _dp]
        L.tor_jacobian_grid.restype = C.c_int
        L.tor_jacobian_grid.argtypes = [C.c_void_p, C.c_int, _ip, _ip, C.c_int, C.c_int, _dp, _dp, _dp, _ip, _ip,
                                        C.c_int, C.c_int, _dp]
        _lib = L
    return _lib


def _cview(z: np.ndarray) -> np.ndarray:
    """complex128 array -> interleaved float64 view (contiguous)."""
    return np.ascontiguousarray(z).view(np.float64)


class Mesh:
    """Oracle-side mesh: geometry, boundary marking and the CSR pattern."""

    def __init__(self, coords: np.ndarray, elems: np.ndarray):
        self.coords = np.ascontiguousarray(coords, np.float64)
        self.elems = np.ascontiguousarray(elems, np.int32)
        self.dim = self.coords.shape[1]
        self.n = self.coords.shape[0]
        self.ne = self.elems.shape[0]
        self._h = lib().tor_mesh_create(self.dim, self.n, self.coords.ravel(), self.ne, self.elems.ravel())
        nnz = lib().tor_mesh_nnz(self._h)
        self.rowptr = np.zeros(self.n + 1, np.int32)
        self.colidx = np.zeros(nnz, np.int32)
        lib().tor_mesh_csr(self._h, self.rowptr, self.colidx)
        self.bnd = np.zeros(self.n, np.uint8)
        lib().tor_mesh_bndnodes(self._h, self.bnd)
        self.size = np.zeros(self.ne)
        lib().tor_mesh_elsize(self._h, self.size)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tor_mesh_free(self._h)
            self._h = None

    @property
    def nnz(self) -> int:
        return int(self.colidx.shape[0])

    def pull_to_boundary(self, p) -> np.ndarray:
        out = np.zeros(self.dim)
        rc = lib().tor_pull_to_boundary(self._h, np.ascontiguousarray(p, np.float64), out)
        if rc:
            raise RuntimeError("PullToBoundary: no boundary side found")
        return out

    def el_found(self, p) -> bool:
        return bool(lib().tor_el_found(self._h, np.ascontiguousarray(p, np.float64)))

    def place_detectors(self, M, fixed: bool) -> np.ndarray:
        """QMMesh::InitM's detector positions (qmmesh.cc:105-147): fixed
        positions outside every element are moved by -1e-4, 0, +1e-4 along
        each axis in turn until one is inside; the others are pulled to the
        boundary (Mesh::PullToBoundary, mesh.cc:1052-1111).  When no boundary
        side takes the projection the reference's fallback writes its result
        to a local point (mesh.cc:1110), so the position stays as read."""
        out = []
        for p in np.asarray(M, np.float64):
            if fixed:
                q = p.copy()
                if not self.el_found(q):
                    found = False
                    for d in range(self.dim):
                        for s in (-1, 0, 1):
                            q = p.copy()
                            q[d] += s * 1e-4
                            if self.el_found(q):
                                found = True
                                break
                        if found:
                            break
                    if not found:
                        raise RuntimeError("no element found to place measurement")
                out.append(q)
            else:
                try:
                    out.append(self.pull_to_boundary(p))
                except RuntimeError:
                    out.append(p.copy())
        return np.array(out).reshape(-1, self.dim)

    def bnd_intersect(self, p1, p2) -> np.ndarray:
        """Mesh::BndIntersect (mesh.cc:1369-1453): the boundary point nearest
        p1 on the segment p1-p2 (2D) or on the line through them (3D)."""
        out = np.zeros(self.dim)
        rc = lib().tor_bnd_intersect(self._h, np.ascontiguousarray(p1, np.float64),
                                     np.ascontiguousarray(p2, np.float64), out)
        if rc:
            raise RuntimeError("BndIntersect: no boundary point found")
        return out

    def external_sources(self, Q, QN=None) -> np.ndarray:
        """QMMesh::LoadQM's "external" source positions (qmmesh.cc:378-391):
        each position moved to the boundary point BndIntersect finds from
        q + |q| n towards q, n the unit normal read with the position (QN) or,
        for a list marked "default" (QN None), the unit vector along -q."""
        out = []
        for i, q in enumerate(np.asarray(Q, np.float64)):
            r = np.zeros(self.dim)
            nrm = None if QN is None else np.ascontiguousarray(QN[i], np.float64)
            rc = lib().tor_external_source(self._h, np.ascontiguousarray(q), None if nrm is None else
                                           nrm.ctypes.data_as(C.c_void_p), r)
            if rc == 2:
                raise RuntimeError("no normal given for an external source")
            if rc:
                raise RuntimeError("BndIntersect: no boundary point found")
            out.append(r)
        return np.array(out).reshape(-1, self.dim)

    def qvec_gaussian(self, cnt, w, neumann=True) -> np.ndarray:
        out = np.zeros(self.n)
        lib().tor_qvec_gaussian(self._h, np.ascontiguousarray(cnt, np.float64), float(w), int(neumann), out)
        return out

    def assemble(self, cmua, ckap, c2a, omega: float, cplx: bool) -> np.ndarray:
        val = np.zeros(self.nnz * (2 if cplx else 1))
        lib().tor_assemble(self._h, np.ascontiguousarray(cmua, np.float64), np.ascontiguousarray(ckap, np.float64),
                           np.ascontiguousarray(c2a, np.float64), float(omega), int(cplx), val)
        return val.view(np.complex128) if cplx else val


def a_keijzer(n: float) -> float:
    return lib().tor_a_keijzer(float(n))


def optical_coefficients(mua, mus, nref):
    """Nodal cmua, ckappa, c2a (src/python/toastmodule.cc:1536-1541, c0 = 0.3 mm/ps)."""
    c0 = 0.3
    mua = np.asarray(mua, float); mus = np.asarray(mus, float); nref = np.asarray(nref, float)
    cmua = mua * c0 / nref
    ckap = c0 / (3.0 * nref * (mua + mus))
    c2a = np.array([c0 / (2.0 * r * a_keijzer(r)) for r in nref])
    return cmua, ckap, c2a


METHODS = {"CG": 0, "BICGSTAB": 1, "GMRES": 2}
PRECONS = {"NONE": 0, "DIAG": 1, "ICH": 2, "DILU": 0}  # DILU is built as no preconditioner (fwdsolver.cc:149-153)


def solve(rowptr, colidx, val, B, method="BICGSTAB", precon="ICH", tol=1e-10, maxit=0, nthreads=1, X0=None):
    """Solve A x_q = b_q for every row of B (nrhs x n).  Returns X, its, errs."""
    cplx = np.iscomplexobj(val)
    n = rowptr.shape[0] - 1
    B = np.ascontiguousarray(B, np.complex128 if cplx else np.float64)
    nrhs = B.shape[0]
    X = np.zeros_like(B) if X0 is None else np.array(X0, dtype=B.dtype, copy=True)
    its = np.zeros(nrhs, np.int32)
    errs = np.zeros(nrhs)
    nf = lib().tor_solve(n, np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colidx, np.int32),
                         _cview(val) if cplx else np.ascontiguousarray(val, np.float64), int(cplx),
                         METHODS[method], PRECONS[precon], float(tol), int(maxit), nrhs,
                         _cview(B).ravel() if cplx else B.ravel(), _cview(X).reshape(-1) if cplx else X.reshape(-1),
                         its, errs, int(nthreads))
    if nf:
        raise RuntimeError(f"oracle solve: {nf} right-hand sides failed (breakdown)")
    return X, its, errs


def rcm(rowptr, colidx):
    """Reverse Cuthill-McKee ordering, perm[new] = old."""
    n = len(rowptr) - 1
    perm = np.zeros(n, np.int32)
    lib().tor_rcm(n, np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colidx, np.int32), perm)
    return perm


def nd_order(rowptr, colidx, coords):
    """Nested dissection by node coordinates, perm[new] = old."""
    n = len(rowptr) - 1
    coords = np.ascontiguousarray(coords, np.float64)
    perm = np.zeros(n, np.int32)
    lib().tor_nd_order(n, np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colidx, np.int32),
                       coords.ravel(), coords.shape[1], perm)
    return perm


class Direct:
    """The reference's LSOLVER_DIRECT path restated: symbolic Cholesky fill,
    left-looking numeric factor and substitution (real; complex systems by the
    same code in complex-symmetric arithmetic).  order: "natural" (the
    reference's: the mesh's own node order), "rcm", or "nd" (nested dissection
    by the node coordinates `coords`); the reorderings only reduce the fill."""

    def __init__(self, rowptr, colidx, val, order="rcm", coords=None):
        self.cplx = np.iscomplexobj(val)
        self.n = len(rowptr) - 1
        rp = np.ascontiguousarray(rowptr, np.int32)
        ci = np.ascontiguousarray(colidx, np.int32)
        if order == "nd":
            perm = nd_order(rp, ci, coords)
        elif order == "rcm":
            perm = rcm(rp, ci)
        else:
            perm = None
        v = _cview(val) if self.cplx else np.ascontiguousarray(val, np.float64)
        self._h = lib().tor_direct_factor(self.n, rp, ci, v, int(self.cplx),
                                          perm.ctypes.data_as(C.c_void_p) if perm is not None else None)
        if not self._h:
            raise MemoryError("oracle direct factor")

    @property
    def nnz_factor(self):
        return lib().tor_direct_nnz(self._h)

    def solve(self, B, nthreads=1):
        B = np.atleast_2d(np.asarray(B, np.complex128 if self.cplx else np.float64))
        X = np.zeros_like(B)
        lib().tor_direct_solve(self._h, int(self.cplx), B.shape[0],
                               _cview(B).ravel() if self.cplx else np.ascontiguousarray(B).ravel(),
                               _cview(X).reshape(-1) if self.cplx else X.reshape(-1), int(nthreads))
        return X

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tor_direct_free(self._h)
            self._h = None


def solve_direct(rowptr, colidx, val, B, order="rcm", coords=None, nthreads=1):
    """Direct FP64 solve of every row of B (nrhs x n)."""
    return Direct(rowptr, colidx, val, order, coords).solve(B, nthreads)


def solve_refined(rowptr, colidx, val, B, method="BICGSTAB", precon="ICH", cw_tol=1e-12, inner_tol=1e-10,
                  max_cycles=12, nthreads=1):
    """An FP64 solve accurate entry by entry: the reference's iterative solve
    (solve()), restarted from the true FP64 residual b - A x until the
    componentwise backward error max_i |r_i| / (|A| |x| + |b|)_i is at most
    cw_tol (|z| = max(|Re z|, |Im z|)).  For meshes too large for the direct
    factorisation.  Returns X and the final backward error per row."""
    import scipy.sparse as sp
    cplx = np.iscomplexobj(val)
    n = len(rowptr) - 1
    A = sp.csr_matrix((val, colidx, rowptr), shape=(n, n))
    absA = sp.csr_matrix((np.maximum(np.abs(np.real(val)), np.abs(np.imag(val))), colidx, rowptr), shape=(n, n))
    B = np.ascontiguousarray(B, np.complex128 if cplx else np.float64)
    X = np.zeros_like(B)
    R = B.copy()

    def mag(z):
        return np.maximum(np.abs(np.real(z)), np.abs(np.imag(z)))

    berr = np.ones(B.shape[0])
    for _ in range(max_cycles):
        D = (absA @ mag(X).T).T + mag(B)
        berr = np.max(np.where(D > 0, mag(R) / np.where(D > 0, D, 1), np.where(mag(R) > 0, np.inf, 0)), axis=1)
        if np.all(berr <= cw_tol):
            break
        act = np.nonzero(berr > cw_tol)[0]
        E, _, _ = solve(rowptr, colidx, val, R[act], method, precon, inner_tol, 0, nthreads)
        X[act] += E
        R[act] = B[act] - (A @ X[act].T).T
    return X, berr


def ic_factor(rowptr, colidx, val):
    cplx = np.iscomplexobj(val)
    n = rowptr.shape[0] - 1
    nl = int((rowptr[-1] - n) // 2) + n
    Lr = np.zeros(n + 1, np.int32)
    Lc = np.zeros(max(nl, 1), np.int32)
    Lv = np.zeros(max(nl, 1) * (2 if cplx else 1))
    d = np.zeros(n * (2 if cplx else 1))
    got = lib().tor_ic_factor(n, rowptr, colidx, _cview(val) if cplx else np.ascontiguousarray(val, np.float64),
                              int(cplx), Lr, Lc, Lv, d)
    Lc = Lc[:got]
    Lv = Lv[:got * (2 if cplx else 1)]
    if cplx:
        return Lr, Lc, Lv.view(np.complex128), d.view(np.complex128)
    return Lr, Lc, Lv, d


def project(phi, mvec, link_ofs, link_m, logscale=True):
    cplx = np.iscomplexobj(phi)
    nq, n = phi.shape
    nqm = int(link_ofs[-1])
    out = np.zeros(nqm * (2 if cplx else 1))
    lib().tor_project(n, nq, _cview(phi).ravel() if cplx else np.ascontiguousarray(phi, np.float64).ravel(),
                      _cview(mvec.astype(np.complex128)).ravel() if cplx else np.ascontiguousarray(mvec, np.float64).ravel(),
                      np.ascontiguousarray(link_ofs, np.int32), np.ascontiguousarray(link_m, np.int32),
                      int(cplx), int(logscale), out)
    return out.view(np.complex128) if cplx else out


def jacobian(mesh: Mesh, dphi, aphi, proj_lin, link_ofs, link_m, logscale=True, nthreads=1):
    cplx = np.iscomplexobj(dphi)
    nq, n = dphi.shape
    nm = aphi.shape[0]
    nqm = int(link_ofs[-1])
    J = np.zeros((2 * nqm, 2 * n) if cplx else (2 * nqm, n))
    lib().tor_jacobian(mesh._h, nq, nm,
                       _cview(dphi).ravel() if cplx else np.ascontiguousarray(dphi, np.float64).ravel(),
                       _cview(aphi).ravel() if cplx else np.ascontiguousarray(aphi, np.float64).ravel(),
                       _cview(proj_lin).ravel() if cplx else np.ascontiguousarray(proj_lin, np.float64).ravel(),
                       np.ascontiguousarray(link_ofs, np.int32), np.ascontiguousarray(link_m, np.int32),
                       int(cplx), int(logscale), J.reshape(-1), int(nthreads))
    return J


def assemble_el(mesh: Mesh, cmua_el, ckap_el, c2a_el, omega, cplx):
    """System matrix values (mesh CSR) from one coefficient per element."""
    val = np.zeros(mesh.nnz * (2 if cplx else 1))
    lib().tor_assemble_el(mesh._h, np.ascontiguousarray(cmua_el, np.float64), np.ascontiguousarray(ckap_el, np.float64),
                          np.ascontiguousarray(c2a_el, np.float64), float(omega), int(cplx), val)
    return val.view(np.complex128) if cplx else val


def jacobian_el(mesh: Mesh, dphi, aphi, proj_lin, link_ofs, link_m, logscale=True):
    """Element-basis Jacobian: complex (2 nQM) x (2 ne), real (2 nQM) x ne."""
    cplx = np.iscomplexobj(dphi)
    nq, n = dphi.shape
    nm = aphi.shape[0]
    nqm = int(link_ofs[-1])
    J = np.zeros((2 * nqm, 2 * mesh.ne) if cplx else (2 * nqm, mesh.ne))
    f = (lambda a: _cview(a).ravel()) if cplx else (lambda a: np.ascontiguousarray(a, np.float64).ravel())
    lib().tor_jacobian_el(mesh._h, nq, nm, f(dphi), f(aphi), f(proj_lin), np.ascontiguousarray(link_ofs, np.int32),
                          np.ascontiguousarray(link_m, np.int32), int(cplx), int(logscale), J.reshape(-1))
    return J


def data_gradient(mesh: Mesh, bdim, sysval, dphi, mvec, proj_lin, proj_log, link_ofs, link_m, data, sd,
                  method="BICGSTAB", precon="ICH", tol=1e-15, gdim=None, kind="pixel"):
    """toast's Gradient on Raster_Pixel(bdim, gdim) (gdim None: bdim; kind
    "cubic": Raster_CubicPixel; kind a BlobRaster: that blob raster) given
    the fields: weights, one adjoint solve per source with the weighted
    detector vectors, then the grid products mapped to the solution basis
    (src/python/toastmodule.cc:1745-1843).  Returns 2 slen."""
    bdim = np.ascontiguousarray(bdim, np.int32)
    gdim = bdim if gdim is None else np.ascontiguousarray(gdim, np.int32)
    nq, n = dphi.shape
    W = np.zeros((nq, n), np.complex128)
    lib().tor_gradient_weights(nq, n, _cview(np.asarray(mvec, np.complex128)).ravel(), _cview(proj_lin).ravel(),
                               _cview(proj_log).ravel(), np.ascontiguousarray(data, np.float64),
                               np.ascontiguousarray(sd, np.float64), np.ascontiguousarray(link_ofs, np.int32),
                               np.ascontiguousarray(link_m, np.int32), W.view(np.float64).reshape(-1))
    wphi, _, _ = solve(mesh.rowptr, mesh.colidx, sysval, W, method, precon, tol)
    if isinstance(kind, BlobRaster):
        grad = np.zeros(2 * kind.slen)
        lib().tor_gradient_blob(mesh._h, kind._h, nq, _cview(dphi).ravel(), _cview(wphi).ravel(), grad)
        return grad
    slen = len(raster_support(mesh, bdim, gdim, kind))
    grad = np.zeros(2 * slen)
    lib().tor_gradient_grid(mesh._h, _KIND[kind], bdim, gdim, nq, _cview(dphi).ravel(), _cview(wphi).ravel(), grad)
    return grad


@dataclass
class RasterPixel:
    """Raster_Pixel with grid == basis: bounding box, element per grid point
    (-1 outside), the grid map matrix B (CSR, natural node numbering) and the
    solution points (grid points inside the mesh, in grid order)."""
    bdim: np.ndarray
    bbmin: np.ndarray
    bbmax: np.ndarray
    elref: np.ndarray
    browptr: np.ndarray
    bcol: np.ndarray
    bval: np.ndarray

    @property
    def sol(self):
        return np.nonzero(self.elref >= 0)[0].astype(np.int32)


def raster_pixel(mesh: Mesh, bdim) -> RasterPixel:
    bdim = np.ascontiguousarray(bdim, np.int32)
    glen = int(np.prod(bdim))
    nn = mesh.elems.shape[1]
    bbmin, bbmax = np.zeros(mesh.dim), np.zeros(mesh.dim)
    elref = np.zeros(glen, np.int32)
    rp = np.zeros(glen + 1, np.int32)
    col = np.zeros(glen * nn, np.int32)
    val = np.zeros(glen * nn)
    lib().tor_raster_pixel(mesh._h, bdim, bbmin, bbmax, elref, rp, col, val)
    return RasterPixel(bdim, bbmin, bbmax, elref, rp, col[:rp[-1]].copy(), val[:rp[-1]].copy())


def raster_support(mesh: Mesh, bdim, gdim=None, kind="pixel") -> np.ndarray:
    """The solution points of the raster as basis indices.  Raster_Pixel:
    without an intermediate grid the grid points inside the mesh; with one,
    the basis points whose subsampled support is positive (raster.cc:55-77).
    Raster_CubicPixel: the basis points whose row of G is not empty
    (raster_cp.cc:170-178)."""
    bdim = np.ascontiguousarray(bdim, np.int32)
    if kind == "cubic":
        gdim = bdim if gdim is None else np.ascontiguousarray(gdim, np.int32)
        r = raster_pixel(mesh, gdim)
        rp = cubic_map(mesh.dim, gdim, bdim, r.bbmin, r.bbmax, r.elref, False)[0]
        return np.nonzero(np.diff(rp) > 0)[0].astype(np.int32)
    if gdim is None or np.array_equal(np.asarray(gdim), bdim):
        return raster_pixel(mesh, bdim).sol
    gdim = np.ascontiguousarray(gdim, np.int32)
    elref = raster_pixel(mesh, gdim).elref
    out = np.zeros(int(np.prod(bdim)), np.int32)
    slen = lib().tor_basis_support(mesh.dim, gdim, bdim, elref, out)
    return out[:slen].copy()


def linpix_map(dim, gdim, bdim, elref, by_grid):
    """Grid2LinPixMatrix (by_grid False: basis x grid, rows normalised) or
    LinPix2GridMatrix (True: grid x basis) as CSR (rowptr, col, val)."""
    gdim = np.ascontiguousarray(gdim, np.int32)
    bdim = np.ascontiguousarray(bdim, np.int32)
    elref = np.ascontiguousarray(elref, np.int32)
    rows = int(np.prod(gdim if by_grid else bdim))
    rp = np.zeros(rows + 1, np.int32)
    nz = lib().tor_linpix_map(dim, gdim, bdim, elref, int(by_grid), rp, None, None)
    col = np.zeros(max(nz, 1), np.int32)
    val = np.zeros(max(nz, 1))
    nz = lib().tor_linpix_map(dim, gdim, bdim, elref, int(by_grid), rp, col.ctypes.data_as(C.c_void_p),
                              val.ctypes.data_as(C.c_void_p))
    return rp, col[:nz].copy(), val[:nz].copy()


_KIND = {"pixel": 0, "cubic": 1}
BLOB_KINDS = {"gauss": 1, "hanning": 2, "ramp": 3, "spline": 4}


class BlobRaster:
    """A blob raster (Raster_Blob, raster_bl.cc, with the Gaussian, Hanning,
    ramp or spline blob of raster_gb.cc / raster_hb.cc / raster_rb.cc /
    raster_sb.cc): basis bdim padded by the support radius, the element per
    padded grid point, the solution points (basis indices) and the node
    values (per node the blob values of the solution points, CSR)."""

    def __init__(self, mesh: Mesh, kind, bdim, sup, sigma=1.0):
        self.mesh = mesh
        self.dim = mesh.dim
        bdim = np.ascontiguousarray(bdim, np.int32)
        self._h = lib().tor_blob_create(mesh._h, BLOB_KINDS[kind], float(sigma), float(sup), bdim)
        pdim = np.zeros(3, np.int32)
        sl, nz, sc = C.c_int(), C.c_int(), C.c_double()
        self.bbmin, self.bbmax = np.zeros(3), np.zeros(3)
        lib().tor_blob_info(self._h, pdim, C.byref(sl), C.byref(nz), C.byref(sc), self.bbmin, self.bbmax)
        self.pdim = pdim[:self.dim].copy()
        self.bbmin, self.bbmax = self.bbmin[:self.dim], self.bbmax[:self.dim]
        self.slen, self.scale = sl.value, sc.value
        self.blen = int(np.prod(self.pdim))
        self.elref = np.zeros(self.blen, np.int32)
        self.sol2basis = np.zeros(max(self.slen, 1), np.int32)
        self.nrp = np.zeros(mesh.n + 1, np.int32)
        self.ncol = np.zeros(max(nz.value, 1), np.int32)
        self.nval = np.zeros(max(nz.value, 1))
        lib().tor_blob_arrays(self._h, self.elref, self.sol2basis, self.nrp, self.ncol, self.nval)
        self.sol2basis = self.sol2basis[:self.slen]

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tor_blob_free(self._h)
            self._h = None

    def mesh_to_basis(self, f):
        """Map_MeshToBasis (raster_bl.cc:170-204): per solution point the
        node-value-weighted sum over the nodes (node order) over the sum of
        the weights; 0 elsewhere."""
        f = np.asarray(f)
        cplx = np.iscomplexobj(f)
        fr, fi, sm = np.zeros(self.slen), np.zeros(self.slen), np.zeros(self.slen)
        for nd in range(self.mesh.n):
            x = complex(f[nd])
            for t in range(self.nrp[nd], self.nrp[nd + 1]):
                j, v = int(self.ncol[t]), float(self.nval[t])
                if cplx:
                    fr[j] += x.real * v
                    fi[j] += x.imag * v
                else:
                    fr[j] += v * x.real
                sm[j] += v
        b = np.zeros(self.blen, np.complex128 if cplx else np.float64)
        for j in range(self.slen):
            if sm[j] != 0.0:
                b[self.sol2basis[j]] = fr[j] / sm[j] + 1j * (fi[j] / sm[j]) if cplx else fr[j] / sm[j]
        return b

    def sol_to_mesh(self, sv):
        """Map_SolToMesh (raster_bl.cc:252-276): per node the sum over the
        solution points of value x node value, in solution order."""
        sv = np.asarray(sv)
        cplx = np.iscomplexobj(sv)
        out = np.zeros(self.mesh.n, np.complex128 if cplx else np.float64)
        for nd in range(self.mesh.n):
            acc = 0j if cplx else 0.0
            for t in range(self.nrp[nd], self.nrp[nd + 1]):
                acc += sv[self.ncol[t]] * float(self.nval[t])
            out[nd] = acc
        return out

    def maps(self, mua, mus):
        """The reference driver's map vectors through a blob raster (grid =
        basis; toast.Raster.Map with raster_bl.cc:140-350): m2g (= M->B),
        m2s, s2m of s + 1, g2m of m2g, m2b, b2m of b + 1, g2b, b2g (copies),
        g2s, s2g of s + 1, complex cm2s of mua + i mus, cs2m of (s + 1) -
        0.5 i s."""
        b = np.arange(1, self.blen + 1, dtype=float)
        sv = np.arange(1, self.slen + 1, dtype=float)
        m2g = self.mesh_to_basis(mua)
        s2g = np.zeros(self.blen)
        s2g[self.sol2basis] = sv
        cs = np.arange(1, self.slen + 1) - 0.5j * np.arange(self.slen)
        return dict(m2g=m2g, m2s=m2g[self.sol2basis], s2m=self.sol_to_mesh(sv),
                    g2m=self.sol_to_mesh(m2g[self.sol2basis]), m2b=m2g, b2m=self.sol_to_mesh(b[self.sol2basis]),
                    g2b=m2g, b2g=b, g2s=m2g[self.sol2basis], s2g=s2g,
                    cm2s=self.mesh_to_basis(np.asarray(mua) + 1j * np.asarray(mus))[self.sol2basis],
                    cs2m=self.sol_to_mesh(cs))

    def jacobian(self, dphi, aphi, proj_lin, link_ofs, link_m, logscale=True):
        """Grid-basis Jacobian on the blob raster: complex (2 nQM) x (2 slen),
        real (2 nQM) x slen."""
        cplx = np.iscomplexobj(dphi)
        nq, nm, nqm = dphi.shape[0], aphi.shape[0], int(link_ofs[-1])
        J = np.zeros((2 * nqm, 2 * self.slen) if cplx else (2 * nqm, self.slen))
        f = (lambda a: _cview(a).ravel()) if cplx else (lambda a: np.ascontiguousarray(a, np.float64).ravel())
        lib().tor_jacobian_blob(self.mesh._h, self._h, nq, nm, f(dphi), f(aphi), f(proj_lin),
                                np.ascontiguousarray(link_ofs, np.int32), np.ascontiguousarray(link_m, np.int32),
                                int(cplx), int(logscale), J.reshape(-1))
        return J


def cubic_map(dim, gdim, bdim, bbmin, bbmax, elref, by_grid):
    """Raster_CubicPixel's G (by_grid False: basis x grid, rows normalised)
    or GI (True: grid x basis, the basis values at the grid points) as CSR."""
    gdim = np.ascontiguousarray(gdim, np.int32)
    bdim = np.ascontiguousarray(bdim, np.int32)
    elref = np.ascontiguousarray(elref, np.int32)
    bbmin = np.ascontiguousarray(bbmin, np.float64)
    bbmax = np.ascontiguousarray(bbmax, np.float64)
    rows = int(np.prod(gdim if by_grid else bdim))
    rp = np.zeros(rows + 1, np.int32)
    nz = lib().tor_cubic_map(dim, gdim, bdim, bbmin, bbmax, elref, int(by_grid), rp, None, None)
    col = np.zeros(max(nz, 1), np.int32)
    val = np.zeros(max(nz, 1))
    lib().tor_cubic_map(dim, gdim, bdim, bbmin, bbmax, elref, int(by_grid), rp, col.ctypes.data_as(C.c_void_p),
                        val.ctypes.data_as(C.c_void_p))
    return rp, col[:nz].copy(), val[:nz].copy()


def csr_ab(a, b, nc):
    """TCompRowMatrix::AB then Shrink of CSR triples a (nr x k) and b (k x nc)."""
    arp, acol, aval = (np.ascontiguousarray(x) for x in a)
    brp, bcol, bval = (np.ascontiguousarray(x) for x in b)
    nr = len(arp) - 1
    crp = np.zeros(nr + 1, np.int32)
    cap = lib().tor_csr_ab(nr, nc, arp, acol, aval, brp, bcol, bval, crp, None, None)
    ccol = np.zeros(max(cap, 1), np.int32)
    cval = np.zeros(max(cap, 1))
    nz = lib().tor_csr_ab(nr, nc, arp, acol, aval, brp, bcol, bval, crp, ccol.ctypes.data_as(C.c_void_p),
                          cval.ctypes.data_as(C.c_void_p))
    return crp, ccol[:nz].copy(), cval[:nz].copy()


def _csr_apply(rp, col, val, x):
    """y = A x row by row in entry order from 0 (RCompRowMatrix::Ax)."""
    y = np.zeros(len(rp) - 1)
    for r in range(len(rp) - 1):
        acc = 0.0
        for j in range(rp[r], rp[r + 1]):
            acc += float(val[j]) * float(x[col[j]])
        y[r] = acc
    return y


def raster_maps(mesh: Mesh, bdim, f_mesh, s_sol):
    """The pixel raster's basis maps (toast.Raster.Map): mesh -> grid (B),
    mesh -> solution (B then the support), solution -> mesh (scatter to the
    grid, then NodeMapMatrix BI), grid -> mesh (BI) of the grid image of
    f_mesh.  Returns (m2g, m2s, s2m, g2m)."""
    r = raster_pixel(mesh, bdim)
    glen = len(r.elref)
    nn = 1 << mesh.dim
    rp = np.zeros(mesh.n + 1, np.int32)
    col = np.zeros(mesh.n * nn, np.int32)
    val = np.zeros(mesh.n * nn)
    lib().tor_node_map(mesh._h, np.ascontiguousarray(bdim, np.int32), r.bbmin, r.bbmax, r.elref, rp, col, val)
    m2g = _csr_apply(r.browptr, r.bcol, r.bval, f_mesh)
    m2s = m2g[r.sol]
    g = np.zeros(glen)
    g[r.sol] = s_sol
    s2m = _csr_apply(rp, col, val, g)
    g2m = _csr_apply(rp, col, val, m2g)
    return m2g, m2s, s2m, g2m


def _csr_apply_c(rp, col, val, x):
    """RCompRowMatrix::Ax_cplx: real matrix, complex vector, the real and
    imaginary sums kept apart (crmatrix_imp.hpp:1302-1327)."""
    x = np.asarray(x, np.complex128)
    return _csr_apply(rp, col, val, x.real) + 1j * _csr_apply(rp, col, val, x.imag)


def raster_basis_maps(mesh: Mesh, bdim, gdim, mua, mus, kind="pixel"):
    """Maps of Raster_Pixel(bdim, gdim) (kind "cubic": Raster_CubicPixel)
    through its basis (toast.Raster.Map, MapBasis src/python/toastmodule.cc:
    718-790; raster.cc:188-408, raster_px.cc:10-176, raster_cp.cc:266-302),
    on the vectors the reference driver maps: real M->B, B->M of b + 1, G->B
    of the grid image of mua, B->G of b + 1, G->S, S->G of s + 1, and the
    complex M->S of mua + i mus and S->M of (s + 1) - 0.5 i s.  The pixel
    raster's real maps use its products C = G B, CI = BI GI and the support
    map D (0 + 1 x); everything else runs the base class's chains through the
    grid.  Also the solution points (sol2basis)."""
    bdim = np.ascontiguousarray(bdim, np.int32)
    gdim = np.ascontiguousarray(gdim, np.int32)
    r = raster_pixel(mesh, gdim)
    glen, blen, n = len(r.elref), int(np.prod(bdim)), mesh.n
    nn = 1 << mesh.dim
    nrp = np.zeros(n + 1, np.int32)
    ncol = np.zeros(n * nn, np.int32)
    nval = np.zeros(n * nn)
    lib().tor_node_map(mesh._h, gdim, r.bbmin, r.bbmax, r.elref, nrp, ncol, nval)
    BI = (nrp, ncol[:nrp[-1]].copy(), nval[:nrp[-1]].copy())
    B = (r.browptr, r.bcol, r.bval)
    if kind == "cubic":
        G = cubic_map(mesh.dim, gdim, bdim, r.bbmin, r.bbmax, r.elref, False)
        GI = cubic_map(mesh.dim, gdim, bdim, r.bbmin, r.bbmax, r.elref, True)
    else:
        G = linpix_map(mesh.dim, gdim, bdim, r.elref, False)
        GI = linpix_map(mesh.dim, gdim, bdim, r.elref, True)
    sol = raster_support(mesh, bdim, gdim, kind)
    slen = len(sol)

    def sel(b):  # Map_BasisToSol: the pixel raster's D->Ax, else a copy
        return b[sol] + 0.0 if kind == "pixel" else (b if slen == blen else b[sol])

    def sct(sv):  # Map_SolToBasis: the pixel raster's D->ATx, else a scatter
        if kind != "pixel" and slen == blen:
            return np.asarray(sv, float)
        b = np.zeros(blen)
        b[sol] += 1.0 * np.asarray(sv)
        return b

    if kind == "pixel":
        Cm = csr_ab(G, B, n)
        CI = csr_ab(BI, GI, blen)
        m2b = lambda m: _csr_apply(*Cm, m)  # noqa: E731
        b2m = lambda b: _csr_apply(*CI, b)  # noqa: E731
    else:
        m2b = lambda m: _csr_apply(*G, _csr_apply(*B, m))  # noqa: E731
        b2m = lambda b: _csr_apply(*BI, _csr_apply(*GI, b))  # noqa: E731
    bvec = np.arange(1, blen + 1, dtype=float)
    svec = np.arange(1, slen + 1, dtype=float)
    m2g = _csr_apply(*B, mua)
    out = dict(sol2basis=sol,
               m2b=m2b(mua),
               b2m=b2m(bvec),
               g2b=_csr_apply(*G, m2g),
               b2g=_csr_apply(*GI, bvec),
               g2s=sel(_csr_apply(*G, m2g)),
               s2g=_csr_apply(*GI, sct(svec)),
               m2s=sel(m2b(mua)),
               s2m=b2m(sct(svec)))
    cm = np.asarray(mua) + 1j * np.asarray(mus)
    cb = _csr_apply_c(*G, _csr_apply_c(*B, cm))
    out["cm2s"] = cb if slen == blen else cb[sol]
    cs = np.arange(1, slen + 1) - 0.5j * np.arange(slen)
    if slen == blen:
        cbs = cs
    else:
        cbs = np.zeros(blen, np.complex128)
        cbs[sol] = cs
    out["cs2m"] = _csr_apply_c(*BI, _csr_apply_c(*GI, cbs))
    return out


def jacobian_grid(mesh: Mesh, bdim, dphi, aphi, proj_lin, link_ofs, link_m, logscale=True, gdim=None,
                  kind="pixel"):
    """Grid-basis Jacobian for Raster_Pixel(bdim, gdim) (gdim None: bdim;
    kind "cubic": Raster_CubicPixel): complex (2 nQM) x (2 slen), real
    (2 nQM) x slen."""
    cplx = np.iscomplexobj(dphi)
    bdim = np.ascontiguousarray(bdim, np.int32)
    gdim = bdim if gdim is None else np.ascontiguousarray(gdim, np.int32)
    nq, n = dphi.shape
    nm = aphi.shape[0]
    nqm = int(link_ofs[-1])
    slen = len(raster_support(mesh, bdim, gdim, kind))
    J = np.zeros((2 * nqm, 2 * slen) if cplx else (2 * nqm, slen))
    f = (lambda a: _cview(a).ravel()) if cplx else (lambda a: np.ascontiguousarray(a, np.float64).ravel())
    lib().tor_jacobian_grid(mesh._h, _KIND[kind], bdim, gdim, nq, nm, f(dphi), f(aphi), f(proj_lin),
                            np.ascontiguousarray(link_ofs, np.int32), np.ascontiguousarray(link_m, np.int32),
                            int(cplx), int(logscale), J.reshape(-1))
    return J


@dataclass
class PathResult:
    qvec: np.ndarray
    mvec: np.ndarray
    sysval: np.ndarray
    dphi: np.ndarray
    aphi: np.ndarray
    proj: np.ndarray           # linear projections (nQM)
    logproj: np.ndarray        # log projections
    J: np.ndarray | None
    its_fwd: np.ndarray
    its_adj: np.ndarray
    times: dict = field(default_factory=dict)


def forward_path(mesh: Mesh, Q, M, link_ofs, link_m, mua, mus, nref, freq_mhz=0.0, qwidth=2.0, mwidth=2.0,
                 method=None, precon="ICH", tol=1e-10, maxit=0, jac=True, nthreads=1) -> PathResult:
    """The whole forward path on the CPU, as the reference's callers run it.
    method "DIRECT" solves with the direct factorisation (an exact FP64 solve
    up to round-off, the accuracy reference of the mixed path)."""
    cplx = freq_mhz != 0.0
    method = method or ("BICGSTAB" if cplx else "CG")
    cmua, ckap, c2a = optical_coefficients(mua, mus, nref)
    omega = freq_mhz * 2.0 * np.pi * 1e-6
    qvec = np.stack([mesh.qvec_gaussian(q, qwidth) for q in Q])
    mvec = np.stack([mesh.qvec_gaussian(m, mwidth) * c2a for m in M])
    t = {}
    t0 = time.perf_counter()
    val = mesh.assemble(cmua, ckap, c2a, omega, cplx)
    t["assemble"] = time.perf_counter() - t0
    dt = np.complex128 if cplx else np.float64
    if method == "DIRECT":
        # LSOLVER_DIRECT (fwdsolver.cc:467-505): one factorisation, substitutions per source
        t0 = time.perf_counter()
        D = Direct(mesh.rowptr, mesh.colidx, val, "nd", mesh.coords)
        dphi = D.solve(qvec.astype(dt), nthreads)
        t["fwd"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        aphi = D.solve(mvec.astype(dt), nthreads)
        t["adj"] = time.perf_counter() - t0
        itf = np.zeros(len(qvec), np.int32)
        ita = np.zeros(len(mvec), np.int32)
    else:
        t0 = time.perf_counter()
        dphi, itf, _ = solve(mesh.rowptr, mesh.colidx, val, qvec.astype(dt), method, precon, tol, maxit, nthreads)
        t["fwd"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        aphi, ita, _ = solve(mesh.rowptr, mesh.colidx, val, mvec.astype(dt), method, precon, tol, maxit, nthreads)
        t["adj"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    proj = project(dphi, mvec.astype(dt), link_ofs, link_m, logscale=False)
    lproj = project(dphi, mvec.astype(dt), link_ofs, link_m, logscale=True)
    t["proj"] = time.perf_counter() - t0
    J = None
    if jac:
        t0 = time.perf_counter()
        J = jacobian(mesh, dphi, aphi, proj, link_ofs, link_m, True, nthreads)
        t["jac"] = time.perf_counter() - t0
    return PathResult(qvec, mvec, val, dphi, aphi, proj, lproj, J, itf, ita, t)
