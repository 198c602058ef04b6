"""ctypes binding of libtoastgpu.so (include/toastgpu.h) and a Python mirror of
the reference's TFwdSolver interface (src/libstoast/fwdsolver.h:77-508) on top
of it.

Host arrays are numpy; device arrays are anything with ``data_ptr()`` (torch
CUDA tensors), passed with ``mem=MEM_DEVICE``.  The library must exist: there
is no CPU fallback, and loading fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtoastgpu.so")

SOLVERS = {"CG": 0, "BICGSTAB": 1, "GMRES": 2, "DIRECT": 3}
PRECONS = {"NONE": 0, "DIAG": 1, "ICH": 2, "DILU": 3}
PRECISIONS = {"fp64": 0, "mixed": 1}
MEM_HOST, MEM_DEVICE = 0, 1
DATA_LIN, DATA_LOG = 1, 2
# status codes (toastgpu.h)
ERR_ARG, ERR_STATE, ERR_CUDA, ERR_NOMEM, ERR_UNSUPPORTED, ERR_BREAKDOWN = 1, 2, 3, 4, 5, 6

EXPORTS = ["tg_mesh_create", "tg_mesh_destroy", "tg_mesh_info", "tg_mesh_csr", "tg_mesh_boundary",
           "tg_qvec_gaussian", "tg_qvec_gaussian_ex", "tg_solver_create", "tg_solver_destroy", "tg_solver_set", "tg_solver_set_refinement", "tg_solver_set_backward_error", "tg_solver_set_reliable_updates", "tg_solver_set_stream", "tg_solver_set_output_stream",
           "tg_solver_sync", "tg_solver_reset", "tg_solver_matrix", "tg_calc_fields", "tg_project_all",
           "tg_jacobian", "tg_forward_path", "tg_project_all_noalloc", "tg_solver_profile", "tg_solver_profile_read", "tg_launch_count", "tg_tuner_log", "tg_solver_reset_basis", "tg_jacobian_el", "tg_mesh_load", "tg_mesh_geometry", "tg_gradient", "tg_raster_create", "tg_raster_create_ex", "tg_raster_create_typed", "tg_raster_create_blob", "tg_raster_destroy", "tg_raster_map", "tg_raster_info", "tg_raster_elref", "tg_raster_basis", "tg_jacobian_grid",
           "tg_qm_load", "tg_qm_info", "tg_qm_positions", "tg_qm_links", "tg_qm_destroy",
           "tg_server_create", "tg_server_destroy", "tg_submit", "tg_poll", "tg_wait", "tg_server_stats",
           "tg_server_reset_stats", "tg_last_error"]
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = range(4)
PROF_SPMM, PROF_SWEEP, PROF_VEC, PROF_JAC, PROF_ASM, PROF_PROJ = range(6)


class ToastGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"toastgpu error {code}: {msg}")
        self.code = code


class TgResult(C.Structure):
    _fields_ = [("it_count", C.c_int), ("status", C.c_int), ("rel_err", C.c_double)]


class TgRequest(C.Structure):
    """tg_request (include/toastgpu.h)."""
    _fields_ = [("mesh", C.c_void_p), ("is_complex", C.c_int), ("method", C.c_int), ("precon", C.c_int),
                ("precision", C.c_int), ("tol", C.c_double), ("maxit", C.c_int), ("cmua", C.c_void_p),
                ("ckappa", C.c_void_p), ("c2a", C.c_void_p), ("omega", C.c_double), ("nq", C.c_int),
                ("qvec", C.c_void_p), ("nm", C.c_int), ("mvec", C.c_void_p), ("link_ofs", C.c_void_p),
                ("link_m", C.c_void_p), ("proj", C.c_void_p), ("logproj", C.c_void_p), ("J", C.c_void_p),
                ("j_fp32", C.c_int), ("res", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with toastpp_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        vp, ip, dp, i_, d_ = C.c_void_p, C.POINTER(C.c_int), C.c_void_p, C.c_int, C.c_double
        sig = {
            "tg_mesh_create": [i_, i_, vp, i_, vp, C.POINTER(C.c_void_p)],
            "tg_mesh_destroy": [vp],
            "tg_mesh_info": [vp, ip, ip, ip, ip, ip, ip],
            "tg_mesh_csr": [vp, vp, vp],
            "tg_mesh_boundary": [vp, vp],
            "tg_qvec_gaussian": [vp, i_, vp, d_, i_, vp],
            "tg_qvec_gaussian_ex": [vp, i_, vp, d_, i_, vp, vp, i_],
            "tg_solver_create": [vp, i_, i_, i_, d_, i_, i_, C.POINTER(C.c_void_p)],
            "tg_solver_destroy": [vp],
            "tg_solver_set": [vp, d_, i_],
            "tg_solver_set_refinement": [vp, d_, i_, i_],
            "tg_solver_set_reliable_updates": [vp, i_],
            "tg_solver_set_backward_error": [vp, d_],
            "tg_solver_set_stream": [vp, vp],
            "tg_solver_set_output_stream": [vp, vp],
            "tg_solver_sync": [vp],
            "tg_solver_reset": [vp, dp, dp, dp, d_, i_],
            "tg_solver_matrix": [vp, dp, i_],
            "tg_calc_fields": [vp, i_, dp, dp, i_, vp],
            "tg_project_all": [vp, i_, dp, i_, dp, vp, vp, i_, dp, i_],
            "tg_jacobian": [vp, i_, dp, i_, dp, dp, vp, vp, i_, vp, i_, i_],
            "tg_forward_path": [vp, dp, dp, dp, d_, i_, dp, i_, dp, vp, vp, dp, dp, dp, dp, vp, i_, i_, vp],
            "tg_project_all_noalloc": [vp, i_, dp, i_, dp, vp, vp, i_, dp],
            "tg_solver_profile": [vp, i_],
            "tg_solver_profile_read": [vp, i_, C.POINTER(C.c_double), ip],
            "tg_launch_count": [C.POINTER(C.c_longlong)],
            "tg_tuner_log": [C.c_char_p, i_],
            "tg_solver_reset_basis": [vp, dp, dp, dp, d_, i_, i_],
            "tg_mesh_load": [C.c_char_p, C.POINTER(C.c_void_p)],
            "tg_gradient": [vp, vp, i_, dp, i_, dp, vp, vp, dp, dp, dp, i_, vp],
            "tg_mesh_geometry": [vp, ip, ip, vp, vp],
            "tg_jacobian_el": [vp, i_, dp, i_, dp, dp, vp, vp, i_, vp, i_, i_],
            "tg_raster_create": [vp, ip, C.POINTER(C.c_void_p)],
            "tg_raster_create_ex": [vp, ip, ip, C.POINTER(C.c_void_p)],
            "tg_raster_create_typed": [vp, i_, ip, ip, C.POINTER(C.c_void_p)],
            "tg_raster_create_blob": [vp, i_, ip, C.c_double, C.c_double, C.POINTER(C.c_void_p)],
            "tg_raster_basis": [vp, ip, ip],
            "tg_raster_destroy": [vp],
            "tg_qm_load": [vp, C.c_char_p, C.POINTER(C.c_void_p)],
            "tg_qm_info": [vp, ip, ip, ip, ip],
            "tg_qm_positions": [vp, vp, vp],
            "tg_qm_links": [vp, vp, vp],
            "tg_qm_destroy": [vp],
            "tg_raster_info": [vp, ip, ip, dp, dp],
            "tg_raster_elref": [vp, ip],
            "tg_raster_map": [vp, C.c_char_p, i_, vp, vp, i_, i_],
            "tg_jacobian_grid": [vp, vp, i_, dp, i_, dp, dp, vp, vp, i_, vp, i_, i_],
            "tg_server_create": [i_, d_, C.POINTER(C.c_void_p)],
            "tg_server_destroy": [vp],
            "tg_submit": [vp, vp, C.POINTER(C.c_longlong)],
            "tg_poll": [vp, C.c_longlong, ip],
            "tg_wait": [vp, C.c_longlong, C.POINTER(C.c_double)],
            "tg_server_stats": [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)],
            "tg_server_reset_stats": [vp],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.tg_last_error.restype = C.c_char_p
        L.tg_last_error.argtypes = []
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise ToastGPUError(rc, lib().tg_last_error().decode())


def _ptr(a):
    """Pointer of a numpy array (host) or a tensor with data_ptr() (device); None -> NULL."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return C.c_void_p(a.ctypes.data)


def _f64(a, cplx):
    a = np.ascontiguousarray(a, dtype=np.complex128 if cplx else np.float64)
    return a


class Mesh:
    """tg_mesh: a P1 triangle or tetrahedron mesh with its CSR and IC(0) structure."""

    def __init__(self, coords, elems):
        coords = np.ascontiguousarray(coords, np.float64)
        elems = np.ascontiguousarray(elems, np.int32)
        self.dim = coords.shape[1]
        self.n = coords.shape[0]
        self.ne = elems.shape[0]
        h = C.c_void_p()
        _check(lib().tg_mesh_create(self.dim, self.n, _ptr(coords), self.ne, _ptr(elems), C.byref(h)))
        self._h = h
        v = [C.c_int() for _ in range(6)]
        _check(lib().tg_mesh_info(self._h, *[C.byref(x) for x in v]))
        self.nnz, self.nbnd, self.nlev_fwd, self.nlev_bwd = v[2].value, v[3].value, v[4].value, v[5].value

    @classmethod
    def load(cls, path):
        """A mesh file in the reference's MeshData 5.0 format, read by the
        library (tg_mesh_load)."""
        h = C.c_void_p()
        _check(lib().tg_mesh_load(os.fsencode(path), C.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        d, nn = C.c_int(), C.c_int()
        _check(lib().tg_mesh_geometry(h, C.byref(d), C.byref(nn), None, None))
        v = [C.c_int() for _ in range(6)]
        _check(lib().tg_mesh_info(h, *[C.byref(x) for x in v]))
        self.dim, self.n, self.ne = d.value, v[0].value, v[1].value
        self.nnz, self.nbnd, self.nlev_fwd, self.nlev_bwd = v[2].value, v[3].value, v[4].value, v[5].value
        return self

    def geometry(self):
        """(coords n x dim, 0-based elements ne x nn)."""
        d, nn = C.c_int(), C.c_int()
        _check(lib().tg_mesh_geometry(self._h, C.byref(d), C.byref(nn), None, None))
        coords = np.zeros((self.n, d.value))
        el = np.zeros((self.ne, nn.value), np.int32)
        _check(lib().tg_mesh_geometry(self._h, None, None, _ptr(coords), _ptr(el)))
        return coords, el

    def close(self):
        if getattr(self, "_h", None):
            lib().tg_mesh_destroy(self._h)
            self._h = None

    __del__ = close

    def csr(self):
        rp = np.zeros(self.n + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        _check(lib().tg_mesh_csr(self._h, _ptr(rp), _ptr(ci)))
        return rp, ci

    def boundary(self):
        b = np.zeros(self.n, np.uint8)
        _check(lib().tg_mesh_boundary(self._h, _ptr(b)))
        return b

    def qvec_gaussian(self, pos, width, neumann=True):
        pos = np.ascontiguousarray(np.atleast_2d(pos), np.float64)
        out = np.zeros((pos.shape[0], self.n))
        _check(lib().tg_qvec_gaussian(self._h, pos.shape[0], _ptr(pos), float(width), int(neumann), _ptr(out)))
        return out

    def qvec_gaussian_device(self, pos, width, neumann=True, scale=None, out=None):
        """tg_qvec_gaussian_ex: the source (or, with scale = c2a, detector)
        vectors formed on the device.  out: a device tensor (npos x n float64)
        for MEM_DEVICE (scale then a device tensor too), else None for a
        host array."""
        pos = np.ascontiguousarray(np.atleast_2d(pos), np.float64)
        if out is None:
            res = np.zeros((pos.shape[0], self.n))
            sc = None if scale is None else np.ascontiguousarray(scale, np.float64)
            _check(lib().tg_qvec_gaussian_ex(self._h, pos.shape[0], _ptr(pos), float(width), int(neumann), _ptr(sc),
                                             _ptr(res), MEM_HOST))
            return res
        _check(lib().tg_qvec_gaussian_ex(self._h, pos.shape[0], _ptr(pos), float(width), int(neumann), _ptr(scale),
                                         _ptr(out), MEM_DEVICE))
        return out


@dataclass
class Links:
    """QMMesh link list: link_ofs[q]..link_ofs[q+1] index link_m (detector per measurement)."""

    ofs: np.ndarray
    m: np.ndarray

    @staticmethod
    def all_to_all(nq, nm):
        return Links(np.arange(nq + 1, dtype=np.int32) * nm, np.tile(np.arange(nm, dtype=np.int32), nq))

    @property
    def nqm(self):
        return int(self.ofs[-1])


class FwdSolver:
    """TFwdSolver<T> on the GPU: T = complex<double> when ``complex`` else double.

    Names follow the reference: Reset, CalcFields, ProjectAll, plus
    GenerateJacobian / GenerateJacobian_cw through ``jacobian``.
    """

    def __init__(self, mesh: Mesh, solver="BICGSTAB", tol=1e-10, precon="ICH", complex=True, maxit=0,
                 precision="fp64"):
        self.mesh = mesh
        self.complex = bool(complex)
        self.precision = precision
        h = C.c_void_p()
        _check(lib().tg_solver_create(mesh._h, int(self.complex), SOLVERS[solver.upper()], PRECONS[precon.upper()],
                                      float(tol), int(maxit), PRECISIONS[precision], C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().tg_solver_destroy(self._h)
            self._h = None

    __del__ = close

    def set_stream(self, stream_handle):
        """Launch on an external cudaStream_t (an int handle, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); 0 restores the own stream."""
        _check(lib().tg_solver_set_stream(self._h, C.c_void_p(stream_handle or None)))

    def profile(self, mask):
        _check(lib().tg_solver_profile(self._h, int(mask)))

    def profile_read(self, cls):
        ms, cnt = C.c_double(), C.c_int()
        _check(lib().tg_solver_profile_read(self._h, int(cls), C.byref(ms), C.byref(cnt)))
        return ms.value, cnt.value

    def forward_path_raw(self, cmua, ckap, c2a, omega, nq, qvec, nm, mvec, links: Links, dphi, aphi, proj, lproj, J,
                         j_fp32, mem, res=None):
        """tg_forward_path with caller-owned buffers (numpy or device tensors)."""
        _check(lib().tg_forward_path(self._h, _ptr(cmua), _ptr(ckap), _ptr(c2a), float(omega), nq, _ptr(qvec), nm,
                                     _ptr(mvec), _ptr(links.ofs), _ptr(links.m), _ptr(dphi), _ptr(aphi), _ptr(proj),
                                     _ptr(lproj), _ptr(J), int(j_fp32), mem, res))

    def set_refinement(self, inner_tol, max_outer=12, inner_ordering=1):
        _check(lib().tg_solver_set_refinement(self._h, float(inner_tol), int(max_outer), int(inner_ordering)))

    def set_backward_error(self, cw_tol=1e-10):
        """Mixed path: refine until max_i |b - A x|_i / (|A||x| + |b|)_i <= cw_tol (0: off)."""
        _check(lib().tg_solver_set_backward_error(self._h, float(cw_tol)))

    def set_reliable_updates(self, mode=2):
        """0 restarted refinement, 1 reliable-update BiCGSTAB, 2 reliable-update COCG (complex)."""
        _check(lib().tg_solver_set_reliable_updates(self._h, int(mode)))

    def sync(self):
        """Wait for the solver's stream and its deferred-output stream."""
        _check(lib().tg_solver_sync(self._h))

    def set_output_stream(self, stream=None):
        """Deferred Jacobian output on a copy stream (cudaStream_t handle), or None."""
        _check(lib().tg_solver_set_output_stream(self._h, C.c_void_p(stream) if stream else None))

    def set_tol(self, tol, maxit=0):
        _check(lib().tg_solver_set(self._h, float(tol), int(maxit)))

    def reset(self, cmua, ckap, c2a, omega=0.0, mem=MEM_HOST):
        if mem == MEM_HOST:
            cmua, ckap, c2a = (np.ascontiguousarray(x, np.float64) for x in (cmua, ckap, c2a))
        _check(lib().tg_solver_reset(self._h, _ptr(cmua), _ptr(ckap), _ptr(c2a), float(omega), mem))

    def reset_elbasis(self, cmua_el, ckap_el, c2a_el, omega=0.0):
        """Reset(sol, omega, elbasis = true): one coefficient per element."""
        a = [np.ascontiguousarray(x, np.float64) for x in (cmua_el, ckap_el, c2a_el)]
        _check(lib().tg_solver_reset_basis(self._h, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), float(omega), MEM_HOST, 1))

    def gradient(self, raster: "Raster", qvec, mvec, links: Links, data, sd, grad=None):
        """toast's Gradient after reset (tg_gradient): returns (grad 2 slen,
        per-solve results: forward then adjoint)."""
        q = _f64(qvec, True)
        mv = _f64(mvec, True)
        g = np.zeros(2 * raster.slen) if grad is None else np.ascontiguousarray(grad, np.float64).copy()
        res = (TgResult * (2 * q.shape[0]))()
        _check(lib().tg_gradient(self._h, raster._h, q.shape[0], _ptr(q), mv.shape[0], _ptr(mv), _ptr(links.ofs),
                                 _ptr(links.m), _ptr(np.ascontiguousarray(data, np.float64)),
                                 _ptr(np.ascontiguousarray(sd, np.float64)), _ptr(g), MEM_HOST, res))
        return g, [(x.it_count, x.status, x.rel_err) for x in res]

    def jacobian_el(self, dphi, aphi, proj, links: Links, scale=DATA_LOG, fp32=False):
        """Element-basis Jacobian (tg_jacobian_el): complex (2 nQM) x (2 ne),
        real (2 nQM) x ne."""
        dphi = _f64(dphi, self.complex)
        aphi = _f64(aphi, self.complex)
        nqm, ne = links.nqm, self.mesh.ne
        J = np.zeros((2 * nqm, 2 * ne if self.complex else ne), np.float32 if fp32 else np.float64)
        pr = None if proj is None else _f64(proj, self.complex)
        _check(lib().tg_jacobian_el(self._h, dphi.shape[0], _ptr(dphi), aphi.shape[0], _ptr(aphi), _ptr(pr),
                                    _ptr(links.ofs), _ptr(links.m), scale, _ptr(J), int(fp32), MEM_HOST))
        return J

    def jacobian_el_raw(self, nq, dphi, nm, aphi, proj, links: Links, scale, J, fp32, mem):
        """tg_jacobian_el with caller-owned buffers (numpy or device tensors)."""
        _check(lib().tg_jacobian_el(self._h, int(nq), _ptr(dphi), int(nm), _ptr(aphi), _ptr(proj), _ptr(links.ofs),
                                    _ptr(links.m), int(scale), _ptr(J), int(fp32), int(mem)))

    def system_matrix(self):
        out = np.zeros(self.mesh.nnz, np.complex128 if self.complex else np.float64)
        _check(lib().tg_solver_matrix(self._h, _ptr(out), MEM_HOST))
        return out

    def calc_fields(self, qvec, phi0=None):
        """Solve for every row of qvec (nrhs x n).  Returns (phi, results)."""
        q = _f64(qvec, self.complex)
        phi = np.zeros_like(q) if phi0 is None else _f64(phi0, self.complex).copy()
        res = (TgResult * q.shape[0])()
        _check(lib().tg_calc_fields(self._h, q.shape[0], _ptr(q), _ptr(phi), MEM_HOST, res))
        return phi, [(r.it_count, r.status, r.rel_err) for r in res]

    def calc_fields_raw(self, k, qvec, phi, mem, res=None):
        """tg_calc_fields with caller-owned buffers (numpy arrays or device
        tensors of k x n values; phi holds the initial guess)."""
        _check(lib().tg_calc_fields(self._h, int(k), _ptr(qvec), _ptr(phi), int(mem), res))

    def project_all(self, mvec, phi, links: Links, scale=DATA_LOG):
        phi = _f64(phi, self.complex)
        mv = _f64(mvec, self.complex)
        out = np.zeros(links.nqm, np.complex128 if self.complex else np.float64)
        _check(lib().tg_project_all(self._h, phi.shape[0], _ptr(phi), mv.shape[0], _ptr(mv), _ptr(links.ofs),
                                    _ptr(links.m), scale, _ptr(out), MEM_HOST))
        return out

    def project_all_noalloc(self, d_phi, nq, d_mvec, nm, links: Links, scale, d_proj):
        """tg_project_all_noalloc: device inputs/outputs, fixed device scratch,
        no device allocation by the library.  d_phi (nq x n), d_mvec (nm x n)
        and d_proj (nQM) are float64 CUDA tensors, complex values as (re, im)
        pairs on a complex solver."""
        w = 2 if self.complex else 1
        n = self.mesh.n
        for name, t, need in (("d_phi", d_phi, nq * n * w), ("d_mvec", d_mvec, nm * n * w),
                              ("d_proj", d_proj, links.nqm * w)):
            if not hasattr(t, "data_ptr") or str(getattr(t, "dtype", "")) != "torch.float64" or not t.is_cuda:
                raise ValueError(f"{name} must be a float64 CUDA tensor")
            if not t.is_contiguous() or t.numel() < need:
                raise ValueError(f"{name} must be contiguous with at least {need} float64 values")
        _check(lib().tg_project_all_noalloc(self._h, int(nq), _ptr(d_phi), int(nm), _ptr(d_mvec), _ptr(links.ofs),
                                            _ptr(links.m), int(scale), _ptr(d_proj)))

    def jacobian_grid(self, raster: "Raster", dphi, aphi, proj, links: Links, scale=DATA_LOG, fp32=False):
        """Grid-basis Jacobian (tg_jacobian_grid): complex (2 nQM) x (2 slen),
        real (2 nQM) x slen."""
        dphi = _f64(dphi, self.complex)
        aphi = _f64(aphi, self.complex)
        nqm, slen = links.nqm, raster.slen
        J = np.zeros((2 * nqm, 2 * slen if self.complex else slen), np.float32 if fp32 else np.float64)
        pr = None if proj is None else _f64(proj, self.complex)
        _check(lib().tg_jacobian_grid(self._h, raster._h, dphi.shape[0], _ptr(dphi), aphi.shape[0], _ptr(aphi),
                                      _ptr(pr), _ptr(links.ofs), _ptr(links.m), scale, _ptr(J), int(fp32), MEM_HOST))
        return J

    def jacobian_grid_raw(self, raster: "Raster", nq, dphi, nm, aphi, proj, links: Links, scale, J, fp32, mem):
        """tg_jacobian_grid with caller-owned buffers (numpy or device tensors)."""
        _check(lib().tg_jacobian_grid(self._h, raster._h, int(nq), _ptr(dphi), int(nm), _ptr(aphi), _ptr(proj),
                                      _ptr(links.ofs), _ptr(links.m), int(scale), _ptr(J), int(fp32), int(mem)))

    def jacobian(self, dphi, aphi, proj, links: Links, scale=DATA_LOG, fp32=False):
        dphi = _f64(dphi, self.complex)
        aphi = _f64(aphi, self.complex)
        n, nqm = self.mesh.n, links.nqm
        J = np.zeros((2 * nqm, 2 * n if self.complex else n), np.float32 if fp32 else np.float64)
        pr = None if proj is None else _f64(proj, self.complex)
        _check(lib().tg_jacobian(self._h, dphi.shape[0], _ptr(dphi), aphi.shape[0], _ptr(aphi), _ptr(pr),
                                 _ptr(links.ofs), _ptr(links.m), scale, _ptr(J), int(fp32), MEM_HOST))
        return J

    def forward_path(self, cmua, ckap, c2a, omega, qvec, mvec, links: Links, want_fields=True, want_jac=True,
                     j_fp32=False):
        """One request through tg_forward_path with host buffers."""
        q = _f64(qvec, self.complex)
        mv = _f64(mvec, self.complex)
        n, nq, nm, nqm = self.mesh.n, q.shape[0], mv.shape[0], links.nqm
        dt = np.complex128 if self.complex else np.float64
        dphi = np.zeros((nq, n), dt) if want_fields else None
        aphi = np.zeros((nm, n), dt) if want_fields else None
        proj = np.zeros(nqm, dt)
        lproj = np.zeros(nqm, dt)
        J = np.zeros((2 * nqm, 2 * n if self.complex else n), np.float32 if j_fp32 else np.float64) if want_jac else None
        res = (TgResult * (nq + nm))()
        cm, ck, ca = (np.ascontiguousarray(x, np.float64) for x in (cmua, ckap, c2a))
        _check(lib().tg_forward_path(self._h, _ptr(cm), _ptr(ck), _ptr(ca), float(omega), nq, _ptr(q), nm, _ptr(mv),
                                     _ptr(links.ofs), _ptr(links.m), _ptr(dphi), _ptr(aphi), _ptr(proj), _ptr(lproj),
                                     _ptr(J), int(j_fp32), MEM_HOST, res))
        its = [(r.it_count, r.status, r.rel_err) for r in res]
        return dict(dphi=dphi, aphi=aphi, proj=proj, logproj=lproj, J=J, results=its)


def tuner_log():
    buf = C.create_string_buffer(1 << 16)
    _check(lib().tg_tuner_log(buf, len(buf)))
    return buf.value.decode()


def launch_count():
    c = C.c_longlong()
    _check(lib().tg_launch_count(C.byref(c)))
    return c.value


def optical_coefficients(mua, mus, nref):
    """cmua, ckappa, c2a from mua, mus', n (src/python/toastmodule.cc:1536-1541;
    A_Keijzer, src/libfe/param.cc:24-32; c0 = 0.3 mm/ps)."""
    c0 = 0.3
    mua = np.asarray(mua, float)
    mus = np.asarray(mus, float)
    nref = np.asarray(nref, float)
    th = np.arcsin(1.0 / nref)
    costh = np.abs(np.cos(th))
    R0 = ((nref - 1.0) * (nref - 1.0)) / ((nref + 1.0) * (nref + 1.0))
    A = (2.0 / (1.0 - R0) - 1.0 + costh * costh * costh) / (1.0 - costh * costh)
    return mua * c0 / nref, c0 / (3.0 * nref * (mua + mus)), c0 / (2.0 * nref * A)


def omega_of(freq_mhz):
    """Modulation frequency [MHz] -> omega [rad/ps] (src/supertoast/fwdfem.cc:116)."""
    return freq_mhz * 2.0 * np.pi * 1e-6


class QM:
    """tg_qm_load: a QM file read against a mesh (QMMesh::LoadQM with
    InitM's detector placement; "external" sources moved to the boundary
    along their normals).  Q, M: positions; links: the link list."""

    def __init__(self, mesh: Mesh, path: str):
        h = C.c_void_p()
        _check(lib().tg_qm_load(mesh._h, os.fsencode(path), C.byref(h)))
        try:
            d, nq, nm, nqm = C.c_int(), C.c_int(), C.c_int(), C.c_int()
            _check(lib().tg_qm_info(h, C.byref(d), C.byref(nq), C.byref(nm), C.byref(nqm)))
            self.Q = np.zeros((nq.value, d.value))
            self.M = np.zeros((nm.value, d.value))
            _check(lib().tg_qm_positions(h, _ptr(self.Q), _ptr(self.M)))
            ofs, lm = np.zeros(nq.value + 1, np.int32), np.zeros(nqm.value, np.int32)
            _check(lib().tg_qm_links(h, _ptr(ofs), _ptr(lm)))
            self.links = Links(ofs, lm)
        finally:
            lib().tg_qm_destroy(h)


# TG_RASTER_PIXEL, TG_RASTER_CUBICPIXEL, and the blob bases
RASTER_KINDS = {"pixel": 0, "cubic": 1, "gauss": 2, "hanning": 3, "ramp": 4, "spline": 5}


class Raster:
    """tg_raster: the pixel raster toast.Raster(mesh, grd, intgrd) builds
    (kind "pixel"), the cubic pixel raster (kind "cubic",
    Raster_CubicPixel), or a blob basis (kind "gauss", "hanning", "ramp",
    "spline": Raster_*Blob, support radius sup, Gaussian width sigma; the
    grid is the padded basis): basis bdim, grid gdim (None: the basis grid)."""

    def __init__(self, mesh: Mesh, bdim, gdim=None, kind="pixel", sup=2.0, sigma=1.0):
        self.mesh = mesh
        self.kind = kind
        self.bdim = np.ascontiguousarray(bdim, np.int32)
        self.gdim = self.bdim.copy() if gdim is None else np.ascontiguousarray(gdim, np.int32)
        h = C.c_void_p()
        if RASTER_KINDS[kind] >= 2:
            _check(lib().tg_raster_create_blob(mesh._h, RASTER_KINDS[kind], self.bdim.ctypes.data_as(C.POINTER(C.c_int)),
                                               float(sup), float(sigma), C.byref(h)))
        else:
            _check(lib().tg_raster_create_typed(mesh._h, RASTER_KINDS[kind],
                                                self.bdim.ctypes.data_as(C.POINTER(C.c_int)),
                                                self.gdim.ctypes.data_as(C.POINTER(C.c_int)), C.byref(h)))
        self._h = h
        gl, sl, bl = C.c_int(), C.c_int(), C.c_int()
        self.bbmin, self.bbmax = np.zeros(len(self.bdim)), np.zeros(len(self.bdim))
        _check(lib().tg_raster_info(self._h, C.byref(gl), C.byref(sl), self.bbmin.ctypes.data_as(C.POINTER(C.c_double)),
                                    self.bbmax.ctypes.data_as(C.POINTER(C.c_double))))
        _check(lib().tg_raster_basis(self._h, C.byref(bl), None))
        self.glen, self.slen, self.blen = gl.value, sl.value, bl.value

    def map(self, kind, x):
        """toast.Raster.Map: kind "X->Y" with X, Y among M (mesh), G (grid),
        B (basis), S (solution); x one vector or a stack (rows), real or
        complex."""
        x = np.asarray(x)
        cplx = np.iscomplexobj(x)
        xs = np.ascontiguousarray(np.atleast_2d(x), np.complex128 if cplx else np.float64)
        sizes = {"M": self.mesh.n, "G": self.glen, "B": self.blen, "S": self.slen}
        out = np.zeros((xs.shape[0], sizes[kind[3]]), xs.dtype)
        _check(lib().tg_raster_map(self._h, kind.encode(), xs.shape[0], _ptr(xs), _ptr(out), 2 if cplx else 1,
                                   MEM_HOST))
        return out[0] if x.ndim == 1 else out

    def sol2basis(self):
        out = np.zeros(max(self.slen, 1), np.int32)
        _check(lib().tg_raster_basis(self._h, None, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out[:self.slen]

    def elref(self):
        out = np.zeros(self.glen, np.int32)
        _check(lib().tg_raster_elref(self._h, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().tg_raster_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Request:
    """One whole request for the server: host inputs and the output buffers it
    fills (proj, logproj, optional J, per-source results)."""

    def __init__(self, mesh: Mesh, cmua, ckap, c2a, omega, qvec, mvec, links: Links, solver=None, precon="ICH",
                 tol=1e-10, precision="mixed", want_jac=True, j_fp32=True, maxit=0, outputs=None):
        """outputs: optional caller-owned (proj, logproj, J) arrays (e.g. views of
        page-locked memory), C-contiguous with the shapes and types the
        request fills; J is None without want_jac."""
        self.complex = omega != 0.0 or np.iscomplexobj(qvec)
        self.mesh = mesh
        cplx = self.complex
        solver = solver or ("BICGSTAB" if cplx else "CG")
        self._keep = [np.ascontiguousarray(x, np.float64) for x in (cmua, ckap, c2a)]
        self.qvec = _f64(qvec, cplx)
        self.mvec = _f64(mvec, cplx)
        self.links = links
        n, nq, nm, nqm = mesh.n, self.qvec.shape[0], self.mvec.shape[0], links.nqm
        dt = np.complex128 if cplx else np.float64
        jshape, jdt = (2 * nqm, 2 * n if cplx else n), np.float32 if j_fp32 else np.float64
        if outputs is None:
            self.proj = np.zeros(nqm, dt)
            self.logproj = np.zeros(nqm, dt)
            self.J = np.zeros(jshape, jdt) if want_jac else None
        else:
            self.proj, self.logproj, self.J = outputs
            for a, shp, t in ((self.proj, (nqm,), dt), (self.logproj, (nqm,), dt)) + \
                    (((self.J, jshape, jdt),) if want_jac else ()):
                if a.shape != shp or a.dtype != t or not a.flags.c_contiguous:
                    raise ValueError(f"output buffer must be a C-contiguous {np.dtype(t).name} array of shape {shp}")
            if not want_jac:
                self.J = None
        self.res = (TgResult * (nq + nm))()
        r = TgRequest()
        r.mesh = mesh._h.value if hasattr(mesh._h, "value") else mesh._h
        r.is_complex = int(cplx)
        r.method, r.precon, r.precision = SOLVERS[solver], PRECONS[precon], PRECISIONS[precision]
        r.tol, r.maxit = float(tol), int(maxit)
        r.cmua, r.ckappa, r.c2a = (x.ctypes.data for x in self._keep)
        r.omega = float(omega)
        r.nq, r.qvec, r.nm, r.mvec = nq, self.qvec.ctypes.data, nm, self.mvec.ctypes.data
        r.link_ofs, r.link_m = links.ofs.ctypes.data, links.m.ctypes.data
        r.proj, r.logproj = self.proj.ctypes.data, self.logproj.ctypes.data
        r.J = self.J.ctypes.data if self.J is not None else None
        r.j_fp32 = int(j_fp32)
        r.res = C.addressof(self.res)
        self.c = r
        self.latency_ms = None

    @property
    def results(self):
        return [(x.it_count, x.status, x.rel_err) for x in self.res]


class Server:
    """tg_server: whole requests admitted by slot and HBM budget, run
    concurrently on per-slot streams (include/toastgpu.h)."""

    def __init__(self, slots=4, hbm_budget_gb=64.0):
        h = C.c_void_p()
        _check(lib().tg_server_create(int(slots), float(hbm_budget_gb), C.byref(h)))
        self._h = h
        self._pending = {}

    def submit(self, req: Request) -> int:
        t = C.c_longlong()
        _check(lib().tg_submit(self._h, C.byref(req.c), C.byref(t)))
        self._pending[t.value] = req
        return t.value

    def poll(self, ticket) -> int:
        st = C.c_int()
        _check(lib().tg_poll(self._h, C.c_longlong(ticket), C.byref(st)))
        return st.value

    def wait(self, ticket) -> Request:
        lat = C.c_double()
        req = self._pending.pop(ticket)
        _check(lib().tg_wait(self._h, C.c_longlong(ticket), C.byref(lat)))
        req.latency_ms = lat.value
        return req

    def stats(self):
        c, f, sv = C.c_longlong(), C.c_longlong(), C.c_longlong()
        p50, p99, el = C.c_double(), C.c_double(), C.c_double()
        _check(lib().tg_server_stats(self._h, C.byref(c), C.byref(f), C.byref(sv), C.byref(p50), C.byref(p99),
                                     C.byref(el)))
        return dict(completed=c.value, failed=f.value, solves=sv.value, p50_ms=p50.value, p99_ms=p99.value,
                    elapsed_s=el.value)

    def reset_stats(self):
        _check(lib().tg_server_reset_stats(self._h))

    def close(self):
        if self._h:
            lib().tg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
