/*
 * toastgpu.h -- C ABI of the GB300 forward-path library (libtoastgpu.so).
 *
 * Drop-in boundary for Toast++'s FEM diffusion forward path.  Every entry
 * point replaces one piece of the reference's C++ interface (paths are within
 * the toastpp project):
 *
 *   tg_mesh_create        Mesh::Setup + MarkBoundary + SparseRowStructure
 *                         (src/libfe/mesh.cc:96-158, 1614-1705, 422-549)
 *   tg_solver_create      TFwdSolver<T>::TFwdSolver(mesh, solver, tol) + SetPrecon
 *                         + Allocate (src/libstoast/fwdsolver.h:85-104, 140, 229;
 *                         fwdsolver.cc:17-34, 143-153, 156-292)
 *   tg_solver_set         SetLinSolver / SetLinSolverMaxit (fwdsolver.h:187, 208)
 *   tg_solver_reset       TFwdSolver<T>::Reset = AssembleSystemMatrix + precon->Reset
 *                         (fwdsolver.cc:337-357, 404-424, 467-505)
 *   tg_solver_matrix      read access to TFwdSolver::F (fwdsolver.h:393-409)
 *   tg_calc_fields        TFwdSolver<T>::CalcFields (fwdsolver.cc:653-750)
 *   tg_project_all        ProjectAll (fwdsolver.h:44-47, fwdsolver.cc:1415-1447)
 *   tg_jacobian           GenerateJacobian(raster=0, ...) nodal basis
 *                         (src/libstoast/jacobian.h:62-82, jacobian.cc:441-497) and
 *                         GenerateJacobian_cw (jacobian.h:101-147, jacobian.cc:132-196, 738-802)
 *   tg_qvec_gaussian      QVec_Gaussian (src/libstoast/source.cc:19-56)
 *   tg_forward_path       the caller sequence of CalcJacobian / CalcJacobianCW
 *                         (src/python/toastmodule.cc:1514-1574, 1630-1684) in one call
 *
 * Conventions
 *   - Every function returns TG_OK (0) or an error code; tg_last_error() gives
 *     the message of the calling thread's last error.  Nothing calls exit().
 *     (The reference reports errors through xERROR -> exit(1), error.cc:37-70.)
 *   - Node and element indices are 0-based, int32.  Elements: 3-noded
 *     triangles (dim 2) or 4-noded tetrahedra (dim 3), positively oriented.
 *   - Complex arrays are interleaved (re, im) doubles.
 *   - Fields and source vectors are source-major: array[q * n + i] (one
 *     TVector<T> per source, as CalcFields takes TVector<T> phi[nQ]).
 *   - mem = TG_MEM_HOST: pointers are host memory (the library copies);
 *     mem = TG_MEM_DEVICE: pointers are device memory of the current device.
 *   - A tg_solver serialises its own calls on its CUDA stream; distinct
 *     solvers may be used from distinct host threads.
 */
#ifndef TOASTGPU_H
#define TOASTGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define TG_OK 0
#define TG_ERR_ARG 1           /* invalid argument */
#define TG_ERR_STATE 2         /* call out of order (e.g. solve before reset) */
#define TG_ERR_CUDA 3          /* CUDA runtime error */
#define TG_ERR_NOMEM 4         /* device allocation failed */
#define TG_ERR_UNSUPPORTED 5   /* combination not implemented */
#define TG_ERR_BREAKDOWN 6     /* a Krylov solve broke down (rho == 0) */

/* LSOLVER / ITMETHOD values (fwdsolver.h:19-21, gsmatrix.h:43-44) */
#define TG_SOLVER_CG 0
#define TG_SOLVER_BICGSTAB 1
#define TG_SOLVER_GMRES 2
/* LSOLVER_DIRECT (fwdsolver.cc:89-123, 467-505: Cholesky for real systems,
   SuperLU for complex ones): a complete F = L L^T factorisation in FP64 at
   each reset (complex systems: complex-symmetric L L^T), in a nested-dissection
   ordering of the nodes; each solve is the two triangular sweeps.  The
   preconditioner and precision settings do not apply.  Per right-hand side
   the result reports 0 iterations and the true relative residual.  A mesh
   whose factor would exceed 2^28 entries gives TG_ERR_UNSUPPORTED at
   tg_solver_create. */
#define TG_SOLVER_DIRECT 3

/* PreconType (src/libmath/precon.h:23-32).  DILU is accepted and, as in
   TFwdSolver::Allocate (fwdsolver.cc:149-153), solved without a preconditioner. */
#define TG_PRECON_NONE 0
#define TG_PRECON_DIAG 1
#define TG_PRECON_ICH 2
#define TG_PRECON_DILU 3

/* arithmetic of the solve: FP64 throughout, or FP32/complex-FP32 inner solves
   inside FP64 iterative refinement */
#define TG_PREC_FP64 0
#define TG_PREC_MIXED 1

#define TG_MEM_HOST 0
#define TG_MEM_DEVICE 1

/* DataScale (fwdsolver.h:28-30) */
#define TG_DATA_LIN 1
#define TG_DATA_LOG 2

typedef struct tg_mesh_s *tg_mesh;
typedef struct tg_solver_s *tg_solver;

/* IterativeSolverResult (src/libmath/matrix.h:34-37), per right-hand side */
typedef struct {
    int it_count;      /* iterations (inner iterations summed for the mixed path) */
    int status;        /* 0 converged, 1 maxit reached, 2 breakdown */
    double rel_err;    /* final |r| / |b| */
} tg_result;

/* ---- mesh ---------------------------------------------------------------- */
int tg_mesh_create(int dim, int n, const double *coords, int ne, const int *elnodes, tg_mesh *out);
/* a mesh file in the reference's MeshData 5.0 text format (operator>> for
   Mesh, src/libfe/mesh.cc:1787-1836): NodeList and an ElementList of 3-noded
   triangles ('o') or 4-noded tetrahedra ('c'); later sections are ignored */
int tg_mesh_load(const char *path, tg_mesh *out);
/* the mesh's dimension, nodes per element and, where the pointers are not
   NULL, its node coordinates (n x dim) and 0-based element nodes (ne x nn) */
int tg_mesh_geometry(tg_mesh mesh, int *dim, int *nn, double *coords, int *elnodes);
int tg_mesh_destroy(tg_mesh mesh);
/* A QM file (QMMesh::LoadQM, src/libfe/qmmesh.cc:319-460): source and
   detector positions and the link list.  Detector positions of a list not
   flagged "fixed" are pulled to the mesh boundary as QMMesh::InitM does
   (Mesh::PullToBoundary, src/libfe/mesh.cc:1052-1111; where no boundary side
   takes the projection the reference keeps the position, and so does this);
   fixed positions outside every element are nudged by 1e-4 along an axis
   (qmmesh.cc:112-127).  An "external" source list moves each source to the
   boundary point Mesh::BndIntersect (mesh.cc:1369-1453) finds from q + |q| n
   towards q, n the unit normal read with the position, or along -q when the
   list's normals flag is "default" (qmmesh.cc:378-391); an "external"
   measurement list is kept as read (LoadQM skips InitM).  A dimension other
   than the mesh's, a missing section, a detector index out of range, a zero
   normal in an external list whose normals are not "default", or an external
   source whose line meets no boundary side give TG_ERR_ARG. */
typedef struct tg_qm_s *tg_qm;
int tg_qm_load(tg_mesh mesh, const char *path, tg_qm *out);
int tg_qm_info(tg_qm qm, int *dim, int *nq, int *nm, int *nqm);
/* Q: nq x dim, M: nm x dim (either may be NULL) */
int tg_qm_positions(tg_qm qm, double *Q, double *M);
/* link_ofs: nq + 1 offsets (Qofs), link_m: nqm detector indices (QMref) */
int tg_qm_links(tg_qm qm, int *link_ofs, int *link_m);
int tg_qm_destroy(tg_qm qm);
/* n, ne, nnz of the CSR pattern, number of boundary nodes, IC(0) levels
   (forward and backward sweep depth) */
int tg_mesh_info(tg_mesh mesh, int *n, int *ne, int *nnz, int *nbnd, int *nlev_fwd, int *nlev_bwd);
int tg_mesh_csr(tg_mesh mesh, int *rowptr, int *colidx);
int tg_mesh_boundary(tg_mesh mesh, unsigned char *bndnode);
/* QVec_Gaussian for npos centres (pos: npos x dim); Neumann mode reproduces the
   boundary source of source.cc:19-56.  out: npos x n, host memory. */
int tg_qvec_gaussian(tg_mesh mesh, int npos, const double *pos, double width, int neumann, double *out);
/* The same on the device (a thread per node and position; the reference's
   summation order): positions on the host, scale (n values, optional, e.g.
   c2a for detector vectors) and out (npos x n) on the host or the device as
   mem says. */
int tg_qvec_gaussian_ex(tg_mesh mesh, int npos, const double *pos, double width, int neumann,
                        const double *scale, double *out, int mem);

/* ---- forward solver ------------------------------------------------------ */
int tg_solver_create(tg_mesh mesh, int is_complex, int method, int precon, double tol, int maxit,
                     int precision, tg_solver *out);
int tg_solver_destroy(tg_solver s);
int tg_solver_set(tg_solver s, double tol, int maxit);
/* mixed precision only: relative tolerance of each FP32 inner solve (default
   1e-4, at least 1e-5: an FP32 recursion does not hold more digits between
   residual replacements), the maximum number of FP64 refinement steps
   (default 12) and the
   elimination ordering of the inner IC(0) preconditioner: 1 (default) a
   colour-major ordering of a greedy colouring, whose colour classes are the
   levels of the triangular sweeps, or 0 the natural ordering of the reference.
   The FP64 path always factors in the natural ordering.  Takes effect at the
   next tg_solver_reset. */
int tg_solver_set_refinement(tg_solver s, double inner_tol, int max_outer, int inner_ordering);
/* mixed precision with BiCGSTAB requested: how the FP32 inner work runs.
   0: restarted refinement (a new FP32 BiCGSTAB solve per FP64 step);
   1: ONE FP32 BiCGSTAB process per right-hand side whose residual is replaced
      by the FP64 residual b - A x whenever it has fallen by inner_tol
      (reliable updates);
   2 (default): as 1 with an FP32 COCG process for complex systems (the
      conjugate-orthogonal CG of the complex symmetric F: one SpMM and one
      IC(0) apply per iteration); real systems use 1.
   The FP64 result meets tol in every mode.  At most 4 * max_outer residual
   replacements per right-hand side. */
/* mixed precision only: the componentwise backward-error bound of every
   solution (default 1e-10; 0 turns the test off).  Besides |b - A x| <= tol |b|
   the FP64 refinement then continues until
       max_i |b - A x|_i / (|A| |x| + |b|)_i <= cw_tol,  |z| = max(|Re z|, |Im z|),
   the Oettli-Prager measure that iterative refinement stops on.  The normwise
   test alone bounds the error of the large entries of a field; the far
   entries, e^-20 of the peak at the far detectors, keep an error of the order
   tol times that dynamic range, which the reference's own solvers carry too.
   With the componentwise bound every entry is as accurate as the bound.  No
   counterpart in the reference (its iterative solvers stop on the normwise
   test, src/libmath/matrix_imp.hpp:93-154, 350-547). */
int tg_solver_set_backward_error(tg_solver s, double cw_tol);
#define TG_MIXED_RESTART 0
#define TG_MIXED_RELIABLE_BICGSTAB 1
#define TG_MIXED_RELIABLE_COCG 2
int tg_solver_set_reliable_updates(tg_solver s, int mode);
/* a cudaStream_t; 0 selects the solver's own stream */
int tg_solver_set_stream(tg_solver s, void *stream);
int tg_solver_sync(tg_solver s);
/* Deferred Jacobian output, for pipelining requests: with a copy stream set
   (a cudaStream_t), tg_forward_path queues the device-to-host copy of a
   page-locked host J on that stream and returns without waiting for it (a
   pageable J is copied before the call returns, as without the stream).  J is complete once
   the work queued on that stream so far has finished (an event recorded on
   it after the call, or tg_solver_sync).  The solver alternates two device J
   buffers and never overwrites one whose copy is still in flight.  NULL
   (default) turns it off: J is in place when tg_forward_path returns. */
int tg_solver_set_output_stream(tg_solver s, void *stream);
/* Reset(sol, omega): nodal cmua, ckappa, c2a (length n); omega in rad/ps
   (0 for real systems).  Assembles F and factors the preconditioner on the GPU. */
int tg_solver_reset(tg_solver s, const double *cmua, const double *ckappa, const double *c2a,
                    double omega, int mem);
/* Reset(sol, omega, elbasis) (fwdsolver.cc:467-505): elbasis = 1 takes one
   cmua / ckappa / c2a value per element (ne each) and assembles with the
   element-basis modes ASSEMBLE_PFF_EL / PDD_EL / BNDPFF_EL
   (src/libfe/mesh.cc:1985-1993); elbasis = 0 is tg_solver_reset. */
int tg_solver_reset_basis(tg_solver s, const double *cmua, const double *ckappa, const double *c2a, double omega,
                          int mem, int elbasis);
/* copy of the assembled system matrix values in CSR order (nnz reals or
   nnz complex) */
int tg_solver_matrix(tg_solver s, double *val, int mem);
/* CalcFields: solve F phi_q = qvec_q for nrhs right-hand sides.  phi holds
   the initial guess on entry (zeros, as CalcFields callers allocate it).
   res (host, optional): per right-hand side result. */
int tg_calc_fields(tg_solver s, int nrhs, const double *qvec, double *phi, int mem, tg_result *res);
/* ProjectAll: proj[l] = dot(phi_q, mvec_m) (non-conjugating) for link l of
   source q with detector m = link_m[l], l in [link_ofs[q], link_ofs[q+1]);
   scale = TG_DATA_LOG returns log (complex log: Re = ln|y|, Im = arg y). */
int tg_project_all(tg_solver s, int nq, const double *phi, int nm, const double *mvec,
                   const int *link_ofs, const int *link_m, int scale, double *proj, int mem);
/* Nodal-basis Jacobian.  Complex: J is (2 nQM) x (2 n) row-major, rows
   [Re; Im] of -PMDF, columns [mua | kappa].  Real (CW): J is Jmua (nQM x n)
   followed by Jkap (nQM x n).  With scale = TG_DATA_LOG each row is divided by
   the linear projection proj[l] (complex for complex systems).
   out_fp32: 0 an FP64 J (FP64-accurate arithmetic: float-float on the GPU's
   FP32 pipes); 1 an FP32 J computed in FP32 (the mixed path's fast J); 2 an
   FP32 J rounded once from the same FP64-accurate sums as 0 (FP32 storage
   of an FP64-accumulated J).  The grid and element bases treat 2 as 1. */
int tg_jacobian(tg_solver s, int nq, const double *dphi, int nm, const double *aphi,
                const double *proj, const int *link_ofs, const int *link_m, int scale,
                void *J, int out_fp32, int mem);

/* The whole path for one request: Reset, CalcFields(qvec), CalcFields(mvec),
   ProjectAll (LIN and LOG) and the Jacobian, on the solver's stream.  Any of
   dphi/aphi/proj/logproj/J may be NULL to skip returning it (J NULL skips the
   Jacobian).  res: 2*nq... per-source results, forward then adjoint (host). */
int tg_forward_path(tg_solver s, const double *cmua, const double *ckappa, const double *c2a,
                    double omega, int nq, const double *qvec, int nm, const double *mvec,
                    const int *link_ofs, const int *link_m, double *dphi, double *aphi,
                    double *proj, double *logproj, void *J, int j_fp32, int mem, tg_result *res);

/* ---- fixed-scratch variant (no counterpart in the reference) -------------
   ProjectAll for callers that cannot call cudaMalloc (a device memory pool
   owned by another runtime, real-time loops that must not allocate, plug-ins
   whose host forbids allocation).  Same result as tg_project_all, but phi,
   mvec and proj are device memory (source-major, as tg_project_all), the
   link list is host memory, and the scratch lives in one fixed file-scope
   device array of TG_NOALLOC_SCRATCH_BYTES held by every GPU that loads the
   library.  No cudaMalloc/cudaFree or allocating routine is called.
   - Problems whose scratch does not fit (about 4 (2n + nQ + nQM) bytes plus
     the detector vectors on their support, nsup x nM values) are rejected
     with TG_ERR_UNSUPPORTED and a message; use tg_project_all for them.
   - The first call on a device looks up the array's device address
     (cudaGetSymbolAddress); make that first call before any stream capture.
   - All calls share the array: calls that overlap on the GPU race, so
     serialise them.  The call synchronises the solver's stream. */
#define TG_NOALLOC_SCRATCH_BYTES (8 * 1024 * 1024)
int tg_project_all_noalloc(tg_solver s, int nq, const double *phi, int nm, const double *mvec,
                           const int *link_ofs, const int *link_m, int scale, double *proj);

/* ---- request server (no counterpart in the reference: its CalcFields is not
   re-entrant, one request per process at a time, fwdsolver.cc:658-731) ------
   Whole requests -- Reset, CalcFields of sources and detectors, ProjectAll
   (LIN and LOG) and optionally the Jacobian -- are submitted from any host
   thread and admitted in arrival order while one of `slots` is free and the
   estimated device working sets of the requests on the device fit in
   hbm_budget_gb (a request larger than the budget runs alone).  Admitted
   requests run concurrently, each on its slot's CUDA stream; each slot keeps
   its solvers resident per (mesh, settings).  Results do not depend on the
   other requests on the device (every reduction has a fixed order).
   All request buffers are host memory owned by the caller until tg_wait
   returns; outputs as tg_forward_path (proj, logproj: nQM values, complex
   interleaved for complex requests; J optional; res: nq + nm entries or NULL). */
typedef struct tg_server_s *tg_server;

typedef struct {
    tg_mesh mesh;
    int is_complex;                 /* 1: frequency domain (omega > 0 allowed), 0: CW */
    int method, precon, precision;  /* TG_SOLVER_*, TG_PRECON_*, TG_PREC_* */
    double tol;
    int maxit;
    const double *cmua, *ckappa, *c2a;   /* nodal, length n */
    double omega;                   /* rad/ps */
    int nq;
    const double *qvec;             /* nq x n, source-major */
    int nm;
    const double *mvec;             /* nm x n */
    const int *link_ofs, *link_m;   /* QMMesh link list */
    double *proj, *logproj;         /* outputs */
    void *J;                        /* output or NULL (no Jacobian) */
    int j_fp32;
    tg_result *res;
} tg_request;

#define TG_REQ_QUEUED 0
#define TG_REQ_RUNNING 1
#define TG_REQ_DONE 2
#define TG_REQ_FAILED 3

int tg_server_create(int slots, double hbm_budget_gb, tg_server *out);
/* waits for every submitted request, then stops the slot threads */
int tg_server_destroy(tg_server server);
int tg_submit(tg_server server, const tg_request *req, long long *ticket);
/* state: TG_REQ_QUEUED / RUNNING / DONE / FAILED */
int tg_poll(tg_server server, long long ticket, int *state);
/* blocks until the request has finished; returns its status code; latency =
   submission to completion.  The ticket is released. */
int tg_wait(tg_server server, long long ticket, double *latency_ms);
/* completed / failed requests, source solves (nq + nm per request), p50 / p99
   latency of the completed requests, seconds since creation or the last reset */
int tg_server_stats(tg_server server, long long *completed, long long *failed, long long *solves,
                    double *p50_ms, double *p99_ms, double *elapsed_s);
int tg_server_reset_stats(tg_server server);

/* ---- measurement (no counterpart in the reference: its timing is
   tic/toc/walltic around calls, src/libmath/timing.h:4-20) ----------------- */
/* kernel classes for tg_solver_profile's mask (bit = 1 << class) */
#define TG_PROF_SPMM 0      /* SpMM / SpMV with fused dot partials */
#define TG_PROF_SWEEP 1     /* one IC(0) apply: all forward + backward level kernels */
#define TG_PROF_VEC 2       /* (reserved) */
#define TG_PROF_JAC 3       /* the Jacobian kernel */
#define TG_PROF_ASM 4       /* assembly + preconditioner factorisation */
#define TG_PROF_PROJ 5      /* projection kernel */
/* record CUDA events around the launches of the selected classes (clears the record) */
int tg_solver_profile(tg_solver s, int mask);
/* total device time and number of recorded launches of one class */
int tg_solver_profile_read(tg_solver s, int cls, double *total_ms, int *count);
/* number of kernels this library has launched in this process */
int tg_launch_count(long long *count);
/* Element-basis Jacobian (GenerateJacobian(RASTER_ELBASIS, ...),
   jacobian.cc:441-497 with IntFG_el / IntGradFGradG_el, 884-939; real:
   GenerateJacobian_cw(RASTER_ELBASIS, ...), 178-193 / 738-802).  Inputs as
   tg_jacobian.  J row-major: complex (2 nQM) x (2 ne) = [-Re mua | -Re kappa ;
   -Im mua | -Im kappa]; real (2 nQM) x ne = [mua ; kappa]. */
int tg_jacobian_el(tg_solver s, int nq, const double *dphi, int nm, const double *aphi, const double *proj,
                   const int *link_ofs, const int *link_m, int scale, void *J, int out_fp32, int mem);

/* ---- grid basis (pixel raster) ----
   Raster_Pixel(bdim, gdim), as toast.Raster(mesh, grd, intgrd) builds it
   (src/python/toastmodule.cc:696; raster.cc:18-83, raster_px.cc:10-48): a
   regular grid of gdim[0] x gdim[1] (x gdim[2]) points over the mesh's
   bounding box carries the mapped fields, a basis of bdim points the
   solution.  Without an intermediate grid (gdim NULL or equal to bdim) the
   solution points are the grid points inside the mesh, in grid order (x
   fastest).  With one, grid and basis are joined by the linear pixel maps
   (Grid2LinPixMatrix / LinPix2GridMatrix, src/libfe/mesh.cc:3138-3320,
   3540-3640) and the solution points are the basis points whose subsampled
   mesh support is positive (SubsampleLinPixel, mesh.cc:3047-3136), in basis
   order.  tg_raster_create(mesh, bdim, out) = tg_raster_create_ex(mesh,
   bdim, NULL, out).
   tg_raster_create_typed with TG_RASTER_CUBICPIXEL builds
   Raster_CubicPixel(bdim, gdim) (src/libstoast/raster_cp.cc:10-186): the
   cubic B-spline basis, joined to the grid by its own G (normalised spline
   weights of the grid points inside the mesh) and GI (the basis functions'
   values at the grid points); its solution points are the basis points with
   a nonempty row of G. */
#define TG_RASTER_PIXEL 0
#define TG_RASTER_CUBICPIXEL 1
#define TG_RASTER_GAUSSBLOB 2
#define TG_RASTER_HANNINGBLOB 3
#define TG_RASTER_RAMPBLOB 4
#define TG_RASTER_SPLINEBLOB 5
typedef struct tg_raster_s *tg_raster;
int tg_raster_create(tg_mesh mesh, const int *bdim, tg_raster *out);
int tg_raster_create_ex(tg_mesh mesh, const int *bdim, const int *gdim, tg_raster *out);
int tg_raster_create_typed(tg_mesh mesh, int type, const int *bdim, const int *gdim, tg_raster *out);
/* The blob bases (Raster_Blob, src/libstoast/raster_bl.cc:9-350, and
   Raster_GaussBlob / HanningBlob / RampBlob / SplineBlob, raster_gb.cc,
   raster_hb.cc, raster_rb.cc, raster_sb.cc): type TG_RASTER_GAUSSBLOB ..
   TG_RASTER_SPLINEBLOB, support radius sup in basis spacings, width sigma
   (Gaussian only).  The basis grid of bdim points is padded by
   ceil(sup - 1e-6) points on every side and is also the grid (glen = blen
   = the padded size); the solution points are the basis points within sup
   of a mesh node.  Fields map to the basis as node-value-weighted averages,
   the basis back to the nodes as node-value-weighted sums. */
int tg_raster_create_blob(tg_mesh mesh, int type, const int *bdim, double sup, double sigma, tg_raster *out);
int tg_raster_destroy(tg_raster r);
/* glen grid points, slen solution points, bounding box (dim values each) */
int tg_raster_info(tg_raster r, int *glen, int *slen, double *bbmin, double *bbmax);
/* element containing each grid point, -1 outside (Raster::Elref) */
int tg_raster_elref(tg_raster r, int *elref);
/* blen basis points and the basis index of each solution point
   (Raster::Sol2Basis, slen values); either may be NULL */
int tg_raster_basis(tg_raster r, int *blen, int *sol2basis);
/* toast.Raster.Map (MapBasis, src/python/toastmodule.cc:718-790): map is
   "X->Y" with X, Y among M (mesh nodes), G (grid), B (basis; the grid itself
   without an intermediate grid) and S (solution points); nvec vectors back
   to back, width doubles per point (1 real, 2 complex interleaved); src,
   dst in host or device memory.  Each map runs the chain the reference's
   raster runs for that vector type (the pixel raster's real vectors: its
   product maps G B and BI GI; otherwise through the grid), summing in the
   reference's order without fused multiply-adds (bit-identical). */
int tg_raster_map(tg_raster r, const char *map, int nvec, const double *src, double *dst, int width, int mem);
/* Grid-basis Jacobian (GenerateJacobian with a raster, jacobian.cc:105-123
   -> GenerateJacobian_grid 289-373; real systems GenerateJacobian_cw with a
   raster, 178-193 -> GenerateJacobian_cw_grid 610-712).  Inputs as
   tg_jacobian (source-major natural fields, projections for LOG data).
   J row-major: complex (2 nQM) x (2 slen) = [Re mua | Re kappa ; Im mua |
   Im kappa]; real (2 nQM) x slen = [mua ; kappa].  out_fp32 selects an FP32
   J computed in FP32, else FP64 throughout. */
int tg_jacobian_grid(tg_solver s, tg_raster r, int nq, const double *dphi, int nm, const double *aphi,
                     const double *proj, const int *link_ofs, const int *link_m, int scale, void *J,
                     int out_fp32, int mem);

/* toast's Gradient on a raster (GetGradient / AddDataGradient,
   src/python/toastmodule.cc:1745-1887), after tg_solver_reset of a complex
   solver: solves the nq sources, projects (model data = ln|y|, arg y), forms
   one adjoint source per source from the data residuals, solves those, and
   subtracts the grid products of the two fields (and of their image
   gradients) from grad.  data, sd: 2 nQM (log amplitude block, then phase
   block); grad: 2 slen [mua | kappa], in/out.  res (optional): 2 nq results,
   the forward solves then the adjoint ones. */
int tg_gradient(tg_solver s, tg_raster r, int nq, const double *qvec, int nm, const double *mvec,
                const int *link_ofs, const int *link_m, const double *data, const double *sd, double *grad, int mem,
                tg_result *res);

/* the SpMM autotuner's decisions so far: one text line per (mesh, value type,
   columns) with every candidate kernel's best launch time and the choice.
   The environment variable TOASTGPU_SPMM_VARIANT (spmm_halo, spmm_vec,
   spmm_wide or spmm_dot) fixes the variant wherever it applies. */
int tg_tuner_log(char *buf, int len);

const char *tg_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* TOASTGPU_H */
