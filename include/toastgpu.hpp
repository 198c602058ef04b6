// toastgpu.hpp -- C++ face of libtoastgpu.so with the names and argument
// meanings of Toast++'s forward-solver interface, so that a caller of
// TFwdSolver / ProjectAll / GenerateJacobian changes types, not code.
//
//   toastgpu::TFwdSolver<T>       TFwdSolver<T> (src/libstoast/fwdsolver.h:77-409),
//                                 T = double (CW) or std::complex<double> (frequency domain)
//   toastgpu::ProjectAll          ProjectAll (fwdsolver.h:44-47, fwdsolver.cc:1415-1447)
//   toastgpu::GenerateJacobian    GenerateJacobian(raster = 0, ...) nodal basis
//                                 (src/libstoast/jacobian.h:62-82) and
//                                 GenerateJacobian_cw (jacobian.h:101-147)
//   toastgpu::Raster_Pixel        Raster_Pixel(bdim, bdim, mesh) (raster_px.cc:10-48), the
//                                 raster toast.Raster(mesh, grd) builds
//   toastgpu::GenerateJacobian    GenerateJacobian(raster, ...) grid basis (jacobian.cc:105-123)
//   toastgpu::GenerateJacobian_el GenerateJacobian(RASTER_ELBASIS, ...) element basis
//   toastgpu::QVec_Gaussian       QVec_Gaussian, Neumann mode (src/libstoast/source.cc:19-56)
//
// Differences a caller sees:
//   - Reset takes the nodal cmua / ckappa / c2a arrays that the reference's
//     Solution holds as OT_CMUA / OT_CKAPPA / OT_C2A (Solution::SetParam).
//   - qvec / mvec and the fields are dense source-major arrays (q * n + i)
//     instead of TCompRowMatrix rows and TVector arrays.
//   - Errors throw toastgpu::Error (the reference calls exit through xERROR).
//   - SetPrecision(TG_PREC_MIXED) selects FP32 inner solves inside FP64
//     refinement; the default is FP64 throughout, as the reference.
#ifndef TOASTGPU_HPP
#define TOASTGPU_HPP

#include <complex>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "toastgpu.h"

namespace toastgpu {

// enumerations with the reference's values (fwdsolver.h:17-30, precon.h:23-32)
enum LSOLVER { LSOLVER_UNDEFINED, LSOLVER_DIRECT, LSOLVER_ITERATIVE };
enum DataScale { DATA_DEFAULT, DATA_LIN, DATA_LOG };
enum PreconType { PRECON_NULL, PRECON_DIAG, PRECON_ICH, PRECON_DILU };

struct IterativeSolverResult {  // src/libmath/matrix.h:34-37
    int it_count;
    double rel_err;
};

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc)
{
    if (rc != TG_OK) throw Error(rc, tg_last_error());
}

// QMMesh link list (qmmesh.h:24-36): Qofs / QMref in source-major order
struct Links {
    std::vector<int> ofs;  // nQ + 1
    std::vector<int> m;    // nQM
    static Links all_to_all(int nq, int nm)
    {
        Links L;
        for (int q = 0; q <= nq; q++) L.ofs.push_back(q * nm);
        for (int q = 0; q < nq; q++)
            for (int j = 0; j < nm; j++) L.m.push_back(j);
        return L;
    }
    int nQM() const { return ofs.empty() ? 0 : ofs.back(); }
};

// Mesh::Setup + MarkBoundary + SparseRowStructure on construction
class Mesh {
public:
    Mesh(int dim, int n, const double* coords, int ne, const int* elnodes)
    {
        check(tg_mesh_create(dim, n, coords, ne, elnodes, &h_));
        check(tg_mesh_info(h_, &n_, &ne_, &nnz_, nullptr, nullptr, nullptr));
        dim_ = dim;
    }
    // operator>> for Mesh (src/libfe/mesh.cc:1787-1836) + Setup: a MeshData 5.0 file
    explicit Mesh(const char* path)
    {
        check(tg_mesh_load(path, &h_));
        check(tg_mesh_info(h_, &n_, &ne_, &nnz_, nullptr, nullptr, nullptr));
        check(tg_mesh_geometry(h_, &dim_, nullptr, nullptr, nullptr));
    }
    ~Mesh() { tg_mesh_destroy(h_); }
    Mesh(const Mesh&) = delete;
    Mesh& operator=(const Mesh&) = delete;
    int nlen() const { return n_; }
    int elen() const { return ne_; }
    int Dimension() const { return dim_; }
    tg_mesh handle() const { return h_; }

private:
    tg_mesh h_ = nullptr;
    int n_ = 0, ne_ = 0, nnz_ = 0, dim_ = 0;
};

// QMMesh::LoadQM (src/libfe/qmmesh.cc:319-460) with InitM's detector
// placement and the boundary projection of "external" sources, against a
// mesh: positions Q, M (row-major, dim per point) and
// the link list (nQMref / QMref as offsets and detector indices)
struct QMData {
    int dim = 0, nQ = 0, nM = 0, nQM = 0;
    std::vector<double> Q, M;
    Links links;
};
inline QMData LoadQM(const Mesh& mesh, const char* path)
{
    tg_qm h = nullptr;
    check(tg_qm_load(mesh.handle(), path, &h));
    QMData d;
    int rc = tg_qm_info(h, &d.dim, &d.nQ, &d.nM, &d.nQM);
    if (rc == TG_OK) {
        d.Q.resize((size_t)d.nQ * d.dim);
        d.M.resize((size_t)d.nM * d.dim);
        d.links.ofs.resize(d.nQ + 1);
        d.links.m.resize(d.nQM);
        rc = tg_qm_positions(h, d.Q.data(), d.M.data());
        if (rc == TG_OK) rc = tg_qm_links(h, d.links.ofs.data(), d.links.m.data());
    }
    tg_qm_destroy(h);
    check(rc);
    return d;
}

// QVec_Gaussian(mesh, cnt, w, SRCMODE_NEUMANN) for one position: n values
inline std::vector<double> QVec_Gaussian(const Mesh& mesh, const double* cnt, double w)
{
    std::vector<double> q(mesh.nlen());
    check(tg_qvec_gaussian(mesh.handle(), 1, cnt, w, 1, q.data()));
    return q;
}

template <class T>
class TFwdSolver {
    static_assert(std::is_same<T, double>::value || std::is_same<T, std::complex<double>>::value,
                  "T = double or std::complex<double>");
    static constexpr bool cplx = std::is_same<T, std::complex<double>>::value;

public:
    // TFwdSolver(mesh, solver, tol, nth) (fwdsolver.h:95-99); nth is accepted
    // and ignored (the GPU solves all sources together)
    TFwdSolver(const Mesh* mesh, const char* solver, double tol = 1e-10, int nth = 1) : mesh_(mesh)
    {
        (void)nth;
        SetLinSolver(solver, tol);
    }
    ~TFwdSolver()
    {
        if (s_) tg_solver_destroy(s_);
    }
    TFwdSolver(const TFwdSolver&) = delete;
    TFwdSolver& operator=(const TFwdSolver&) = delete;

    void SetDataScaling(DataScale scale) { dscale_ = scale; }
    DataScale GetDataScaling() const { return dscale_; }
    void SetPrecon(PreconType type) { precon_ = type; drop(); }
    // "CG", "BICGSTAB" or "GMRES" (case-insensitive, fwdsolver.cc:1279-1296);
    // DIRECT / BICG / Gauss-Seidel are not part of this library
    void SetLinSolver(const char* solver, double tol = 1e-10)
    {
        std::string s(solver);
        for (auto& c : s) c = (char)toupper((unsigned char)c);
        if (s == "CG") method_ = TG_SOLVER_CG;
        else if (s == "BICGSTAB") method_ = TG_SOLVER_BICGSTAB;
        else if (s == "GMRES") method_ = TG_SOLVER_GMRES;
        else throw Error(TG_ERR_UNSUPPORTED, "linear solver " + s + " is not provided by the GPU path");
        tol_ = tol;
        if (s_) check(tg_solver_set(s_, tol_, maxit_));
        else drop();
    }
    double GetLinSolverTol() const { return tol_; }
    void SetLinSolverMaxit(int maxit)
    {
        maxit_ = maxit;
        if (s_) check(tg_solver_set(s_, tol_, maxit_));
    }
    void SetPrecision(int precision) { precision_ = precision; drop(); }
    LSOLVER LinSolver() const { return LSOLVER_ITERATIVE; }

    // Allocate (fwdsolver.cc:156-292)
    void Allocate()
    {
        if (!s_) {
            int p = precon_ == PRECON_DILU ? TG_PRECON_DILU : (int)precon_;
            check(tg_solver_create(mesh_->handle(), cplx ? 1 : 0, method_, p, tol_, maxit_, precision_, &s_));
        }
    }
    // Reset(sol, omega) (fwdsolver.cc:467-505): assembly and preconditioner
    // Reset(sol, omega, elbasis) (fwdsolver.cc:467-505): elbasis = true takes
    // one coefficient per element (mesh.elen() values each)
    void Reset(const double* cmua, const double* ckappa, const double* c2a, double omega = 0, bool elbasis = false)
    {
        Allocate();
        check(tg_solver_reset_basis(s_, cmua, ckappa, c2a, omega, TG_MEM_HOST, elbasis ? 1 : 0));
    }
    // CalcFields(qvec, phi, res) (fwdsolver.cc:653-750): phi holds the
    // initial guess; res gets the summed iterations and the largest error
    void CalcFields(int nq, const T* qvec, T* phi, IterativeSolverResult* res = nullptr) const
    {
        std::vector<tg_result> r(nq);
        check(tg_calc_fields(s_, nq, (const double*)qvec, (double*)phi, TG_MEM_HOST, r.data()));
        if (res) {
            res->it_count = 0;
            res->rel_err = 0;
            for (auto& x : r) {
                res->it_count += x.it_count;
                if (x.rel_err > res->rel_err) res->rel_err = x.rel_err;
            }
        }
    }
    // ProjectAll(mvec, phi, scale) (fwdsolver.cc:826-860)
    std::vector<T> ProjectAll(int nm, const T* mvec, int nq, const T* phi, const Links& L,
                              DataScale scale = DATA_DEFAULT) const
    {
        std::vector<T> y(L.nQM());
        const int sc = (scale == DATA_DEFAULT ? dscale_ : scale) == DATA_LOG ? TG_DATA_LOG : TG_DATA_LIN;
        check(tg_project_all(s_, nq, (const double*)phi, nm, (const double*)mvec, L.ofs.data(), L.m.data(), sc,
                             (double*)y.data(), TG_MEM_HOST));
        return y;
    }
    // read access to the assembled system matrix values, CSR order
    std::vector<T> SystemMatrixValues() const
    {
        int nnz = 0;
        check(tg_mesh_info(mesh_->handle(), nullptr, nullptr, &nnz, nullptr, nullptr, nullptr));
        std::vector<T> v(nnz);
        check(tg_solver_matrix(s_, (double*)v.data(), TG_MEM_HOST));
        return v;
    }
    tg_solver handle() const { return s_; }
    const Mesh* meshptr() const { return mesh_; }

private:
    void drop()
    {
        if (s_) { tg_solver_destroy(s_); s_ = nullptr; }
    }
    const Mesh* mesh_;
    tg_solver s_ = nullptr;
    int method_ = TG_SOLVER_BICGSTAB, precision_ = TG_PREC_FP64, maxit_ = 0;
    PreconType precon_ = PRECON_NULL;
    DataScale dscale_ = DATA_LIN;
    double tol_ = 1e-10;
};

// GenerateJacobian(0, mesh, mvec, dphi, aphi, proj, dscale, J) nodal basis:
// J is (2 nQM) x (2 n) row-major, rows [Re; Im] of -PMDF, columns [mua | kappa]
// (jacobian.cc:441-497); proj = linear projections, used for DATA_LOG
template <class T>
void GenerateJacobian(const TFwdSolver<T>& fws, int nq, const T* dphi, int nm, const T* aphi, const T* proj,
                      const Links& L, DataScale dscale, double* J)
{
    check(tg_jacobian(fws.handle(), nq, (const double*)dphi, nm, (const double*)aphi, (const double*)proj,
                      L.ofs.data(), L.m.data(), dscale == DATA_LOG ? TG_DATA_LOG : TG_DATA_LIN, J, 0, TG_MEM_HOST));
}

// GenerateJacobian(RASTER_ELBASIS, mesh, dphi, aphi, proj, dscale, J) element
// basis: complex J (2 nQM) x (2 ne) row-major [-Re mua | -Re kappa ; -Im mua |
// -Im kappa] (jacobian.cc:441-497); real J (2 nQM) x ne [mua ; kappa]
// (GenerateJacobian_cw(RASTER_ELBASIS, ...), jacobian.cc:178-193, 738-802)
template <class T>
void GenerateJacobian_el(const TFwdSolver<T>& fws, int nq, const T* dphi, int nm, const T* aphi, const T* proj,
                         const Links& L, DataScale dscale, double* J)
{
    check(tg_jacobian_el(fws.handle(), nq, (const double*)dphi, nm, (const double*)aphi, (const double*)proj,
                         L.ofs.data(), L.m.data(), dscale == DATA_LOG ? TG_DATA_LOG : TG_DATA_LIN, J, 0, TG_MEM_HOST));
}

// Raster_Pixel(bdim, gdim, mesh): a grid of gdim points per axis over the
// mesh's bounding box and a basis of bdim points; SLen() solution points
// (without an intermediate grid: the grid points inside the mesh)
class Raster_Pixel {
public:
    Raster_Pixel(const int* bdim, const Mesh& mesh) : Raster_Pixel(bdim, nullptr, mesh) {}
    Raster_Pixel(const int* bdim, const int* gdim, const Mesh& mesh)
    {
        check(tg_raster_create_ex(mesh.handle(), bdim, gdim, &h_));
        check(tg_raster_info(h_, &glen_, &slen_, nullptr, nullptr));
        check(tg_raster_basis(h_, &blen_, nullptr));
    }
    ~Raster_Pixel() { tg_raster_destroy(h_); }
    Raster_Pixel(const Raster_Pixel&) = delete;
    Raster_Pixel& operator=(const Raster_Pixel&) = delete;
    int GLen() const { return glen_; }
    int BLen() const { return blen_; }
    int SLen() const { return slen_; }
    std::vector<int> Elref() const
    {
        std::vector<int> e(glen_);
        check(tg_raster_elref(h_, e.data()));
        return e;
    }
    tg_raster handle() const { return h_; }

private:
    tg_raster h_ = nullptr;
    int glen_ = 0, blen_ = 0, slen_ = 0;
};

// Raster_CubicPixel(bdim, gdim, mesh) (src/libstoast/raster_cp.cc): the
// cubic B-spline basis of bdim points over a grid of gdim points
class Raster_CubicPixel {
public:
    Raster_CubicPixel(const int* bdim, const int* gdim, const Mesh& mesh)
    {
        check(tg_raster_create_typed(mesh.handle(), TG_RASTER_CUBICPIXEL, bdim, gdim, &h_));
        check(tg_raster_info(h_, &glen_, &slen_, nullptr, nullptr));
        check(tg_raster_basis(h_, &blen_, nullptr));
    }
    ~Raster_CubicPixel() { tg_raster_destroy(h_); }
    Raster_CubicPixel(const Raster_CubicPixel&) = delete;
    Raster_CubicPixel& operator=(const Raster_CubicPixel&) = delete;
    int GLen() const { return glen_; }
    int BLen() const { return blen_; }
    int SLen() const { return slen_; }
    tg_raster handle() const { return h_; }

private:
    tg_raster h_ = nullptr;
    int glen_ = 0, blen_ = 0, slen_ = 0;
};

// GenerateJacobian(raster, mesh, dphi, aphi, proj, dscale, J) grid basis:
// complex J (2 nQM) x (2 SLen) row-major [Re mua | Re kappa ; Im mua | Im
// kappa] (jacobian.cc:289-373); real J (2 nQM) x SLen [mua ; kappa]
// (GenerateJacobian_cw with a raster, jacobian.cc:178-193, 610-712)
template <class T>
void GenerateJacobian(const Raster_Pixel& raster, const TFwdSolver<T>& fws, int nq, const T* dphi, int nm,
                      const T* aphi, const T* proj, const Links& L, DataScale dscale, double* J)
{
    check(tg_jacobian_grid(fws.handle(), raster.handle(), nq, (const double*)dphi, nm, (const double*)aphi,
                           (const double*)proj, L.ofs.data(), L.m.data(),
                           dscale == DATA_LOG ? TG_DATA_LOG : TG_DATA_LIN, J, 0, TG_MEM_HOST));
}

}  // namespace toastgpu

#endif  // TOASTGPU_HPP
