// jacobian_gpu.cc -- the reference's GenerateJacobian / GenerateJacobian_cw
// (src/libstoast/jacobian.h:62-147) on the GPU.
//
// Defines the five public functions of the reference's jacobian.h by
// forwarding to the C ABI: the nodal basis (raster RASTER_NDBASIS), the
// element basis (RASTER_ELBASIS) and the grid basis of a Raster_Pixel, with
// or without an intermediate grid (the raster toast.Raster(mesh, grd,
// intgrd) builds), or of a Raster_CubicPixel; other rasters stop with
// xERROR.  The shim Makefile weakens these
// five symbols in the reference's own jacobian object, which stays linked
// for the rest of what it holds (ImageGradient, used by the regularisation
// and raster code), so these definitions take their place.
//
// As the reference: Jacobian rows are source-major links (Qofs / QMref);
// complex J is (2 nQM) x (2 nsol) [Re; Im] x [mua | kappa]; CW gives Jmua and
// Jkap (nQM x nsol each), scaled row by row by 1/y for log data.  The
// projection-from-mvec overloads project first, then proceed as the
// projection overloads (so the element-basis kappa block sits at offset ne in
// both; jacobian.cc:397 offsets it by n in the mvec overload).
#define STOASTLIB_IMPLEMENTATION
#include "stoastlib.h"

#include <complex>
#include <vector>

#include "toastgpu.h"
#include "shim_common.h"

using namespace tgshim;

namespace {

// the basis of a raster argument: 0 nodal, 1 element, 2 grid (Raster_Pixel
// or Raster_CubicPixel)
int basis_of(const Raster* raster)
{
    if (raster == RASTER_NDBASIS) return 0;
    if (raster == RASTER_ELBASIS) return 1;
    if (!dynamic_cast<const Raster_Pixel*>(raster) && !dynamic_cast<const Raster_CubicPixel*>(raster))
        xERROR("libtoastgpu: only pixel and cubic pixel rasters are provided");
    return 2;
}

template <class T>
std::vector<double> dense_fields(const TVector<T>* phi, int k, int n)
{
    const bool cplx = sizeof(T) == 16;
    std::vector<double> out((size_t)k * n * (cplx ? 2 : 1));
    for (int q = 0; q < k; q++) {
        const T* p = phi[q].data_buffer();
        memcpy(&out[(size_t)q * n * (cplx ? 2 : 1)], p, sizeof(T) * n);
    }
    return out;
}

// J (row-major doubles, rows x cols) for the given basis and data scale
void jacobian(const Raster* raster, const QMMesh* mesh, bool cplx, const std::vector<double>& f,
              const std::vector<double>& a, const double* proj, int scale, std::vector<double>& J, int& ncol)
{
    tg_mesh gm = nullptr;
    tg_solver s = mesh_solver(mesh, cplx, &gm);
    std::vector<int> ofs, lm;
    links_of(mesh, ofs, lm);
    const int nq = mesh->nQ, nm = mesh->nM, nqm = (int)lm.size();
    const int basis = basis_of(raster);
    int nsol = mesh->nlen();
    tg_raster r = nullptr;
    if (basis == 1) nsol = mesh->elen();
    if (basis == 2) {
        const IVector& b = raster->BDim();
        const IVector& g = raster->GDim();
        int bdim[3] = {b[0], b[1], b.Dim() > 2 ? b[2] : 1};
        int gdim[3] = {g[0], g[1], g.Dim() > 2 ? g[2] : 1};
        const int type = dynamic_cast<const Raster_CubicPixel*>(raster) ? TG_RASTER_CUBICPIXEL : TG_RASTER_PIXEL;
        check(tg_raster_create_typed(gm, type, bdim, gdim, &r), "tg_raster_create_typed");
        int glen = 0;
        check(tg_raster_info(r, &glen, &nsol, nullptr, nullptr), "tg_raster_info");
    }
    ncol = cplx ? 2 * nsol : nsol;
    J.assign((size_t)2 * nqm * ncol, 0.0);
    int rc;
    if (basis == 0)
        rc = tg_jacobian(s, nq, f.data(), nm, a.data(), proj, ofs.data(), lm.data(), scale, J.data(), 0,
                         TG_MEM_HOST);
    else if (basis == 1)
        rc = tg_jacobian_el(s, nq, f.data(), nm, a.data(), proj, ofs.data(), lm.data(), scale, J.data(), 0,
                            TG_MEM_HOST);
    else
        rc = tg_jacobian_grid(s, r, nq, f.data(), nm, a.data(), proj, ofs.data(), lm.data(), scale, J.data(), 0,
                              TG_MEM_HOST);
    if (r) tg_raster_destroy(r);
    check(rc, "GenerateJacobian");
}

void to_dense(RDenseMatrix& M, const double* src, int rows, int cols)
{
    M.New(rows, cols);
    memcpy(M.ValPtr(), src, sizeof(double) * (size_t)rows * cols);
}

}  // namespace

void GenerateJacobian(const Raster* raster, const QMMesh* mesh, const CVector* dphi, const CVector* aphi,
                      const CVector* proj, DataScale dscale, RDenseMatrix& J)
{
    const int n = mesh->nlen();
    std::vector<double> f = dense_fields(dphi, mesh->nQ, n), a = dense_fields(aphi, mesh->nM, n), Jd;
    int ncol = 0;
    jacobian(raster, mesh, true, f, a, dscale == DATA_LOG ? (const double*)proj->data_buffer() : nullptr,
             dscale == DATA_LOG ? TG_DATA_LOG : TG_DATA_LIN, Jd, ncol);
    to_dense(J, Jd.data(), 2 * mesh->nQM, ncol);
}

void GenerateJacobian(const Raster* raster, const QMMesh* mesh, const CCompRowMatrix& mvec, const CVector* dphi,
                      const CVector* aphi, DataScale dscale, RDenseMatrix& J)
{
    CVector proj;
    if (dscale == DATA_LOG) proj = ProjectAll(mesh, mvec, dphi, DATA_LIN);
    GenerateJacobian(raster, mesh, dphi, aphi, &proj, dscale, J);
}

void GenerateJacobian_cw(const Raster* raster, const QMMesh* mesh, const RVector* dphi, const RVector* aphi,
                         RDenseMatrix* Jmua, RDenseMatrix* Jkap)
{
    GenerateJacobian_cw(raster, mesh, dphi, aphi, (const RVector*)0, DATA_LIN, Jmua, Jkap);
}

void GenerateJacobian_cw(const Raster* raster, const QMMesh* mesh, const RVector* dphi, const RVector* aphi,
                         const RVector* proj, DataScale dscale, RDenseMatrix* Jmua, RDenseMatrix* Jkap)
{
    const int n = mesh->nlen(), nqm = mesh->nQM;
    std::vector<double> f = dense_fields(dphi, mesh->nQ, n), a = dense_fields(aphi, mesh->nM, n), Jd;
    int ncol = 0;
    jacobian(raster, mesh, false, f, a, dscale == DATA_LOG ? proj->data_buffer() : nullptr,
             dscale == DATA_LOG ? TG_DATA_LOG : TG_DATA_LIN, Jd, ncol);
    if (Jmua) to_dense(*Jmua, Jd.data(), nqm, ncol);
    if (Jkap) to_dense(*Jkap, Jd.data() + (size_t)nqm * ncol, nqm, ncol);
}

void GenerateJacobian_cw(const Raster* raster, const QMMesh* mesh, const RCompRowMatrix& mvec, const RVector* dphi,
                         const RVector* aphi, DataScale dscale, RDenseMatrix* Jmua, RDenseMatrix* Jkap)
{
    RVector proj;
    if (dscale == DATA_LOG) proj = ProjectAll(mesh, mvec, dphi, DATA_LIN);
    GenerateJacobian_cw(raster, mesh, dphi, aphi, &proj, dscale, Jmua, Jkap);
}
