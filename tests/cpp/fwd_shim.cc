// A caller written against the C++ face (include/toastgpu.hpp) in the
// sequence of the reference's fwdfem / CalcJacobian callers
// (src/supertoast/fwdfem.cc:180-250, src/python/toastmodule.cc:1514-1574):
// Allocate, Reset, CalcFields for sources and detectors, ProjectAll (LIN and
// LOG), GenerateJacobian.  Input and output are raw binary files.
//
//   fwd_shim IN OUT
//   IN : int32 dim, n, ne, nq, nm, cplx ; double freq_mhz, width ;
//        n*dim coords ; ne*(dim+1) int32 elements ; n cmua ; n ckappa ; n c2a ;
//        nq*dim source positions ; nm*dim detector positions
//   OUT: nQM logproj values, then the Jacobian (doubles; complex interleaved),
//        then the grid-basis Jacobian of Raster_Pixel(12 points per axis)
//
//   fwd_shim qm MESH QMFILE OUT
//   reads a mesh file and a QM file through the face (Mesh(path), LoadQM) and
//   writes int32 dim, nQ, nM, nQM ; Q ; M (doubles) ; link offsets ; detectors
#include <cmath>
#include <complex>
#include <cstdio>
#include <string>
#include <vector>

#include "toastgpu.hpp"

using namespace toastgpu;

template <class T>
static int run(int dim, int n, int nq, int nm, double omega, double width, const std::vector<double>& xy,
               const std::vector<int>& el, int ne, const std::vector<double>& prm, const std::vector<double>& qp,
               const std::vector<double>& mp, FILE* out)
{
    Mesh mesh(dim, n, xy.data(), ne, el.data());
    const double* cmua = prm.data();
    const double* ckap = prm.data() + n;
    const double* c2a = prm.data() + 2 * n;
    std::vector<T> qvec((size_t)nq * n), mvec((size_t)nm * n);
    for (int q = 0; q < nq; q++) {
        std::vector<double> v = QVec_Gaussian(mesh, &qp[(size_t)q * dim], width);
        for (int i = 0; i < n; i++) qvec[(size_t)q * n + i] = v[i];
    }
    for (int m = 0; m < nm; m++) {
        std::vector<double> v = QVec_Gaussian(mesh, &mp[(size_t)m * dim], width);
        for (int i = 0; i < n; i++) mvec[(size_t)m * n + i] = v[i] * c2a[i];
    }
    TFwdSolver<T> FWS(&mesh, std::is_same<T, double>::value ? "CG" : "BICGSTAB", 1e-12);
    FWS.SetPrecon(PRECON_ICH);
    FWS.SetDataScaling(DATA_LOG);
    FWS.Allocate();
    FWS.Reset(cmua, ckap, c2a, omega);
    std::vector<T> dphi((size_t)nq * n), aphi((size_t)nm * n);
    IterativeSolverResult res;
    FWS.CalcFields(nq, qvec.data(), dphi.data(), &res);
    FWS.CalcFields(nm, mvec.data(), aphi.data(), &res);
    Links L = Links::all_to_all(nq, nm);
    std::vector<T> proj = FWS.ProjectAll(nm, mvec.data(), nq, dphi.data(), L, DATA_LIN);
    std::vector<T> lproj = FWS.ProjectAll(nm, mvec.data(), nq, dphi.data(), L, DATA_LOG);
    const int cols = std::is_same<T, double>::value ? n : 2 * n;
    std::vector<double> J((size_t)2 * L.nQM() * cols);
    GenerateJacobian(FWS, nq, dphi.data(), nm, aphi.data(), proj.data(), L, DATA_LOG, J.data());
    const int bdim[3] = {12, 12, 12};
    Raster_Pixel raster(bdim, mesh);
    const int gcols = std::is_same<T, double>::value ? raster.SLen() : 2 * raster.SLen();
    std::vector<double> Jg((size_t)2 * L.nQM() * gcols);
    GenerateJacobian(raster, FWS, nq, dphi.data(), nm, aphi.data(), proj.data(), L, DATA_LOG, Jg.data());
    fwrite(lproj.data(), sizeof(T), lproj.size(), out);
    fwrite(J.data(), sizeof(double), J.size(), out);
    fwrite(Jg.data(), sizeof(double), Jg.size(), out);
    return 0;
}

static int qm_main(const char* meshf, const char* qmf, const char* outf)
{
    Mesh mesh(meshf);
    QMData qm = LoadQM(mesh, qmf);
    FILE* o = fopen(outf, "wb");
    if (!o) return 2;
    const int hdr[4] = {qm.dim, qm.nQ, qm.nM, qm.nQM};
    fwrite(hdr, sizeof(int), 4, o);
    fwrite(qm.Q.data(), sizeof(double), qm.Q.size(), o);
    fwrite(qm.M.data(), sizeof(double), qm.M.size(), o);
    fwrite(qm.links.ofs.data(), sizeof(int), qm.links.ofs.size(), o);
    fwrite(qm.links.m.data(), sizeof(int), qm.links.m.size(), o);
    fclose(o);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc == 5 && std::string(argv[1]) == "qm") return qm_main(argv[2], argv[3], argv[4]);
    if (argc != 3) { fprintf(stderr, "usage: fwd_shim IN OUT | fwd_shim qm MESH QMFILE OUT\n"); return 2; }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[6];
    double fw[2];
    if (fread(hdr, sizeof(int), 6, f) != 6 || fread(fw, sizeof(double), 2, f) != 2) return 2;
    const int dim = hdr[0], n = hdr[1], ne = hdr[2], nq = hdr[3], nm = hdr[4], cplx = hdr[5];
    std::vector<double> xy((size_t)n * dim), prm((size_t)3 * n), qp((size_t)nq * dim), mp((size_t)nm * dim);
    std::vector<int> el((size_t)ne * (dim + 1));
    bool ok = fread(xy.data(), sizeof(double), xy.size(), f) == xy.size() &&
              fread(el.data(), sizeof(int), el.size(), f) == el.size() &&
              fread(prm.data(), sizeof(double), prm.size(), f) == prm.size() &&
              fread(qp.data(), sizeof(double), qp.size(), f) == qp.size() &&
              fread(mp.data(), sizeof(double), mp.size(), f) == mp.size();
    fclose(f);
    if (!ok) return 2;
    FILE* out = fopen(argv[2], "wb");
    if (!out) return 2;
    const double omega = fw[0] * 2.0 * M_PI * 1e-6;
    int rc;
    try {
        rc = cplx ? run<std::complex<double>>(dim, n, nq, nm, omega, fw[1], xy, el, ne, prm, qp, mp, out)
                  : run<double>(dim, n, nq, nm, 0.0, fw[1], xy, el, ne, prm, qp, mp, out);
    } catch (const Error& e) {
        fprintf(stderr, "%s\n", e.what());
        rc = 1;
    }
    fclose(out);
    return rc;
}
