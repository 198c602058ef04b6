// ref_driver.cc -- runs the reference's own forward path (compiled from the
// reference tree by oracle/Makefile.ref) on one problem and writes the results
// as raw little-endian binary, so that the oracle restatement and the GPU path
// can be compared against the reference itself.
//
// The call sequence mirrors the reference's own callers:
//   src/supertoast/fwdfem.cc:56-250        (fields + ProjectAll, LOG data)
//   src/python/toastmodule.cc:1514-1574    (CalcJacobian, complex)
//   src/python/toastmodule.cc:1630-1684    (CalcJacobianCW, real)
//   src/python/toastmodule.cc:1189-1220    (measurement vectors scaled by c2a)
//
// Usage (key=value arguments):
//   ref_driver mesh=M.msh (qm=F.qm | optodes=O.bin) out=PREFIX
//              dtype=real|complex solver=CG|BICGSTAB|GMRES precon=NONE|DIAG|ICH
//              tol=1e-10 maxit=0 freq=100 qwidth=2 mwidth=2 nth=1
//              (params=P.bin | mua=0.025 mus=2 nref=1.4) jac=0|1 fields=0|1
//              sysmat=0|1 qsub=0 msub=0 grid=NX,NY[,NZ]
// optodes.bin: int32 dim,nQ,nM ; nQ*dim doubles ; nM*dim doubles (all-to-all links)
// params.bin : n*3 doubles, node-major (mua, mus', nref)
// qsub/msub  : if >0, only the first qsub sources / msub detectors are solved
//              (bounded CPU baseline samples); the Jacobian is then skipped.
// elparams   : E.bin, ne*3 doubles (mua, mus', nref per element): Reset in
//              the element basis (Reset(sol, omega, true), fwdsolver.cc:467-505)
//              and the element-basis Jacobian (GenerateJacobian(RASTER_ELBASIS,
//              ...), jacobian.cc:441-497; CW 738-802), PREFIX_Jel.bin; the
//              nodal params still give c2a for the detector vectors
// gradient   : with grid, data=D.bin and sd=S.bin (2 nQM doubles each: log
//              amplitude then phase), also the data gradient of toast's
//              Gradient (GetGradient / AddDataGradient,
//              src/python/toastmodule.cc:1745-1887) on the raster, run as that
//              code runs it with this library's calls: PREFIX_grad.bin
// grid       : also the grid-basis Jacobian for Raster_Pixel(bdim = grid,
//              gdim) (src/python/toastmodule.cc:696, raster_px.cc:10-48),
//              LOG data, written with the raster's element reference per grid
//              point (PREFIX_Jgrid.bin, PREFIX_elref.bin).  gdim=NX,NY[,NZ]
//              gives the intermediate grid (default: the basis grid); with
//              it the solution points' basis indices (PREFIX_sol2basis.bin)
//              and the maps through the basis are written too.  raster=cubic
//              builds a Raster_CubicPixel(bdim, gdim) instead, raster=gauss
//              (sigma=, sup=), hanning, ramp or spline (sup=) a blob basis;
//              the raster's own grid size is written (PREFIX_rgdim.bin).
// qmdump     : with qm, write what QMMesh::LoadQM (qmmesh.cc:319-460, with
//              InitM's detector placement) made of the file and stop:
//              PREFIX_qpos.bin, PREFIX_mpos.bin (nQ / nM x dim doubles),
//              PREFIX_nqmref.bin (nQ int32), PREFIX_qmref.bin (nQM int32)
#include "stoastlib.h"
#include <fstream>
#include <iostream>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

using namespace std;

static map<string, string> g_args;
static string arg(const char* k, const char* def) {
    auto it = g_args.find(k);
    return it == g_args.end() ? string(def) : it->second;
}

static void wbin(const string& fn, const void* p, size_t bytes) {
    FILE* f = fopen(fn.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", fn.c_str()); exit(2); }
    if (bytes) fwrite(p, 1, bytes, f);
    fclose(f);
}

static std::vector<char> rbin(const string& fn) {
    FILE* f = fopen(fn.c_str(), "rb");
    if (!f) { fprintf(stderr, "cannot read %s\n", fn.c_str()); exit(2); }
    fseek(f, 0, SEEK_END); long sz = ftell(f); fseek(f, 0, SEEK_SET);
    std::vector<char> buf(sz);
    if (sz && fread(buf.data(), 1, sz, f) != (size_t)sz) exit(2);
    fclose(f);
    return buf;
}

// Sets the QMMesh link tables for all-to-all links without LoadQM (positions
// are used exactly as given; InitM is not run because nothing on the path
// reads Mel/Mcosingder).
static void setup_optodes(QMMesh& mesh, const string& fn) {
    std::vector<char> b = rbin(fn);
    const int* hdr = (const int*)b.data();
    int dim = hdr[0], nq = hdr[1], nm = hdr[2];
    const double* xy = (const double*)(b.data() + 3 * sizeof(int));
    mesh.nQ = nq; mesh.nM = nm;
    mesh.Q = new Point[nq]; mesh.M = new Point[nm];
    for (int i = 0; i < nq; i++) { mesh.Q[i].New(dim); for (int d = 0; d < dim; d++) mesh.Q[i][d] = xy[i * dim + d]; }
    for (int i = 0; i < nm; i++) { mesh.M[i].New(dim); for (int d = 0; d < dim; d++) mesh.M[i][d] = xy[(nq + i) * dim + d]; }
    mesh.nQMref = new int[nq]; mesh.Qofs = new int[nq];
    mesh.QMref = new int*[nq]; mesh.QMofs = new int*[nq];
    for (int q = 0; q < nq; q++) {
        mesh.nQMref[q] = nm;
        mesh.Qofs[q] = q * nm;
        mesh.QMref[q] = new int[nm];
        mesh.QMofs[q] = new int[nm];
        for (int m = 0; m < nm; m++) { mesh.QMref[q][m] = m; mesh.QMofs[q][m] = q * nm + m; }
    }
    mesh.nQM = nq * nm;
}

template <class T> static const double* rawd(const TVector<T>& v) {
    return (const double*)v.data_buffer();
}

// The raster's basis maps (toast.Raster.Map, src/python/toastmodule.cc:
// 718-790) of a nodal field (mua) and of a solution-basis vector (s + 1 at
// solution point s): PREFIX_m2g.bin (mesh -> grid), _m2s.bin (mesh ->
// solution), _s2m.bin (solution -> mesh), _g2m.bin (grid -> mesh, the grid
// vector being the mesh -> grid map of mua)
static void write_maps(Raster& raster, const RVector& mua, const string& out)
{
    const int glen = raster.GLen(), slen = raster.SLen(), n = mua.Dim();
    RVector g(glen), sv(slen), m(n), sin(slen);
    raster.Map_MeshToGrid(mua, g);
    wbin(out + "_m2g.bin", g.data_buffer(), glen * sizeof(double));
    raster.Map_MeshToSol(mua, sv);
    wbin(out + "_m2s.bin", sv.data_buffer(), slen * sizeof(double));
    for (int i = 0; i < slen; i++) sin[i] = i + 1.0;
    raster.Map_SolToMesh(sin, m);
    wbin(out + "_s2m.bin", m.data_buffer(), n * sizeof(double));
    raster.Map_GridToMesh(g, m);
    wbin(out + "_g2m.bin", m.data_buffer(), n * sizeof(double));
}

// With an intermediate grid (gdim != bdim): the maps through the basis
// (toast.Raster.Map "M->B", "B->M", "G->B", "B->G", "G->S", "S->G", and the
// complex "M->S" / "S->M", which the pixel raster runs through the grid,
// raster.cc:236-270, 374-408): PREFIX_m2b, _b2m (basis vector b + 1 at basis
// point b), _g2b (of the grid image of mua), _b2g, _g2s, _s2g (s + 1), and
// _cm2s, _cs2m (mua + i mus'-like second field, interleaved complex)
static void write_basis_maps(Raster& raster, const RVector& mua, const RVector& mus, const string& out)
{
    const int glen = raster.GLen(), blen = raster.BLen(), slen = raster.SLen(), n = mua.Dim();
    RVector g(glen), b(blen), m(n), sv(slen), bin(blen), sin(slen);
    raster.Map_MeshToBasis(mua, b);
    wbin(out + "_m2b.bin", b.data_buffer(), blen * sizeof(double));
    for (int i = 0; i < blen; i++) bin[i] = i + 1.0;
    raster.Map_BasisToMesh(bin, m);
    wbin(out + "_b2m.bin", m.data_buffer(), n * sizeof(double));
    raster.Map_MeshToGrid(mua, g);
    raster.Map_GridToBasis(g, b);
    wbin(out + "_g2b.bin", b.data_buffer(), blen * sizeof(double));
    raster.Map_BasisToGrid(bin, g);
    wbin(out + "_b2g.bin", g.data_buffer(), glen * sizeof(double));
    raster.Map_MeshToGrid(mua, g);
    raster.Map_GridToSol(g, sv);
    wbin(out + "_g2s.bin", sv.data_buffer(), slen * sizeof(double));
    for (int i = 0; i < slen; i++) sin[i] = i + 1.0;
    raster.Map_SolToGrid(sin, g);
    wbin(out + "_s2g.bin", g.data_buffer(), glen * sizeof(double));
    CVector cm(n), cs(slen), cmo(n);
    for (int i = 0; i < n; i++) cm[i] = std::complex<double>(mua[i], mus[i]);
    raster.Map_MeshToSol(cm, cs);
    wbin(out + "_cm2s.bin", (const double*)cs.data_buffer(), slen * 2 * sizeof(double));
    for (int i = 0; i < slen; i++) cs[i] = std::complex<double>(i + 1.0, -0.5 * i);
    raster.Map_SolToMesh(cs, cmo);
    wbin(out + "_cs2m.bin", (const double*)cmo.data_buffer(), n * 2 * sizeof(double));
    std::vector<int> s2b(slen);
    for (int i = 0; i < slen; i++) s2b[i] = raster.Sol2Basis(i);
    wbin(out + "_sol2basis.bin", s2b.data(), slen * sizeof(int));
    // the raster's own grid and basis sizes (a blob basis pads both)
    std::vector<int> dims;
    for (int d = 0; d < raster.Dim(); d++) dims.push_back(raster.GDim()[d]);
    for (int d = 0; d < raster.Dim(); d++) dims.push_back(raster.BDim()[d]);
    wbin(out + "_rgdim.bin", dims.data(), dims.size() * sizeof(int));
}

// The data gradient on a raster, in the sequence of toast's GetGradient /
// AddDataGradient (src/python/toastmodule.cc:1745-1843), with the model data
// from ProjectAll_real (LOG: log amplitude, phase) of the fields already
// solved: per source, weights from the data residuals, one adjoint solve of
// the weighted detector vectors, then the products of the two fields and of
// their image gradients on the grid, subtracted into the gradient.
static void ref_data_gradient(QMMesh& mesh, Raster& raster, CFwdSolver& FWS, const RVector& data, const RVector& sd,
                              CVector* dphi, const CCompRowMatrix& mvec, RVector& grad)
{
    const int glen = raster.GLen(), slen = raster.SLen(), dim = raster.Dim(), nQM = mesh.nQM;
    RVector proj = FWS.ProjectAll_real(mvec, dphi, DATA_LOG);
    RVector gmua(grad, 0, slen), gkap(grad, slen, slen);
    int omod = 0, oarg = nQM;
    for (int q = 0; q < mesh.nQ; q++) {
        CVector df(glen);
        CVector* dg = new CVector[dim];
        raster.Map_MeshToGrid(dphi[q], df);
        ImageGradient(raster.GDim(), raster.GSize(), df, dg, raster.Elref());
        const int nl = mesh.nQMref[q];
        CVector cp = ProjectSingle(&mesh, q, mvec, dphi[q]);
        CVector w(mesh.nlen());
        for (int m = 0, k = 0; m < mesh.nM; m++) {
            if (!mesh.Connected(q, m)) continue;
            const CVector row = mvec.Row(m);
            const double rp = cp[k].real(), ip = cp[k].imag(), dn = 1.0 / (rp * rp + ip * ip);
            const double bm = (data[omod + k] - proj[omod + k]) / sd[omod + k];
            const double ba = (data[oarg + k] - proj[oarg + k]) / sd[oarg + k];
            double t = -2.0 * bm / (1.0 * sd[omod + k]);
            w += row * std::complex<double>(t * rp * dn, -t * ip * dn);
            t = -2.0 * ba / (1.0 * sd[oarg + k]);
            w += row * std::complex<double>(-t * ip * dn, -t * rp * dn);
            k++;
        }
        CVector wa(mesh.nlen());
        FWS.CalcField(w, wa);
        CVector af(glen);
        CVector* ag = new CVector[dim];
        raster.Map_MeshToGrid(wa, af);
        ImageGradient(raster.GDim(), raster.GSize(), af, ag, raster.Elref());
        CVector dgr(slen);
        raster.Map_GridToSol(df * af, dgr);
        gmua -= Re(dgr);
        CVector gk(glen);
        for (int i = 0; i < glen; i++)
            for (int d = 0; d < dim; d++) gk[i] += dg[d][i] * ag[d][i];
        raster.Map_GridToSol(gk, dgr);
        gkap -= Re(dgr);
        delete[] dg;
        delete[] ag;
        omod += nl;
        oarg += nl;
    }
}

// the raster of the grid arguments: Raster_Pixel, or with raster=cubic
// Raster_CubicPixel (raster_cp.cc), raster=gauss|hanning|ramp|spline the
// blob bases (raster_gb.cc, raster_hb.cc, raster_rb.cc, raster_sb.cc) of
// support radius sup (and width sigma for gauss)
static Raster* make_raster(const IVector& bdim, const IVector& gdim, QMMesh& mesh)
{
    const string kind = arg("raster", "pixel");
    const double sup = atof(arg("sup", "2").c_str());
    if (kind == "cubic") return new Raster_CubicPixel(bdim, gdim, &mesh);
    if (kind == "gauss") return new Raster_GaussBlob(bdim, gdim, &mesh, atof(arg("sigma", "1").c_str()), sup);
    if (kind == "hanning") return new Raster_HanningBlob(bdim, gdim, &mesh, sup);
    if (kind == "ramp") return new Raster_RampBlob(bdim, gdim, &mesh, sup);
    if (kind == "spline") return new Raster_SplineBlob(bdim, gdim, &mesh, sup);
    return new Raster_Pixel(bdim, gdim, &mesh);
}

int main(int argc, char** argv) {
    for (int i = 1; i < argc; i++) {
        const char* eq = strchr(argv[i], '=');
        if (!eq) { fprintf(stderr, "bad arg %s\n", argv[i]); return 2; }
        g_args[string(argv[i], eq - argv[i])] = string(eq + 1);
    }
    const double c0 = 0.3;
    string out = arg("out", "ref");
    bool cplx = arg("dtype", "complex") == "complex";
    string solver = arg("solver", cplx ? "BICGSTAB" : "CG");
    string precon = arg("precon", "ICH");
    double tol = atof(arg("tol", "1e-10").c_str());
    int maxit = atoi(arg("maxit", "0").c_str());
    double freq = atof(arg("freq", cplx ? "100" : "0").c_str());
    double qwidth = atof(arg("qwidth", "2").c_str());
    double mwidth = atof(arg("mwidth", "2").c_str());
    int nth = atoi(arg("nth", "1").c_str());
    bool want_jac = atoi(arg("jac", "0").c_str()) != 0;
    bool want_fields = atoi(arg("fields", "0").c_str()) != 0;
    bool want_sys = atoi(arg("sysmat", "0").c_str()) != 0;
    int qsub = atoi(arg("qsub", "0").c_str());
    std::vector<int> grid;
    {
        string g = arg("grid", "");
        for (size_t a = 0; a < g.size();) {
            size_t b = g.find(',', a);
            if (b == string::npos) b = g.size();
            grid.push_back(atoi(g.substr(a, b - a).c_str()));
            a = b + 1;
        }
    }
    int msub = atoi(arg("msub", "0").c_str());
    std::vector<int> igrid;  // intermediate grid; empty: the basis grid
    {
        string g = arg("gdim", "");
        for (size_t a = 0; a < g.size();) {
            size_t b = g.find(',', a);
            if (b == string::npos) b = g.size();
            igrid.push_back(atoi(g.substr(a, b - a).c_str()));
            a = b + 1;
        }
    }

    Task_Init(nth);
    toastVerbosity = 0;

    QMMesh mesh;
    {
        ifstream ifs(arg("mesh", "").c_str());
        ifs >> mesh;
        mesh.Setup();
    }
    if (g_args.count("qm")) {
        ifstream ifs(arg("qm", "").c_str());
        mesh.LoadQM(ifs);
        if (atoi(arg("qmdump", "0").c_str())) {
            const int d = mesh.Dimension();
            std::vector<double> qp, mp;
            for (int i = 0; i < mesh.nQ; i++) for (int k = 0; k < d; k++) qp.push_back(mesh.Q[i][k]);
            for (int i = 0; i < mesh.nM; i++) for (int k = 0; k < d; k++) mp.push_back(mesh.M[i][k]);
            std::vector<int> nref(mesh.nQMref, mesh.nQMref + mesh.nQ), ref;
            for (int i = 0; i < mesh.nQ; i++) for (int j = 0; j < mesh.nQMref[i]; j++) ref.push_back(mesh.QMref[i][j]);
            string out = arg("out", "ref");
            wbin(out + "_qpos.bin", qp.data(), qp.size() * sizeof(double));
            wbin(out + "_mpos.bin", mp.data(), mp.size() * sizeof(double));
            wbin(out + "_nqmref.bin", nref.data(), nref.size() * sizeof(int));
            wbin(out + "_qmref.bin", ref.data(), ref.size() * sizeof(int));
            return 0;
        }
    } else {
        setup_optodes(mesh, arg("optodes", ""));
    }
    int n = mesh.nlen(), nQ = mesh.nQ, nM = mesh.nM, nQM = mesh.nQM;
    int dim = mesh.Dimension();

    RVector mua(n), mus(n), ref(n);
    if (g_args.count("params")) {
        std::vector<char> b = rbin(arg("params", ""));
        const double* p = (const double*)b.data();
        for (int i = 0; i < n; i++) { mua[i] = p[3 * i]; mus[i] = p[3 * i + 1]; ref[i] = p[3 * i + 2]; }
    } else {
        mua = atof(arg("mua", "0.025").c_str());
        mus = atof(arg("mus", "2").c_str());
        ref = atof(arg("nref", "1.4").c_str());
    }
    Solution msol(OT_NPARAM, n);
    msol.SetParam(OT_CMUA, mua * c0 / ref);
    msol.SetParam(OT_CKAPPA, c0 / (3.0 * ref * (mua + mus)));
    msol.SetParam(OT_N, ref);
    RVector c2a(n);
    for (int i = 0; i < n; i++) c2a[i] = c0 / (2.0 * ref[i] * A_Keijzer(ref[i]));
    msol.SetParam(OT_C2A, c2a);
    double omega = freq * 2.0 * Pi * 1e-6;
    const bool elbasis = g_args.count("elparams") > 0;
    const int ne = mesh.elen();
    Solution msol_el(OT_NPARAM, elbasis ? ne : 1);
    if (elbasis) {
        std::vector<char> b = rbin(arg("elparams", ""));
        const double* p = (const double*)b.data();
        RVector emua(ne), emus(ne), eref(ne), ec2a(ne);
        for (int e = 0; e < ne; e++) { emua[e] = p[3 * e]; emus[e] = p[3 * e + 1]; eref[e] = p[3 * e + 2]; }
        for (int e = 0; e < ne; e++) ec2a[e] = c0 / (2.0 * eref[e] * A_Keijzer(eref[e]));
        msol_el.SetParam(OT_CMUA, emua * c0 / eref);
        msol_el.SetParam(OT_CKAPPA, c0 / (3.0 * eref * (emua + emus)));
        msol_el.SetParam(OT_N, eref);
        msol_el.SetParam(OT_C2A, ec2a);
    }

    // detector positions as used (after LoadQM/InitM pulled them to the boundary)
    {
        std::vector<double> optpos;
        for (int i = 0; i < nQ; i++) for (int d = 0; d < dim; d++) optpos.push_back(mesh.Q[i][d]);
        for (int i = 0; i < nM; i++) for (int d = 0; d < dim; d++) optpos.push_back(mesh.M[i][d]);
        wbin(out + "_optodes.bin", optpos.data(), optpos.size() * sizeof(double));
    }

    PreconType pt = precon == "ICH" ? PRECON_ICH : precon == "DIAG" ? PRECON_DIAG
                  : precon == "DILU" ? PRECON_DILU : PRECON_NULL;
    int nq_solve = qsub > 0 ? min(qsub, nQ) : nQ;
    int nm_solve = msub > 0 ? min(msub, nM) : nM;
    bool sampled = qsub > 0 || msub > 0;

    FILE* info = fopen((out + "_info.txt").c_str(), "w");
    fprintf(info, "n %d\nnQ %d\nnM %d\nnQM %d\ndim %d\nelen %d\n", n, nQ, nM, nQM, dim, mesh.elen());

    if (cplx) {
        CCompRowMatrix qvec(nQ, n), mvec(nM, n);
        for (int i = 0; i < nQ; i++) {
            CVector q(n);
            SetReal(q, QVec_Gaussian(mesh, mesh.Q[i], qwidth, SRCMODE_NEUMANN));
            qvec.SetRow(i, q);
        }
        for (int i = 0; i < nM; i++) {
            CVector m(n);
            SetReal(m, QVec_Gaussian(mesh, mesh.M[i], mwidth, SRCMODE_NEUMANN) * c2a);
            mvec.SetRow(i, m);
        }
        CFwdSolver FWS(&mesh, solver.c_str(), tol);
        FWS.SetPrecon(pt);
        FWS.SetLinSolverMaxit(maxit);
        FWS.SetDataScaling(DATA_LOG);
        FWS.Allocate();
        double t0 = walltic();
        if (elbasis) FWS.Reset(msol_el, omega, true);
        else FWS.Reset(msol, omega);
        fprintf(info, "t_reset %.9g\n", walltoc(t0));
        if (want_sys) {
            const CCompRowMatrix& F = *FWS.F;
            wbin(out + "_rowptr.bin", F.rowptr, (n + 1) * sizeof(int));
            wbin(out + "_colidx.bin", F.colidx, F.nVal() * sizeof(int));
            wbin(out + "_sysval.bin", F.ValPtr(), F.nVal() * sizeof(std::complex<double>));
        }
        CVector* dphi = new CVector[nQ];
        CVector* aphi = new CVector[nM];
        for (int i = 0; i < nQ; i++) dphi[i].New(n);
        for (int i = 0; i < nM; i++) aphi[i].New(n);
        IterativeSolverResult res;
        CCompRowMatrix qs(nq_solve, n), ms(nm_solve, n);
        for (int i = 0; i < nq_solve; i++) qs.SetRow(i, qvec.Row(i));
        for (int i = 0; i < nm_solve; i++) ms.SetRow(i, mvec.Row(i));
        t0 = walltic();
        FWS.CalcFields(qs, dphi, &res);
        fprintf(info, "t_fwd %.9g\nit_fwd %d\nerr_fwd %.6g\n", walltoc(t0), res.it_count, res.rel_err);
        t0 = walltic();
        FWS.CalcFields(ms, aphi, &res);
        fprintf(info, "t_adj %.9g\nit_adj %d\nerr_adj %.6g\n", walltoc(t0), res.it_count, res.rel_err);
        if (!sampled) {
            t0 = walltic();
            CVector proj = FWS.ProjectAll(mvec, dphi, DATA_LIN);
            CVector lproj = FWS.ProjectAll(mvec, dphi, DATA_LOG);
            fprintf(info, "t_proj %.9g\n", walltoc(t0));
            wbin(out + "_proj.bin", rawd(proj), nQM * sizeof(std::complex<double>));
            wbin(out + "_logproj.bin", rawd(lproj), nQM * sizeof(std::complex<double>));
            if (want_jac) {
                RDenseMatrix J(2 * nQM, 2 * n);
                t0 = walltic();
                GenerateJacobian(0, &mesh, dphi, aphi, &proj, DATA_LOG, J);
                fprintf(info, "t_jac %.9g\n", walltoc(t0));
                wbin(out + "_J.bin", J.ValPtr(), (size_t)2 * nQM * 2 * n * sizeof(double));
            }
            if (elbasis) {
                RDenseMatrix Je(2 * nQM, 2 * ne);
                GenerateJacobian(RASTER_ELBASIS, &mesh, dphi, aphi, &proj, DATA_LOG, Je);
                wbin(out + "_Jel.bin", Je.ValPtr(), (size_t)2 * nQM * 2 * ne * sizeof(double));
            }
            if ((int)grid.size() == dim) {
                IVector bdim(dim, grid.data());
                IVector gdim(dim, ((int)igrid.size() == dim ? igrid : grid).data());
                std::unique_ptr<Raster> rowner(make_raster(bdim, gdim, mesh));
                Raster& raster = *rowner;
                int slen = raster.SLen(), glen = raster.GLen();
                RDenseMatrix Jg(2 * nQM, 2 * slen);
                GenerateJacobian(&raster, &mesh, dphi, aphi, &proj, DATA_LOG, Jg);
                wbin(out + "_Jgrid.bin", Jg.ValPtr(), (size_t)2 * nQM * 2 * slen * sizeof(double));
                wbin(out + "_elref.bin", raster.Elref(), (size_t)glen * sizeof(int));
                fprintf(info, "slen %d\nglen %d\n", slen, glen);
                write_maps(raster, mua, out);
                if ((int)igrid.size() == dim || arg("raster", "pixel") != "pixel")
                    write_basis_maps(raster, mua, mus, out);
                if (g_args.count("data")) {
                    std::vector<char> db = rbin(arg("data", "")), sb = rbin(arg("sd", ""));
                    RVector data(2 * nQM, (double*)db.data()), sd(2 * nQM, (double*)sb.data());
                    RVector grad(2 * slen);
                    ref_data_gradient(mesh, raster, FWS, data, sd, dphi, mvec, grad);
                    wbin(out + "_grad.bin", grad.data_buffer(), (size_t)2 * slen * sizeof(double));
                }
            }
        }
        if (want_fields) {
            FILE* f = fopen((out + "_dphi.bin").c_str(), "wb");
            for (int i = 0; i < nq_solve; i++) fwrite(rawd(dphi[i]), sizeof(std::complex<double>), n, f);
            fclose(f);
            f = fopen((out + "_aphi.bin").c_str(), "wb");
            for (int i = 0; i < nm_solve; i++) fwrite(rawd(aphi[i]), sizeof(std::complex<double>), n, f);
            fclose(f);
        }
        delete[] dphi;
        delete[] aphi;
    } else {
        RCompRowMatrix qvec(nQ, n), mvec(nM, n);
        for (int i = 0; i < nQ; i++) qvec.SetRow(i, QVec_Gaussian(mesh, mesh.Q[i], qwidth, SRCMODE_NEUMANN));
        for (int i = 0; i < nM; i++) mvec.SetRow(i, QVec_Gaussian(mesh, mesh.M[i], mwidth, SRCMODE_NEUMANN) * c2a);
        RFwdSolver FWS(&mesh, solver.c_str(), tol);
        FWS.SetPrecon(pt);
        FWS.SetLinSolverMaxit(maxit);
        FWS.SetDataScaling(DATA_LOG);
        FWS.Allocate();
        double t0 = walltic();
        if (elbasis) FWS.Reset(msol_el, 0, true);
        else FWS.Reset(msol, 0);
        fprintf(info, "t_reset %.9g\n", walltoc(t0));
        if (want_sys) {
            const RCompRowMatrix& F = *FWS.F;
            wbin(out + "_rowptr.bin", F.rowptr, (n + 1) * sizeof(int));
            wbin(out + "_colidx.bin", F.colidx, F.nVal() * sizeof(int));
            wbin(out + "_sysval.bin", F.ValPtr(), F.nVal() * sizeof(double));
        }
        RVector* dphi = new RVector[nQ];
        RVector* aphi = new RVector[nM];
        for (int i = 0; i < nQ; i++) dphi[i].New(n);
        for (int i = 0; i < nM; i++) aphi[i].New(n);
        IterativeSolverResult res;
        RCompRowMatrix qs(nq_solve, n), ms(nm_solve, n);
        for (int i = 0; i < nq_solve; i++) qs.SetRow(i, qvec.Row(i));
        for (int i = 0; i < nm_solve; i++) ms.SetRow(i, mvec.Row(i));
        t0 = walltic();
        FWS.CalcFields(qs, dphi, &res);
        fprintf(info, "t_fwd %.9g\nit_fwd %d\nerr_fwd %.6g\n", walltoc(t0), res.it_count, res.rel_err);
        t0 = walltic();
        FWS.CalcFields(ms, aphi, &res);
        fprintf(info, "t_adj %.9g\nit_adj %d\nerr_adj %.6g\n", walltoc(t0), res.it_count, res.rel_err);
        if (!sampled) {
            t0 = walltic();
            RVector proj = FWS.ProjectAll(mvec, dphi, DATA_LIN);
            RVector lproj = FWS.ProjectAll(mvec, dphi, DATA_LOG);
            fprintf(info, "t_proj %.9g\n", walltoc(t0));
            wbin(out + "_proj.bin", rawd(proj), nQM * sizeof(double));
            wbin(out + "_logproj.bin", rawd(lproj), nQM * sizeof(double));
            if (want_jac) {
                RDenseMatrix Jmua, Jkap;
                t0 = walltic();
                GenerateJacobian_cw(0, &mesh, mvec, dphi, aphi, DATA_LOG, &Jmua, &Jkap);
                fprintf(info, "t_jac %.9g\n", walltoc(t0));
                FILE* f = fopen((out + "_J.bin").c_str(), "wb");
                fwrite(Jmua.ValPtr(), sizeof(double), (size_t)nQM * n, f);
                fwrite(Jkap.ValPtr(), sizeof(double), (size_t)nQM * n, f);
                fclose(f);
            }
            if (elbasis) {
                RDenseMatrix Jmua, Jkap;
                GenerateJacobian_cw(RASTER_ELBASIS, &mesh, dphi, aphi, &proj, DATA_LOG, &Jmua, &Jkap);
                FILE* f = fopen((out + "_Jel.bin").c_str(), "wb");
                fwrite(Jmua.ValPtr(), sizeof(double), (size_t)nQM * ne, f);
                fwrite(Jkap.ValPtr(), sizeof(double), (size_t)nQM * ne, f);
                fclose(f);
            }
            if ((int)grid.size() == dim) {
                IVector bdim(dim, grid.data());
                IVector gdim(dim, ((int)igrid.size() == dim ? igrid : grid).data());
                std::unique_ptr<Raster> rowner(make_raster(bdim, gdim, mesh));
                Raster& raster = *rowner;
                int slen = raster.SLen(), glen = raster.GLen();
                RDenseMatrix Jmua, Jkap;
                GenerateJacobian_cw(&raster, &mesh, dphi, aphi, &proj, DATA_LOG, &Jmua, &Jkap);
                FILE* f = fopen((out + "_Jgrid.bin").c_str(), "wb");
                fwrite(Jmua.ValPtr(), sizeof(double), (size_t)nQM * slen, f);
                fwrite(Jkap.ValPtr(), sizeof(double), (size_t)nQM * slen, f);
                fclose(f);
                wbin(out + "_elref.bin", raster.Elref(), (size_t)glen * sizeof(int));
                fprintf(info, "slen %d\nglen %d\n", slen, glen);
                write_maps(raster, mua, out);
                if ((int)igrid.size() == dim || arg("raster", "pixel") != "pixel")
                    write_basis_maps(raster, mua, mus, out);
            }
        }
        if (want_fields) {
            FILE* f = fopen((out + "_dphi.bin").c_str(), "wb");
            for (int i = 0; i < nq_solve; i++) fwrite(rawd(dphi[i]), sizeof(double), n, f);
            fclose(f);
            f = fopen((out + "_aphi.bin").c_str(), "wb");
            for (int i = 0; i < nm_solve; i++) fwrite(rawd(aphi[i]), sizeof(double), n, f);
            fclose(f);
        }
        delete[] dphi;
        delete[] aphi;
    }
    fclose(info);
    return 0;
}
