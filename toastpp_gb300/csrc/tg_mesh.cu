// tg_mesh.cu -- per-mesh preprocessing and device upload.
//
// Follows the reference's mesh set-up: element geometry of Triangle3 /
// Tetrahedron4 (src/libfe/tri3.cc:79-119, tet4.cc:113-171), boundary sides =
// sides not shared by two elements (Mesh::MarkBoundary, mesh.cc:1614-1705),
// cached element integrals (element.cc:540-545), the CSR pattern of all node
// pairs sharing an element (Mesh::SparseRowStructure, mesh.cc:422-549) and the
// IC(0) pattern = strict lower part of that pattern
// (CalculateIncompleteCholeskyFillin, crmatrix_imp.hpp:2077-2102).
#include <algorithm>
#include <array>
#include <cstring>
#include <numeric>
#include "tg_mesh.cuh"

namespace tg {

static const int TRI_SIDE[3][2] = {{0, 1}, {1, 2}, {2, 0}};
static const int TET_SIDE[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};

static double dist(const double* a, const double* b, int dim)
{
    double s = 0.0;
    for (int i = 0; i < dim; i++) s += (a[i] - b[i]) * (a[i] - b[i]);
    return std::sqrt(s);
}

static void geometry(MeshHost& m)
{
    m.geo.assign((size_t)m.ne * 16, 0.0);
    m.rec.assign((size_t)m.ne * EL_REC, 0.0);
    for (int e = 0; e < m.ne; e++) {
        const int* nd = &m.el[(size_t)e * m.nn];
        double* g = &m.geo[(size_t)e * 16];
        double* r = &m.rec[(size_t)e * EL_REC];
        if (m.dim == 2) {
            const double *p0 = &m.coords[2 * nd[0]], *p1 = &m.coords[2 * nd[1]], *p2 = &m.coords[2 * nd[2]];
            double x0 = p0[0], y0 = p0[1], x1 = p1[0], y1 = p1[1], x2 = p2[0], y2 = p2[1];
            g[0] = x1 * y2 - x2 * y1; g[3] = y1 - y2; g[6] = x2 - x1;
            g[1] = x2 * y0 - x0 * y2; g[4] = y2 - y0; g[7] = x0 - x2;
            g[2] = x0 * y1 - x1 * y0; g[5] = y0 - y1; g[8] = x1 - x0;
            r[0] = 0.5 * (g[0] + g[1] + g[2]);
        } else {
            const double *p0 = &m.coords[3 * nd[0]], *p1 = &m.coords[3 * nd[1]];
            const double *p2 = &m.coords[3 * nd[2]], *p3 = &m.coords[3 * nd[3]];
            double x0 = p0[0], y0 = p0[1], z0 = p0[2], x1 = p1[0], y1 = p1[1], z1 = p1[2];
            double x2 = p2[0], y2 = p2[1], z2 = p2[2], x3 = p3[0], y3 = p3[1], z3 = p3[2];
            double *a = g, *b = g + 4, *c = g + 8, *d = g + 12;
            a[0] = x1*(y2*z3-y3*z2) - x2*(y1*z3-y3*z1) + x3*(y1*z2-y2*z1);
            a[1] = x0*(y3*z2-y2*z3) - x2*(y3*z0-y0*z3) + x3*(y2*z0-y0*z2);
            a[2] = x0*(y1*z3-y3*z1) - x1*(y0*z3-y3*z0) + x3*(y0*z1-y1*z0);
            a[3] = x0*(y2*z1-y1*z2) - x1*(y2*z0-y0*z2) + x2*(y1*z0-y0*z1);
            b[0] = y1*(z3-z2) + y2*(z1-z3) + y3*(z2-z1);
            b[1] = y0*(z2-z3) + y2*(z3-z0) + y3*(z0-z2);
            b[2] = y0*(z3-z1) + y1*(z0-z3) + y3*(z1-z0);
            b[3] = y0*(z1-z2) + y1*(z2-z0) + y2*(z0-z1);
            c[0] = x1*(z2-z3) + x2*(z3-z1) + x3*(z1-z2);
            c[1] = x0*(z3-z2) + x2*(z0-z3) + x3*(z2-z0);
            c[2] = x0*(z1-z3) + x1*(z3-z0) + x3*(z0-z1);
            c[3] = x0*(z2-z1) + x1*(z0-z2) + x2*(z1-z0);
            d[0] = x1*(y3-y2) + x2*(y1-y3) + x3*(y2-y1);
            d[1] = x0*(y2-y3) + x2*(y3-y0) + x3*(y0-y2);
            d[2] = x0*(y3-y1) + x1*(y0-y3) + x3*(y1-y0);
            d[3] = x0*(y1-y2) + x1*(y2-y0) + x2*(y0-y1);
            for (int s = 0; s < 4; s++) {  // face areas by Heron's formula (TriangleArea)
                const double* q1 = &m.coords[3 * nd[TET_SIDE[s][0]]];
                const double* q2 = &m.coords[3 * nd[TET_SIDE[s][1]]];
                const double* q3 = &m.coords[3 * nd[TET_SIDE[s][2]]];
                double aa = dist(q1, q2, 3), bb = dist(q2, q3, 3), cc = dist(q3, q1, 3);
                double sp = 0.5 * (aa + bb + cc);
                r[17 + s] = std::sqrt(sp * (sp - aa) * (sp - bb) * (sp - cc));
            }
            r[0] = (1.0 / 6.0) * (a[0] + a[1] + a[2] + a[3]);
        }
    }
}

static void mark_boundary(MeshHost& m)
{
    int nside = m.dim == 2 ? 3 : 4, nsn = m.dim == 2 ? 2 : 3;
    struct Side { std::array<int, 3> nd; int el, sd; };
    std::vector<Side> sides((size_t)m.ne * nside);
    for (int e = 0; e < m.ne; e++)
        for (int s = 0; s < nside; s++) {
            Side& x = sides[(size_t)e * nside + s];
            x.el = e; x.sd = s; x.nd = {-1, -1, -1};
            for (int k = 0; k < nsn; k++)
                x.nd[k] = m.el[(size_t)e * m.nn + (m.dim == 2 ? TRI_SIDE[s][k] : TET_SIDE[s][k])];
            std::sort(x.nd.begin(), x.nd.begin() + nsn);
        }
    std::sort(sides.begin(), sides.end(), [](const Side& a, const Side& b) { return a.nd < b.nd; });
    m.bndside.assign((size_t)m.ne * nside, 0);
    m.bndnode.assign(m.n, 0);
    for (size_t i = 0; i < sides.size(); i++) {
        bool b = true;
        if (i > 0 && sides[i].nd == sides[i - 1].nd) b = false;
        if (b && i + 1 < sides.size() && sides[i].nd == sides[i + 1].nd) b = false;
        if (!b) continue;
        m.bndside[(size_t)sides[i].el * nside + sides[i].sd] = 1;
        for (int k = 0; k < nsn; k++) m.bndnode[sides[i].nd[k]] = 1;
    }
}

static void element_records(MeshHost& m)
{
    int nn = m.nn;
    m.intbff.assign((size_t)m.ne * nn * nn, 0.0);
    static const int T[4][4][4] = {  // Tet4 boundary face mass tables (tet4.cc:1039-1068), x 2/24
        {{2,1,1,0},{1,2,1,0},{1,1,2,0},{0,0,0,0}},
        {{2,1,0,1},{1,2,0,1},{0,0,0,0},{1,1,0,2}},
        {{2,0,1,1},{0,0,0,0},{1,0,2,1},{1,0,1,2}},
        {{0,0,0,0},{0,2,1,1},{0,1,2,1},{0,1,1,2}}};
    for (int e = 0; e < m.ne; e++) {
        const double* g = &m.geo[(size_t)e * 16];
        double* r = &m.rec[(size_t)e * EL_REC];
        double* bff = &m.intbff[(size_t)e * nn * nn];
        double sz = r[0];
        const int* nd = &m.el[(size_t)e * nn];
        if (m.dim == 2) {
            const double *b = g + 3, *c = g + 6;
            double scale = 0.25 / sz;  // Triangle3::ComputeIntDD (tri3.cc:490-506)
            for (int i = 0; i < 3; i++)
                for (int j = 0; j <= i; j++) {
                    double v = scale * (b[i] * b[j] + c[i] * c[j]);
                    r[1 + i * 3 + j] = r[1 + j * 3 + i] = v;
                }
            for (int s = 0; s < 3; s++) {  // Triangle3::ComputeBndIntFF (tri3.cc:561-582)
                if (!m.bndside[(size_t)e * 3 + s]) continue;
                int n0 = TRI_SIDE[s][0], n1 = TRI_SIDE[s][1];
                double dx = m.coords[2 * nd[n0]] - m.coords[2 * nd[n1]];
                double dy = m.coords[2 * nd[n0] + 1] - m.coords[2 * nd[n1] + 1];
                double d = std::hypot(dx, dy);
                for (int i = 0; i < 3; i++) {
                    if (i != n0 && i != n1) continue;
                    bff[i * 3 + i] += d / 3.0;
                    for (int j = 0; j < i; j++)
                        if (j == n0 || j == n1) bff[i * 3 + j] += d / 6.0;
                }
            }
            for (int i = 0; i < 3; i++) for (int j = 0; j < i; j++) bff[j * 3 + i] = bff[i * 3 + j];
            for (int k = 0; k < 9; k++) r[10 + k] = bff[k];
        } else {
            const double *b = g + 4, *c = g + 8, *d = g + 12;
            double scale = 1.0 / (144.0 * sz);  // Tetrahedron4::IntFDD (tet4.cc:380-412)
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) {
                    int p = std::min(i, j), q = std::max(i, j);
                    r[1 + i * 4 + j] = (b[p] * b[q] + c[p] * c[q] + d[p] * d[q]) * scale;
                }
            int mask = 0;
            for (int s = 0; s < 4; s++) {
                if (!m.bndside[(size_t)e * 4 + s]) continue;
                mask |= 1 << s;
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 4; j++) bff[i * 4 + j] += (T[s][i][j] * (2.0 / 24.0)) * r[17 + s];
            }
            r[21] = (double)mask;
        }
    }
}

static void csr_pattern(MeshHost& m)
{
    std::vector<std::vector<int>> adj(m.n);
    for (int e = 0; e < m.ne; e++)
        for (int i = 0; i < m.nn; i++)
            for (int j = 0; j < m.nn; j++) adj[m.el[(size_t)e * m.nn + i]].push_back(m.el[(size_t)e * m.nn + j]);
    m.rowptr.assign(m.n + 1, 0);
    m.colidx.clear();
    m.diagpos.assign(m.n, -1);
    for (int i = 0; i < m.n; i++) {
        auto& a = adj[i];
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
        for (int c : a) {
            if (c == i) m.diagpos[i] = (int)m.colidx.size();
            m.colidx.push_back(c);
        }
        m.rowptr[i + 1] = (int)m.colidx.size();
    }
}

static int find_col(const std::vector<int>& rowptr, const std::vector<int>& colidx, int r, int c)
{
    auto b = colidx.begin() + rowptr[r], e = colidx.begin() + rowptr[r + 1];
    auto it = std::lower_bound(b, e, c);
    return (it != e && *it == c) ? (int)(it - colidx.begin()) : -1;
}

static void ic_pattern(MeshHost& m)
{
    int n = m.n;
    m.Lrowptr.assign(n + 1, 0);
    m.Lcolidx.clear();
    m.Lapos.clear();
    for (int i = 0; i < n; i++) {
        for (int k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
            if (m.colidx[k] >= i) break;
            m.Lcolidx.push_back(m.colidx[k]);
            m.Lapos.push_back(k);
        }
        m.Lrowptr[i + 1] = (int)m.Lcolidx.size();
    }
    int nl = m.Lrowptr[n];
    // column view: for column i, rows r > i ascending, with the L index
    m.Ucolptr.assign(n + 1, 0);
    for (int k = 0; k < nl; k++) m.Ucolptr[m.Lcolidx[k] + 1]++;
    for (int i = 0; i < n; i++) m.Ucolptr[i + 1] += m.Ucolptr[i];
    m.Urow.assign(nl, 0);
    m.Umap.assign(nl, 0);
    std::vector<int> fill(n, 0);
    for (int r = 0; r < n; r++)
        for (int k = m.Lrowptr[r]; k < m.Lrowptr[r + 1]; k++) {
            int c = m.Lcolidx[k], p = m.Ucolptr[c] + fill[c]++;
            m.Urow[p] = r;
            m.Umap[p] = k;
        }
    // level schedules: forward depth through L rows, backward through L columns
    std::vector<int> lev(n, 0), blev(n, 0);
    int nlf = 0, nlb = 0;
    for (int i = 0; i < n; i++) {
        int l = 0;
        for (int k = m.Lrowptr[i]; k < m.Lrowptr[i + 1]; k++) l = std::max(l, lev[m.Lcolidx[k]] + 1);
        lev[i] = l;
        nlf = std::max(nlf, l + 1);
    }
    for (int i = n - 1; i >= 0; i--) {
        int l = 0;
        for (int k = m.Ucolptr[i]; k < m.Ucolptr[i + 1]; k++) l = std::max(l, blev[m.Urow[k]] + 1);
        blev[i] = l;
        nlb = std::max(nlb, l + 1);
    }
    auto group = [n](const std::vector<int>& lv, int nlev, std::vector<int>& ptr, std::vector<int>& rows) {
        ptr.assign(nlev + 1, 0);
        for (int i = 0; i < n; i++) ptr[lv[i] + 1]++;
        for (int l = 0; l < nlev; l++) ptr[l + 1] += ptr[l];
        rows.assign(n, 0);
        std::vector<int> f(nlev, 0);
        for (int i = 0; i < n; i++) rows[ptr[lv[i]] + f[lv[i]]++] = i;
    };
    group(lev, nlf, m.fwd_lev_ptr, m.fwd_lev_rows);
    group(blev, nlb, m.bwd_lev_ptr, m.bwd_lev_rows);
}

static void gather_maps(MeshHost& m)
{
    int nnz = m.rowptr[m.n];
    std::vector<int> cnt(nnz + 1, 0);
    std::vector<int> slot((size_t)m.ne * m.nn * m.nn);
    for (int e = 0; e < m.ne; e++)
        for (int i = 0; i < m.nn; i++)
            for (int j = 0; j < m.nn; j++) {
                int k = find_col(m.rowptr, m.colidx, m.el[(size_t)e * m.nn + i], m.el[(size_t)e * m.nn + j]);
                slot[((size_t)e * m.nn + i) * m.nn + j] = k;
                cnt[k + 1]++;
            }
    for (int k = 0; k < nnz; k++) cnt[k + 1] += cnt[k];
    m.asm_ptr = cnt;
    m.asm_list.assign(cnt[nnz], 0);
    std::vector<int> f(nnz, 0);
    for (int e = 0; e < m.ne; e++)  // element order, as the reference assembles
        for (int i = 0; i < m.nn; i++)
            for (int j = 0; j < m.nn; j++) {
                int k = slot[((size_t)e * m.nn + i) * m.nn + j];
                m.asm_list[m.asm_ptr[k] + f[k]++] = e * 16 + i * 4 + j;
            }
    m.nel_ptr.assign(m.n + 1, 0);
    for (int e = 0; e < m.ne; e++)
        for (int i = 0; i < m.nn; i++) m.nel_ptr[m.el[(size_t)e * m.nn + i] + 1]++;
    for (int i = 0; i < m.n; i++) m.nel_ptr[i + 1] += m.nel_ptr[i];
    m.nel_list.assign(m.nel_ptr[m.n], 0);
    std::vector<int> g(m.n, 0);
    for (int e = 0; e < m.ne; e++)
        for (int i = 0; i < m.nn; i++) {
            int nd = m.el[(size_t)e * m.nn + i];
            m.nel_list[m.nel_ptr[nd] + g[nd]++] = e * 4 + i;
        }
}

template <class T>
static T* upload(const std::vector<T>& v)
{
    T* p = nullptr;
    size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
    if (cudaMalloc(&p, bytes) != cudaSuccess) throw Error{4, "cudaMalloc failed for mesh data"};
    if (!v.empty()) TG_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}

Mesh::~Mesh()
{
    void* ptrs[] = {d.rec, d.el, d.rowptr, d.colidx, d.diagpos, d.Lrowptr, d.Lcolidx, d.Lapos, d.Ucolptr,
                    d.Urow, d.Umap, d.fwd_lev_rows, d.bwd_lev_rows, d.asm_ptr, d.asm_list, d.nel_ptr,
                    d.nel_list, d.bndnode};
    for (void* p : ptrs) if (p) cudaFree(p);
}

Mesh* mesh_build(int dim, int n, const double* coords, int ne, const int* el)
{
    TG_CHECK(dim == 2 || dim == 3, 1, "dim must be 2 or 3");
    TG_CHECK(n > 0 && ne > 0 && coords && el, 1, "empty mesh");
    Mesh* M = new Mesh();
    MeshHost& m = M->h;
    m.dim = dim; m.n = n; m.ne = ne; m.nn = dim == 2 ? 3 : 4;
    m.coords.assign(coords, coords + (size_t)n * dim);
    m.el.assign(el, el + (size_t)ne * m.nn);
    for (int v : m.el)
        if (v < 0 || v >= n) { delete M; throw Error{1, "element node index out of range"}; }
    geometry(m);
    mark_boundary(m);
    element_records(m);
    csr_pattern(m);
    for (int i = 0; i < n; i++)
        if (m.diagpos[i] < 0) { delete M; throw Error{1, "node not referenced by any element"}; }
    ic_pattern(m);
    gather_maps(m);
    cudaGetDevice(&M->device);
    MeshDev& d = M->d;
    d.dim = dim; d.n = n; d.ne = ne; d.nn = m.nn;
    d.nnz = m.rowptr[n];
    d.nnzL = m.Lrowptr[n];
    d.nlev_fwd = (int)m.fwd_lev_ptr.size() - 1;
    d.nlev_bwd = (int)m.bwd_lev_ptr.size() - 1;
    d.rec = upload(m.rec);
    d.el = upload(m.el);
    d.rowptr = upload(m.rowptr);
    d.colidx = upload(m.colidx);
    d.diagpos = upload(m.diagpos);
    d.Lrowptr = upload(m.Lrowptr);
    d.Lcolidx = upload(m.Lcolidx);
    d.Lapos = upload(m.Lapos);
    d.Ucolptr = upload(m.Ucolptr);
    d.Urow = upload(m.Urow);
    d.Umap = upload(m.Umap);
    d.fwd_lev_rows = upload(m.fwd_lev_rows);
    d.bwd_lev_rows = upload(m.bwd_lev_rows);
    d.asm_ptr = upload(m.asm_ptr);
    d.asm_list = upload(m.asm_list);
    d.nel_ptr = upload(m.nel_ptr);
    d.nel_list = upload(m.nel_list);
    d.bndnode = upload(m.bndnode);
    M->fwd_lev_ptr_h = m.fwd_lev_ptr;
    M->bwd_lev_ptr_h = m.bwd_lev_ptr;
    return M;
}

// QVec_Gaussian (src/libstoast/source.cc:19-56): host-side input generation.
void qvec_gaussian_host(const MeshHost& m, const double* cnt, double w, bool neumann, double* q)
{
    const double PI = 3.14159265358979323846;
    double w2 = w * w;
    double fac1 = 1.0 / (std::sqrt(2.0 * PI) * w);
    if (m.dim == 3) fac1 /= (std::sqrt(2.0 * PI) * w);
    if (!neumann) fac1 /= (std::sqrt(2.0 * PI) * w);
    double fac2 = -0.5 / w2;
    std::fill(q, q + m.n, 0.0);
    for (int e = 0; e < m.ne; e++) {
        const int* nd = &m.el[(size_t)e * m.nn];
        for (int i = 0; i < m.nn; i++) {
            int is = nd[i];
            if (neumann && !m.bndnode[is]) continue;
            double d = dist(cnt, &m.coords[(size_t)is * m.dim], m.dim);
            double s = std::exp(d * d * fac2) * fac1;
            for (int j = 0; j < m.nn; j++) {
                int js = nd[j];
                if (neumann) {
                    if (m.bndnode[js]) q[js] += s * m.intbff[((size_t)e * m.nn + i) * m.nn + j];
                } else {
                    double ff = (i == j ? 2.0 : 1.0) * (m.dim == 2 ? 1.0 / 12.0 : 1.0 / 20.0);
                    q[js] += s * (ff * m.rec[(size_t)e * EL_REC]);
                }
            }
        }
    }
}

}  // namespace tg
