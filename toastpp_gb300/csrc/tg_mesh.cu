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
#include <atomic>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
#include "tg_mesh.cuh"
#include "../../include/toastgpu.h"

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

// Morton (Z-order) layout of the nodes: rows that are close in space are
// close in memory, so the neighbours a row gathers are shared by nearby rows.
// distinct source rows of every ROW_TILE-row tile of the layout CSR: the
// SpMM stages them once per tile in shared memory instead of gathering one
// row per entry
static void halo_lists(MeshHost& m)
{
    const int n = m.n, nt = (n + ROW_TILE - 1) / ROW_TILE;
    m.halo_ptr.assign(nt + 1, 0);
    m.halo_col.clear();
    m.lcol.assign(m.lcolidx.size(), 0);
    m.halo_max = 0;
    std::vector<int> cols;
    for (int t = 0; t < nt; t++) {
        const int r0 = t * ROW_TILE, r1 = std::min(n, r0 + ROW_TILE);
        cols.assign(m.lcolidx.begin() + m.lrowptr[r0], m.lcolidx.begin() + m.lrowptr[r1]);
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        if (cols.size() > 65535) throw Error{1, "tile halo too large"};
        for (int e = m.lrowptr[r0]; e < m.lrowptr[r1]; e++)
            m.lcol[e] = (unsigned short)(std::lower_bound(cols.begin(), cols.end(), m.lcolidx[e]) - cols.begin());
        m.halo_col.insert(m.halo_col.end(), cols.begin(), cols.end());
        m.halo_ptr[t + 1] = (int)m.halo_col.size();
        m.halo_max = std::max(m.halo_max, (int)cols.size());
    }
}

static void layout_order(MeshHost& m)
{
    int n = m.n, dim = m.dim;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < n; i++)
        for (int d = 0; d < dim; d++) {
            lo[d] = std::min(lo[d], m.coords[(size_t)i * dim + d]);
            hi[d] = std::max(hi[d], m.coords[(size_t)i * dim + d]);
        }
    const int bits = dim == 2 ? 16 : 10;
    std::vector<std::pair<uint64_t, int>> key(n);
    for (int i = 0; i < n; i++) {
        uint64_t code = 0;
        unsigned q[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) {
            double t = hi[d] > lo[d] ? (m.coords[(size_t)i * dim + d] - lo[d]) / (hi[d] - lo[d]) : 0.0;
            q[d] = (unsigned)std::min((double)((1u << bits) - 1), std::floor(t * (1u << bits)));
        }
        for (int b = bits - 1; b >= 0; b--)
            for (int d = 0; d < dim; d++) code = (code << 1) | ((q[d] >> b) & 1u);
        key[i] = {code, i};
    }
    std::sort(key.begin(), key.end());
    m.perm.assign(n, 0);
    m.iperm.assign(n, 0);
    for (int p = 0; p < n; p++) { m.iperm[p] = key[p].second; m.perm[key[p].second] = p; }
    // layout CSR: layout row p = natural row iperm[p], entries in natural column order
    m.lrowptr.assign(n + 1, 0);
    m.lcolidx.clear();
    m.lay2nat.clear();
    m.ldiagpos.assign(n, -1);
    for (int p = 0; p < n; p++) {
        int i = m.iperm[p];
        for (int q = m.rowptr[i]; q < m.rowptr[i + 1]; q++) {
            if (m.colidx[q] == i) m.ldiagpos[p] = (int)m.lcolidx.size();
            m.lcolidx.push_back(m.perm[m.colidx[q]]);
            m.lay2nat.push_back(q);
        }
        m.lrowptr[p + 1] = (int)m.lcolidx.size();
    }
    m.jcolidx.resize(m.colidx.size());
    for (size_t q = 0; q < m.colidx.size(); q++) m.jcolidx[q] = m.perm[m.colidx[q]];
}

static void ic_finish(const MeshHost& m, ICHost& c);

// IC(0) structure for the ordering given by key[natural node] (a rank): see ICHost.
static void ic_pattern(MeshHost& m, const std::vector<int>& keynat, ICHost& c)
{
    int n = m.n;
    c.key.assign(n, 0);
    for (int p = 0; p < n; p++) c.key[p] = keynat[m.iperm[p]];
    c.Lrowptr.assign(n + 1, 0);
    c.Lcolidx.clear();
    c.Lapos.clear();
    c.Lkey.clear();
    std::vector<std::pair<int, int>> ent;
    for (int p = 0; p < n; p++) {
        ent.clear();
        for (int e = m.lrowptr[p]; e < m.lrowptr[p + 1]; e++) {
            int kj = c.key[m.lcolidx[e]];
            if (kj < c.key[p]) ent.push_back({kj, e});
        }
        std::sort(ent.begin(), ent.end());
        for (auto& pr : ent) {
            c.Lcolidx.push_back(m.lcolidx[pr.second]);
            c.Lkey.push_back(pr.first);
            c.Lapos.push_back(pr.second);
        }
        c.Lrowptr[p + 1] = (int)c.Lcolidx.size();
    }
    ic_finish(m, c);
}

// The column view, the level schedules and the level ELL layouts of an L
// pattern whose rows (Lrowptr, Lcolidx, Lkey, Lapos) and ranks (key) are set.
static void ic_finish(const MeshHost& m, ICHost& c)
{
    const int n = m.n;
    int nl = c.Lrowptr[n];
    std::vector<int> byrank(n);  // layout rows in ascending rank
    for (int p = 0; p < n; p++) byrank[p] = p;
    std::sort(byrank.begin(), byrank.end(), [&](int a, int b) { return c.key[a] < c.key[b]; });
    c.Ucolptr.assign(n + 1, 0);
    for (int q = 0; q < nl; q++) c.Ucolptr[c.Lcolidx[q] + 1]++;
    for (int p = 0; p < n; p++) c.Ucolptr[p + 1] += c.Ucolptr[p];
    c.Urow.assign(nl, 0);
    c.Umap.assign(nl, 0);
    std::vector<int> fill(n, 0);
    for (int p : byrank)  // rows of each column in ascending rank
        for (int q = c.Lrowptr[p]; q < c.Lrowptr[p + 1]; q++) {
            int col = c.Lcolidx[q], pos = c.Ucolptr[col] + fill[col]++;
            c.Urow[pos] = p;
            c.Umap[pos] = q;
        }
    std::vector<int> lev(n, 0), blev(n, 0);  // by layout row
    int nlf = 0, nlb = 0;
    for (int p : byrank) {
        int l = 0;
        for (int q = c.Lrowptr[p]; q < c.Lrowptr[p + 1]; q++) l = std::max(l, lev[c.Lcolidx[q]] + 1);
        lev[p] = l;
        nlf = std::max(nlf, l + 1);
    }
    for (int t = n - 1; t >= 0; t--) {
        int p = byrank[t], l = 0;
        for (int u = c.Ucolptr[p]; u < c.Ucolptr[p + 1]; u++) l = std::max(l, blev[c.Urow[u]] + 1);
        blev[p] = l;
        nlb = std::max(nlb, l + 1);
    }
    auto group = [&](const std::vector<int>& lv, int nlev, std::vector<int>& ptr, std::vector<int>& rows) {
        ptr.assign(nlev + 1, 0);
        for (int p = 0; p < n; p++) ptr[lv[p] + 1]++;
        for (int l = 0; l < nlev; l++) ptr[l + 1] += ptr[l];
        rows.assign(n, 0);
        std::vector<int> f(nlev, 0);
        for (int p = 0; p < n; p++) rows[ptr[lv[p]] + f[lv[p]]++] = p;  // layout order inside a level
    };
    group(lev, nlf, c.fwd_lev_ptr, c.fwd_lev_rows);
    group(blev, nlb, c.bwd_lev_ptr, c.bwd_lev_rows);
    auto ell = [&](bool fwd, const std::vector<int>& ptr, const std::vector<int>& rows, std::vector<int>& w,
                   std::vector<int>& off, std::vector<int>& col, std::vector<int>& src) {
        int nlev = (int)ptr.size() - 1;
        w.assign(nlev, 0);
        off.assign(nlev + 1, 0);
        for (int l = 0; l < nlev; l++) {
            int mw = 1;
            for (int t = ptr[l]; t < ptr[l + 1]; t++) {
                int p = rows[t];
                mw = std::max(mw, fwd ? c.Lrowptr[p + 1] - c.Lrowptr[p] : c.Ucolptr[p + 1] - c.Ucolptr[p]);
            }
            w[l] = mw;
            off[l + 1] = off[l] + (ptr[l + 1] - ptr[l]) * mw;
        }
        col.assign(off[nlev], -1);
        src.assign(off[nlev], -1);
        for (int l = 0; l < nlev; l++)
            for (int t = ptr[l]; t < ptr[l + 1]; t++) {
                int p = rows[t], base = off[l] + (t - ptr[l]) * w[l];
                if (fwd)
                    for (int q = c.Lrowptr[p]; q < c.Lrowptr[p + 1]; q++) {
                        col[base + q - c.Lrowptr[p]] = c.Lcolidx[q];
                        src[base + q - c.Lrowptr[p]] = q;
                    }
                else  // descending rank, the order CholeskySubst subtracts them
                    for (int u = c.Ucolptr[p + 1] - 1, j = 0; u >= c.Ucolptr[p]; u--, j++) {
                        col[base + j] = c.Urow[u];
                        src[base + j] = c.Umap[u];
                    }
            }
    };
    ell(true, c.fwd_lev_ptr, c.fwd_lev_rows, c.fwd_ell_w, c.fwd_ell_off, c.fwd_ell_col, c.fwd_ell_src);
    ell(false, c.bwd_lev_ptr, c.bwd_lev_rows, c.bwd_ell_w, c.bwd_ell_off, c.bwd_ell_col, c.bwd_ell_src);
}

// ---------------------------------------------------------------------------
// Complete factor for the direct solver (LSOLVER_DIRECT): a fill-reducing
// nested-dissection ordering and the symbolic Cholesky pattern, in the same
// ICHost form as the IC(0) patterns so the same factor and sweep kernels run
// on it (IC on a pattern closed under fill is the exact factorisation).
// ---------------------------------------------------------------------------
namespace {
struct NDState {
    const MeshHost* m;
    std::vector<int> mark, sep;
    int stamp = 0;
    double coord(int p, int d) const { return m->coords[(size_t)m->iperm[p] * m->dim + d]; }
};

// orders idx[lo, hi) into out: lower half, upper half (both recursively),
// then the separator (upper-half nodes adjacent to the lower half); the
// halves split at the median of the longest extent; sets of at most 32
// nodes keep their layout (spatial) order
void nd_order(NDState& S, std::vector<int>& idx, int lo, int hi, std::vector<int>& out)
{
    const MeshHost& m = *S.m;
    const int cnt = hi - lo;
    if (cnt <= 32) {
        std::sort(idx.begin() + lo, idx.begin() + hi);
        out.insert(out.end(), idx.begin() + lo, idx.begin() + hi);
        return;
    }
    double ext = -1.0;
    int ax = 0;
    for (int d = 0; d < m.dim; d++) {
        double a = 1e300, b = -1e300;
        for (int t = lo; t < hi; t++) {
            const double v = S.coord(idx[t], d);
            a = std::min(a, v);
            b = std::max(b, v);
        }
        if (b - a > ext) { ext = b - a; ax = d; }
    }
    const int mid = lo + cnt / 2;
    std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi, [&](int a, int b) {
        const double u = S.coord(a, ax), v = S.coord(b, ax);
        return u < v || (u == v && a < b);
    });
    const int tag = ++S.stamp;
    for (int t = lo; t < mid; t++) S.mark[idx[t]] = tag;
    const size_t s0 = S.sep.size();
    int w = mid;
    for (int t = mid; t < hi; t++) {
        const int p = idx[t];
        bool adj = false;
        for (int e = m.lrowptr[p]; e < m.lrowptr[p + 1] && !adj; e++) adj = S.mark[m.lcolidx[e]] == tag;
        if (adj) S.sep.push_back(p);
        else idx[w++] = p;
    }
    std::vector<int> sep(S.sep.begin() + s0, S.sep.end());
    S.sep.resize(s0);
    nd_order(S, idx, lo, mid, out);
    nd_order(S, idx, mid, w, out);
    std::sort(sep.begin(), sep.end());
    out.insert(out.end(), sep.begin(), sep.end());
}
}  // namespace

void direct_pattern(const MeshHost& m, ICHost& c, long long max_nnz)
{
    const int n = m.n;
    NDState S;
    S.m = &m;
    S.mark.assign(n, 0);
    std::vector<int> idx(n), order;
    for (int p = 0; p < n; p++) idx[p] = p;
    order.reserve(n);
    nd_order(S, idx, 0, n, order);
    c.key.assign(n, 0);
    for (int r = 0; r < n; r++) c.key[order[r]] = r;
    // symbolic factorisation in rank space: column j holds the ranks i > j of
    // its neighbours and of its elimination-tree children's columns
    std::vector<std::vector<int>> col(n);
    std::vector<std::vector<int>> kids(n);
    std::vector<int> seen(n, -1);
    long long total = 0;
    for (int j = 0; j < n; j++) {
        const int p = order[j];
        std::vector<int>& cj = col[j];
        seen[j] = j;
        for (int e = m.lrowptr[p]; e < m.lrowptr[p + 1]; e++) {
            const int i = c.key[m.lcolidx[e]];
            if (i > j && seen[i] != j) { seen[i] = j; cj.push_back(i); }
        }
        for (int ch : kids[j]) {
            for (int i : col[ch])
                if (i > j && seen[i] != j) { seen[i] = j; cj.push_back(i); }
        }
        std::sort(cj.begin(), cj.end());
        if (!cj.empty()) kids[cj[0]].push_back(j);
        total += (long long)cj.size();
        TG_CHECK(total <= max_nnz, TG_ERR_UNSUPPORTED, "direct solver: the factor's fill exceeds its limit");
    }
    // rows of L by layout row, entries in ascending rank (the transpose of
    // the columns, which come in ascending rank)
    std::vector<int> rcnt(n + 1, 0);
    for (int j = 0; j < n; j++)
        for (int i : col[j]) rcnt[order[i] + 1]++;
    c.Lrowptr.assign(n + 1, 0);
    for (int p = 0; p < n; p++) c.Lrowptr[p + 1] = c.Lrowptr[p] + rcnt[p + 1];
    const size_t nl = (size_t)c.Lrowptr[n];
    c.Lcolidx.assign(nl, 0);
    c.Lkey.assign(nl, 0);
    c.Lapos.assign(nl, -1);
    std::vector<int> fill(c.Lrowptr.begin(), c.Lrowptr.end() - 1);
    for (int j = 0; j < n; j++) {
        for (int i : col[j]) {
            const int pr = order[i];
            const int q = fill[pr]++;
            c.Lcolidx[q] = order[j];
            c.Lkey[q] = j;
        }
        std::vector<int>().swap(col[j]);
    }
    // Lapos: the entry of A at (row, column), or -1 for a fill entry
    std::vector<int> where(n, -1);
    for (int p = 0; p < n; p++) {
        for (int e = m.lrowptr[p]; e < m.lrowptr[p + 1]; e++) where[m.lcolidx[e]] = e;
        for (int q = c.Lrowptr[p]; q < c.Lrowptr[p + 1]; q++) c.Lapos[q] = where[c.Lcolidx[q]];
        for (int e = m.lrowptr[p]; e < m.lrowptr[p + 1]; e++) where[m.lcolidx[e]] = -1;
    }
    ic_finish(m, c);
}

// greedy colouring in natural order; key = colour-major rank (colour, natural index)
static std::vector<int> colour_key(MeshHost& m)
{
    int n = m.n;
    std::vector<int> col(n, -1);
    std::vector<int> mark;
    int nc = 0;
    for (int i = 0; i < n; i++) {
        mark.assign(nc + 1, 0);
        for (int q = m.rowptr[i]; q < m.rowptr[i + 1]; q++) {
            int j = m.colidx[q];
            if (j != i && col[j] >= 0) mark[col[j]] = 1;
        }
        int c = 0;
        while (c < nc && mark[c]) c++;
        col[i] = c;
        if (c == nc) nc++;
    }
    m.ncolors = nc;
    std::vector<int> cnt(nc + 1, 0);
    for (int i = 0; i < n; i++) cnt[col[i] + 1]++;
    for (int c = 0; c < nc; c++) cnt[c + 1] += cnt[c];
    std::vector<int> key(n);
    for (int i = 0; i < n; i++) key[i] = cnt[col[i]]++;
    return key;
}

static void gather_maps(MeshHost& m)
{
    int nnz = m.rowptr[m.n];
    std::vector<int> nat2lay(nnz);
    for (int e = 0; e < nnz; e++) nat2lay[m.lay2nat[e]] = e;
    std::vector<int> cnt(nnz + 1, 0);
    std::vector<int> slot((size_t)m.ne * m.nn * m.nn);
    for (int e = 0; e < m.ne; e++)
        for (int i = 0; i < m.nn; i++)
            for (int j = 0; j < m.nn; j++) {
                int k = nat2lay[find_col(m.rowptr, m.colidx, m.el[(size_t)e * m.nn + i], m.el[(size_t)e * m.nn + j])];
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
    m.nel_pos.assign(m.nel_ptr[m.n], 0u);
    std::vector<int> g(m.n, 0);
    for (int e = 0; e < m.ne; e++)
        for (int i = 0; i < m.nn; i++) {
            int nd = m.el[(size_t)e * m.nn + i];
            int slot = m.nel_ptr[nd] + g[nd]++;
            m.nel_list[slot] = e * 4 + i;
            unsigned packed = 0;
            for (int j = 0; j < m.nn; j++) {
                int p = find_col(m.rowptr, m.colidx, nd, m.el[(size_t)e * m.nn + j]) - m.rowptr[nd];
                if (p < 0 || p > 255) throw Error{1, "node degree above 255 is not supported"};
                packed |= (unsigned)p << (8 * j);
            }
            m.nel_pos[slot] = packed;
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
    void* ptrs[] = {d.rec, d.el, d.rowptr, d.colidx, d.diagpos, d.perm, d.iperm, d.jrowptr, d.jcolidx, d.asm_ptr,
                    d.asm_list, d.nel_ptr, d.nel_list, d.nel_pos, d.bndnode, d.halo_ptr, d.halo_col, d.lcol,
                    d.intbff};
    for (void* p : ptrs) if (p) cudaFree(p);
    for (auto& g : d.ic) {
        void* q[] = {g.key, g.Lrowptr, g.Lcolidx, g.Lapos, g.Lkey, g.Ucolptr, g.Urow, g.Umap, g.fwd_lev_rows,
                     g.bwd_lev_rows, g.fwd_ell_col, g.fwd_ell_src, g.bwd_ell_col, g.bwd_ell_src, g.fwd_lev_ptr,
                     g.bwd_lev_ptr, g.fwd_ell_w, g.bwd_ell_w, g.fwd_ell_off, g.bwd_ell_off};
        for (void* p : q) if (p) cudaFree(p);
    }
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
    layout_order(m);
    halo_lists(m);
    {
        std::vector<int> natkey(n);
        for (int i = 0; i < n; i++) natkey[i] = i;
        ic_pattern(m, natkey, m.ic[0]);
        ic_pattern(m, colour_key(m), m.ic[1]);
    }
    gather_maps(m);
    static std::atomic<long long> next_uid{1};
    M->uid = next_uid.fetch_add(1);
    cudaGetDevice(&M->device);
    MeshDev& d = M->d;
    d.dim = dim; d.n = n; d.ne = ne; d.nn = m.nn;
    d.nnz = m.rowptr[n];
    d.rec = upload(m.rec);
    d.intbff = upload(m.intbff);
    d.el = upload(m.el);
    d.rowptr = upload(m.lrowptr);
    d.colidx = upload(m.lcolidx);
    d.diagpos = upload(m.ldiagpos);
    d.perm = upload(m.perm);
    d.iperm = upload(m.iperm);
    d.jrowptr = upload(m.rowptr);
    d.jcolidx = upload(m.jcolidx);
    d.halo_ptr = upload(m.halo_ptr);
    d.halo_col = upload(m.halo_col);
    d.lcol = upload(m.lcol);
    d.halo_max = m.halo_max;
    d.asm_ptr = upload(m.asm_ptr);
    d.asm_list = upload(m.asm_list);
    d.nel_ptr = upload(m.nel_ptr);
    d.nel_list = upload(m.nel_list);
    d.nel_pos = upload(m.nel_pos);
    d.bndnode = upload(m.bndnode);
    for (int t = 0; t < 2; t++) {
        const ICHost& c = m.ic[t];
        ICDev& g = d.ic[t];
        g.nnzL = c.Lrowptr[n];
        g.nlev_fwd = (int)c.fwd_lev_ptr.size() - 1;
        g.nlev_bwd = (int)c.bwd_lev_ptr.size() - 1;
        g.nell_fwd = (int)c.fwd_ell_col.size();
        g.nell_bwd = (int)c.bwd_ell_col.size();
        g.key = upload(c.key);
        g.Lrowptr = upload(c.Lrowptr);
        g.Lcolidx = upload(c.Lcolidx);
        g.Lapos = upload(c.Lapos);
        g.Lkey = upload(c.Lkey);
        g.Ucolptr = upload(c.Ucolptr);
        g.Urow = upload(c.Urow);
        g.Umap = upload(c.Umap);
        g.fwd_lev_rows = upload(c.fwd_lev_rows);
        g.bwd_lev_rows = upload(c.bwd_lev_rows);
        g.fwd_ell_col = upload(c.fwd_ell_col);
        g.fwd_ell_src = upload(c.fwd_ell_src);
        g.bwd_ell_col = upload(c.bwd_ell_col);
        g.bwd_ell_src = upload(c.bwd_ell_src);
        g.fwd_lev_ptr = upload(c.fwd_lev_ptr);
        g.bwd_lev_ptr = upload(c.bwd_lev_ptr);
        g.fwd_ell_w = upload(c.fwd_ell_w);
        g.bwd_ell_w = upload(c.bwd_ell_w);
        g.fwd_ell_off = upload(c.fwd_ell_off);
        g.bwd_ell_off = upload(c.bwd_ell_off);
    }
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

// Element_Unstructured::GContains (element.cc:553-563): the element's bounding
// box widened by 1e-8, then LContains(Local(p)) with the padded test
// (tri3.cc:134-144 / 191-200, tet4.cc:186-196 / 268-279)
bool el_gcontains(const MeshHost& m, int e, const double* p)
{
    const int dim = m.dim, nn = m.nn;
    const int* nd = &m.el[(size_t)e * nn];
    for (int d = 0; d < dim; d++) {
        double lo = 1e10, hi = -1e10;
        for (int i = 0; i < nn; i++) {
            const double v = m.coords[(size_t)nd[i] * dim + d];
            lo = std::min(lo, v);
            hi = std::max(hi, v);
        }
        if (p[d] < lo - 1e-8 || p[d] > hi + 1e-8) return false;
    }
    const double* g = &m.geo[(size_t)e * 16];
    const double EPS = 1e-8;
    if (dim == 2) {
        const double scale = 1.0 / (g[0] + g[1] + g[2]);
        const double l0 = (g[1] + g[4] * p[0] + g[7] * p[1]) * scale;
        const double l1 = (g[2] + g[5] * p[0] + g[8] * p[1]) * scale;
        return l0 + EPS >= 0.0 && l1 + EPS >= 0.0 && l0 + l1 - EPS <= 1.0;
    }
    const double *a = g, *b = g + 4, *c = g + 8, *dd = g + 12;
    const double scale = 1.0 / (a[0] + a[1] + a[2] + a[3]);
    double l[3];
    for (int r = 0; r < 3; r++) l[r] = (a[r + 1] + b[r + 1] * p[0] + c[r + 1] * p[1] + dd[r + 1] * p[2]) * scale;
    return l[0] + EPS >= 0.0 && l[1] + EPS >= 0.0 && l[2] + EPS >= 0.0 && l[0] + l[1] + l[2] - EPS <= 1.0;
}


// Mesh::PullToBoundary (mesh.cc:1052-1111) with sub = 0 for P1 elements: the
// boundary node nearest p (the first of equal distance), then the elements
// around it in order; in each, the sides whose nodes are all boundary nodes
// (Element::BndSideList, element.cc:338-348) in side order: p in the
// element's local coordinates (Triangle3::Local, tri3.cc:134-144;
// Tetrahedron4::Local, tet4.cc:186-196) is projected along the side's local
// normal (LNormal, tri3.cc:172-182, tet4.cc:254-266, the reference's
// truncated constants) and the first projection inside the element
// (LContains with padding, tri3.cc:191-200, tet4.cc:268-279) is mapped back
// (Element::Global, element.cc:164-176).  Returns false when none is.
static bool pull_to_boundary(const MeshHost& m, const double* p, double* out)
{
    const int dim = m.dim, nn = m.nn;
    int nmin = -1;
    double dmin = 1e10;
    for (int k = 0; k < m.n; k++) {
        if (!m.bndnode[k]) continue;
        const double d = dist(p, &m.coords[(size_t)k * dim], dim);
        if (d < dmin) {
            dmin = d;
            nmin = k;
        }
    }
    static const double LN2[3][2] = {{0, -1}, {0.7071067814, 0.7071067814}, {-1, 0}};
    static const double LN3[4][3] = {{0, 0, -1}, {0, -1, 0}, {-1, 0, 0}, {0.577350269, 0.577350269, 0.577350269}};
    const int nside = dim == 2 ? 3 : 4, nsn = dim == 2 ? 2 : 3;
    for (int e = 0; e < m.ne && nmin >= 0; e++) {
        const int* nd = &m.el[(size_t)e * nn];
        bool has = false;
        for (int i = 0; i < nn; i++) has |= nd[i] == nmin;
        if (!has) continue;
        const double* g = &m.geo[(size_t)e * 16];
        // local coordinates of a global point
        auto local = [&](const double* x, double* l) {
            if (dim == 2) {
                const double scale = 1.0 / (g[0] + g[1] + g[2]);
                l[0] = (g[1] + g[4] * x[0] + g[7] * x[1]) * scale;
                l[1] = (g[2] + g[5] * x[0] + g[8] * x[1]) * scale;
            } else {
                const double *a = g, *b = g + 4, *c = g + 8, *d = g + 12;
                const double scale = 1.0 / (a[0] + a[1] + a[2] + a[3]);
                for (int r = 0; r < 3; r++) l[r] = (a[r + 1] + b[r + 1] * x[0] + c[r + 1] * x[1] + d[r + 1] * x[2]) * scale;
            }
        };
        for (int sd = 0; sd < nside; sd++) {
            bool bnd = true;
            for (int k = 0; k < nsn && bnd; k++)
                if (!m.bndnode[nd[dim == 2 ? TRI_SIDE[sd][k] : TET_SIDE[sd][k]]]) bnd = false;
            if (!bnd) continue;
            const double* ln = dim == 2 ? LN2[sd] : LN3[sd];
            double ploc[3], nloc[3], l[3];
            local(p, ploc);
            local(&m.coords[(size_t)nd[dim == 2 ? TRI_SIDE[sd][0] : TET_SIDE[sd][0]] * dim], nloc);
            double pd = 0.0;
            for (int r = 0; r < dim; r++) pd += (ploc[r] - nloc[r]) * ln[r];
            for (int r = 0; r < dim; r++) l[r] = ploc[r] - ln[r] * pd;
            const double EPS = 1e-8;
            bool in = true;
            double sum = 0.0;
            for (int r = 0; r < dim; r++) {
                in = in && l[r] + EPS >= 0.0;
                sum = r ? sum + l[r] : l[r];
            }
            if (!in || sum - EPS > 1.0) continue;
            double u[4];
            u[0] = dim == 2 ? 1.0 - l[0] - l[1] : 1.0 - l[0] - l[1] - l[2];
            for (int r = 0; r < dim; r++) u[r + 1] = l[r];
            for (int c = 0; c < dim; c++) {
                double v = 0.0;
                for (int j = 0; j < nn; j++) v += u[j] * m.coords[(size_t)nd[j] * dim + c];
                out[c] = v;
            }
            return true;
        }
    }
    return false;
}

bool el_found(const MeshHost& m, const double* p)
{
    for (int e = 0; e < m.ne; e++)
        if (el_gcontains(m, e, p)) return true;
    return false;
}

// The line (or segment) p1-p2 against one element's boundary sides, in the
// element's local frame; up to 4 points into s, their count returned.
//  - Triangle3::Intersection (tri3.cc:698-780), boundary sides only: side 0
//    is tested against the edge y = 0, the flag of side 1 against x = 0 and
//    that of side 2 against x + y = 1 (the reference pairs them so, although
//    side 1 joins nodes 1-2 and side 2 nodes 2-0, tri3.cc:121-127); points
//    off the segment p1-p2 are dropped.
//  - Tetrahedron4::Intersection (tet4.cc:1222-1283): the whole line against
//    the boundary faces' planes, each point kept inside its face.
static int side_intersections(const MeshHost& m, int e, const double* p1, const double* p2, double s[4][3])
{
    const unsigned char* bs = &m.bndside[(size_t)e * (m.dim == 2 ? 3 : 4)];
    int k = 0;
    if (m.dim == 2) {
        const double EPS = 1e-12;
        if (bs[0] && p1[1] * p2[1] < 0.0) {
            const double xs = p1[0] - p1[1] / (p2[1] - p1[1]) * (p2[0] - p1[0]);
            if (xs > -EPS && xs < 1.0 + EPS) { s[k][0] = xs; s[k][1] = 0.0; k++; }
        }
        if (bs[1] && p1[0] * p2[0] < 0.0) {
            const double ys = p1[1] - p1[0] / (p2[0] - p1[0]) * (p2[1] - p1[1]);
            if (ys > -EPS && ys < 1.0 + EPS) { s[k][0] = 0.0; s[k][1] = ys; k++; }
        }
        if (bs[2]) {
            double xs = p1[0];
            if (std::fabs(p1[0] - p2[0]) > EPS) {
                const double a = (p1[1] - p2[1]) / (p1[0] - p2[0]);
                const double c = p1[1] - a * p1[0];
                xs = (1.0 - c) / (a + 1.0);
            }
            if (xs > -EPS && xs < 1.0 + EPS) { s[k][0] = xs; s[k][1] = 1.0 - xs; k++; }
        }
        if (k) {
            int d = 0, j = 0;
            double dp = p2[0] - p1[0];
            if (std::fabs(dp) < EPS) { d = 1; dp = p2[1] - p1[1]; }
            for (int i = 0; i < k; i++) {
                const double a = (s[i][d] - p1[d]) / dp;
                if (a < -EPS || a > 1.0 + EPS) continue;
                s[j][0] = s[i][0];
                s[j][1] = s[i][1];
                j++;
            }
            k = j;
        }
        return k;
    }
    const double sx = p1[0], sy = p1[1], sz = p1[2];
    const double dx = p2[0] - p1[0], dy = p2[1] - p1[1], dz = p2[2] - p1[2];
    auto keep = [&](double x, double y, double z) { s[k][0] = x; s[k][1] = y; s[k][2] = z; k++; };
    if (bs[0] && dz != 0.0) {
        const double a = -sz / dz, rx = sx + a * dx, ry = sy + a * dy;
        if (rx >= 0 && ry >= 0 && rx + ry <= 1) keep(rx, ry, 0.0);
    }
    if (bs[1] && dy != 0.0) {
        const double a = -sy / dy, rx = sx + a * dx, rz = sz + a * dz;
        if (rx >= 0 && rz >= 0 && rx + rz <= 1) keep(rx, 0.0, rz);
    }
    if (bs[2] && dx != 0.0) {
        const double a = -sx / dx, ry = sy + a * dy, rz = sz + a * dz;
        if (ry >= 0 && rz >= 0 && ry + rz <= 1) keep(0.0, ry, rz);
    }
    if (bs[3] && (dx + dy + dz) != 0.0) {
        const double a = (1 - sx - sy - sz) / (dx + dy + dz);
        const double rx = sx + a * dx, ry = sy + a * dy, rz = sz + a * dz;
        if (rx >= 0 && ry >= 0 && rx + ry <= 1) keep(rx, ry, rz);
    }
    return k;
}

// Mesh::BndIntersect (mesh.cc:1369-1453): in 3D the line must cross the
// mesh's bounding box (BoundingBox, mesh.cc:1341-1360, no padding) on one of
// its faces; then every element with a boundary side intersects it in its
// local frame (Element::GlobalIntersection, element.cc:505-511), the points
// are mapped back (Element::Global, element.cc:164-176) and the one nearest
// p1 (the first of equal distance, element order) is the result.
static bool bnd_intersect(const MeshHost& m, const double* p1, const double* p2, double* out)
{
    const int dim = m.dim, nn = m.nn, nside = dim == 2 ? 3 : 4;
    if (dim > 2) {
        const double EPS = 1e-12;
        double lo[3] = {1e6, 1e6, 1e6}, hi[3] = {-1e6, -1e6, -1e6};
        for (int k = 0; k < m.n; k++)
            for (int d = 0; d < 3; d++) {
                const double v = m.coords[(size_t)k * 3 + d];
                lo[d] = v < lo[d] ? v : lo[d];
                hi[d] = v > hi[d] ? v : hi[d];
            }
        const double d[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
        // the box faces normal to z, then y, then x; (u, v) the other axes
        static const int AX[3][3] = {{2, 0, 1}, {1, 0, 2}, {0, 1, 2}};
        bool hit = false;
        for (int f = 0; f < 3 && !hit; f++) {
            const int w = AX[f][0], u = AX[f][1], v = AX[f][2];
            if (d[w] == 0.0) continue;
            for (int side = 0; side < 2 && !hit; side++) {
                const double a = ((side ? hi[w] : lo[w]) - p1[w]) / d[w];
                const double ru = p1[u] + a * d[u], rv = p1[v] + a * d[v];
                hit = ru > lo[u] - EPS && ru < hi[u] + EPS && rv > lo[v] - EPS && rv < hi[v] + EPS;
            }
        }
        if (!hit) return false;
    }
    double dmin = 1e10;
    bool found = false;
    for (int e = 0; e < m.ne; e++) {
        bool any = false;
        for (int sd = 0; sd < nside; sd++) any |= m.bndside[(size_t)e * nside + sd] != 0;
        if (!any) continue;
        const double* g = &m.geo[(size_t)e * 16];
        double l1[3], l2[3], s[4][3];
        if (dim == 2) {
            const double scale = 1.0 / (g[0] + g[1] + g[2]);
            l1[0] = (g[1] + g[4] * p1[0] + g[7] * p1[1]) * scale;
            l1[1] = (g[2] + g[5] * p1[0] + g[8] * p1[1]) * scale;
            l2[0] = (g[1] + g[4] * p2[0] + g[7] * p2[1]) * scale;
            l2[1] = (g[2] + g[5] * p2[0] + g[8] * p2[1]) * scale;
        } else {
            const double *a = g, *b = g + 4, *c = g + 8, *dd = g + 12;
            const double scale = 1.0 / (a[0] + a[1] + a[2] + a[3]);
            for (int r = 0; r < 3; r++) {
                l1[r] = (a[r + 1] + b[r + 1] * p1[0] + c[r + 1] * p1[1] + dd[r + 1] * p1[2]) * scale;
                l2[r] = (a[r + 1] + b[r + 1] * p2[0] + c[r + 1] * p2[1] + dd[r + 1] * p2[2]) * scale;
            }
        }
        const int k = side_intersections(m, e, l1, l2, s);
        const int* nd = &m.el[(size_t)e * nn];
        for (int j = 0; j < k; j++) {
            double u[4], glob[3];
            u[0] = dim == 2 ? 1.0 - s[j][0] - s[j][1] : 1.0 - s[j][0] - s[j][1] - s[j][2];
            for (int r = 0; r < dim; r++) u[r + 1] = s[j][r];
            for (int c = 0; c < dim; c++) {
                glob[c] = 0.0;
                for (int i = 0; i < nn; i++) glob[c] += u[i] * m.coords[(size_t)nd[i] * dim + c];
            }
            const double dst = dist(p1, glob, dim);
            if (dst < dmin) {
                dmin = dst;
                for (int c = 0; c < dim; c++) out[c] = glob[c];
                found = true;
            }
        }
    }
    return found;
}

// qmmesh.cc:378-391: n = the normal read (or -q), scaled by the reciprocal of
// its length (TVector::operator/=, vector_imp.hpp:672-677); the start point
// q + |q| n; lengths are plain roots of sums of squares (l2norm,
// vector_imp.hpp:1117-1120, 1290-1298)
int qm_external_source(const MeshHost& m, const double* q, const double* nrm, double* out)
{
    const int dim = m.dim;
    double n[3], s = 0.0, sq = 0.0, p1[3];
    for (int c = 0; c < dim; c++) n[c] = nrm ? nrm[c] : -q[c];
    for (int c = 0; c < dim; c++) s += std::fabs(n[c]) * std::fabs(n[c]);
    if (nrm && !(std::sqrt(s) > 0.0)) return 2;
    const double inv = 1.0 / std::sqrt(s);
    for (int c = 0; c < dim; c++) n[c] *= inv;
    for (int c = 0; c < dim; c++) sq += std::fabs(q[c]) * std::fabs(q[c]);
    const double len = std::sqrt(sq);
    for (int c = 0; c < dim; c++) p1[c] = q[c] + len * n[c];
    return bnd_intersect(m, p1, q, out) ? 0 : 1;
}

bool qm_place_detector(const MeshHost& m, bool fixed, double* p)
{
    if (!fixed) {
        // when no side takes the projection, the reference's fallback
        // (PullToBoundary_old) writes to a local point (mesh.cc:1110): the
        // position stays as read
        double q[3];
        if (pull_to_boundary(m, p, q))
            for (int c = 0; c < m.dim; c++) p[c] = q[c];
        return true;
    }
    // a fixed position outside every element moves by -1e-4, 0, +1e-4 along
    // each axis in turn until an element contains it (qmmesh.cc:112-127)
    if (el_found(m, p)) return true;
    double p0[3] = {p[0], p[1], m.dim > 2 ? p[2] : 0.0};
    const double eps = 1e-4;
    for (int d = 0; d < m.dim; d++)
        for (int s = -1; s <= 1; s++) {
            for (int c = 0; c < m.dim; c++) p[c] = p0[c];
            p[d] += s * eps;
            if (el_found(m, p)) return true;
        }
    return false;
}

}  // namespace tg
