// tg_grid.cuh -- the grid-basis Jacobian of a pixel raster.
//
// Reference: GenerateJacobian_grid (src/libstoast/jacobian.cc:289-373,
// complex, projections given) and GenerateJacobian_cw_grid (516-712, real)
// with Raster_Pixel (raster_px.cc:10-48).  The PMDFs are formed on the
// raster's grid; where the basis is coarser than the grid (an intermediate
// grid) the rows are then mapped to the basis by G (grid_to_sol_rows_kernel).
//
// Per request the fields (source-major, natural numbering) are resampled on
// the grid column by column (gm[c * glen + g]), then the values and the
// central or one-sided differences of ImageGradient (jacobian.cc:944-1060) at
// the solution points (the grid points inside the mesh) go to planes
// P[(c * (1 + dim) + comp) * slen + s] (comp 0 the value, 1..dim the
// gradient), so that a thread per solution point reads every plane of a
// source or detector coalesced.  Then one thread per solution point and
// group of sources walks the sources' links and writes its column of every
// link row.
#pragma once
#include "tg_kernels.cuh"

namespace tg {

struct GridDev {
    int dim, nx, ny, nz, glen, slen;
    double ih[3];                // 1 / (gsize / n) per axis (ImageGradient's spacing)
    const int* elref;            // glen: containing element or -1
    const int* sol;              // slen: grid index of each solution point
    const int* rowptr;           // glen + 1: grid map matrix B (natural node columns)
    const int* col;
    const double* val;
};

// Map_MeshToGrid (raster.cc:188-199; complex: Ax_cplx, crmatrix_imp.hpp:
// 1302-1327): gm[g * k + c] = sum_j B(g, j) x[row(col_j) * ld + c], x
// node-major, rows in the natural numbering (perm null) or in a layout
// (row = perm[natural]); a warp per grid point, lanes over columns
template <class V>
__global__ void grid_map_kernel(GridDev G, int k, const V* __restrict__ x, int ld, const int* __restrict__ perm,
                                V* __restrict__ gm)
{
    const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (g >= G.glen) return;
    const int j0 = G.rowptr[g], j1 = G.rowptr[g + 1];
    for (int c = lane; c < k; c += 32) {
        V acc = vzero<V>();
        for (int j = j0; j < j1; j++) {
            const int r = perm ? perm[G.col[j]] : G.col[j];
            acc = vadd(acc, vscale(x[(size_t)r * ld + c], G.val[j]));
        }
        gm[(size_t)g * k + c] = acc;
    }
}

// value (comp 0) or ImageGradient component comp - 1 of column c at grid
// point g: central or one-sided differences as jacobian.cc:944-1060 takes
// them; masked: neighbours outside the element mask do not count, else every
// grid point does
template <class V>
__device__ __forceinline__ V grid_component(const GridDev& G, int k, const V* __restrict__ gm, int g, int c,
                                            int comp, int masked)
{
    const V v0 = gm[(size_t)g * k + c];
    if (comp == 0) return v0;
    const int d = comp - 1;
    const int co = d == 0 ? g % G.nx : (d == 1 ? (g / G.nx) % G.ny : g / (G.nx * G.ny));
    const int len = d == 0 ? G.nx : (d == 1 ? G.ny : G.nz), st = d == 0 ? 1 : (d == 1 ? G.nx : G.nx * G.ny);
    const bool blo = co > 0 && (!masked || G.elref[g - st] >= 0);
    const bool bhi = co < len - 1 && (!masked || G.elref[g + st] >= 0);
    using R = typename vt<V>::R;
    if (blo && bhi) return vscale(vsub(gm[(size_t)(g + st) * k + c], gm[(size_t)(g - st) * k + c]), (R)(0.5 * G.ih[d]));
    // a point outside the mask (a blob basis's solution point off the
    // mesh) without both neighbours inside: 0 (ImageGradient,
    // jacobian.cc:944-1060)
    if (masked && G.elref[g] < 0) return vzero<V>();
    if (blo) return vscale(vsub(v0, gm[(size_t)(g - st) * k + c]), (R)G.ih[d]);
    if (bhi) return vscale(vsub(gm[(size_t)(g + st) * k + c], v0), (R)G.ih[d]);
    return vzero<V>();
}

// Field planes P[(c * (1 + dim) + comp) * slen + s] from the grid fields:
// block = 32 solution points x 32 columns; each component is formed with
// lanes over columns (coalesced reads of gm) into a shared tile, then
// written with lanes over solution points (coalesced planes)
template <class V, class OUT>
__global__ void __launch_bounds__(256) grid_planes_kernel(GridDev G, int k, const V* __restrict__ gm, int masked,
                                                          OUT* __restrict__ planes)
{
    __shared__ OUT tile[32][33];
    const int s0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    const int np = 1 + G.dim;
    for (int comp = 0; comp < np; comp++) {
        for (int r = ty; r < 32; r += 8) {
            const int s = s0 + r, c = c0 + tx;
            if (s < G.slen && c < k) tile[r][tx] = vcast<OUT, V>(grid_component(G, k, gm, G.sol[s], c, comp, masked));
        }
        __syncthreads();
        for (int r = ty; r < 32; r += 8) {
            const int c = c0 + r, s = s0 + tx;
            if (s < G.slen && c < k) planes[((size_t)c * np + comp) * G.slen + s] = tile[tx][r];
        }
        __syncthreads();
    }
}

// Map_MeshToGrid of source-major columns, column-major result:
// gm[c * glen + g] = sum_j B(g, j) x[c * n + col_j] in the arithmetic type A;
// columns c < k0 from x0, the others from x1.  A thread per grid point keeps
// its row of B (at most four entries for linear elements) in registers for
// MAPC columns; neighbouring grid points gather from neighbouring nodes.
constexpr int MAPC = 8;
template <class A, class V>
__global__ void __launch_bounds__(256) grid_map_cm_kernel(GridDev G, int n, int k, int k0, const V* __restrict__ x0,
                                                          const V* __restrict__ x1, A* __restrict__ gm)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G.glen) return;
    using R = typename vt<A>::R;
    const int j0 = G.rowptr[g], nj = G.rowptr[g + 1] - j0;
    int col[4];
    R w[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        col[j] = j < nj ? G.col[j0 + j] : 0;
        w[j] = j < nj ? (R)G.val[j0 + j] : (R)0;
    }
    const int c1 = min(k, (int)(blockIdx.y + 1) * MAPC);
    for (int c = blockIdx.y * MAPC; c < c1; c++) {
        const V* x = c < k0 ? x0 + (size_t)c * n : x1 + (size_t)(c - k0) * n;
        A acc = vzero<A>();
        if (nj <= 4) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (j < nj) acc = vadd(acc, vscale(vcast<A, V>(x[col[j]]), w[j]));
        } else {
            for (int j = j0; j < j0 + nj; j++) acc = vadd(acc, vscale(vcast<A, V>(x[G.col[j]]), (R)G.val[j]));
        }
        gm[(size_t)c * G.glen + g] = acc;
    }
}

// Field planes P[(c * (1 + dim) + comp) * slen + s] from the column-major grid
// fields: a thread per solution point finds, once, the neighbours and weight
// of each axis's difference under the masked and the unmasked rule of
// grid_component, then forms MAPC columns; columns c < kmask are masked, the
// others when mask_rest is set.  Reads and writes run along s.
template <class A>
__global__ void __launch_bounds__(256) grid_planes_cm_kernel(GridDev G, int k, int kmask, int mask_rest,
                                                             const A* __restrict__ gm, A* __restrict__ planes)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= G.slen) return;
    using R = typename vt<A>::R;
    const int g = G.sol[s], np = 1 + G.dim;
    const int co[3] = {g % G.nx, (g / G.nx) % G.ny, g / (G.nx * G.ny)};
    const int len[3] = {G.nx, G.ny, G.nz}, st[3] = {1, G.nx, G.nx * G.ny};
    int lo[2][3], hi[2][3];
    R w[2][3];
#pragma unroll
    for (int mk = 0; mk < 2; mk++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            lo[mk][d] = hi[mk][d] = g;
            w[mk][d] = (R)0;
            if (d >= G.dim) continue;
            const bool blo = co[d] > 0 && (!mk || G.elref[g - st[d]] >= 0);
            const bool bhi = co[d] < len[d] - 1 && (!mk || G.elref[g + st[d]] >= 0);
            // one-sided differences only at points inside the mask
            const bool in = !mk || G.elref[g] >= 0;
            if (blo) lo[mk][d] = g - st[d];
            if (bhi) hi[mk][d] = g + st[d];
            if ((blo && bhi) || (in && (blo || bhi))) w[mk][d] = (R)((blo && bhi ? 0.5 : 1.0) * G.ih[d]);
        }
    const int c1 = min(k, (int)(blockIdx.y + 1) * MAPC);
    for (int c = blockIdx.y * MAPC; c < c1; c++) {
        const A* x = gm + (size_t)c * G.glen;
        const int mk = (c < kmask || mask_rest) ? 1 : 0;
        A* P = planes + (size_t)c * np * G.slen + s;
        P[0] = x[g];
#pragma unroll
        for (int d = 0; d < 3; d++)
            if (d < G.dim) P[(size_t)(d + 1) * G.slen] = vscale(vsub(x[hi[mk][d]], x[lo[mk][d]]), w[mk][d]);
    }
}

// Smith's complex division (Smith 1962)
__device__ __forceinline__ cd cdiv_smith(cd a, cd b)
{
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, den = b.x + b.y * r;
        return cd{(a.x + a.y * r) / den, (a.y - a.x * r) / den};
    }
    const double r = b.x / b.y, den = b.x * r + b.y;
    return cd{(a.x * r + a.y) / den, (a.y * r - a.x) / den};
}

// The factor of each link's row: sc / y for log data (Smith's division for
// complex y), sc for linear data (y null), in FP64, then cast to the
// Jacobian's arithmetic type
template <class C, class V64>
__global__ void grid_yscale_kernel(int nqm, const V64* __restrict__ y, double sc, C* __restrict__ ysc)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nqm) return;
    if constexpr (vt<V64>::cplx) {
        const cd r = y ? cdiv_smith(cd{1.0, 0.0}, y[l]) : cd{1.0, 0.0};
        ysc[l] = vcast<C, cd>(cd{r.x * sc, r.y * sc});
    } else {
        ysc[l] = vcast<C, double>(y ? sc / y[l] : sc);
    }
}

// J stores bypass L2 retention (evict-first), so the 2.4 GB stream of rows
// does not push the field planes out of L2
__device__ __forceinline__ void st_stream(float* p, float v) { __stcs(p, v); }
__device__ __forceinline__ void st_stream(double* p, double v) { __stcs(p, v); }

// The links of a block's GQ sources for LT detectors at a time, in shared
// memory: the link index (or -1) and its factor, read by every thread of the
// block from there instead of from the pair table and the factor array
// (element_jacobian_kernel: 4.10 -> 3.76 ms on the 3D cylinder; the grid
// kernel, at 80 registers with it, lost as much at 48^3 as it gained at 32^3).
constexpr int LT = 64;
template <class V, int GQ>
struct LinkTile {
    int l[GQ][LT];
    V y[GQ][LT];
    // detectors m0 .. m0 + LT - 1 of sources q0 .. q0 + GQ - 1; the caller
    // syncs the block before (the previous tile's readers) and after
    __device__ __forceinline__ void fill(int m0, int q0, int nq, int nm, const int* __restrict__ pair,
                                         const V* __restrict__ ysc)
    {
        for (int i = threadIdx.x; i < GQ * LT; i += blockDim.x) {
            const int g = i / LT, j = i % LT, m = m0 + j;
            const int k = (m < nm && q0 + g < nq) ? pair[(size_t)(q0 + g) * nm + m] : -1;
            l[g][j] = k;
            y[g][j] = k >= 0 ? ysc[k] : vzero<V>();
        }
    }
};

// One thread per (solution point, group of GQ sources): the sources' planes
// stay in registers while the detectors' planes stream past, each loaded once
// per group, the next detector's while this one's entries form.  PMDF_mua =
// -(f a), PMDF_kap = -sum_d (grad_d f)(grad_d a) (jacobian.cc:58-72); LOG
// data are divided by y (complex: PMDF_log, 76-79; real:
// GenerateJacobian_cw, 178-193) and every entry is multiplied by the voxel
// scale (365-370).  ysc[l] carries -scale / y of the link (-scale for LINEAR
// data), so an entry costs one complex product more than its PMDF: a
// division per entry would run on the FP64 pipe.  NP = 1 + dim planes.
// pair[q * nm + m]: link index or -1.  J rows: complex [Re mua | Re kap] at l
// and [Im mua | Im kap] at nQM + l (2 slen columns); real mua at l and kap at
// nQM + l (slen).  With l0 > 0 the kernel serves the sources of one chunk
// whose links are l0 .. l0 + nqm - 1: row l - l0 and nqm + l - l0.
template <class V, class JT, int GQ, int NP>
__global__ void __launch_bounds__(256) grid_jacobian_kernel(int slen, int nq, int nm, int nqm, const V* __restrict__ Fp,
                                                            const V* __restrict__ Ap, const int* __restrict__ pair,
                                                            const V* __restrict__ ysc, JT* __restrict__ J, int l0)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x, q0 = blockIdx.y * GQ;
    if (s >= slen) return;
    V f[GQ][NP];
#pragma unroll
    for (int g = 0; g < GQ; g++)
#pragma unroll
        for (int d = 0; d < NP; d++) f[g][d] = Fp[((size_t)min(q0 + g, nq - 1) * NP + d) * slen + s];
    constexpr bool CPLX = vt<V>::cplx;
    const size_t cols = CPLX ? 2 * (size_t)slen : (size_t)slen;
    V an[NP];
#pragma unroll
    for (int d = 0; d < NP; d++) an[d] = Ap[(size_t)d * slen + s];
    for (int m = 0; m < nm; m++) {
        V a[NP];
#pragma unroll
        for (int d = 0; d < NP; d++) {
            a[d] = an[d];
            if (m + 1 < nm) an[d] = Ap[((size_t)(m + 1) * NP + d) * slen + s];
        }
        int lk[GQ];
        bool any = false;
#pragma unroll
        for (int g = 0; g < GQ; g++) {
            lk[g] = q0 + g < nq ? pair[(size_t)(q0 + g) * nm + m] : -1;
            any |= lk[g] >= 0;
        }
        if (!any) continue;
#pragma unroll
        for (int g = 0; g < GQ; g++) {
            const int l = lk[g];
            if (l < 0) continue;
            const V y = ysc[l];
            V t = vmul(f[g][1], a[1]);
#pragma unroll
            for (int d = 2; d < NP; d++) t = vfma(t, f[g][d], a[d]);
            const V pm = vmul(vmul(f[g][0], a[0]), y), pk = vmul(t, y);
            JT* r0 = J + (size_t)(l - l0) * cols + s;
            JT* r1 = J + (size_t)(l - l0 + nqm) * cols + s;
            if constexpr (CPLX) {
                st_stream(r0, (JT)re(pm));
                st_stream(r1, (JT)im(pm));
                st_stream(r0 + slen, (JT)re(pk));
                st_stream(r1 + slen, (JT)im(pk));
            } else {
                st_stream(r0, (JT)pm);
                st_stream(r1, (JT)pk);
            }
        }
    }
}

// Element-basis Jacobian (GenerateJacobian_mesh with elbasis, jacobian.cc:
// 441-497; CW 738-802 and the LOG scaling 178-193), with IntFG_el /
// IntGradFGradG_el (884-939): per element e and link (q, m),
// sum_ij f_i g_j IntFF(i,j) and sum_ij f_i g_j IntDD(i,j), formed as
// sum_i f_i h_i with h = W g once per (element, detector) and shared by the
// group's GQ sources.  IntFF(i,j) = size (1 + [i = j]) / 12 (triangles) or
// / 20 (tetrahedra), so h_i = size / 12 (or 20) (a_i + sum_j a_j).  NN nodes
// per element (3 or 4).  Fields source-major in the natural numbering.
// ysc[l] = -1 / y for LOG data, -1 for LINEAR.  J: complex (2 nQM) x (2 ne)
// rows -Re / -Im, kappa at column ne + e; real (2 nQM) x ne [mua ; kappa].
template <class V, class JT, int GQ, int NN>
__global__ void __launch_bounds__(256) element_jacobian_kernel(MeshDev m, int nq, int nm, int nqm,
                                                               const V* __restrict__ F, const V* __restrict__ A,
                                                               const int* __restrict__ pair,
                                                               const V* __restrict__ ysc, JT* __restrict__ J)
{
    __shared__ LinkTile<V, GQ> tile;
    const int q0 = blockIdx.y * GQ;
    // threads past ne take part in the tile fills only
    const bool act = blockIdx.x * blockDim.x + threadIdx.x < m.ne;
    const int e = min((int)(blockIdx.x * blockDim.x + threadIdx.x), m.ne - 1);
    using R = typename vt<V>::R;
    const int n = m.n;
    const int* nd = m.el + (size_t)e * NN;
    const double* r = m.rec + (size_t)e * EL_REC;
    const R cff = (R)((NN == 3 ? 1.0 / 12.0 : 1.0 / 20.0) * r[0]);
    R wdd[NN][NN];
    int node[NN];
#pragma unroll
    for (int i = 0; i < NN; i++) {
        node[i] = nd[i];
#pragma unroll
        for (int j = 0; j < NN; j++)
            // IntDD: the record's value for triangles, 4 x it for tetrahedra
            wdd[i][j] = (R)((NN == 4 ? 4.0 : 1.0) * r[1 + i * NN + j]);
    }
    V f[GQ][NN];
#pragma unroll
    for (int g = 0; g < GQ; g++)
#pragma unroll
        for (int i = 0; i < NN; i++) f[g][i] = F[(size_t)min(q0 + g, nq - 1) * n + node[i]];
    constexpr bool CPLX = vt<V>::cplx;
    const size_t cols = CPLX ? 2 * (size_t)m.ne : (size_t)m.ne;
    // the next detector's nodal values load while this one's entries form
    V an[NN];
#pragma unroll
    for (int j = 0; j < NN; j++) an[j] = A[node[j]];
    for (int mm = 0; mm < nm; mm++) {
        const int jt = mm % LT;
        if (jt == 0) {
            __syncthreads();
            tile.fill(mm, q0, nq, nm, pair, ysc);
            __syncthreads();
        }
        V a[NN];
#pragma unroll
        for (int j = 0; j < NN; j++) {
            a[j] = an[j];
            if (mm + 1 < nm) an[j] = A[(size_t)(mm + 1) * n + node[j]];
        }
        bool any = false;
#pragma unroll
        for (int g = 0; g < GQ; g++) any |= tile.l[g][jt] >= 0;
        if (!any || !act) continue;
        V hm[NN], hk[NN];
        V sa = vzero<V>();
#pragma unroll
        for (int j = 0; j < NN; j++) sa = vadd(sa, a[j]);
#pragma unroll
        for (int i = 0; i < NN; i++) {
            hm[i] = vscale(vadd(sa, a[i]), cff);
            hk[i] = vscale(a[0], wdd[i][0]);
#pragma unroll
            for (int j = 1; j < NN; j++) hk[i] = vadd(hk[i], vscale(a[j], wdd[i][j]));
        }
#pragma unroll
        for (int g = 0; g < GQ; g++) {
            const int l = tile.l[g][jt];
            if (l < 0) continue;
            V pm = vmul(f[g][0], hm[0]), pk = vmul(f[g][0], hk[0]);
#pragma unroll
            for (int i = 1; i < NN; i++) {
                pm = vfma(pm, f[g][i], hm[i]);
                pk = vfma(pk, f[g][i], hk[i]);
            }
            const V y = tile.y[g][jt];
            pm = vmul(pm, y);
            pk = vmul(pk, y);
            JT* r0 = J + (size_t)l * cols;
            JT* r1 = J + (size_t)(l + nqm) * cols;
            if constexpr (CPLX) {
                st_stream(r0 + e, (JT)re(pm));
                st_stream(r1 + e, (JT)im(pm));
                st_stream(r0 + m.ne + e, (JT)re(pk));
                st_stream(r1 + m.ne + e, (JT)im(pk));
            } else {
                st_stream(r0 + e, (JT)pm);
                st_stream(r1 + e, (JT)pk);
            }
        }
    }
}

// The data gradient of toast's Gradient (GetGradient / AddDataGradient,
// src/python/toastmodule.cc:1745-1887).  Per link: with y = r + i i the
// linear projection, dn = 1/|y|^2, b = (data - model) / sd for the log
// amplitude and the phase (model = ln|y|, arg y), a = -2 b_mod / sd_mod and
// p = -2 b_arg / sd_arg, the detector vector enters the source's adjoint
// right-hand side twice: times (a r dn, -a i dn), then times (-p i dn, -p r dn).
__global__ void gradient_coef_kernel(int nqm, const cd* __restrict__ ylin, const cd* __restrict__ ylog,
                                     const double* __restrict__ data, const double* __restrict__ sd,
                                     cd* __restrict__ coef)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nqm) return;
    const double rp = ylin[l].x, ip = ylin[l].y, dn = 1.0 / (rp * rp + ip * ip);
    const double bm = (data[l] - ylog[l].x) / sd[l];
    const double ba = (data[nqm + l] - ylog[l].y) / sd[nqm + l];
    double t = -2.0 * bm / (1.0 * sd[l]);
    coef[2 * l] = cd{t * rp * dn, -t * ip * dn};
    t = -2.0 * ba / (1.0 * sd[nqm + l]);
    coef[2 * l + 1] = cd{-t * ip * dn, -t * rp * dn};
}

// adjoint right-hand sides w_q = sum over q's links (in order) of
// mvec_m coef1 + mvec_m coef2, written node-major in the solver's layout
__global__ void gradient_weights_kernel(int n, int nq, const cd* __restrict__ mvec, const int* __restrict__ link_ofs,
                                        const int* __restrict__ link_m, const cd* __restrict__ coef,
                                        const int* __restrict__ perm, cd* __restrict__ W)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
    if (i >= n || q >= nq) return;
    cd w = cd{0.0, 0.0};
    for (int l = link_ofs[q]; l < link_ofs[q + 1]; l++) {
        const cd r = mvec[(size_t)link_m[l] * n + i];
        w = vadd(w, vmul(r, coef[2 * l]));
        w = vadd(w, vmul(r, coef[2 * l + 1]));
    }
    W[(size_t)perm[i] * nq + q] = w;
}

// grad_mua[s] -= Re(f a), grad_kappa[s] -= Re(sum_d grad_d f grad_d a),
// summed over the sources in order (no voxel scaling); grad in/out
__global__ void gradient_accum_kernel(int dim, int slen, int nq, const cd* __restrict__ Pf, const cd* __restrict__ Pa,
                                      double* __restrict__ grad)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= slen) return;
    const int np = 1 + dim;
    double gm = grad[s], gk = grad[slen + s];
    for (int q = 0; q < nq; q++) {
        const cd* f = Pf + (size_t)q * np * slen + s;
        const cd* a = Pa + (size_t)q * np * slen + s;
        gm -= re(vmul(f[0], a[0]));
        cd k = cd{0.0, 0.0};
        for (int d = 1; d < np; d++) k = vadd(k, vmul(f[(size_t)d * slen], a[(size_t)d * slen]));
        gk -= re(k);
    }
    grad[s] = gm;
    grad[slen + s] = gk;
}

// Map_GridToSol (raster.cc:374-390) of Jacobian rows computed on the grid of
// a raster with an intermediate grid: row r of Jg (nb blocks of gslen grid
// points inside the mesh) -> row row0(r) of J (nb blocks of slen solution
// points): J[k] = sum over G's row of the solution point k of w Jg[col], in
// the row's entry order (RCompRowMatrix::Ax).  Rows r < half go to row0 + r,
// the others to row0 + r - half + hoff (the Im / kappa rows of a chunk of
// links).  add: J += instead of J = (the data gradient).  A thread per
// output entry.
template <class JT>
__global__ void grid_to_sol_rows_kernel(long long rows, int half, long long row0, long long hoff, int nb, int gslen,
                                        int slen, const int* __restrict__ rp, const int* __restrict__ col,
                                        const double* __restrict__ val, const JT* __restrict__ Jg,
                                        JT* __restrict__ J, int add)
{
    const long long total = rows * nb * (long long)slen;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % slen);
        const long long rb = t / slen;
        const int b = (int)(rb % nb);
        const long long r = rb / nb;
        const JT* x = Jg + (size_t)r * nb * gslen + (size_t)b * gslen;
        JT acc = (JT)0;
        for (int j = rp[k]; j < rp[k + 1]; j++) acc += (JT)val[j] * x[col[j]];
        const long long orow = r < half ? row0 + r : row0 + r - half + hoff;
        JT* y = J + (size_t)orow * nb * slen + (size_t)b * slen + k;
        *y = add ? *y + acc : acc;
    }
}

// Raster basis maps: y = A x row by row in entry order (RCompRowMatrix::Ax,
// crmatrix_imp.hpp:1168-1189; complex vectors component by component,
// Ax_cplx 1302-1327), one thread per (row, vector), `width` doubles per point.
// div (optional): each row's sum divided by div[row], 0 where that is 0 (a
// blob basis's node average, raster_bl.cc:170-204).
__global__ void csr_apply_kernel(int rows, int cols, int width, const int* __restrict__ rp,
                                 const int* __restrict__ col, const double* __restrict__ val,
                                 const double* __restrict__ x, double* __restrict__ y, const double* __restrict__ div)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y;
    if (r >= rows) return;
    const double* xv = x + (size_t)v * cols * width;
    for (int c = 0; c < width; c++) {
        double acc = 0.0;
        for (int j = rp[r]; j < rp[r + 1]; j++) acc = __dadd_rn(acc, __dmul_rn(val[j], xv[(size_t)col[j] * width + c]));
        if (div) acc = div[r] != 0.0 ? __ddiv_rn(acc, div[r]) : 0.0;
        y[((size_t)v * rows + r) * width + c] = acc;
    }
}

// basis -> solution points (Map_BasisToSol, raster.cc:292-315).  d: the
// pixel raster's real map D->Ax (raster_px.cc:147-150), 0 + 1 x, which
// turns -0 into +0
__global__ void gather_points_kernel(int slen, int glen, int width, const int* __restrict__ sol,
                                     const double* __restrict__ g, double* __restrict__ s, int d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y;
    if (i >= slen) return;
    for (int c = 0; c < width; c++) {
        const double x = g[((size_t)v * glen + sol[i]) * width + c];
        s[((size_t)v * slen + i) * width + c] = d ? __dadd_rn(0.0, x) : x;
    }
}

// solution points -> basis, zeros elsewhere (Map_SolToBasis, raster.cc:
// 318-345; d: the real D->ATx, 0 + 1 x)
__global__ void scatter_points_kernel(int slen, int glen, int width, const int* __restrict__ sol,
                                      const double* __restrict__ s, double* __restrict__ g, int d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y;
    if (i >= slen) return;
    for (int c = 0; c < width; c++) {
        const double x = s[((size_t)v * slen + i) * width + c];
        g[((size_t)v * glen + sol[i]) * width + c] = d ? __dadd_rn(0.0, x) : x;
    }
}

// QVec_Gaussian (src/libstoast/source.cc:19-56) for npos positions on the
// device: a thread per (node, position) gathers the contributions the
// reference scatters, in the reference's order (elements ascending, then the
// element's source nodes i ascending): q[js] += s_i BndIntFF(i, j) (Neumann:
// boundary source and receiving nodes only) or s_i IntFF(i, j), with
// s_i = exp(-d_i^2 / 2w^2) fac1.  scale (optional, n values) multiplies the
// result (detector vectors times c2a, toastmodule.cc:1189-1220).
__global__ void qvec_gaussian_kernel(int n, int dim, int nn, const double* __restrict__ coords,
                                     const int* __restrict__ el, const int* __restrict__ nel_ptr,
                                     const int* __restrict__ nel_list, const unsigned char* __restrict__ bnd,
                                     const double* __restrict__ intbff, const double* __restrict__ rec, int rec_len,
                                     int npos, const double* __restrict__ pos, double fac1, double fac2, int neumann,
                                     const double* __restrict__ scale, double* __restrict__ q)
{
    const int js = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y;
    if (js >= n || p >= npos) return;
    double acc = 0.0;
    if (!neumann || bnd[js]) {
        const double* c = pos + (size_t)p * dim;
        for (int t = nel_ptr[js]; t < nel_ptr[js + 1]; t++) {
            const int e = nel_list[t] >> 2, j = nel_list[t] & 3;
            const int* nd = el + (size_t)e * nn;
            for (int i = 0; i < nn; i++) {
                const int is = nd[i];
                if (neumann && !bnd[is]) continue;
                double d2 = 0.0;
                for (int k = 0; k < dim; k++) {
                    const double dk = c[k] - coords[(size_t)is * dim + k];
                    d2 += dk * dk;
                }
                const double d = sqrt(d2);
                const double sv = exp(d * d * fac2) * fac1;
                if (neumann) acc += sv * intbff[((size_t)e * nn + i) * nn + j];
                else acc += sv * ((i == j ? 2.0 : 1.0) * (dim == 2 ? 1.0 / 12.0 : 1.0 / 20.0) * rec[(size_t)e * rec_len]);
            }
        }
    }
    q[(size_t)p * n + js] = scale ? acc * scale[js] : acc;
}

}  // namespace tg
