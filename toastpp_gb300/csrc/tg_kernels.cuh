// tg_kernels.cuh -- device kernels of the forward path.
//
// Block-vector layout: node-major, X[i * ld + c] (ld >= k right-hand sides).
// Dot products that steer the Krylov methods are computed in a fixed order
// that does not depend on how many right-hand sides share the launch: every
// ROW_TILE-row tile of a column is summed sequentially in row order into a
// partial (one thread per column), and the partials of a column are reduced by
// reduce_finalize_kernel in a fixed tree.  A column therefore gets bitwise the
// same scalars alone and inside any batch.
#pragma once
#include "tg_common.cuh"
#include "tg_mesh.cuh"

namespace tg {

// Per-column Krylov state (one right-hand side each).  active: 1 iterating,
// 0 finished, -1 finishing on the |s| test of the real BiCGSTAB variant.
struct ColState {
    double rho, rhop, alpha, omega, beta, dnew, dold, bnorm, err, tol;
    int its, active, status, maxit;
    int rel;  // reliable update of the mixed path: 1 resume the Krylov process, 2 restart it
    // mixed path: the FP32 process works on (true residual) / scale, a power
    // of two of the last true residual norm, so its values stay O(1)
    double scale, scale_prev;
    // COCG (complex symmetric CG) scalars, complex: rho = r.z, alpha, beta
    double zr, zi, ar, ai, br, bi;
    int nupd;  // residual replacements this column has taken
    // mixed path: componentwise backward error of the FP64 solution at its
    // last true residual (max_i |r_i| / (|A| |x| + |b|)_i)
    double berr;
};

// 2^floor(log2 x) for x > 0 finite, else 1: scaling by it is exact
__host__ __device__ __forceinline__ double pow2_floor(double x)
{
    return (x > 0.0 && isfinite(x)) ? ldexp(1.0, ilogb(x)) : 1.0;
}

// ---------------------------------------------------------------------------
// Assembly: one thread per CSR entry gathers its element contributions in
// element order, mode by mode, as TFwdSolver::AssembleSystemMatrix does with
// one thread (src/libstoast/fwdsolver.cc:337-357, 404-424; AddToElMatrix,
// src/libfe/mesh.cc:1958-2129; AddToSysMatrix iCFF, mesh.cc:2252-2282).
// ---------------------------------------------------------------------------

static __constant__ int c_tet_fff[4][4][4] = {  // Tet4 IntFFF planes x120 (tet4.cc:49-77)
    {{6,2,2,2},{2,2,1,1},{2,1,2,1},{2,1,1,2}},
    {{2,2,1,1},{2,6,2,2},{1,2,2,1},{1,2,1,2}},
    {{2,1,2,1},{1,2,2,1},{2,2,6,2},{1,1,2,2}},
    {{2,1,1,2},{1,2,1,2},{1,1,2,2},{2,2,2,6}}};
// the same divided by 120, as the reference divides each entry (folded here:
// the quotient is the correctly rounded one either way)
static __constant__ double c_tet_fff120[4][4][4] = {
    {{6.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0}, {2.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0, 1.0 / 120.0}, {2.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0}, {2.0 / 120.0, 1.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0}},
    {{2.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0, 1.0 / 120.0}, {2.0 / 120.0, 6.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0}, {1.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0}, {1.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0}},
    {{2.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0}, {1.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0}, {2.0 / 120.0, 2.0 / 120.0, 6.0 / 120.0, 2.0 / 120.0}, {1.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0}},
    {{2.0 / 120.0, 1.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0}, {1.0 / 120.0, 2.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0}, {1.0 / 120.0, 1.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0}, {2.0 / 120.0, 2.0 / 120.0, 2.0 / 120.0, 6.0 / 120.0}}};
static __constant__ int c_tet_bfff[4][4][4][4] = {  // Tet4 face IntFFF tables x60 (tet4.cc:724-817)
    { {{6,2,2,0},{2,2,1,0},{2,1,2,0},{0,0,0,0}}, {{2,2,1,0},{2,6,2,0},{1,2,2,0},{0,0,0,0}},
      {{2,1,2,0},{1,2,2,0},{2,2,6,0},{0,0,0,0}}, {{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0}} },
    { {{6,2,0,2},{2,2,0,1},{0,0,0,0},{2,1,0,2}}, {{2,2,0,1},{2,6,0,2},{0,0,0,0},{1,2,0,2}},
      {{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0}}, {{2,1,0,2},{1,2,0,2},{0,0,0,0},{2,2,0,6}} },
    { {{6,0,2,2},{0,0,0,0},{2,0,2,1},{2,0,1,2}}, {{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0}},
      {{2,0,2,1},{0,0,0,0},{2,0,6,2},{1,0,2,2}}, {{2,0,1,2},{0,0,0,0},{1,0,2,2},{2,0,2,6}} },
    { {{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0}}, {{0,0,0,0},{0,6,2,2},{0,2,2,1},{0,2,1,2}},
      {{0,0,0,0},{0,2,2,1},{0,2,6,2},{0,1,2,2}}, {{0,0,0,0},{0,2,1,2},{0,1,2,2},{0,2,2,6}} } };

// Triangle3::IntPFF (tri3.cc:325-353)
__device__ __forceinline__ double tri_intpff(double sz, int i, int j, double p0, double p1, double p2)
{
    const double i30 = 1.0 / 30.0;
    if (i < j) { int t = i; i = j; j = t; }
    switch (i * 3 + j) {
    case 0: return sz * i30 * (3.0 * p0 + p1 + p2);
    case 3: return sz * i30 * (p0 + p1 + 0.5 * p2);
    case 4: return sz * i30 * (p0 + 3.0 * p1 + p2);
    case 6: return sz * i30 * (p0 + 0.5 * p1 + p2);
    case 7: return sz * i30 * (0.5 * p0 + p1 + p2);
    default: return sz * i30 * (p0 + p1 + 3.0 * p2);
    }
}

template <bool CPLX>
__global__ void assemble_kernel(MeshDev m, const double* __restrict__ cmua, const double* __restrict__ ckap,
                                const double* __restrict__ c2a, double omega, double* __restrict__ val)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.nnz) return;
    double pff = 0.0, pdd = 0.0, bnd = 0.0, iff = 0.0;
    for (int c = m.asm_ptr[k]; c < m.asm_ptr[k + 1]; c++) {
        int code = m.asm_list[c];
        int e = code >> 4, i = (code >> 2) & 3, j = code & 3;
        const double* r = m.rec + (size_t)e * EL_REC;
        const int* nd = m.el + (size_t)e * m.nn;
        double sz = r[0];
        if (m.dim == 2) {
            pff += tri_intpff(sz, i, j, cmua[nd[0]], cmua[nd[1]], cmua[nd[2]]);
            pdd += r[1 + i * 3 + j] * ((ckap[nd[0]] + ckap[nd[1]] + ckap[nd[2]]) / 3.0);
            bnd += r[10 + i * 3 + j] * ((c2a[nd[0]] + c2a[nd[1]] + c2a[nd[2]]) / 3.0);
            if (CPLX) iff += (((i == j ? 2.0 : 1.0) * (1.0 / 12.0)) * sz) * omega;
        } else {
            double p0 = cmua[nd[0]], p1 = cmua[nd[1]], p2 = cmua[nd[2]], p3 = cmua[nd[3]];
            pff += (c_tet_fff120[0][i][j] * p0 + c_tet_fff120[1][i][j] * p1 + c_tet_fff120[2][i][j] * p2 +
                    c_tet_fff120[3][i][j] * p3) * sz;
            double res = 0.0;
            for (int q = 0; q < 4; q++) res += ckap[nd[q]];
            pdd += res * r[1 + i * 4 + j];
            int mask = (int)r[21];
            double b = 0.0;
            if (mask) {
                for (int sd = 0; sd < 4; sd++) {
                    if (!(mask & (1 << sd))) continue;
                    double sres = 0.0;
                    for (int q = 0; q < 4; q++) sres += c2a[nd[q]] * (c_tet_bfff[sd][q][i][j] * (2.0 / 120.0));
                    b += sres * r[17 + sd];
                }
            }
            bnd += b;
            if (CPLX) iff += (((i == j ? 2.0 : 1.0) * (1.0 / 20.0)) * sz) * omega;
        }
    }
    double v = 0.0;
    v += pff;
    v += pdd;
    v += bnd;
    if (CPLX) { val[2 * k] = v; val[2 * k + 1] = iff; }
    else val[k] = v;
}

// Element-basis assembly (AddToElMatrix modes ASSEMBLE_PFF_EL, PDD_EL,
// BNDPFF_EL, src/libfe/mesh.cc:1985-1993, for TFwdSolver::Reset with
// elbasis, fwdsolver.cc:337-357 / 404-424): one coefficient per element,
// entry = IntFF(i,j) c_e (tri3.cc:285-292, tet4.cc:348-355), IntDD(i,j) k_e,
// BndIntFF(i,j) a_e; the three passes summed in the reference's order
template <bool CPLX>
__global__ void assemble_el_kernel(MeshDev m, const double* __restrict__ cmua, const double* __restrict__ ckap,
                                   const double* __restrict__ c2a, double omega, double* __restrict__ val)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.nnz) return;
    double pff = 0.0, pdd = 0.0, bnd = 0.0, iff = 0.0;
    const int nn = m.nn;
    const double ffd = m.dim == 2 ? 1.0 / 12.0 : 1.0 / 20.0;
    for (int c = m.asm_ptr[k]; c < m.asm_ptr[k + 1]; c++) {
        int code = m.asm_list[c];
        int e = code >> 4, i = (code >> 2) & 3, j = code & 3;
        const double* r = m.rec + (size_t)e * EL_REC;
        const double sz = r[0];
        const double intff = ((i == j ? 2.0 : 1.0) * ffd) * sz;
        pff += intff * cmua[e];
        // the record holds IntDD for triangles and IntDD / 4 (the IntFDD
        // factor, exact) for tetrahedra (Tetrahedron4::ComputeIntDD, tet4.cc:1016-1031)
        pdd += (m.dim == 3 ? 4.0 * r[1 + i * nn + j] : r[1 + i * nn + j]) * ckap[e];
        bnd += m.intbff[((size_t)e * nn + i) * nn + j] * c2a[e];
        if (CPLX) iff += intff * omega;
    }
    double v = 0.0;
    v += pff;
    v += pdd;
    v += bnd;
    if (CPLX) { val[2 * k] = v; val[2 * k + 1] = iff; }
    else val[k] = v;
}

// ---------------------------------------------------------------------------
// IC(0) (IncompleteCholeskyFactorize, src/libmath/crmatrix_imp.hpp:2166-2203,
// recover = true; complex pivots compared by squared magnitude,
// src/libmath/mathdef.h:128-132) and its apply (CholeskySubst,
// crmatrix_imp.hpp:2267-2295: forward (L + D) y = b by rows, backward
// (D + L^T) x = y by columns), both scheduled by levels of the dependency
// graph of the natural ordering, so the arithmetic is the reference's.
// L(j,i) lives at Umap[u] for column i; its A entry a_ji is at Lapos[Umap[u]].
// ---------------------------------------------------------------------------
// Whole IC(0) apply in one launch: one CTA per group of CG right-hand-side
// columns walks every forward level, then every backward level, of the
// dependency schedule; the only synchronisation is __syncthreads between
// levels (the columns of one CTA never depend on another CTA).  Rows of a
// level are spread over the CTA's threads; each thread does CG columns.
// ---------------------------------------------------------------------------
template <class V>
__global__ void ic_factor_level(MeshDev m, ICDev ic, const int* __restrict__ rows, int nrows, const V* __restrict__ A,
                                V* __restrict__ L, V* __restrict__ dinv)
{
    // a warp per row: every lane forms the pivot (the same sums in the same
    // order), then the lanes share the column's entries L(j, i), each of
    // which depends only on rows of earlier levels
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (t >= nrows) return;
    int i = rows[t];
    const int ikey = ic.key[i];
    V diag = A[m.diagpos[i]];
    V x = vzero<V>();
    int l0 = ic.Lrowptr[i], l1 = ic.Lrowptr[i + 1];
    for (int k = l0; k < l1; k++) x = vfma(x, L[k], L[k]);
    V di;
    bool pos = vt<V>::cplx ? (nrm2(diag) > nrm2(x)) : (re(diag) > re(x));
    if (pos) {
        if constexpr (vt<V>::cplx) di = csqrt_d(vsub(diag, x));
        else di = sqrt(diag - x);
    } else {
        if constexpr (vt<V>::cplx) di = V{1e-10, 0.0};
        else di = 1e-10;
    }
    for (int u = ic.Ucolptr[i] + lane; u < ic.Ucolptr[i + 1]; u += 32) {
        int j = ic.Urow[u];
        // row_mult (crmatrix_imp.hpp:1971-2009): sum over columns ranked before i of L(i,c) L(j,c)
        V s = vzero<V>();
        int a = l0, b = ic.Lrowptr[j], be = ic.Lrowptr[j + 1];
        while (a < l1 && b < be) {
            int ca = ic.Lkey[a], cb = ic.Lkey[b];  // ranks in the elimination ordering (the merge order)
            if (cb >= ikey) break;
            if (ca < cb) a++;
            else if (ca > cb) b++;
            else { s = vfma(s, L[a], L[b]); a++; b++; }
        }
        // a_ji = a_ij (symmetric pattern and values); a fill entry of a
        // complete factor has no entry in A (Lapos -1)
        const int ap = ic.Lapos[ic.Umap[u]];
        V aij = ap >= 0 ? A[ap] : vzero<V>();
        L[ic.Umap[u]] = vdiv(vsub(aij, s), di);
    }
    if (lane == 0) dinv[i] = vrecip(di);
}

// Level-scheduled sweeps of the IC(0) apply: one kernel per level, spread
// over the whole GPU (lane -> (row of the level, column)).
template <class V, class S>
__global__ void ic_fwd_level(ICDev ic, const int* __restrict__ rows, int nrows, int k, int ld, int cw,
                             const V* __restrict__ L, const V* __restrict__ dinv, const V* __restrict__ b,
                             V* __restrict__ y, const ColState* __restrict__ st)
{
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    int lane = threadIdx.x & 31;
    int rpw = 32 / cw;                         // rows per warp
    int ncg = (k + cw - 1) / cw;               // column groups
    int item = gw * rpw + lane / cw;           // (row, column group) item
    if (item >= nrows * ncg) return;
    int r = item / ncg, cg = item % ncg;
    int c = cg * cw + (lane % cw);
    if (c >= k || (st && st[c].active != 1)) return;
    int i = rows[r];
    V s = b[(size_t)i * ld + c];
    for (int q = ic.Lrowptr[i]; q < ic.Lrowptr[i + 1]; q++) s = vfms(s, L[q], y[(size_t)ic.Lcolidx[q] * ld + c]);
    y[(size_t)i * ld + c] = vmul(s, dinv[i]);
}

template <class V, class S>
__global__ void ic_bwd_level(ICDev ic, const int* __restrict__ rows, int nrows, int k, int ld, int cw,
                             const V* __restrict__ L, const V* __restrict__ dinv, V* __restrict__ x,
                             const ColState* __restrict__ st)
{
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    int lane = threadIdx.x & 31;
    int rpw = 32 / cw;
    int ncg = (k + cw - 1) / cw;
    int item = gw * rpw + lane / cw;
    if (item >= nrows * ncg) return;
    int r = item / ncg, cg = item % ncg;
    int c = cg * cw + (lane % cw);
    if (c >= k || (st && st[c].active != 1)) return;
    int i = rows[r];
    V s = x[(size_t)i * ld + c];
    for (int u = ic.Ucolptr[i + 1] - 1; u >= ic.Ucolptr[i]; u--) s = vfms(s, L[ic.Umap[u]], x[(size_t)ic.Urow[u] * ld + c]);
    x[(size_t)i * ld + c] = vmul(s, dinv[i]);
}


// ---------------------------------------------------------------------------
// Tile dot partials.  A ROW_TILE-row tile is split into TILE_RG interleaved
// row groups (rows r0+g, r0+g+TILE_RG, ...); each (group, column) is summed
// sequentially by one thread, and the groups are then added in ascending
// order.  The order depends only on the row numbering, never on k.
// ---------------------------------------------------------------------------
constexpr int TILE_RG = 8;
constexpr int TILE_CK = 128;  // columns per chunk of the shared-memory staging

struct TileAcc {
    // sh: [np][TILE_RG][TILE_CK]
    double* sh;
    __device__ void put(int p, int g, int cc, double v) { sh[(p * TILE_RG + g) * TILE_CK + cc] = v; }
    __device__ double sum(int p, int cc) const
    {
        double a = 0.0;
        for (int g = 0; g < TILE_RG; g++) a += sh[(p * TILE_RG + g) * TILE_CK + cc];
        return a;
    }
};

// y-dots of a tile: part0 = sum Re(conj(w) y) (w != null), part1 = sum |y|^2
template <class V>
__device__ __forceinline__ void tile_dots(int r0, int r1, int k, int ld, const V* __restrict__ y,
                                          const V* __restrict__ w, int want_n2, double* __restrict__ part, int np,
                                          int ntiles, int tile, const ColState* __restrict__ st, int cbeg = 0)
{
    // want_n2: 0 -> [Re(conj(w) y)], 1 -> [Re(conj(w) y)], |y|^2 (the first
    // only with w), 2 -> the bilinear w.y as [Re, Im] (COCG)
    // columns [cbeg, k) of the tile (a block that owns a column range passes
    // its range; the per-column order is the same)
    using S = typename vt<V>::R;  // a thread's few rows sum in the value's own precision
    __shared__ double sh[2 * TILE_RG * TILE_CK];
    TileAcc T{sh};
    for (int c0 = cbeg; c0 < k; c0 += TILE_CK) {
        const int ck = min(TILE_CK, k - c0);
        for (int it = threadIdx.x; it < ck * TILE_RG; it += blockDim.x) {
            const int cc = it % ck, g = it / ck, c = c0 + cc;
            S d0 = 0, d1 = 0;
            if (!(st && st[c].active != 1))
#pragma unroll 4
                for (int r = r0 + g; r < r1; r += TILE_RG) {
                    V yv = y[(size_t)r * ld + c];
                    if (want_n2 == 2) {
                        const V pr = vmul(w[(size_t)r * ld + c], yv);
                        d0 += re(pr);
                        d1 += im(pr);
                        continue;
                    }
                    if (w) d0 += redot(w[(size_t)r * ld + c], yv);
                    if (want_n2) d1 += nrm2(yv);
                }
            T.put(0, g, cc, (double)d0);
            T.put(1, g, cc, (double)d1);
        }
        __syncthreads();
        for (int cc = threadIdx.x; cc < ck; cc += blockDim.x) {
            const int c = c0 + cc;
            if (st && st[c].active != 1) continue;
            if (want_n2 == 2) {
                part[((size_t)c * np) * ntiles + tile] = T.sum(0, cc);
                part[((size_t)c * np + 1) * ntiles + tile] = T.sum(1, cc);
                continue;
            }
            int p = 0;
            if (w) part[((size_t)c * np + p++) * ntiles + tile] = T.sum(0, cc);
            if (want_n2) part[((size_t)c * np + p) * ntiles + tile] = T.sum(1, cc);
        }
        __syncthreads();
    }
}

// warp shuffle of value types
__device__ __forceinline__ double shfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float shfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ cd shfl(cd v, int src) { return cd{__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src)}; }
__device__ __forceinline__ cf shfl(cf v, int src) { return cf{__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src)}; }

// Sparse row times a block of k >= 32 columns, one warp: the row's (up to 32
// per pass) indices and values are loaded cooperatively and broadcast by
// shuffle; lane owns columns lane + 32 j (j < NJ); the gathers of UNR entries
// are issued together so that many loads are in flight per lane.
template <class V, int NJ, bool MINUS>
__device__ __forceinline__ void warp_row_gather(const int* __restrict__ cidx, const V* __restrict__ vals,
                                                const int* __restrict__ vmap, int q0, int q1, int k, int ld,
                                                const V* __restrict__ x, V (&acc)[NJ], int lane)
{
    constexpr int UNR = 4;
    for (int base = q0; base < q1; base += 32) {
        int cnt = min(32, q1 - base);
        int my_c = 0;
        V my_v = vzero<V>();
        if (lane < cnt) {
            my_c = cidx[base + lane];
            my_v = vals[vmap ? vmap[base + lane] : base + lane];
        }
        for (int e = 0; e < cnt; e += UNR) {
            int cc[UNR];
            V av[UNR];
#pragma unroll
            for (int u = 0; u < UNR; u++) {
                cc[u] = __shfl_sync(0xffffffffu, my_c, min(e + u, 31));
                av[u] = shfl(my_v, min(e + u, 31));
            }
            V g[UNR][NJ];
#pragma unroll
            for (int u = 0; u < UNR; u++)
#pragma unroll
                for (int j = 0; j < NJ; j++) {
                    int c = lane + 32 * j;
                    g[u][j] = (e + u < cnt && c < k) ? x[(size_t)cc[u] * ld + c] : vzero<V>();
                }
#pragma unroll
            for (int u = 0; u < UNR; u++)
                if (e + u < cnt)
#pragma unroll
                    for (int j = 0; j < NJ; j++)
                        acc[j] = MINUS ? vfms(acc[j], av[u], g[u][j]) : vfma(acc[j], av[u], g[u][j]);
        }
    }
}

// SpMM for k >= 32 (NJ = ceil(k/32) <= 8): warp per row within a row tile,
// then the tile-sequential dot partials.
template <class V, int NJ>
__global__ void __launch_bounds__(256) spmm_wide_kernel(int n, const int* __restrict__ rowptr,
                                                        const int* __restrict__ colidx, const V* __restrict__ A, int k,
                                                        int ld, const V* __restrict__ x, V* __restrict__ y,
                                                        const V* __restrict__ w, int want_n2, double* __restrict__ part,
                                                        int np, int ntiles, const ColState* __restrict__ st)
{
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int r = r0 + warp; r < r1; r += nwarp) {
        V acc[NJ];
#pragma unroll
        for (int j = 0; j < NJ; j++) acc[j] = vzero<V>();
        warp_row_gather<V, NJ, false>(colidx, A, nullptr, rowptr[r], rowptr[r + 1], k, ld, x, acc, lane);
#pragma unroll
        for (int j = 0; j < NJ; j++) {
            int c = lane + 32 * j;
            if (c < k && !(st && st[c].active != 1)) y[(size_t)r * ld + c] = acc[j];
        }
    }
    if (!w && !want_n2) return;
    __syncthreads();
    tile_dots<V>(r0, r1, k, ld, y, w, want_n2, part, np, ntiles, tile, st);
}

// 16-byte words of a block-vector row: P = values per word
template <class V>
struct alignas(16) W16 {
    static constexpr int P = 16 / sizeof(V);
    V v[P];
};

// SpMM for k a multiple of W16<V>::P: warp per row of the tile, lane owns the
// 16-byte words lane + 32 j (j < NW) of the row.  Every lane reads the entry's
// column and value itself (one broadcast transaction), so an entry costs one
// address computation and NW 128-bit gathers.
template <class V, int NW>
__global__ void __launch_bounds__(256) spmm_vec_kernel(int n, const int* __restrict__ rowptr,
                                                       const int* __restrict__ colidx, const V* __restrict__ A, int k,
                                                       int ld, const V* __restrict__ x, V* __restrict__ y,
                                                       const V* __restrict__ w, int want_n2,
                                                       double* __restrict__ part, int np, int ntiles,
                                                       const ColState* __restrict__ st)
{
    constexpr int P = W16<V>::P;
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    const int nwords = k / P, ldw = ld / P;
    const W16<V>* X = reinterpret_cast<const W16<V>*>(x);
    W16<V>* Y = reinterpret_cast<W16<V>*>(y);
    for (int r = r0 + warp; r < r1; r += nwarp) {
        W16<V> acc[NW];
#pragma unroll
        for (int j = 0; j < NW; j++)
#pragma unroll
            for (int p = 0; p < P; p++) acc[j].v[p] = vzero<V>();
        const int q1 = rowptr[r + 1];
        int q = rowptr[r];
        for (; q + 2 <= q1; q += 2) {
            const int c0 = colidx[q], c1 = colidx[q + 1];
            const V a0 = A[q], a1 = A[q + 1];
            const W16<V>* x0 = X + (size_t)c0 * ldw;
            const W16<V>* x1 = X + (size_t)c1 * ldw;
            W16<V> g0[NW], g1[NW];
#pragma unroll
            for (int j = 0; j < NW; j++) {
                const int wi = lane + 32 * j;
                if (wi < nwords) { g0[j] = x0[wi]; g1[j] = x1[wi]; }
            }
#pragma unroll
            for (int j = 0; j < NW; j++)
#pragma unroll
                for (int p = 0; p < P; p++) {
                    acc[j].v[p] = vfma(acc[j].v[p], a0, g0[j].v[p]);
                    acc[j].v[p] = vfma(acc[j].v[p], a1, g1[j].v[p]);
                }
        }
        if (q < q1) {
            const int c0 = colidx[q];
            const V a0 = A[q];
            const W16<V>* x0 = X + (size_t)c0 * ldw;
#pragma unroll
            for (int j = 0; j < NW; j++) {
                const int wi = lane + 32 * j;
                if (wi < nwords) {
                    W16<V> g = x0[wi];
#pragma unroll
                    for (int p = 0; p < P; p++) acc[j].v[p] = vfma(acc[j].v[p], a0, g.v[p]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NW; j++) {
            const int wi = lane + 32 * j;
            if (wi >= nwords) continue;
            if (st) {  // inactive columns keep their values
                W16<V> o = acc[j];
                bool all = true;
#pragma unroll
                for (int p = 0; p < P; p++) all &= st[wi * P + p].active == 1;
                if (all) { Y[(size_t)r * ldw + wi] = o; continue; }
#pragma unroll
                for (int p = 0; p < P; p++)
                    if (st[wi * P + p].active == 1) y[(size_t)r * ld + wi * P + p] = o.v[p];
            } else {
                Y[(size_t)r * ldw + wi] = acc[j];
            }
        }
    }
    if (!w && !want_n2) return;
    __syncthreads();
    tile_dots<V>(r0, r1, k, ld, y, w, want_n2, part, np, ntiles, tile, st);
}

// asynchronous global -> shared copy of one value (LDGSTS), B = 4, 8 or 16 bytes
template <int B>
__device__ __forceinline__ void cp_async_val(void* dst, const void* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (B == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// SpMM with the tile's source rows staged in shared memory.  The ROW_TILE
// rows of a tile reference halo_ptr[t+1] - halo_ptr[t] distinct rows of x
// (about a third of their entries on a Morton-ordered 3D mesh).  Block =
// (tile, chunk of HALO_CW 16-byte words): it copies that chunk of the
// distinct rows once (cp.async) and the tile's values and local indices,
// then HALO_CW lanes per row apply the entries in CSR order (as
// spmm_vec_kernel) from shared memory, and the block forms the dot partials
// of its own columns.  Small blocks and no chunk loop: many blocks per SM
// hide the gather latency.
constexpr int HALO_CW = 8;       // 16-byte words per block = lanes per row
constexpr int HALO_MAXE = 1024;  // entries of a tile held in shared memory

template <class V>
__global__ void __launch_bounds__(256) spmm_halo_kernel(int n, const int* __restrict__ rowptr,
                                                        const unsigned short* __restrict__ lcol,
                                                        const int* __restrict__ halo_ptr,
                                                        const int* __restrict__ halo_col, const V* __restrict__ A,
                                                        int k, int ld, const V* __restrict__ x, V* __restrict__ y,
                                                        const V* __restrict__ w, int want_n2,
                                                        double* __restrict__ part, int np, int ntiles,
                                                        const ColState* __restrict__ st, int hmax)
{
    constexpr int P = W16<V>::P;
    extern __shared__ __align__(16) unsigned char hsm[];
    W16<V>* sx = reinterpret_cast<W16<V>*>(hsm);                       // [hmax][HALO_CW]
    V* sa = reinterpret_cast<V*>(sx + (size_t)hmax * HALO_CW);          // [HALO_MAXE]
    unsigned short* sl = reinterpret_cast<unsigned short*>(sa + HALO_MAXE);  // [HALO_MAXE]
    __shared__ int srp[ROW_TILE + 1];
    const int tile = blockIdx.x, w0 = blockIdx.y * HALO_CW;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    const int h0 = halo_ptr[tile], nh = halo_ptr[tile + 1] - h0;
    const int nwords = k / P, ldw = ld / P;
    const int cw = min(HALO_CW, nwords - w0);
    const W16<V>* X = reinterpret_cast<const W16<V>*>(x);
    W16<V>* Y = reinterpret_cast<W16<V>*>(y);
    for (int e = threadIdx.x; e < nh * cw; e += blockDim.x) {
        const int h = e / cw, ww = e - h * cw;
        cp_async_val<16>(&sx[h * HALO_CW + ww], &X[(size_t)halo_col[h0 + h] * ldw + w0 + ww]);
    }
    cp_async_commit();
    const int e0 = rowptr[r0], ne = rowptr[r1] - e0;
    const bool sm_entries = ne <= HALO_MAXE;
    for (int t = threadIdx.x; t <= r1 - r0; t += blockDim.x) srp[t] = rowptr[r0 + t] - e0;
    if (sm_entries)
        for (int t = threadIdx.x; t < ne; t += blockDim.x) { sa[t] = A[e0 + t]; sl[t] = lcol[e0 + t]; }
    cp_async_wait<0>();
    __syncthreads();
    const int grp = threadIdx.x / HALO_CW, l = threadIdx.x % HALO_CW, ngrp = blockDim.x / HALO_CW;
    if (l < cw) {
        const int wi = w0 + l;
        for (int r = r0 + grp; r < r1; r += ngrp) {
            W16<V> acc;
#pragma unroll
            for (int p = 0; p < P; p++) acc.v[p] = vzero<V>();
            const int q0 = srp[r - r0], q1 = srp[r - r0 + 1];
            if (sm_entries) {
#pragma unroll 4
                for (int q = q0; q < q1; q++) {
                    const V a = sa[q];
                    const W16<V> g = sx[sl[q] * HALO_CW + l];
#pragma unroll
                    for (int p = 0; p < P; p++) acc.v[p] = vfma(acc.v[p], a, g.v[p]);
                }
            } else {
#pragma unroll 4
                for (int q = q0; q < q1; q++) {
                    const V a = A[e0 + q];
                    const W16<V> g = sx[lcol[e0 + q] * HALO_CW + l];
#pragma unroll
                    for (int p = 0; p < P; p++) acc.v[p] = vfma(acc.v[p], a, g.v[p]);
                }
            }
            if (st) {  // inactive columns keep their values
                bool all = true;
#pragma unroll
                for (int p = 0; p < P; p++) all &= st[wi * P + p].active == 1;
                if (all) Y[(size_t)r * ldw + wi] = acc;
                else
#pragma unroll
                    for (int p = 0; p < P; p++)
                        if (st[wi * P + p].active == 1) y[(size_t)r * ld + wi * P + p] = acc.v[p];
            } else {
                Y[(size_t)r * ldw + wi] = acc;
            }
        }
    }
    if (!w && !want_n2) return;
    __syncthreads();
    tile_dots<V>(r0, r1, (w0 + cw) * P, ld, y, w, want_n2, part, np, ntiles, tile, st, w0 * P);
}

// IC(0) level kernel on the level's ELL entries (k >= 32): warp per (slot,
// column group); the slot's entries sit at slot * w, so the row's indices,
// values, right-hand side and pivot load in one round and the gathers in the
// next.  blockIdx.y selects the group of 32 * NJ columns a warp owns: a row's
// columns split over gridDim.y warps, so a level of few rows still fills the
// GPU and each warp carries fewer gathers.
// Launched as a programmatic dependent of the previous level: it lets the
// next level start at once (griddepcontrol.launch_dependents), loads what no
// kernel of the sweep writes (the level's rows, ELL indices and values,
// pivots), and only then waits for the previous level's completion
// (griddepcontrol.wait, a no-op after an ordinary launch).
template <class V, int NJ, bool FWD>
__global__ void __launch_bounds__(256) ic_level_ell(const int* __restrict__ rows, int nrows, int w,
                                                    const int* __restrict__ ecol, const V* __restrict__ eval, int k,
                                                    int ld, const V* __restrict__ dinv, const V* __restrict__ b,
                                                    V* __restrict__ y, const ColState* __restrict__ st)
{
    const int slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int c0 = blockIdx.y * 32 * NJ;  // this warp's first column
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const bool live = slot < nrows && c0 < k;
    int i = 0, my_c0 = -1;
    V di = vzero<V>(), my_v0 = vzero<V>();
    if (live) {
        i = rows[slot];
        di = dinv[i];
        if (lane < min(32, w)) {
            my_c0 = ecol[(size_t)slot * w + lane];
            my_v0 = eval[(size_t)slot * w + lane];
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (!live) return;
    V acc[NJ];
#pragma unroll
    for (int j = 0; j < NJ; j++) {
        int c = c0 + lane + 32 * j;
        acc[j] = c < k ? (FWD ? b[(size_t)i * ld + c] : y[(size_t)i * ld + c]) : vzero<V>();
    }
    constexpr int UNR = 4;  // entries whose gathers are in flight together
    for (int base = 0; base < w; base += 32) {
        const int cnt = min(32, w - base);
        int my_c = my_c0;
        V my_v = my_v0;
        if (base > 0) {
            my_c = -1;
            my_v = vzero<V>();
            if (lane < cnt) {
                my_c = ecol[(size_t)slot * w + base + lane];
                my_v = eval[(size_t)slot * w + base + lane];
            }
        }
        for (int e = 0; e < cnt; e += UNR) {
            int cc[UNR];
            V av[UNR];
#pragma unroll
            for (int u = 0; u < UNR; u++) {
                cc[u] = __shfl_sync(0xffffffffu, my_c, min(e + u, 31));
                av[u] = shfl(my_v, min(e + u, 31));
            }
            V g[UNR][NJ];
#pragma unroll
            for (int u = 0; u < UNR; u++)
#pragma unroll
                for (int j = 0; j < NJ; j++) {
                    int c = c0 + lane + 32 * j;
                    g[u][j] = (e + u < cnt && cc[u] >= 0 && c < k) ? y[(size_t)cc[u] * ld + c] : vzero<V>();
                }
#pragma unroll
            for (int u = 0; u < UNR; u++)
                if (e + u < cnt && cc[u] >= 0)
#pragma unroll
                    for (int j = 0; j < NJ; j++) acc[j] = vfms(acc[j], av[u], g[u][j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NJ; j++) {
        int c = c0 + lane + 32 * j;
        if (c < k && !(st && st[c].active != 1)) y[(size_t)i * ld + c] = vmul(acc[j], di);
    }
}

// ---------------------------------------------------------------------------
// The whole IC(0) apply (forward then backward sweep) as ONE persistent
// cooperative launch: every warp walks the rows of a level (warp-strided),
// and the levels are separated by a grid barrier instead of a kernel
// boundary.  A level of the 30k cylinder's colour ordering takes about 2 us
// of dependent gathers, against 5.6 us per level as separate launches.
//
// Blocks of 1024 threads, one or two per SM, so that few blocks arrive at
// each barrier's counter.  The barrier spins with a bound: a block that
// waits more than about half a second (it cannot, in a cooperative launch, whose blocks are all resident)
// sets *err and goes on, later barriers stop waiting, the launch ends with
// wrong values and the host reports the flag as an error.
// ---------------------------------------------------------------------------
template <class V>
struct IcSweepArgs {
    int nlev_f, nlev_b;
    const int *lev_f, *lev_b;           // first row of each level (nlev + 1)
    const int *w_f, *w_b, *off_f, *off_b;  // ELL width and offset per level
    const int *rows_f, *rows_b, *ecol_f, *ecol_b;
    const V *eval_f, *eval_b;
    int k, ld;
    const V* dinv;
    const V* b;                         // right-hand side (forward sweep)
    V* y;                               // result (written by both sweeps)
    const ColState* st;
    unsigned* bar;                      // barrier arrival count, zero at launch
    int* err;                           // set when a barrier wait gave up
};

__device__ __forceinline__ void grid_barrier_bounded(unsigned* count, unsigned target, int* err)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(count, 1u);
        if (!*(volatile int*)err) {
            for (unsigned it = 0;; it++) {
                unsigned v;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
                if (v >= target) break;
                if (it > (1u << 20)) { atomicExch(err, 1); break; }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// one row (ELL slot) of a level, columns lane + 32 j: the body of
// ic_level_ell.  Plain loads of y are safe after the barrier: its fences
// and acquire load order them after every other block's writes of the
// earlier levels (the grid synchronisation pattern of cooperative groups).
template <class V, int NJ, bool FWD>
__device__ __forceinline__ void ic_ell_row(int slot, int lane, const int* __restrict__ rows, int w,
                                           const int* __restrict__ ecol, const V* __restrict__ eval, int k, int ld,
                                           const V* __restrict__ dinv, const V* __restrict__ b, V* __restrict__ y,
                                           const ColState* __restrict__ st)
{
    const int i = rows[slot];
    const V di = dinv[i];
    V acc[NJ];
#pragma unroll
    for (int j = 0; j < NJ; j++) {
        int c = lane + 32 * j;
        acc[j] = c < k ? (FWD ? b[(size_t)i * ld + c] : y[(size_t)i * ld + c]) : vzero<V>();
    }
    constexpr int UNR = 4;
    for (int base = 0; base < w; base += 32) {
        const int cnt = min(32, w - base);
        int my_c = -1;
        V my_v = vzero<V>();
        if (lane < cnt) {
            my_c = ecol[(size_t)slot * w + base + lane];
            my_v = eval[(size_t)slot * w + base + lane];
        }
        for (int e = 0; e < cnt; e += UNR) {
            int cc[UNR];
            V av[UNR];
#pragma unroll
            for (int u = 0; u < UNR; u++) {
                cc[u] = __shfl_sync(0xffffffffu, my_c, min(e + u, 31));
                av[u] = shfl(my_v, min(e + u, 31));
            }
            V g[UNR][NJ];
#pragma unroll
            for (int u = 0; u < UNR; u++)
#pragma unroll
                for (int j = 0; j < NJ; j++) {
                    int c = lane + 32 * j;
                    g[u][j] = (e + u < cnt && cc[u] >= 0 && c < k) ? y[(size_t)cc[u] * ld + c] : vzero<V>();
                }
#pragma unroll
            for (int u = 0; u < UNR; u++)
                if (e + u < cnt && cc[u] >= 0)
#pragma unroll
                    for (int j = 0; j < NJ; j++) acc[j] = vfms(acc[j], av[u], g[u][j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NJ; j++) {
        int c = lane + 32 * j;
        if (c < k && !(st && st[c].active != 1)) y[(size_t)i * ld + c] = vmul(acc[j], di);
    }
}

template <class V, int NJ>
__global__ void __launch_bounds__(1024) ic_sweep_persistent(IcSweepArgs<V> a)
{
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    unsigned nbar = 0;
    for (int l = 0; l < a.nlev_f; l++) {
        if (l) grid_barrier_bounded(a.bar, gridDim.x * ++nbar, a.err);
        const int r0 = a.lev_f[l], nr = a.lev_f[l + 1] - r0, w = a.w_f[l], eo = a.off_f[l];
        for (int slot = gw; slot < nr; slot += nw)
            ic_ell_row<V, NJ, true>(slot, lane, a.rows_f + r0, w, a.ecol_f + eo, a.eval_f + eo, a.k, a.ld, a.dinv,
                                    a.b, a.y, a.st);
    }
    for (int l = 0; l < a.nlev_b; l++) {
        grid_barrier_bounded(a.bar, gridDim.x * ++nbar, a.err);
        const int r0 = a.lev_b[l], nr = a.lev_b[l + 1] - r0, w = a.w_b[l], eo = a.off_b[l];
        for (int slot = gw; slot < nr; slot += nw)
            ic_ell_row<V, NJ, false>(slot, lane, a.rows_b + r0, w, a.ecol_b + eo, a.eval_b + eo, a.k, a.ld, a.dinv,
                                     a.b, a.y, a.st);
    }
}

// factor values into the ELL layouts (padding -> 0)
template <class V>
__global__ void ell_gather_kernel(int cnt, const int* __restrict__ src, const V* __restrict__ L, V* __restrict__ out)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    int q = src[t];
    out[t] = q >= 0 ? L[q] : vzero<V>();
}


// ---------------------------------------------------------------------------
// SpMM y = A x with optional fused dot partials over ROW_TILE-row tiles:
//   part0[c] = sum Re(conj(w) y)      (w != null)
//   part1[c] = sum |y|^2              (want_n2)
// One block per row tile.  Partials are written to part[(c * np + p) * ntiles + tile].
// ---------------------------------------------------------------------------
template <class V>
__global__ void spmm_dot_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ colidx,
                                const V* __restrict__ A, int k, int ld, const V* __restrict__ x,
                                V* __restrict__ y, const V* __restrict__ w, int want_n2,
                                double* __restrict__ part, int np, int ntiles, const ColState* __restrict__ st)
{
    int tile = blockIdx.x;
    int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    int cw = k >= 32 ? 32 : (k >= 16 ? 16 : (k >= 8 ? 8 : (k >= 4 ? 4 : (k >= 2 ? 2 : 1))));
    int ncg = (k + cw - 1) / cw;
    int rpw = 32 / cw;
    int warp = threadIdx.x / 32, lane = threadIdx.x & 31, nwarp = blockDim.x / 32;
    int items = (r1 - r0) * ncg;
    for (int it = warp * rpw + lane / cw; it < items; it += nwarp * rpw) {
        int r = r0 + it / ncg, c = (it % ncg) * cw + (lane % cw);
        if (c >= k || (st && st[c].active != 1)) continue;
        V s = vzero<V>();
        for (int q = rowptr[r]; q < rowptr[r + 1]; q++) s = vfma(s, A[q], x[(size_t)colidx[q] * ld + c]);
        y[(size_t)r * ld + c] = s;
    }
    if (!w && !want_n2) return;
    __syncthreads();
    tile_dots<V>(r0, r1, k, ld, y, w, want_n2, part, np, ntiles, tile, st);
}

// single right-hand side: warp per row, lanes over the row's entries
template <class V>
__global__ void spmv1_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ colidx,
                             const V* __restrict__ A, const V* __restrict__ x, V* __restrict__ y)
{
    int r = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x & 31;
    if (r >= n) return;
    V s = vzero<V>();
    for (int q = rowptr[r] + lane; q < rowptr[r + 1]; q += 32) s = vfma(s, A[q], x[colidx[q]]);
    for (int o = 16; o; o >>= 1) {
        if constexpr (vt<V>::cplx) { s.x += __shfl_down_sync(0xffffffffu, s.x, o); s.y += __shfl_down_sync(0xffffffffu, s.y, o); }
        else s += __shfl_down_sync(0xffffffffu, s, o);
    }
    if (lane == 0) y[r] = s;
}

// ---------------------------------------------------------------------------
// Per-column Krylov state and the deterministic reduce + finalize step.
// ---------------------------------------------------------------------------


// a value from (re, im) (the imaginary part is dropped for real types)
template <class V> __device__ __forceinline__ V vmake(double re_, double im_);
template <> __device__ __forceinline__ double vmake<double>(double re_, double) { return re_; }
template <> __device__ __forceinline__ float vmake<float>(double re_, double) { return (float)re_; }
template <> __device__ __forceinline__ cd vmake<cd>(double re_, double im_) { return cd{re_, im_}; }
template <> __device__ __forceinline__ cf vmake<cf>(double re_, double im_) { return cf{(float)re_, (float)im_}; }

enum Phase : int {
    PH_BNORM = 0,        // part0 = |b|^2 -> bnorm; (re)activate
    PH_BICG_RHO0,        // part0 = rd.r  -> rho (iteration 0)
    PH_BICG_ALPHA,       // part0 = rd.v  -> alpha = rho / aden
    PH_BICG_S,           // part0 = |s|^2 (real variant early exit)
    PH_BICG_OMEGA,       // part0 = t.s, part1 = |t|^2 -> omega
    PH_BICG_END,         // part0 = |r|^2, part1 = rd.r -> err, convergence, next beta/rho
    PH_PCG_INIT,         // part0 = r.d -> dnew
    PH_PCG_ALPHA,        // part0 = d.q -> alpha
    PH_PCG_END,          // part0 = r.q (dnew), part1 = |r|^2 -> beta, err, convergence
    PH_RESID,            // part0 = |r|^2 -> err (refinement residual)
    PH_REL_RESUME,       // part0 = rd.r after a residual replacement -> rho, beta; reactivate
    PH_COCG_RHO0,        // part0 + i part1 = r.z (bilinear) -> rho
    PH_COCG_ALPHA,       // part0 + i part1 = p.q -> alpha = rho / (p.q)
    PH_COCG_RES,         // part0 = |r|^2 -> err, convergence
    PH_COCG_BETA,        // part0 + i part1 = r.z -> beta = rho' / rho, rho = rho'
};

template <int NP>
__global__ void reduce_finalize_kernel(int k, int ntiles, const double* __restrict__ part, ColState* __restrict__ st,
                                       int phase, int real_variant, int iter_base)
{
    int c = blockIdx.x;
    if (c >= k) return;
    __shared__ double sh[NP][256];
    double acc[NP];
    for (int p = 0; p < NP; p++) acc[p] = 0.0;
    for (int t = threadIdx.x; t < ntiles; t += 256)
        for (int p = 0; p < NP; p++) acc[p] += part[((size_t)c * NP + p) * ntiles + t];
    for (int p = 0; p < NP; p++) sh[p][threadIdx.x] = acc[p];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int p = 0; p < NP; p++) sh[p][threadIdx.x] += sh[p][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x) return;
    ColState& S = st[c];
    double v0 = sh[0][0], v1 = NP > 1 ? sh[NP - 1][0] : 0.0;
    switch (phase) {
    case PH_BNORM:
        // columns the caller switched off stay off (refinement steps)
        S.bnorm = sqrt(v0);
        S.its = 0; S.status = 0; S.err = 0.0;
        S.active = (S.active == 1 && S.bnorm > 0.0) ? 1 : 0;
        break;
    case PH_BICG_RHO0:
        if (!S.active) break;
        S.rho = v0;
        if (v0 == 0.0) { S.active = 0; S.status = 2; S.its = iter_base; }
        break;
    case PH_BICG_ALPHA:
        if (!S.active) break;
        S.alpha = S.rho / v0;
        if (!isfinite(S.alpha)) { S.active = 0; S.status = 2; S.its = S.its; }  // rd.v = 0: breakdown
        break;
    case PH_BICG_S:
        if (!S.active) break;
        S.err = sqrt(v0);  // real variant only: |s| < tol |b| ends the solve (matrix_imp.hpp:512-517)
        if (real_variant && S.err < S.tol * S.bnorm) { S.active = -1; S.rel = -1; }  // -1: finish with x += alpha pd
        break;
    case PH_BICG_OMEGA:
        if (S.active != 1) break;
        S.omega = v0 / v1;
        break;
    case PH_BICG_END: {
        if (S.active == -1) { S.active = 0; S.status = 0; break; }
        if (!S.active) break;
        S.err = sqrt(v0);
        S.its++;
        if (S.err <= S.tol * S.bnorm) { S.active = 0; S.status = 0; S.its--; break; }
        if (S.omega == 0.0) { S.active = 0; S.status = 1; S.its--; break; }
        if (S.its >= S.maxit) { S.active = 0; S.status = 1; break; }
        S.rhop = S.rho;
        S.rho = v1;
        if (v1 == 0.0) { S.active = 0; S.status = 2; S.its--; break; }
        S.beta = (S.rho * S.alpha) / (S.rhop * S.omega);
        break;
    }
    case PH_PCG_INIT:
        if (!S.active) break;
        S.dnew = v0;
        break;
    case PH_PCG_ALPHA:
        if (!S.active) break;
        S.alpha = S.dnew / v0;
        if (S.alpha == 0.0 || isnan(S.alpha)) { S.active = 0; S.status = 2; S.err = S.err; }
        break;
    case PH_PCG_END: {
        if (!S.active) break;
        S.dold = S.dnew;
        S.dnew = v0;
        S.beta = S.dnew / S.dold;
        S.its++;
        if (S.beta == 0.0 || isnan(S.beta)) { S.active = 0; S.status = 2; S.its--; break; }
        S.err = sqrt(v1);
        if (S.err <= S.tol * S.bnorm) { S.active = 0; S.status = 0; S.its--; break; }
        if (S.its >= S.maxit) { S.active = 0; S.status = 1; break; }
        break;
    }
    case PH_RESID:
        S.err = sqrt(v0);
        break;
    case PH_COCG_RHO0:
        if (S.active != 1) break;
        S.zr = v0; S.zi = v1;
        if (v0 == 0.0 && v1 == 0.0) { S.active = 0; S.status = 2; }
        break;
    case PH_COCG_ALPHA: {
        if (S.active != 1) break;
        const cd a = cdiv(cd{S.zr, S.zi}, cd{v0, v1});
        S.ar = a.x; S.ai = a.y;
        if (!isfinite(a.x) || !isfinite(a.y)) { S.active = 0; S.status = 2; }
        break;
    }
    case PH_COCG_RES:
        if (S.active != 1) break;
        S.err = sqrt(v0);
        S.its++;
        if (S.err <= S.tol * S.bnorm) { S.active = 0; S.status = 0; break; }
        if (S.its >= S.maxit) { S.active = 0; S.status = 1; }
        break;
    case PH_COCG_BETA: {
        if (S.active != 1) break;
        if (S.rel == 2) {  // restarted process: p = z
            S.br = 0.0; S.bi = 0.0;
        } else {
            const cd b = cdiv(cd{v0, v1}, cd{S.zr, S.zi});
            S.br = b.x; S.bi = b.y;
        }
        S.rel = 0;
        S.zr = v0; S.zi = v1;
        if ((v0 == 0.0 && v1 == 0.0) || !isfinite(S.br) || !isfinite(S.bi)) { S.active = 0; S.status = 2; }
        break;
    }
    case PH_REL_RESUME:
        // the replaced residual continues the same BiCGSTAB process
        // (rel 1: the END step's rho / beta update with the new r) or
        // starts a new one from it (rel 2, after a breakdown)
        if (!S.rel) break;
        if (S.rel == 1) {
            S.rhop = S.rho;
            S.rho = v0;
            S.beta = (S.rho * S.alpha) / (S.rhop * S.omega);
        } else {
            S.rho = v0;
            S.beta = 0.0;
            S.omega = 1.0;
        }
        S.rel = 0;
        S.status = 0;
        S.active = 1;
        if (v0 == 0.0 || !isfinite(S.beta)) { S.active = 0; S.status = 2; }
        break;
    }
}

// generic column dot partials over row tiles: part0 = sum Re(conj(a) b),
// optional part1 = sum Re(conj(c2) d2)
template <class V>
__global__ void dot_tiles_kernel(int n, int k, int ld, const V* __restrict__ a, const V* __restrict__ b,
                                 const V* __restrict__ c2, const V* __restrict__ d2, double* __restrict__ part,
                                 int np, int ntiles, const ColState* __restrict__ st)
{
    __shared__ double sh[2 * TILE_RG * TILE_CK];
    TileAcc T{sh};
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    for (int c0 = 0; c0 < k; c0 += TILE_CK) {
        const int ck = min(TILE_CK, k - c0);
        for (int it = threadIdx.x; it < ck * TILE_RG; it += blockDim.x) {
            const int cc = it % ck, g = it / ck, c = c0 + cc;
            typename vt<V>::R d0 = 0, d1 = 0;
            if (!(st && st[c].active != 1))
                for (int r = r0 + g; r < r1; r += TILE_RG) {
                    size_t o = (size_t)r * ld + c;
                    d0 += redot(a[o], b[o]);
                    if (c2) d1 += redot(c2[o], d2[o]);
                }
            T.put(0, g, cc, (double)d0);
            T.put(1, g, cc, (double)d1);
        }
        __syncthreads();
        for (int cc = threadIdx.x; cc < ck; cc += blockDim.x) {
            const int c = c0 + cc;
            if (st && st[c].active != 1) continue;
            part[((size_t)c * np) * ntiles + tile] = T.sum(0, cc);
            if (c2) part[((size_t)c * np + 1) * ntiles + tile] = T.sum(1, cc);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// BiCGSTAB elementwise steps (matrix_imp.hpp:350-413 complex, 479-547 real).
// S = real scalar type of V.  ColState is read per column.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool col_on(const ColState* st, int c) { return st[c].active == 1; }

// p = r (first iteration) or r + beta (p - omega v); for diagonal/no
// preconditioner also pd = M^-1 p.  precon: 0 none, 1 diag.
template <class V, class S>
__global__ void bicg_p_kernel(int n, int k, int ld, const ColState* st, int first, const V* __restrict__ r,
                              V* __restrict__ p, const V* __restrict__ v, V* __restrict__ pd,
                              const V* __restrict__ idiag, int precon)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    int i = (int)(t / k), c = (int)(t % k);
    if (!col_on(st, c)) return;
    size_t o = (size_t)i * ld + c;
    V pv;
    if (first) pv = r[o];
    else {
        S beta = (S)st[c].beta, omega = (S)st[c].omega;
        pv = vadd(r[o], vscale(vsub(p[o], vscale(v[o], omega)), beta));
    }
    p[o] = pv;
    if (precon == 1) pd[o] = vmul(pv, idiag[i]);
    else if (precon == 0) pd[o] = pv;
}

// s = r - alpha v with |s|^2 partials; sd = M^-1 s for diag/none
template <class V, class S>
__global__ void bicg_s_kernel(int n, int k, int ld, const ColState* st, const V* __restrict__ r,
                              const V* __restrict__ v, V* __restrict__ s, V* __restrict__ sd,
                              const V* __restrict__ idiag, int precon, double* __restrict__ part, int ntiles)
{
    __shared__ double sh[2 * TILE_RG * TILE_CK];
    TileAcc T{sh};
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    for (int c0 = 0; c0 < k; c0 += TILE_CK) {
        const int ck = min(TILE_CK, k - c0);
        for (int it = threadIdx.x; it < ck * TILE_RG; it += blockDim.x) {
            const int cc = it % ck, g = it / ck, c = c0 + cc;
            S acc = 0;
            if (col_on(st, c)) {
                const S alpha = (S)st[c].alpha;
#pragma unroll 4
                for (int i = r0 + g; i < r1; i += TILE_RG) {
                    size_t o = (size_t)i * ld + c;
                    V sv = vsub(r[o], vscale(v[o], alpha));
                    s[o] = sv;
                    if (precon == 1) sd[o] = vmul(sv, idiag[i]);
                    else if (precon == 0) sd[o] = sv;
                    acc += nrm2(sv);
                }
            }
            T.put(0, g, cc, (double)acc);
        }
        __syncthreads();
        for (int cc = threadIdx.x; cc < ck; cc += blockDim.x)
            if (col_on(st, c0 + cc)) part[(size_t)(c0 + cc) * ntiles + tile] = T.sum(0, cc);
        __syncthreads();
    }
}

// x += alpha pd + omega sd ; r = s - omega t ; partials |r|^2, Re(conj(rd) r).
// Columns that ended on |s| (real variant) take x += alpha pd only.
template <class V, class S>
__global__ void bicg_xr_kernel(int n, int k, int ld, const ColState* st, V* __restrict__ x, V* __restrict__ r,
                               const V* __restrict__ rd, const V* __restrict__ pd, const V* __restrict__ sd,
                               const V* __restrict__ s, const V* __restrict__ t, double* __restrict__ part, int ntiles)
{
    __shared__ double sh[2 * TILE_RG * TILE_CK];
    TileAcc T{sh};
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    for (int c0 = 0; c0 < k; c0 += TILE_CK) {
        const int ck = min(TILE_CK, k - c0);
        for (int it = threadIdx.x; it < ck * TILE_RG; it += blockDim.x) {
            const int cc = it % ck, g = it / ck, c = c0 + cc;
            const int a = st[c].active;
            S n2 = 0, rr = 0;
            if (a != 0) {
                const S alpha = (S)st[c].alpha, omega = (S)st[c].omega;
#pragma unroll 4
                for (int i = r0 + g; i < r1; i += TILE_RG) {
                    size_t o = (size_t)i * ld + c;
                    if (a == -1) { x[o] = vadd(x[o], vscale(pd[o], alpha)); continue; }
                    x[o] = vadd(x[o], vadd(vscale(pd[o], alpha), vscale(sd[o], omega)));
                    V rv = vsub(s[o], vscale(t[o], omega));
                    r[o] = rv;
                    n2 += nrm2(rv);
                    rr += redot(rd[o], rv);
                }
            }
            T.put(0, g, cc, (double)n2);
            T.put(1, g, cc, (double)rr);
        }
        __syncthreads();
        for (int cc = threadIdx.x; cc < ck; cc += blockDim.x) {
            const int c = c0 + cc;
            if (st[c].active == 0) continue;
            part[((size_t)c * 2) * ntiles + tile] = T.sum(0, cc);
            part[((size_t)c * 2 + 1) * ntiles + tile] = T.sum(1, cc);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// PCG elementwise steps (matrix_imp.hpp:93-154)
// ---------------------------------------------------------------------------
// x += alpha d ; r -= alpha q ; for diag/none: z = M^-1 r and partials r.z, |r|^2
template <class V, class S>
__global__ void pcg_xr_kernel(int n, int k, int ld, const ColState* st, V* __restrict__ x, V* __restrict__ r,
                              const V* __restrict__ d, const V* __restrict__ q, V* __restrict__ z,
                              const V* __restrict__ idiag, int precon, double* __restrict__ part, int ntiles)
{
    __shared__ double sh[2 * TILE_RG * TILE_CK];
    TileAcc T{sh};
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    for (int c0 = 0; c0 < k; c0 += TILE_CK) {
        const int ck = min(TILE_CK, k - c0);
        for (int it = threadIdx.x; it < ck * TILE_RG; it += blockDim.x) {
            const int cc = it % ck, g = it / ck, c = c0 + cc;
            S rz = 0, n2 = 0;
            if (col_on(st, c)) {
                const S alpha = (S)st[c].alpha;
                for (int i = r0 + g; i < r1; i += TILE_RG) {
                    size_t o = (size_t)i * ld + c;
                    x[o] = vadd(x[o], vscale(d[o], alpha));
                    V rv = vsub(r[o], vscale(q[o], alpha));
                    r[o] = rv;
                    if (precon != 2) {
                        V zv = precon == 1 ? vmul(rv, idiag[i]) : rv;
                        z[o] = zv;
                        rz += redot(rv, zv);
                        n2 += nrm2(rv);
                    }
                }
            }
            T.put(0, g, cc, (double)rz);
            T.put(1, g, cc, (double)n2);
        }
        __syncthreads();
        if (precon != 2)
            for (int cc = threadIdx.x; cc < ck; cc += blockDim.x) {
                const int c = c0 + cc;
                if (!col_on(st, c)) continue;
                part[((size_t)c * 2) * ntiles + tile] = T.sum(0, cc);
                part[((size_t)c * 2 + 1) * ntiles + tile] = T.sum(1, cc);
            }
        __syncthreads();
    }
}

// d = d beta + z
template <class V, class S>
__global__ void pcg_d_kernel(int n, int k, int ld, const ColState* st, V* __restrict__ d, const V* __restrict__ z)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    int i = (int)(t / k), c = (int)(t % k);
    if (!col_on(st, c)) return;
    size_t o = (size_t)i * ld + c;
    d[o] = vadd(vscale(d[o], (S)st[c].beta), z[o]);
}

// ---------------------------------------------------------------------------
// small elementwise helpers
// ---------------------------------------------------------------------------
// r = b - r (in place on r), rd = r, optional |b|^2 partials are separate
template <class V>
__global__ void resid_kernel(int n, int k, int ld, const V* __restrict__ b, V* __restrict__ r, V* __restrict__ rd)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    size_t o = (size_t)(t / k) * ld + (t % k);
    V v = vsub(b[o], r[o]);
    r[o] = v;
    if (rd) rd[o] = v;
}

template <class V>
__global__ void scale_diag_kernel(int n, int k, int ld, const V* __restrict__ a, const V* __restrict__ idiag,
                                  V* __restrict__ out, int precon)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    int i = (int)(t / k);
    size_t o = (size_t)i * ld + (t % k);
    out[o] = precon == 1 ? vmul(a[o], idiag[i]) : a[o];
}

// source-major (q*n + i) <-> node-major (i*ld + q) transposes with precision cast
// perm (nullable): natural node -> layout row of the node-major block
template <class To, class From>
__global__ void to_nodemajor_kernel(int n, int k, int ld, const From* __restrict__ src, To* __restrict__ dst,
                                    const int* __restrict__ perm)
{
    __shared__ From tile[32][33];
    int i0 = blockIdx.x * 32, q0 = blockIdx.y * 32;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        int q = q0 + yy, i = i0 + threadIdx.x;
        if (q < k && i < n) tile[yy][threadIdx.x] = src[(size_t)q * n + i];
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        int i = i0 + yy, q = q0 + threadIdx.x;
        if (q < k && i < n) dst[(size_t)(perm ? perm[i] : i) * ld + q] = vcast<To, From>(tile[threadIdx.x][yy]);
    }
}

template <class To, class From>
__global__ void to_srcmajor_kernel(int n, int k, int ld, const From* __restrict__ src, To* __restrict__ dst,
                                   const int* __restrict__ perm)
{
    __shared__ From tile[32][33];
    int i0 = blockIdx.x * 32, q0 = blockIdx.y * 32;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        int i = i0 + yy, q = q0 + threadIdx.x;
        if (q < k && i < n) tile[yy][threadIdx.x] = src[(size_t)(perm ? perm[i] : i) * ld + q];
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        int q = q0 + yy, i = i0 + threadIdx.x;
        if (q < k && i < n) dst[(size_t)q * n + i] = vcast<To, From>(tile[threadIdx.x][yy]);
    }
}

template <class To, class From>
__global__ void cast_kernel(size_t cnt, const From* __restrict__ a, To* __restrict__ b)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) b[t] = vcast<To, From>(a[t]);
}

// node-major block with leading dimension ld (k used columns) -> dense k columns, cast
template <class To, class From>
__global__ void strided_cast_kernel(int n, int k, const From* __restrict__ a, int ld, To* __restrict__ b)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    size_t i = t / k, c = t % k;
    b[t] = vcast<To, From>(a[i * ld + c]);
}

// x += e (refinement update, FP64 x, low-precision e)
template <class V, class E>
__global__ void add_correction_kernel(size_t cnt, V* __restrict__ x, const E* __restrict__ e)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) x[t] = vadd(x[t], vcast<V, E>(e[t]));
}

// restarted refinement: the inner solve of column c works on r / scale_c
// (scale_c a power of two of |r|, so the FP32 values stay O(1) down to the
// rounding floor); its correction is added back times scale_c.  A column
// whose inner solve broke down (status 2) adds nothing.
static __global__ void refine_scale_kernel(int k, const ColState* __restrict__ outer, ColState* __restrict__ inner)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    inner[c].scale = pow2_floor(outer[c].err);
}

template <class V64, class V32>
__global__ void add_scaled_correction_kernel(int n, int k, const ColState* __restrict__ inner, V64* __restrict__ x,
                                             const V32* __restrict__ e)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    const int c = (int)(t % k);
    if (inner[c].status == 2) return;
    x[t] = vadd(x[t], vscale(vcast<V64, V32>(e[t]), inner[c].scale));
}

// 1/diag(A) for the Diag preconditioner (TPrecon_Diag::Reset,
// src/libmath/precon_imp.hpp:56-64): 1 where the diagonal is zero.
template <class V>
__global__ void diag_inv_kernel(int n, const int* __restrict__ diagpos, const V* __restrict__ A, V* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V d = A[diagpos[i]];
    bool z = re(d) == 0 && im(d) == 0;
    if constexpr (vt<V>::cplx) out[i] = z ? V{1.0, 0.0} : vrecip(d);
    else out[i] = z ? 1.0 : 1.0 / d;
}

static __global__ void count_active_kernel(int k, const ColState* __restrict__ cst, int* out)
{
    __shared__ int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    int c = 0;
    for (int i = threadIdx.x; i < k; i += blockDim.x) c += cst[i].active != 0;
    atomicAdd(&s, c);
    __syncthreads();
    if (threadIdx.x == 0) *out = s;
}

// ---------------------------------------------------------------------------
// Reliable updates of the mixed-precision BiCGSTAB (residual replacement,
// Sleijpen & van der Vorst 1996): the FP32 process runs until its recursive
// residual has fallen by the trigger factor; then the FP32 correction is
// added to the FP64 solution, the true residual b - A x is formed in FP64 and
// replaces the FP32 residual, and the same Krylov process continues.
// ---------------------------------------------------------------------------
// out[0] outer columns active, out[1] inner columns iterating, out[2] waiting
// for an update (outer active, inner stopped)
static __global__ void rel_flags_kernel(int k, const ColState* __restrict__ co, const ColState* __restrict__ ci,
                                        int* out)
{
    __shared__ int s[3];
    if (threadIdx.x < 3) s[threadIdx.x] = 0;
    __syncthreads();
    int a = 0, b = 0, f = 0;
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        const bool oa = co[c].active == 1, ia = ci[c].active == 1;
        a += oa;
        b += ia;
        f += oa && !ia;
    }
    atomicAdd(&s[0], a);
    atomicAdd(&s[1], b);
    atomicAdd(&s[2], f);
    __syncthreads();
    if (threadIdx.x < 3) out[threadIdx.x] = s[threadIdx.x];
}

// ---------------------------------------------------------------------------
// Componentwise backward error of an FP64 solution (the Oettli-Prager
// measure that iterative refinement stops on): for each listed column c,
//   berr_c = max_i |r_ic| / (|A| |x_c| + |b_c|)_i,   r = b - A x,
// with |z| = max(|Re z|, |Im z|) and the sums in FP32 (the test needs the
// magnitude of the denominator, not its digits).  A solution whose berr is at
// the FP64 rounding level is exact for a matrix and right-hand side perturbed
// by that relative amount entry by entry, so its small entries (far from the
// source, where the fields are e^-20 of their peak) are as accurate as its
// large ones, which a normwise residual test does not give.
// A block handles BERR_ROWS rows of the kf listed columns (idx, or all k
// columns when idx is null) and folds its maxima into cmax[c] as the bits of
// a non-negative float: an integer maximum of those bits is the float
// maximum, exact and independent of the order (NaN bits sort above inf, so a
// NaN never passes the test).  cmax must be zeroed before the launch.
// ---------------------------------------------------------------------------
constexpr int BERR_ROWS = 32;

template <class V64>
__global__ void berr_kernel(int n, int k, int kf, const int* __restrict__ idx, const int* __restrict__ rowptr,
                            const int* __restrict__ colidx, const float* __restrict__ absA,
                            const V64* __restrict__ x, const V64* __restrict__ b, const V64* __restrict__ r,
                            unsigned* __restrict__ cmax)
{
    extern __shared__ unsigned sm_berr[];  // kf entries
    for (int j = threadIdx.x; j < kf; j += blockDim.x) sm_berr[j] = 0u;
    __syncthreads();
    const int r0 = blockIdx.x * BERR_ROWS, r1 = min(n, r0 + BERR_ROWS);
    const int cnt = (r1 - r0) * kf;
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
        const int i = r0 + t / kf, j = t % kf;
        const int c = idx ? idx[j] : j;
        float d = 0.f;
        for (int e = rowptr[i]; e < rowptr[i + 1]; e++) d = fmaf(absA[e], mag1f(x[(size_t)colidx[e] * k + c]), d);
        const size_t o = (size_t)i * k + c;
        d += mag1f(b[o]);
        const float rr = mag1f(r[o]);
        const float q = rr == 0.f ? 0.f : (d > 0.f ? rr / d : INFINITY);
        atomicMax(&sm_berr[j], __float_as_uint(q));
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kf; j += blockDim.x)
        if (sm_berr[j]) atomicMax(&cmax[idx ? idx[j] : j], sm_berr[j]);
}

// |Re a| + |Im a| of each system-matrix entry, in FP32, for berr_kernel
template <class V64>
__global__ void abs_values_kernel(int nnz, const V64* __restrict__ a, float* __restrict__ out)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nnz) out[t] = mag1f(a[t]);
}

// the column passes both tests: normwise |r| <= tol |b| and, when cwtol > 0,
// the componentwise backward error from cmax (berr_kernel) <= cwtol
__device__ __forceinline__ bool col_converged(ColState& O, int c, double cwtol, const unsigned* cmax)
{
    if (cwtol > 0.0 && cmax) O.berr = (double)__uint_as_float(cmax[c]);
    if (!(O.err <= O.tol * O.bnorm)) return false;
    if (cwtol <= 0.0) return true;
    if (!cmax) return O.err == 0.0;
    return O.berr <= cwtol;  // false for NaN
}

// inner columns start from the outer residual, scaled to O(1): scale =
// pow2_floor(|r|), bnorm = |r| / scale, trigger tol.  With a componentwise
// test (cwtol > 0) only an exact initial guess (r = 0) stops here.
static __global__ void rel_init_kernel(int k, ColState* __restrict__ co, ColState* __restrict__ ci, double trig,
                                       int maxit, double cwtol)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    ColState& O = co[c];
    O.berr = 1.0;
    if (O.active == 1 && col_converged(O, c, cwtol, nullptr)) { O.active = 0; O.status = 0; O.berr = 0.0; }
    ColState s;
    memset(&s, 0, sizeof(s));
    s.tol = trig;
    s.maxit = maxit;
    s.scale = s.scale_prev = pow2_floor(O.err);
    s.bnorm = O.err / s.scale;
    s.active = O.active;
    ci[c] = s;
}

// r32 = r / scale for every column (the start of the process)
template <class V64, class V32>
__global__ void rel_scaled_cast_kernel(int n, int k, const ColState* __restrict__ ci, const V64* __restrict__ r64,
                                       V32* __restrict__ r)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    int c = (int)(t % k);
    r[t] = vcast<V32, V64>(vscale(r64[t], 1.0 / ci[c].scale));
}

// waiting columns: rel = 1 (the trigger was reached: resume) or 2 (breakdown,
// omega = 0 or the iteration limit: restart the process)
static __global__ void rel_mark_kernel(int k, const ColState* __restrict__ co, ColState* __restrict__ ci)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    ColState& I = ci[c];
    // a half-step exit (rel -1, real variant) leaves no consistent direction: restart
    I.rel = (co[c].active == 1 && I.active != 1) ? ((I.status == 0 && I.rel != -1) ? 1 : 2) : 0;
}

// at the iteration limit every active column takes its last update
static __global__ void rel_mark_all_kernel(int k, const ColState* __restrict__ co, ColState* __restrict__ ci)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    if (co[c].active == 1 && !ci[c].rel) ci[c].rel = 1;
}

// x += scale * x32 and x32 = 0 on the marked columns
template <class V64, class V32>
__global__ void rel_accumulate_kernel(int n, int k, const ColState* __restrict__ ci, V64* __restrict__ x,
                                      V32* __restrict__ x32)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    int c = (int)(t % k);
    if (!ci[c].rel) return;
    x[t] = vadd(x[t], vscale(vcast<V64, V32>(x32[t]), ci[c].scale));
    x32[t] = vzero<V32>();
}

// after |b - A x| of the marked columns is in co.err: converged columns stop,
// the others restart their trigger from the new residual; at the update or
// iteration limit every active column stops with status 1
// limit: the iteration limit was reached; max_upd: replacements per column
static __global__ void rel_outer_kernel(int k, ColState* __restrict__ co, ColState* __restrict__ ci, int limit,
                                        int cocg, int max_upd, double cwtol, const unsigned* __restrict__ cmax)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    ColState& O = co[c];
    ColState& I = ci[c];
    if (O.active != 1 || !I.rel) return;
    if (col_converged(O, c, cwtol, cmax)) { O.active = 0; O.status = 0; I.rel = 0; return; }
    if (limit || ++I.nupd >= max_upd) { O.active = 0; O.status = 1; I.rel = 0; return; }
    // a true residual far above the recursive one means the process no longer
    // follows the FP64 system (at the rounding floor of the FP64 residual the
    // true residual stops falling while the recursion goes on): resuming it
    // with the old directions stagnates, so it restarts from the true residual
    if (O.err > 8.0 * I.err * I.scale) I.rel = 2;
    // rescale the process to the new residual (exact: powers of two)
    I.scale_prev = I.scale;
    I.scale = pow2_floor(O.err);
    I.bnorm = O.err / I.scale;
    const double f = I.scale_prev / I.scale;
    if (cocg) { I.zr *= f * f; I.zi *= f * f; }  // r.z: both factors rescale
    else I.rho *= f;                             // rd.r: rd stays
}

// the marked columns take the true residual; restarted columns also reset the
// shadow residual and the search directions
template <class V64, class V32>
__global__ void rel_replace_kernel(int n, int k, const ColState* __restrict__ ci, const V64* __restrict__ r64,
                                   V32* __restrict__ r, V32* __restrict__ rd, V32* __restrict__ p,
                                   V32* __restrict__ v)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    int c = (int)(t % k);
    const int rel = ci[c].rel;
    if (!rel) return;
    const V32 x = vcast<V32, V64>(vscale(r64[t], 1.0 / ci[c].scale));
    r[t] = x;
    if (rel == 2) {
        if (rd) rd[t] = x;
        p[t] = vzero<V32>();
        if (v) v[t] = vzero<V32>();
    } else {
        using S32 = typename vt<V32>::R;
        const S32 f = (S32)(ci[c].scale_prev / ci[c].scale);
        p[t] = vscale(p[t], f);
        if (v) v[t] = vscale(v[t], f);
    }
}

static __global__ void rel_finish_kernel(int k, ColState* __restrict__ co, const ColState* __restrict__ ci)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    co[c].its = ci[c].its;
    if (co[c].active == 1) { co[c].active = 0; co[c].status = 1; }
}

// the marked columns (rel != 0) as a list, in column order (one block)
static __global__ void rel_compact_kernel(int k, const ColState* __restrict__ ci, int* __restrict__ idx,
                                          int* __restrict__ cnt)
{
    __shared__ int base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int c0 = 0; c0 < k; c0 += blockDim.x) {
        const int c = c0 + threadIdx.x;
        const int f = (c < k && ci[c].rel) ? 1 : 0;
        // ordered compaction of this chunk: warp ballots, then warp offsets
        const unsigned b = __ballot_sync(0xffffffffu, f);
        __shared__ int wcnt[32];
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) wcnt[wid] = __popc(b);
        __syncthreads();
        int off = base;
        for (int w = 0; w < wid; w++) off += wcnt[w];
        if (f) idx[off + __popc(b & ((1u << lane) - 1))] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += wcnt[w];
            base += t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *cnt = base;
}

// dst (n x kf) = src columns idx (n x k)
template <class V>
__global__ void gather_cols_kernel(int n, int k, int kf, const int* __restrict__ idx, const V* __restrict__ src,
                                   V* __restrict__ dst)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * kf) return;
    const size_t i = t / kf;
    const int j = (int)(t % kf);
    dst[t] = src[i * k + idx[j]];
}

// r[:, idx] = b[:, idx] - ax (ax: n x kf)
template <class V>
__global__ void scatter_resid_kernel(int n, int k, int kf, const int* __restrict__ idx, const V* __restrict__ b,
                                     const V* __restrict__ ax, V* __restrict__ r)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * kf) return;
    const size_t i = t / kf;
    const int c = idx[t % kf];
    r[i * k + c] = vsub(b[i * k + c], ax[t]);
}

// ---------------------------------------------------------------------------
// COCG, the conjugate-orthogonal CG for complex symmetric A = A^T with a
// complex symmetric preconditioner (IC(0): M = L~ L~^T): CG with the bilinear
// product x.y = sum x_i y_i in place of the inner product, one SpMM and one
// preconditioner apply per iteration.  Used as the FP32 inner process of the
// mixed path for complex systems.
// ---------------------------------------------------------------------------
// x += alpha p, r -= alpha q on the active columns, |r|^2 partials
template <class V>
__global__ void cocg_xr_kernel(int n, int k, int ld, const ColState* __restrict__ st, V* __restrict__ x,
                               V* __restrict__ r, const V* __restrict__ p, const V* __restrict__ q,
                               double* __restrict__ part, int ntiles)
{
    __shared__ double sh[2 * TILE_RG * TILE_CK];
    TileAcc T{sh};
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    for (int c0 = 0; c0 < k; c0 += TILE_CK) {
        const int ck = min(TILE_CK, k - c0);
        for (int it = threadIdx.x; it < ck * TILE_RG; it += blockDim.x) {
            const int cc = it % ck, g = it / ck, c = c0 + cc;
            typename vt<V>::R acc = 0;  // a thread's few rows in the value's precision
            if (st[c].active == 1) {
                const V a = vmake<V>(st[c].ar, st[c].ai);
#pragma unroll 4
                for (int i = r0 + g; i < r1; i += TILE_RG) {
                    const size_t o = (size_t)i * ld + c;
                    x[o] = vfma(x[o], a, p[o]);
                    const V rv = vfms(r[o], a, q[o]);
                    r[o] = rv;
                    acc += nrm2(rv);
                }
            }
            T.put(0, g, cc, (double)acc);
        }
        __syncthreads();
        for (int cc = threadIdx.x; cc < ck; cc += blockDim.x)
            if (st[c0 + cc].active == 1) part[(size_t)(c0 + cc) * ntiles + tile] = T.sum(0, cc);
        __syncthreads();
    }
}

// p = z (first) or p = z + beta p on the active columns
template <class V>
__global__ void cocg_p_kernel(int n, int k, int ld, const ColState* __restrict__ st, int first,
                              const V* __restrict__ z, V* __restrict__ p)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    const int c = (int)(t % k);
    if (st[c].active != 1) return;
    const size_t o = (t / k) * ld + c;
    p[o] = first ? z[o] : vfma(z[o], vmake<V>(st[c].br, st[c].bi), p[o]);
}

// reactivate the columns that took a residual replacement (COCG continues
// with z = M r, beta and p; a restart keeps rel = 2 until the beta step)
static __global__ void rel_reactivate_kernel(int k, ColState* __restrict__ ci)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k || !ci[c].rel) return;
    ci[c].active = 1;
    ci[c].status = 0;
}

// bilinear column products sum a_i b_i (no conjugation) as [Re, Im] tile partials
template <class V>
__global__ void bdot_tiles_kernel(int n, int k, int ld, const V* __restrict__ a, const V* __restrict__ b,
                                  double* __restrict__ part, int ntiles, const ColState* __restrict__ st)
{
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    tile_dots<V>(r0, r1, k, ld, b, a, 2, part, 2, ntiles, tile, st);
}

}  // namespace tg
