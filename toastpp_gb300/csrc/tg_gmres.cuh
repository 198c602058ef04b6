// tg_gmres.cuh -- batched GMRES(m) with per-column state, following the
// reference's gmres (src/libmath/gmres_imp.hpp:39-230; restart 20 from
// IterativeSolve, gsmatrix_imp.hpp:539): preconditioned right-hand side,
// modified Gram-Schmidt with conjugated products, Givens rotations without
// conjugation (complex square root), back substitution, restart residual
// Mb - M A x.  Every column runs its own cycles; columns that leave the inner
// loop early wait for the restart step of the batch.
#pragma once
#include "tg_kernels.cuh"

namespace tg {

constexpr int GM_M = 20;

template <class W>  // W = double or cd: the small dense arithmetic in FP64
struct GmCol {
    W H[GM_M][GM_M + 1];   // H(j,k), as the reference's TDenseMatrix(M, M+1)
    W s[GM_M + 1], c1[GM_M], c2[GM_M], y[GM_M];
    double norm_b, hn;     // |M b|; |w| of the current inner step before its rotation
    int j, jend, inner, cycle, maxc, xsmall;
};

TGHD double wabs(double a) { return fabs(a); }
TGHD double wabs(cd a) { return hypot(a.x, a.y); }
TGHD cd wsqrt(cd a) { return csqrt_d(a); }
TGHD double wsqrt(double a) { return sqrt(a); }
TGHD cd wdiv(cd a, cd b) { return cdiv(a, b); }
TGHD double wdiv(double a, double b) { return a / b; }
TGHD cd wneg(cd a) { return cd{-a.x, -a.y}; }
TGHD double wneg(double a) { return -a; }
template <class W> TGHD W wfromre(double r);
template <> TGHD double wfromre<double>(double r) { return r; }
template <> TGHD cd wfromre<cd>(double r) { return cd{r, 0.0}; }
template <class W> TGHD W wfrom2(double re_, double im_);
template <> TGHD double wfrom2<double>(double re_, double) { return re_; }
template <> TGHD cd wfrom2<cd>(double re_, double im_) { return cd{re_, im_}; }

// sum over the tile of a * conj(b), real and imaginary parts (np = 2), after
// an optional w -= h_prev * vprev update of a (the fused modified
// Gram-Schmidt step); or |a|^2 alone (np = 1) after a final update.
template <class V, class W>
__global__ void gm_mgs_kernel(int n, int k, int ld, const ColState* __restrict__ st, const GmCol<W>* __restrict__ g,
                              int need_inner, int jj, int kprev, V* __restrict__ w, const V* __restrict__ vprev,
                              const V* __restrict__ vk, double* __restrict__ part, int ntiles)
{
    using S = typename vt<V>::R;
    __shared__ double sh[2 * TILE_RG * TILE_CK];
    TileAcc T{sh};
    const int tile = blockIdx.x;
    const int r0 = tile * ROW_TILE, r1 = min(n, r0 + ROW_TILE);
    for (int c0 = 0; c0 < k; c0 += TILE_CK) {
        const int ck = min(TILE_CK, k - c0);
        for (int it = threadIdx.x; it < ck * TILE_RG; it += blockDim.x) {
            const int cc = it % ck, grp = it / ck, c = c0 + cc;
            double d0 = 0.0, d1 = 0.0;
            if (st[c].active == 1 && (!need_inner || g[c].inner)) {
                V h = vzero<V>();
                if (vprev) {
                    W hw = g[c].H[jj][kprev];
                    if constexpr (vt<V>::cplx) h = V{(S)re(hw), (S)im(hw)};
                    else h = (V)re(hw);
                }
                for (int i = r0 + grp; i < r1; i += TILE_RG) {
                    size_t o = (size_t)i * ld + c;
                    V a = w[o];
                    if (vprev) { a = vfms(a, h, vprev[o]); w[o] = a; }
                    if (vk) {
                        V b = vk[o];  // a * conj(b)
                        d0 += (double)re(a) * (double)re(b) + (double)im(a) * (double)im(b);
                        d1 += (double)im(a) * (double)re(b) - (double)re(a) * (double)im(b);
                    } else {
                        d0 += (double)nrm2(a);
                    }
                }
            }
            T.put(0, grp, cc, d0);
            T.put(1, grp, cc, d1);
        }
        __syncthreads();
        for (int cc = threadIdx.x; cc < ck; cc += blockDim.x) {
            const int c = c0 + cc;
            part[((size_t)c * 2) * ntiles + tile] = T.sum(0, cc);
            part[((size_t)c * 2 + 1) * ntiles + tile] = T.sum(1, cc);
        }
        __syncthreads();
    }
}

enum GmPhase : int { GM_NORMB = 0, GM_NORMX, GM_OUTER, GM_H, GM_HNORM };

// deterministic reduction of the tile partials (two parts) + the column's
// GMRES bookkeeping for the phase
template <class W>
__global__ void gm_reduce_kernel(int k, int ntiles, const double* __restrict__ part, ColState* __restrict__ st,
                                 GmCol<W>* __restrict__ g, int phase, int jj, int kk, double elim_n)
{
    const int c = blockIdx.x;
    if (c >= k) return;
    __shared__ double sh[2][256];
    double a0 = 0.0, a1 = 0.0;
    for (int t = threadIdx.x; t < ntiles; t += 256) {
        a0 += part[((size_t)c * 2) * ntiles + t];
        a1 += part[((size_t)c * 2 + 1) * ntiles + t];
    }
    sh[0][threadIdx.x] = a0;
    sh[1][threadIdx.x] = a1;
    __syncthreads();
    for (int s2 = 128; s2 > 0; s2 >>= 1) {
        if (threadIdx.x < s2) { sh[0][threadIdx.x] += sh[0][threadIdx.x + s2]; sh[1][threadIdx.x] += sh[1][threadIdx.x + s2]; }
        __syncthreads();
    }
    if (threadIdx.x) return;
    ColState& S = st[c];
    GmCol<W>& G = g[c];
    const double v0 = sh[0][0], v1 = sh[1][0];
    const double elim = S.tol;
    switch (phase) {
    case GM_NORMB:  // norm_b = |M b|
        G.norm_b = sqrt(v0);
        S.bnorm = G.norm_b;
        G.cycle = 0;
        S.its = 0;
        S.status = 0;
        S.active = (S.active == 1 && G.norm_b > 0.0) ? 1 : 0;
        break;
    case GM_NORMX:  // |x| < elim N selects v0 = Mb (gmres_imp.hpp:78-84)
        G.xsmall = sqrt(v0) < elim * elim_n;
        break;
    case GM_OUTER: {  // outer loop test and cycle start (gmres_imp.hpp:95-120)
        if (S.active != 1) break;
        const double norm_v = sqrt(v0);
        S.err = norm_v;
        if (!(norm_v > elim * G.norm_b && G.cycle < G.maxc)) {
            S.active = 0;
            S.status = norm_v > elim * G.norm_b ? 1 : 0;
            S.its = G.cycle;
            break;
        }
        G.s[0] = wfromre<W>(norm_v);
        G.j = -1;
        G.cycle++;
        S.its = G.cycle;
        G.inner = (wabs(G.s[0]) > elim * G.norm_b) && (G.j < GM_M - 1) && (G.cycle < G.maxc);
        G.jend = -1;
        break;
    }
    case GM_H:  // H(jj,kk) = sum w conj(v_kk)
        if (S.active == 1 && G.inner) G.H[jj][kk] = wfrom2<W>(v0, v1);
        break;
    case GM_HNORM: {  // H(jj,jj+1) = |w|, Givens rotations, next inner test
        if (!(S.active == 1 && G.inner)) break;
        const int j = jj;
        G.j = j;
        G.jend = j;
        G.hn = sqrt(v0);
        G.H[j][j + 1] = wfromre<W>(G.hn);
        for (int q = 0; q < j; q++) {
            W h1 = vadd(vmul(G.c1[q], G.H[j][q]), vmul(G.c2[q], G.H[j][q + 1]));
            W h2 = vadd(vmul(wneg(G.c2[q]), G.H[j][q]), vmul(G.c1[q], G.H[j][q + 1]));
            G.H[j][q] = h1;
            G.H[j][q + 1] = h2;
        }
        W r = wsqrt(vadd(vmul(G.H[j][j], G.H[j][j]), vmul(G.H[j][j + 1], G.H[j][j + 1])));
        G.c1[j] = wdiv(G.H[j][j], r);
        G.c2[j] = wdiv(G.H[j][j + 1], r);
        G.H[j][j] = r;
        G.H[j][j + 1] = wfromre<W>(0.0);
        G.s[j + 1] = vmul(wneg(G.c2[j]), G.s[j]);
        G.s[j] = vmul(G.s[j], G.c1[j]);
        G.inner = (wabs(G.s[j + 1]) > elim * G.norm_b) && (j < GM_M - 1) && (G.cycle < G.maxc);
        break;
    }
    }
}

// v = v / s0 (first basis vector) or v = v * (1 / H(jj,jj+1)) (new basis vector)
template <class V, class W>
__global__ void gm_scale_kernel(int n, int k, int ld, const ColState* __restrict__ st, const GmCol<W>* __restrict__ g,
                                int mode, int jj, V* __restrict__ v)
{
    using S = typename vt<V>::R;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    const int c = (int)(t % k);
    if (st[c].active != 1) return;
    const GmCol<W>& G = g[c];
    size_t o = (t / k) * ld + c;
    if (mode == 0) {
        if constexpr (vt<V>::cplx) {
            cd q = cdiv(cd{(double)v[o].x, (double)v[o].y}, cd{re(G.s[0]), im(G.s[0])});
            v[o] = V{(S)q.x, (S)q.y};
        } else {
            v[o] = (V)((double)v[o] / re(G.s[0]));
        }
    } else {
        if (G.jend != jj) return;  // column did not take this inner step
        const double tmp = 1.0 / G.hn;
        v[o] = vscale(v[o], (S)tmp);
    }
}

// back substitution H y = s (gmres_imp.hpp:175-182), one thread per column
template <class W>
__global__ void gm_solve_kernel(int k, const ColState* __restrict__ st, GmCol<W>* __restrict__ g)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k || st[c].active != 1) return;
    GmCol<W>& G = g[c];
    for (int l = G.jend; l >= 0; l--) {
        G.y[l] = wdiv(G.s[l], G.H[l][l]);
        for (int q = l - 1; q >= 0; q--) G.s[q] = vsub(G.s[q], vmul(G.H[l][q], G.y[l]));
    }
}

// x += sum_{l = jend..0} y_l v_l (gmres_imp.hpp:186-188); basis vectors at V + l * vstride
template <class V, class W>
__global__ void gm_update_kernel(int n, int k, int ld, const ColState* __restrict__ st,
                                 const GmCol<W>* __restrict__ g, const V* __restrict__ basis, size_t vstride,
                                 V* __restrict__ x)
{
    using S = typename vt<V>::R;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    const int c = (int)(t % k);
    if (st[c].active != 1) return;
    const GmCol<W>& G = g[c];
    size_t o = (t / k) * ld + c;
    V xv = x[o];
    for (int l = G.jend; l >= 0; l--) {
        V yl;
        if constexpr (vt<V>::cplx) yl = V{(S)re(G.y[l]), (S)im(G.y[l])};
        else yl = (V)re(G.y[l]);
        xv = vadd(xv, vmul(yl, basis[(size_t)l * vstride + o]));
    }
    x[o] = xv;
}

// v0 = Mb - t (t = M A x), or v0 = Mb where |x| < elim N on the first pass
template <class V, class W>
__global__ void gm_resid_kernel(int n, int k, int ld, const ColState* __restrict__ st,
                                const GmCol<W>* __restrict__ g, int first, const V* __restrict__ mb,
                                const V* __restrict__ t, V* __restrict__ v0)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * k) return;
    const int c = (int)(i % k);
    if (st[c].active != 1) return;
    size_t o = (i / k) * ld + c;
    v0[o] = (first && g[c].xsmall) ? mb[o] : vsub(mb[o], t[o]);
}

// number of columns still in the inner loop of their cycle
template <class W>
__global__ void gm_count_kernel(int k, const ColState* __restrict__ st, const GmCol<W>* __restrict__ g, int* out)
{
    __shared__ int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    int c = 0;
    for (int i = threadIdx.x; i < k; i += blockDim.x) c += (st[i].active == 1 && g[i].inner) ? 1 : 0;
    atomicAdd(&s, c);
    __syncthreads();
    if (threadIdx.x == 0) *out = s;
}

template <class W>
__global__ void gm_init_kernel(int k, GmCol<W>* __restrict__ g, int maxc)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    g[c].maxc = maxc;
    g[c].cycle = 0;
    g[c].inner = 0;
    g[c].j = -1;
    g[c].jend = -1;
}

}  // namespace tg
