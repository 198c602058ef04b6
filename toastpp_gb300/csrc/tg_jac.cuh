// tg_jac.cuh -- ProjectAll and the nodal-basis Jacobian.
#pragma once
#include "tg_kernels.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// ProjectAll (src/libstoast/fwdsolver.cc:1415-1447): y_l = sum_i phi_q[i] mvec_m[i]
// (non-conjugating) for each link l = (q, m).  The detector vectors are stored
// compressed to their common support (boundary nodes for Neumann detectors):
// Msup[s * nm + m] at node sup[s].  One warp per link; the log option gives
// ln|y| + i arg(y) (std::log of a complex).
// ---------------------------------------------------------------------------
// support of the detector vectors: nodes where any detector is nonzero
template <class V>
__global__ void support_flag_kernel(int n, int nm, const V* __restrict__ mvec, int* __restrict__ flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int f = 0;
    for (int m = 0; m < nm && !f; m++) { V v = mvec[(size_t)m * n + i]; f = (re(v) != 0 || im(v) != 0); }
    flag[i] = f;
}

// ordered compaction by one block (deterministic): sup = indices with flag set
static __global__ void support_scan_kernel(int n, const int* __restrict__ flag, int* __restrict__ sup, int* __restrict__ nsup)
{
    __shared__ int cnt[1024];
    int t = threadIdx.x, nt = blockDim.x;
    int per = (n + nt - 1) / nt, b = t * per, e = min(n, b + per);
    int c = 0;
    for (int i = b; i < e; i++) c += flag[i];
    cnt[t] = c;
    __syncthreads();
    if (t == 0) {
        int acc = 0;
        for (int j = 0; j < nt; j++) { int v = cnt[j]; cnt[j] = acc; acc += v; }
        *nsup = acc;
    }
    __syncthreads();
    int o = cnt[t];
    for (int i = b; i < e; i++) if (flag[i]) sup[o++] = i;
}

template <class V>
__global__ void support_gather_kernel(int n, int nm, const int* __restrict__ nsup, const int* __restrict__ sup,
                                      const V* __restrict__ mvec, V* __restrict__ Msup)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    int ns = *nsup;
    if (t >= (size_t)ns * nm) return;
    int s = (int)(t / nm), m = (int)(t % nm);
    Msup[t] = mvec[(size_t)m * n + sup[s]];
}

template <class To, class From>
__global__ void recip_cast_kernel(int cnt, const From* __restrict__ y, To* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    out[i] = vcast<To, From>(vrecip(y[i]));
}

template <class V>
__global__ void project_kernel(const int* __restrict__ nsup_p, const int* __restrict__ sup,
                               const int* __restrict__ perm, const V* __restrict__ X, int ldx,
                               const V* __restrict__ Msup, int nm, const int* __restrict__ link_q,
                               const int* __restrict__ link_m, int nqm, int logscale, V* __restrict__ lin,
                               V* __restrict__ lg)
{
    int l = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x & 31;
    if (l >= nqm) return;
    int q = link_q[l], m = link_m[l], nsup = *nsup_p;
    V s = vzero<V>();
    for (int t = lane; t < nsup; t += 32) s = vfma(s, X[(size_t)perm[sup[t]] * ldx + q], Msup[(size_t)t * nm + m]);
    for (int o = 16; o; o >>= 1) {
        if constexpr (vt<V>::cplx) { s.x += __shfl_down_sync(0xffffffffu, s.x, o); s.y += __shfl_down_sync(0xffffffffu, s.y, o); }
        else s += __shfl_down_sync(0xffffffffu, s, o);
    }
    if (lane) return;
    if (lin) lin[l] = s;
    if (lg) {
        if constexpr (vt<V>::cplx) lg[l] = V{log(hypot(s.x, s.y)), atan2(s.y, s.x)};
        else lg[l] = log(s);
    }
}

// ---------------------------------------------------------------------------
// Nodal Jacobian (GenerateJacobian_mesh, src/libstoast/jacobian.cc:441-497;
// GenerateJacobian_cw_mesh, 738-802).  For node k, with N(k) the nodes that
// share an element with k (CSR row k):
//   PMDF_mua[q,m,k] = sum_{a in N(k)} f_q(a) Hm_k[a,m],
//     Hm_k[a,m] = sum_{e ∋ k} sum_{j: node(e,j)=a} sum_l IntFFF_e(i_k,j,l) g_m(node(e,l))
//   PMDF_kap[q,m,k] = same with IntFDD_e (IntFG / IntGradFGradG, 806-872),
// i.e. the reference's element loops regrouped per node (f = forward field,
// g = adjoint field, no conjugation).  J = -Re / -Im of PMDF (divided by the
// linear projection for log data, PMDF_log 76-79).
//
// CTA: KT consecutive nodes (one per lane) x JM detectors, looping over the
// sources in chunks of JQ.  Phase B builds Hm/Hk for the tile in shared
// memory (thread = node x detector); phase C gives each lane JR_Q sources x
// JR_M detectors of its node, so a warp writes KT consecutive J columns
// (coalesced) for each of its pairs.
constexpr int JM = 8, JQ = 8, JR_Q = 2, JR_M = 4;

template <class V>
struct JacArgs {
    MeshDev m;
    int nq, nm, nqm;
    const V* F; int ldf;          // forward fields, node-major (column q of row i at i*ldf + q)
    const V* G; int ldg;          // adjoint fields, node-major
    const int* pairidx;           // nq*nm -> link index or -1
    const V* yinv;                // per link 1/y (log data) or null
    void* J;                      // output
    int out_fp32;
};

__device__ __forceinline__ double el_intfff(const MeshDev& m, const double* r, int i, int j, int l)
{
    if (m.dim == 2) {
        // Triangle3::IntFFF (tri3.cc:294-297): size * {1/60, 1/30, 1/10}[#equal]
        int eq = (i == j) + (i == l) + (j == l);
        double sc = eq == 0 ? 1.0 / 60.0 : (eq == 1 ? 1.0 / 30.0 : 1.0 / 10.0);
        return r[0] * sc;
    }
    return c_tet_fff[i][j][l] / 120.0 * r[0];  // Tetrahedron4::IntFFF (tet4.cc:357-361)
}

__device__ __forceinline__ double el_intfdd(const MeshDev& m, const double* r, int j, int l)
{
    if (m.dim == 2) return r[1 + j * 3 + l] * 0.3333333333;  // tri3.h:196-197 (sic)
    return r[1 + j * 4 + l];                                  // tet4.cc:380-412
}

template <class V, class OUT>
__device__ __forceinline__ void jac_store(OUT* J, size_t idx, typename vt<V>::R v) { J[idx] = (OUT)v; }

template <class V, int KT>
__global__ void __launch_bounds__(256) jacobian_kernel(JacArgs<V> a)
{
    using S = typename vt<V>::R;
    extern __shared__ __align__(16) unsigned char jsm[];
    const MeshDev& m = a.m;
    const int k0 = blockIdx.x * KT;
    const int m0 = blockIdx.y * JM;
    const int kend = min(m.n, k0 + KT);
    const int base = m.jrowptr[k0];
    const int R = m.jrowptr[kend] - base;
    V* Gs = (V*)jsm;                    // R x JM
    V* Hm = Gs + (size_t)R * JM;        // R x JM
    V* Hk = Hm + (size_t)R * JM;        // R x JM
    V* Fs = Hk + (size_t)R * JM;        // R x JQ
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < R * JM; e += nt) {
        int rr = e / JM, mm = e % JM, mg = m0 + mm;
        Gs[e] = mg < a.nm ? a.G[(size_t)m.jcolidx[base + rr] * a.ldg + mg] : vzero<V>();
        Hm[e] = vzero<V>();
        Hk[e] = vzero<V>();
    }
    __syncthreads();
    // Phase B: Hm/Hk rows of every node of the tile; thread = (node, detector).
    // The IntFFF weights of P1 elements are size/D x {6 all equal, 2 two equal,
    // 1 distinct} (D = 60 triangles, 120 tetrahedra), so for the element node
    // i = k:  sum_l IntFFF(i,j,l) g_l = size/D (2 SG + 4 g_i) for j = i and
    // size/D (SG + g_i + g_j) otherwise, SG = sum of g over the element.
    for (int w = tid; w < KT * JM; w += nt) {
        int t = w / JM, mm = w % JM, k = k0 + t;
        if (k >= kend) continue;
        const int rk = m.jrowptr[k] - base;
        const S inv_d = (S)(m.dim == 2 ? 1.0 / 60.0 : 1.0 / 120.0);
        for (int p = m.nel_ptr[k]; p < m.nel_ptr[k + 1]; p++) {
            const int code = m.nel_list[p];
            const int e = code >> 2, i = code & 3;
            const unsigned pk = m.nel_pos[p];
            const double* r = m.rec + (size_t)e * EL_REC;
            int pos[4];
            V g[4];
            V sg = vzero<V>();
            for (int j = 0; j < m.nn; j++) {
                pos[j] = rk + (int)((pk >> (8 * j)) & 255u);
                g[j] = Gs[pos[j] * JM + mm];
                sg = vadd(sg, g[j]);
            }
            const S cf = (S)r[0] * inv_d;
            for (int j = 0; j < m.nn; j++) {
                V wm = j == i ? vadd(vscale(sg, (S)2), vscale(g[i], (S)4)) : vadd(vadd(sg, g[i]), g[j]);
                V hk = vzero<V>();
                for (int l = 0; l < m.nn; l++) hk = vadd(hk, vscale(g[l], (S)el_intfdd(m, r, j, l)));
                Hm[pos[j] * JM + mm] = vadd(Hm[pos[j] * JM + mm], vscale(wm, cf));
                Hk[pos[j] * JM + mm] = vadd(Hk[pos[j] * JM + mm], hk);
            }
        }
    }
    __syncthreads();
    // Phase C: lane = node of the tile; warp = a group of JR_Q x JR_M pairs
    const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
    const int t = lane, k = k0 + t;
    const bool kin = (t < KT) && (k < kend);
    const int rb = kin ? m.jrowptr[k] - base : 0, re2 = kin ? m.jrowptr[k + 1] - base : 0;
    const int n = m.n;
    constexpr int GQ = JQ / JR_Q, GM = JM / JR_M;  // pair groups per chunk
    for (int q0 = 0; q0 < a.nq; q0 += JQ) {
        for (int e = tid; e < R * JQ; e += nt) {
            int rr = e / JQ, c = e % JQ;
            Fs[e] = (q0 + c) < a.nq ? a.F[(size_t)m.jcolidx[base + rr] * a.ldf + q0 + c] : vzero<V>();
        }
        __syncthreads();
        for (int grp = warp; grp < GQ * GM; grp += nwarp) {
            int qq0 = (grp / GM) * JR_Q, mm0 = (grp % GM) * JR_M;
            V am[JR_Q][JR_M], ak[JR_Q][JR_M];
#pragma unroll
            for (int a1 = 0; a1 < JR_Q; a1++)
#pragma unroll
                for (int b1 = 0; b1 < JR_M; b1++) { am[a1][b1] = vzero<V>(); ak[a1][b1] = vzero<V>(); }
            for (int rr = rb; rr < re2; rr++) {
                V f[JR_Q], hm[JR_M], hk[JR_M];
#pragma unroll
                for (int a1 = 0; a1 < JR_Q; a1++) f[a1] = Fs[rr * JQ + qq0 + a1];
#pragma unroll
                for (int b1 = 0; b1 < JR_M; b1++) { hm[b1] = Hm[rr * JM + mm0 + b1]; hk[b1] = Hk[rr * JM + mm0 + b1]; }
#pragma unroll
                for (int a1 = 0; a1 < JR_Q; a1++)
#pragma unroll
                    for (int b1 = 0; b1 < JR_M; b1++) {
                        am[a1][b1] = vfma(am[a1][b1], f[a1], hm[b1]);
                        ak[a1][b1] = vfma(ak[a1][b1], f[a1], hk[b1]);
                    }
            }
            if (!kin) continue;
#pragma unroll
            for (int a1 = 0; a1 < JR_Q; a1++)
#pragma unroll
                for (int b1 = 0; b1 < JR_M; b1++) {
                    int q = q0 + qq0 + a1, mg = m0 + mm0 + b1;
                    if (q >= a.nq || mg >= a.nm) continue;
                    int l = a.pairidx[(size_t)q * a.nm + mg];
                    if (l < 0) continue;
                    V xm = am[a1][b1], xk = ak[a1][b1];
                    if (a.yinv) { V yi = a.yinv[l]; xm = vmul(xm, yi); xk = vmul(xk, yi); }
                    if constexpr (vt<V>::cplx) {
                        size_t r0 = (size_t)l * 2 * n + k, r1 = (size_t)(l + a.nqm) * 2 * n + k;
                        if (a.out_fp32) {
                            float* J = (float*)a.J;
                            J[r0] = (float)-re(xm); J[r1] = (float)-im(xm);
                            J[r0 + n] = (float)-re(xk); J[r1 + n] = (float)-im(xk);
                        } else {
                            double* J = (double*)a.J;
                            J[r0] = -re(xm); J[r1] = -im(xm);
                            J[r0 + n] = -re(xk); J[r1 + n] = -im(xk);
                        }
                    } else {
                        size_t r0 = (size_t)l * n + k, r1 = (size_t)(l + a.nqm) * n + k;
                        if (a.out_fp32) {
                            float* J = (float*)a.J;
                            J[r0] = (float)-xm; J[r1] = (float)-xk;
                        } else {
                            double* J = (double*)a.J;
                            J[r0] = -xm; J[r1] = -xk;
                        }
                    }
                }
        }
        __syncthreads();
    }
}

}  // namespace tg
