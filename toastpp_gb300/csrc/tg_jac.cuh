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
__global__ void project_kernel(const int* __restrict__ nsup_p, const int* __restrict__ sup, const V* __restrict__ X, int ldx,
                               const V* __restrict__ Msup, int nm, const int* __restrict__ link_q,
                               const int* __restrict__ link_m, int nqm, int logscale, V* __restrict__ lin,
                               V* __restrict__ lg)
{
    int l = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x & 31;
    if (l >= nqm) return;
    int q = link_q[l], m = link_m[l], nsup = *nsup_p;
    V s = vzero<V>();
    for (int t = lane; t < nsup; t += 32) s = vfma(s, X[(size_t)sup[t] * ldx + q], Msup[(size_t)t * nm + m]);
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
// CTA: JT_NODES consecutive nodes x JT_M detectors, looping over sources in
// chunks of JT_Q; thread (qq, mm) writes JT_NODES consecutive J columns.
// ---------------------------------------------------------------------------
constexpr int JT_NODES = 8, JT_M = 8, JT_Q = 16;

template <class V>
struct JacArgs {
    MeshDev m;
    int nq, nm, nqm;
    const V* F; int ldf;          // forward fields, node-major
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

template <class V>
__global__ void __launch_bounds__(JT_Q * JT_M) jacobian_kernel(JacArgs<V> a)
{
    using S = typename vt<V>::R;
    extern __shared__ __align__(16) unsigned char jsm[];
    const MeshDev& m = a.m;
    int k0 = blockIdx.x * JT_NODES;
    int m0 = blockIdx.y * JT_M;
    int kend = min(m.n, k0 + JT_NODES);
    int base = m.rowptr[k0];
    int R = m.rowptr[kend] - base;
    V* Gs = (V*)jsm;                    // R x JT_M
    V* Hm = Gs + (size_t)R * JT_M;      // R x JT_M
    V* Hk = Hm + (size_t)R * JT_M;      // R x JT_M
    V* Fs = Hk + (size_t)R * JT_M;      // R x JT_Q
    int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < R * JT_M; e += nt) {
        int rr = e / JT_M, mm = e % JT_M;
        int mg = m0 + mm;
        Gs[e] = mg < a.nm ? a.G[(size_t)m.colidx[base + rr] * a.ldg + mg] : vzero<V>();
        Hm[e] = vzero<V>();
        Hk[e] = vzero<V>();
    }
    __syncthreads();
    // Phase B: H for each node of the tile (thread = node x detector)
    for (int w = tid; w < JT_NODES * JT_M; w += nt) {
        int t = w / JT_M, mm = w % JT_M;
        int k = k0 + t;
        if (k >= kend) continue;
        int rs = m.rowptr[k], re_ = m.rowptr[k + 1];
        for (int p = m.nel_ptr[k]; p < m.nel_ptr[k + 1]; p++) {
            int code = m.nel_list[p];
            int e = code >> 2, i = code & 3;
            const int* nd = m.el + (size_t)e * m.nn;
            const double* r = m.rec + (size_t)e * EL_REC;
            int pos[4];
            for (int j = 0; j < m.nn; j++) {  // position of node(e,j) in row k
                int lo = rs, hi = re_ - 1, target = nd[j];
                while (lo < hi) { int mid = (lo + hi) >> 1; if (m.colidx[mid] < target) lo = mid + 1; else hi = mid; }
                pos[j] = lo - base;
            }
            for (int j = 0; j < m.nn; j++) {
                V hm = Hm[pos[j] * JT_M + mm], hk = Hk[pos[j] * JT_M + mm];
                for (int l = 0; l < m.nn; l++) {
                    V g = Gs[pos[l] * JT_M + mm];
                    hm = vadd(hm, vscale(g, (S)el_intfff(m, r, i, j, l)));
                    hk = vadd(hk, vscale(g, (S)el_intfdd(m, r, j, l)));
                }
                Hm[pos[j] * JT_M + mm] = hm;
                Hk[pos[j] * JT_M + mm] = hk;
            }
        }
    }
    __syncthreads();
    int qq = tid / JT_M, mm = tid % JT_M;
    int mg = m0 + mm;
    int n = m.n;
    for (int q0 = 0; q0 < a.nq; q0 += JT_Q) {
        for (int e = tid; e < R * JT_Q; e += nt) {
            int rr = e / JT_Q, c = e % JT_Q;
            Fs[e] = (q0 + c) < a.nq ? a.F[(size_t)m.colidx[base + rr] * a.ldf + q0 + c] : vzero<V>();
        }
        __syncthreads();
        int q = q0 + qq;
        int l = (q < a.nq && mg < a.nm) ? a.pairidx[(size_t)q * a.nm + mg] : -1;
        if (l >= 0) {
            V yi = a.yinv ? a.yinv[l] : vzero<V>();
            S om[JT_NODES], ok[JT_NODES], oim[JT_NODES], oik[JT_NODES];
            for (int t = 0; t < JT_NODES; t++) {
                int k = k0 + t;
                V am = vzero<V>(), ak = vzero<V>();
                if (k < kend) {
                    for (int rr = m.rowptr[k] - base; rr < m.rowptr[k + 1] - base; rr++) {
                        V f = Fs[rr * JT_Q + qq];
                        am = vfma(am, f, Hm[rr * JT_M + mm]);
                        ak = vfma(ak, f, Hk[rr * JT_M + mm]);
                    }
                }
                if (a.yinv) { am = vmul(am, yi); ak = vmul(ak, yi); }
                om[t] = -re(am); ok[t] = -re(ak); oim[t] = -im(am); oik[t] = -im(ak);
            }
            int cnt = kend - k0;
            if constexpr (vt<V>::cplx) {
                size_t r0 = (size_t)l * 2 * n, r1 = (size_t)(l + a.nqm) * 2 * n;
                if (a.out_fp32) {
                    float* J = (float*)a.J;
                    for (int t = 0; t < cnt; t++) {
                        J[r0 + k0 + t] = (float)om[t]; J[r1 + k0 + t] = (float)oim[t];
                        J[r0 + n + k0 + t] = (float)ok[t]; J[r1 + n + k0 + t] = (float)oik[t];
                    }
                } else {
                    double* J = (double*)a.J;
                    for (int t = 0; t < cnt; t++) {
                        J[r0 + k0 + t] = om[t]; J[r1 + k0 + t] = oim[t];
                        J[r0 + n + k0 + t] = ok[t]; J[r1 + n + k0 + t] = oik[t];
                    }
                }
            } else {
                size_t r0 = (size_t)l * n, r1 = (size_t)(l + a.nqm) * n;
                if (a.out_fp32) {
                    float* J = (float*)a.J;
                    for (int t = 0; t < cnt; t++) { J[r0 + k0 + t] = (float)om[t]; J[r1 + k0 + t] = (float)ok[t]; }
                } else {
                    double* J = (double*)a.J;
                    for (int t = 0; t < cnt; t++) { J[r0 + k0 + t] = om[t]; J[r1 + k0 + t] = ok[t]; }
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace tg
