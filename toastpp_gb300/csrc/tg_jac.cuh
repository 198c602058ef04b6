// tg_jac.cuh -- ProjectAll and the nodal-basis Jacobian.
#pragma once
#include <cuda_bf16.h>
#include <type_traits>
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
// Layout.  Tile = 32 consecutive (natural) nodes, one per lane.  Each node's
// neighbours are "slots" (i, t) = i * 32 + t, i < D (the largest node degree):
// slot (i, t) is the i-th entry of CSR row k0 + t, or padding.  All per-slot
// arrays in shared memory are column-major [column][slot] with an odd column
// stride SP, so a warp reading slot i of its 32 nodes touches 32 consecutive
// words (no bank conflicts), and the writes of J along k are coalesced.
//
// The element integrals are gathered per node once per mesh (they depend on
// the geometry only): Wm_k[i][j] = sum_{e ∋ k} IntFFF_e(k, a_i, a_j) and
// Wk_k[i][j] = sum_{e ∋ k} IntFDD_e(a_i, a_j), stored tile-interleaved
// W[((tile * D + i) * D + j) * 32 + t].  Then Hm_k[a_i, m] =
// sum_j Wm_k[i][j] g_m(a_j) (and Hk likewise) is a small dense product.
//
// CTA = one tile x JM detectors; the sources are streamed in chunks of JQ
// through two cp.async buffers (the next chunk loads while this one is used).
// Phase C: lane = node, warp = JRQ x JRM (source, detector) pairs.
constexpr int JKT = 32;

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
    const typename vt<V>::R* Wm;  // per-node element weights (tile-interleaved)
    const typename vt<V>::R* Wk;
    int D, SP, nmc;               // slots per node, column stride, detector chunks
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

// per-node weights, FP64, into zeroed Wm/Wk; thread = node (its own slots only)
static __global__ void jac_weights_kernel(MeshDev m, int D, double* __restrict__ Wm, double* __restrict__ Wk)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n) return;
    const size_t tb = (size_t)(k / JKT) * D * D * JKT + (k % JKT);
    for (int p = m.nel_ptr[k]; p < m.nel_ptr[k + 1]; p++) {
        const int code = m.nel_list[p], e = code >> 2, i = code & 3;
        const unsigned pk = m.nel_pos[p];
        const double* r = m.rec + (size_t)e * EL_REC;
        for (int x = 0; x < m.nn; x++) {
            const int px = (int)((pk >> (8 * x)) & 255u);
            for (int y = 0; y < m.nn; y++) {
                const int py = (int)((pk >> (8 * y)) & 255u);
                const size_t o = tb + ((size_t)px * D + py) * JKT;
                Wm[o] += el_intfff(m, r, i, x, y);
                Wk[o] += el_intfdd(m, r, x, y);
            }
        }
    }
}

// packed FP32x2 arithmetic (sm_100+ fma.rn.f32x2): one instruction, two lanes
__device__ __forceinline__ unsigned long long f2_pack(float a, float b)
{
    unsigned long long d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long a)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a));
    return r;
}

// Phase C for complex FP32: sum_i f_i h_i kept as four real sums, two per
// packed register: P = (sum fr hr, sum fr hi), Q = (sum fi hr, sum fi hi);
// then Re = P.x - Q.y, Im = P.y + Q.x.
template <int JRQ, int JRM>
__device__ __forceinline__ void jac_pairs_c32(const cf* __restrict__ Fs, const cf* __restrict__ Hm,
                                              const cf* __restrict__ Hk, int SP, int qq0, int mm0, int dmax,
                                              int lane, cf (&am)[JRQ][JRM], cf (&ak)[JRQ][JRM])
{
    unsigned long long pm[JRQ][JRM], qm[JRQ][JRM], pk[JRQ][JRM], qk[JRQ][JRM];
#pragma unroll
    for (int x = 0; x < JRQ; x++)
#pragma unroll
        for (int y = 0; y < JRM; y++) pm[x][y] = qm[x][y] = pk[x][y] = qk[x][y] = 0ull;
    const unsigned long long* F = reinterpret_cast<const unsigned long long*>(Fs) + (size_t)qq0 * SP + lane;
    const unsigned long long* M = reinterpret_cast<const unsigned long long*>(Hm) + (size_t)mm0 * SP + lane;
    const unsigned long long* K = reinterpret_cast<const unsigned long long*>(Hk) + (size_t)mm0 * SP + lane;
#pragma unroll 2
    for (int i = 0; i < dmax; i++) {
        const int s = i * JKT;
        unsigned long long frr[JRQ], fii[JRQ], hm[JRM], hk[JRM];
#pragma unroll
        for (int x = 0; x < JRQ; x++) {
            const float2 f = f2_unpack(F[(size_t)x * SP + s]);
            frr[x] = f2_pack(f.x, f.x);
            fii[x] = f2_pack(f.y, f.y);
        }
#pragma unroll
        for (int y = 0; y < JRM; y++) { hm[y] = M[(size_t)y * SP + s]; hk[y] = K[(size_t)y * SP + s]; }
#pragma unroll
        for (int x = 0; x < JRQ; x++)
#pragma unroll
            for (int y = 0; y < JRM; y++) {
                pm[x][y] = f2_fma(frr[x], hm[y], pm[x][y]);
                qm[x][y] = f2_fma(fii[x], hm[y], qm[x][y]);
                pk[x][y] = f2_fma(frr[x], hk[y], pk[x][y]);
                qk[x][y] = f2_fma(fii[x], hk[y], qk[x][y]);
            }
    }
#pragma unroll
    for (int x = 0; x < JRQ; x++)
#pragma unroll
        for (int y = 0; y < JRM; y++) {
            const float2 p = f2_unpack(pm[x][y]), q = f2_unpack(qm[x][y]);
            const float2 u = f2_unpack(pk[x][y]), v = f2_unpack(qk[x][y]);
            am[x][y] = cf{p.x - q.y, p.y + q.x};
            ak[x][y] = cf{u.x - v.y, u.y + v.x};
        }
}

template <class V, int JQ, int JM, int JRQ, int JRM, int NT>
__global__ void __launch_bounds__(NT) jacobian_kernel(JacArgs<V> a)
{
    using S = typename vt<V>::R;
    static_assert(JM <= JQ, "the adjoint block shares a source buffer");
    extern __shared__ __align__(16) unsigned char jsm[];
    const MeshDev& m = a.m;
    const int SP = a.SP, D = a.D;
    const int tile = blockIdx.x / a.nmc, m0 = (blockIdx.x % a.nmc) * JM;
    const int k0 = tile * JKT;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    V* Hm = (V*)jsm;                          // [JM][SP]
    V* Hk = Hm + (size_t)JM * SP;             // [JM][SP]
    V* Fb = Hk + (size_t)JM * SP;             // 2 x [JQ][SP]
    V* yis = Fb + (size_t)2 * JQ * SP;             // [nq][JM]: 1 / y of the link (log data)
    int* lidx = (int*)(yis + (size_t)a.nq * JM);   // [nq][JM]: link index or -1
    int* sidx = lidx + (size_t)a.nq * JM;          // [D * 32]: field row of each slot, -1 padding
    const int k = k0 + lane;
    const bool kin = k < m.n;
    const int deg = kin ? m.jrowptr[k + 1] - m.jrowptr[k] : 0;
    const int dmax = __reduce_max_sync(0xffffffffu, deg);
    const int nslot = dmax * JKT;
    for (int s = tid; s < nslot; s += blockDim.x) {
        const int i = s / JKT, kk = k0 + s % JKT;
        int r = -1;
        if (kk < m.n) {
            const int b = m.jrowptr[kk];
            if (i < m.jrowptr[kk + 1] - b) r = m.jcolidx[b + i];
        }
        sidx[s] = r;
    }
    for (int e = tid; e < a.nq * JM; e += blockDim.x) {
        const int q = e / JM, mg = m0 + e % JM;
        const int l = mg < a.nm ? a.pairidx[(size_t)q * a.nm + mg] : -1;
        lidx[e] = l;
        if (a.yinv) yis[e] = l >= 0 ? a.yinv[l] : vzero<V>();
    }
    __syncthreads();
    auto load_chunk = [&](int q0, V* Fs) {
        for (int e = tid; e < JQ * nslot; e += blockDim.x) {
            const int c = e % JQ, s = e / JQ, r = sidx[s];
            V* dst = Fs + (size_t)c * SP + s;
            if (r >= 0 && q0 + c < a.nq) cp_async_val<sizeof(V)>(dst, a.F + (size_t)r * a.ldf + q0 + c);
            else *dst = vzero<V>();
        }
        cp_async_commit();
    };
    load_chunk(0, Fb);
    // adjoint fields of the slots into the second buffer
    V* Gs = Fb + (size_t)JQ * SP;
    for (int e = tid; e < JM * nslot; e += blockDim.x) {
        const int mm = e % JM, s = e / JM, r = sidx[s], mg = m0 + mm;
        Gs[(size_t)mm * SP + s] = (r >= 0 && mg < a.nm) ? a.G[(size_t)r * a.ldg + mg] : vzero<V>();
    }
    __syncthreads();
    // Phase B: H[mm][slot(i, t)] = sum_j W_t[i][j] Gs[mm][slot(j, t)].  Warp =
    // rows i; each weight is loaded once (coalesced over the tile's nodes) and
    // used for every detector of the block.
    {
        const size_t tb = (size_t)tile * D * D * JKT + lane;
        for (int i = warp; i < dmax; i += blockDim.x / 32) {
            V hm[JM], hk[JM];
#pragma unroll
            for (int mm = 0; mm < JM; mm++) { hm[mm] = vzero<V>(); hk[mm] = vzero<V>(); }
            const S* wm = a.Wm + tb + (size_t)i * D * JKT;
            const S* wk = a.Wk + tb + (size_t)i * D * JKT;
#pragma unroll 4
            for (int j = 0; j < dmax; j++) {
                const S xm = wm[(size_t)j * JKT], xk = wk[(size_t)j * JKT];
#pragma unroll
                for (int mm = 0; mm < JM; mm++) {
                    const V g = Gs[(size_t)mm * SP + j * JKT + lane];
                    hm[mm] = vadd(hm[mm], vscale(g, xm));
                    hk[mm] = vadd(hk[mm], vscale(g, xk));
                }
            }
#pragma unroll
            for (int mm = 0; mm < JM; mm++) {
                Hm[(size_t)mm * SP + i * JKT + lane] = hm[mm];
                Hk[(size_t)mm * SP + i * JKT + lane] = hk[mm];
            }
        }
    }
    __syncthreads();
    const int n = m.n;
    constexpr int GM = JM / JRM, NG = (JQ / JRQ) * GM;
    const int nch = (a.nq + JQ - 1) / JQ;
    for (int ch = 0; ch < nch; ch++) {
        if (ch + 1 < nch) {
            load_chunk((ch + 1) * JQ, Fb + (size_t)((ch + 1) & 1) * JQ * SP);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const V* Fs = Fb + (size_t)(ch & 1) * JQ * SP;
        const int q0 = ch * JQ;
        for (int grp = warp; grp < NG; grp += blockDim.x / 32) {
            const int qq0 = (grp / GM) * JRQ, mm0 = (grp % GM) * JRM;
            V am[JRQ][JRM], ak[JRQ][JRM];
            if constexpr (std::is_same<V, cf>::value) {
                jac_pairs_c32<JRQ, JRM>(Fs, Hm, Hk, SP, qq0, mm0, dmax, lane, am, ak);
            } else {
#pragma unroll
            for (int x = 0; x < JRQ; x++)
#pragma unroll
                for (int y = 0; y < JRM; y++) { am[x][y] = vzero<V>(); ak[x][y] = vzero<V>(); }
#pragma unroll 2
            for (int i = 0; i < dmax; i++) {
                const int s = i * JKT + lane;
                V f[JRQ], hm[JRM], hk[JRM];
#pragma unroll
                for (int x = 0; x < JRQ; x++) f[x] = Fs[(size_t)(qq0 + x) * SP + s];
#pragma unroll
                for (int y = 0; y < JRM; y++) { hm[y] = Hm[(size_t)(mm0 + y) * SP + s]; hk[y] = Hk[(size_t)(mm0 + y) * SP + s]; }
#pragma unroll
                for (int x = 0; x < JRQ; x++)
#pragma unroll
                    for (int y = 0; y < JRM; y++) {
                        am[x][y] = vfma(am[x][y], f[x], hm[y]);
                        ak[x][y] = vfma(ak[x][y], f[x], hk[y]);
                    }
            }
            }
            if (!kin) continue;
#pragma unroll
            for (int x = 0; x < JRQ; x++)
#pragma unroll
                for (int y = 0; y < JRM; y++) {
                    const int q = q0 + qq0 + x, mg = m0 + mm0 + y;
                    if (q >= a.nq || mg >= a.nm) continue;
                    const int l = lidx[q * JM + mm0 + y];
                    if (l < 0) continue;
                    V xm = am[x][y], xk = ak[x][y];
                    if (a.yinv) { const V yi = yis[q * JM + mm0 + y]; xm = vmul(xm, yi); xk = vmul(xk, yi); }
                    if constexpr (vt<V>::cplx) {
                        const size_t r0 = (size_t)l * 2 * n + k, r1 = (size_t)(l + a.nqm) * 2 * n + k;
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
                        const size_t r0 = (size_t)l * n + k, r1 = (size_t)(l + a.nqm) * n + k;
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


// ---------------------------------------------------------------------------
// Nodal Jacobian with FP64 accuracy at FP32 throughput ("float-float").
//
// GB300 issues FP64 at about 1/60 of its FP32 rate, and the Jacobian's pair
// loop (two complex products per neighbour, per (source, detector, node)) is
// 44 GFLOP for the 30k cylinder, so the plain FP64 kernel is bound by the
// FP64 pipe.  Here every FP64 quantity is carried as an unevaluated sum of
// two floats hi + lo (|lo| <= ulp(hi)/2): products are made exact with a
// fused multiply-add (p = a*b, e = fma(a, b, -p)), the cross terms a_hi b_lo
// and a_lo b_hi join the error, and each sum is compensated (TwoSum: the
// rounding error of every addition is recovered exactly and accumulated).
// The result carries about 44 significant bits, well past what an FP64 J
// from FP64 fields needs.  The mua and kappa parts share every field value,
// so they travel as the two halves of packed f32x2 registers.  FP32 range:
// the fields and their products stay within 1e-38..1e38 for these models
// (they decay by at most e^-40 across a domain).
// Layout as jacobian_kernel: tile of 32 nodes (lane = node), slots i*32+t.
// ---------------------------------------------------------------------------
typedef unsigned long long f2x;  // packed (mua, kappa) floats

__device__ __forceinline__ f2x f2_add(f2x a, f2x b)
{
    f2x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b)
{
    f2x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b)
{
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_neg(f2x a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ f2x f2_bcast(float a) { return f2_pack(a, a); }

// (sh, sl) += (ah, al) * (bh, bl), lane by lane: exact product by FMA plus
// the cross terms, TwoSum of the leading parts, errors into sl
__device__ __forceinline__ void ff2_mac(f2x& sh, f2x& sl, f2x ah, f2x al, f2x bh, f2x bl)
{
    const f2x p = f2_mul(ah, bh);
    f2x e = f2_fma(ah, bh, f2_neg(p));  // a*b - p, exact
    e = f2_fma(ah, bl, e);
    e = f2_fma(al, bh, e);
    const f2x t = f2_add(sh, p);
    const f2x bp = f2_sub(t, sh);
    const f2x err = f2_add(f2_sub(sh, f2_sub(t, bp)), f2_sub(p, bp));
    sh = t;
    sl = f2_add(sl, f2_add(err, e));
}

// hi + lo as a double: a TwoSum in FP32 first (so the parts no longer
// overlap), then the two exact conversions and one FP64 addition
__device__ __forceinline__ double ff_to_double(float h, float l)
{
    const float t = __fadd_rn(h, l);
    const float bp = __fsub_rn(t, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(t, bp)), __fsub_rn(l, bp));
    return (double)t + (double)e;
}

// a double as (hi, lo)
__device__ __forceinline__ float2 ff_split(double x)
{
    const float h = __double2float_rn(x);
    return make_float2(h, __double2float_rn(x - (double)h));
}

// node-major FP64 fields (n rows, columns c < k at stride ld) as float-float:
// complex -> float4 (re_hi, re_lo, im_hi, im_lo), real -> float2 (hi, lo)
template <bool CPLX>
__global__ void ff_split_fields_kernel(int n, int k, const double* __restrict__ a, int ld, void* __restrict__ out)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * k) return;
    const size_t i = t / k, c = t % k;
    if constexpr (CPLX) {
        const double re = a[2 * (i * ld + c)], im = a[2 * (i * ld + c) + 1];
        const float2 r = ff_split(re), q = ff_split(im);
        ((float4*)out)[t] = make_float4(r.x, r.y, q.x, q.y);
    } else {
        ((float2*)out)[t] = ff_split(a[i * ld + c]);
    }
}

// per-node weights (FP64, tile-interleaved) as packed float-float:
// float4 (Wm_hi, Wk_hi, Wm_lo, Wk_lo)
static __global__ void ff_split_weights_kernel(size_t cnt, const double* __restrict__ wm, const double* __restrict__ wk,
                                               float4* __restrict__ out)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const float2 a = ff_split(wm[t]), b = ff_split(wk[t]);
    out[t] = make_float4(a.x, b.x, a.y, b.y);
}

struct JacFFArgs {
    MeshDev m;
    int nq, nm, nqm, cplx;
    const void* F;                // float-float forward fields, node-major, ld nq
    const void* G;                // float-float adjoint fields, node-major, ld nm
    const int* pairidx;           // nq*nm -> link index or -1
    const float4* yinv;           // per link 1/y as (re_hi, re_lo, im_hi, im_lo), or null
    double* J;                    // FP64 output, or
    float* J32;                   // FP32 output (each hi + lo rounded once to float)
    const float4* W;              // packed float-float weights
    int D, SP, nmc;
};

// CTA = one 32-node tile x JM detectors, sources streamed in chunks of JQ;
// phase B forms H = W G for the JM detectors (packed mua/kappa, float-float),
// phase C has one (source, detector) pair per warp, lane = node.
template <bool CPLX, int JQ, int JM, int NT>
__global__ void __launch_bounds__(NT) jacobian_ff_kernel(JacFFArgs a)
{
    // field items: complex float4 (re_hi, re_lo, im_hi, im_lo), real float2
    using FI = typename std::conditional<CPLX, float4, float2>::type;
    // H words: complex re_hi, re_lo, im_hi, im_lo; real hi, lo (packed f2x)
    constexpr int HW = CPLX ? 4 : 2;
    static_assert(JM <= JQ, "the adjoint block shares a source buffer");
    extern __shared__ __align__(16) unsigned char jsm[];
    const MeshDev& m = a.m;
    const int SP = a.SP, D = a.D;
    const int tile = blockIdx.x / a.nmc, m0 = (blockIdx.x % a.nmc) * JM;
    const int k0 = tile * JKT;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    f2x* Hs = (f2x*)jsm;                                   // [HW][JM][SP]
    FI* Fb = (FI*)(Hs + (size_t)JM * SP * HW);             // 2 x [JQ][SP]
    float4* yis = (float4*)(Fb + (size_t)2 * JQ * SP);     // [nq][JM]
    int* lidx = (int*)(yis + (size_t)a.nq * JM);           // [nq][JM]
    int* sidx = lidx + (size_t)a.nq * JM;                  // [D * 32]
    const FI* F = (const FI*)a.F;
    const FI* G = (const FI*)a.G;
    const int k = k0 + lane;
    const bool kin = k < m.n;
    const int deg = kin ? m.jrowptr[k + 1] - m.jrowptr[k] : 0;
    const int dmax = __reduce_max_sync(0xffffffffu, deg);
    const int nslot = dmax * JKT;
    for (int s = tid; s < nslot; s += blockDim.x) {
        const int i = s / JKT, kk = k0 + s % JKT;
        int r = -1;
        if (kk < m.n) {
            const int b = m.jrowptr[kk];
            if (i < m.jrowptr[kk + 1] - b) r = m.jcolidx[b + i];
        }
        sidx[s] = r;
    }
    for (int e = tid; e < a.nq * JM; e += blockDim.x) {
        const int q = e / JM, mg = m0 + e % JM;
        const int l = mg < a.nm ? a.pairidx[(size_t)q * a.nm + mg] : -1;
        lidx[e] = l;
        if (a.yinv) yis[e] = l >= 0 ? a.yinv[l] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    FI zero;
    memset(&zero, 0, sizeof(FI));
    auto load_chunk = [&](int q0, FI* Fs) {
        for (int e = tid; e < JQ * nslot; e += blockDim.x) {
            const int c = e % JQ, s = e / JQ, r = sidx[s];
            FI* dst = Fs + (size_t)c * SP + s;
            if (r >= 0 && q0 + c < a.nq) cp_async_val<sizeof(FI)>(dst, F + (size_t)r * a.nq + q0 + c);
            else *dst = zero;
        }
        cp_async_commit();
    };
    load_chunk(0, Fb);
    FI* Gs = Fb + (size_t)JQ * SP;
    for (int e = tid; e < JM * nslot; e += blockDim.x) {
        const int mm = e % JM, s = e / JM, r = sidx[s], mg = m0 + mm;
        Gs[(size_t)mm * SP + s] = (r >= 0 && mg < a.nm) ? G[(size_t)r * a.nm + mg] : zero;
    }
    __syncthreads();
    // Phase B: H[mm][slot(i)] = sum_j W[i][j] g[mm][slot(j)], packed (Wm, Wk)
    {
        const size_t tb = (size_t)tile * D * D * JKT + lane;
        for (int i = warp; i < dmax; i += blockDim.x / 32) {
            f2x h[JM][HW];
#pragma unroll
            for (int mm = 0; mm < JM; mm++)
#pragma unroll
                for (int w = 0; w < HW; w++) h[mm][w] = 0ull;
            const float4* wr = a.W + tb + (size_t)i * D * JKT;
#pragma unroll 2
            for (int j = 0; j < dmax; j++) {
                const float4 wv = wr[(size_t)j * JKT];
                const f2x wh = f2_pack(wv.x, wv.y), wl = f2_pack(wv.z, wv.w);
#pragma unroll
                for (int mm = 0; mm < JM; mm++) {
                    const FI g = Gs[(size_t)mm * SP + j * JKT + lane];
                    if constexpr (CPLX) {
                        ff2_mac(h[mm][0], h[mm][1], wh, wl, f2_bcast(g.x), f2_bcast(g.y));
                        ff2_mac(h[mm][2], h[mm][3], wh, wl, f2_bcast(g.z), f2_bcast(g.w));
                    } else {
                        ff2_mac(h[mm][0], h[mm][1], wh, wl, f2_bcast(g.x), f2_bcast(g.y));
                    }
                }
            }
#pragma unroll
            for (int mm = 0; mm < JM; mm++)
#pragma unroll
                for (int w = 0; w < HW; w++) Hs[((size_t)w * JM + mm) * SP + i * JKT + lane] = h[mm][w];
        }
    }
    __syncthreads();
    const int n = m.n;
    constexpr int NG = JQ * JM;
    const int nch = (a.nq + JQ - 1) / JQ;
    for (int ch = 0; ch < nch; ch++) {
        if (ch + 1 < nch) {
            load_chunk((ch + 1) * JQ, Fb + (size_t)((ch + 1) & 1) * JQ * SP);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const FI* Fs = Fb + (size_t)(ch & 1) * JQ * SP;
        const int q0 = ch * JQ;
        for (int grp = warp; grp < NG; grp += blockDim.x / 32) {
            const int qq = grp / JM, mm = grp % JM;
            const int q = q0 + qq, mg = m0 + mm;
            if (q >= a.nq || mg >= a.nm) continue;
            const int l = lidx[q * JM + mm];
            if (l < 0) continue;
            // packed (mua, kappa) sums: re (hi, lo), im (hi, lo)
            f2x srh = 0ull, srl = 0ull, sih = 0ull, sil = 0ull;
            const FI* fp = Fs + (size_t)qq * SP + lane;
            const f2x* hp = Hs + (size_t)mm * SP + lane;
            const size_t hw = (size_t)JM * SP;  // stride between the H words
            // the loads of neighbour i + 1 are issued before the products of
            // neighbour i (shared-memory latency off the critical path)
            FI f = fp[0];
            f2x h0 = hp[0], h1 = hp[hw], h2 = 0ull, h3 = 0ull;
            if constexpr (CPLX) { h2 = hp[2 * hw]; h3 = hp[3 * hw]; }
            for (int i = 0; i < dmax; i++) {
                const int in = i + 1 < dmax ? i + 1 : i;
                const FI fn = fp[(size_t)in * JKT];
                const f2x* hq = hp + (size_t)in * JKT;
                const f2x n0 = hq[0], n1 = hq[hw];
                f2x n2 = 0ull, n3 = 0ull;
                if constexpr (CPLX) { n2 = hq[2 * hw]; n3 = hq[3 * hw]; }
                if constexpr (CPLX) {
                    const f2x frh = f2_bcast(f.x), frl = f2_bcast(f.y), fih = f2_bcast(f.z), fil = f2_bcast(f.w);
                    const f2x nih = f2_bcast(-f.z), nil = f2_bcast(-f.w);
                    // re += fr hr - fi hi ; im += fr hi + fi hr (no conjugation)
                    ff2_mac(srh, srl, frh, frl, h0, h1);
                    ff2_mac(sih, sil, frh, frl, h2, h3);
                    ff2_mac(srh, srl, nih, nil, h2, h3);
                    ff2_mac(sih, sil, fih, fil, h0, h1);
                } else {
                    ff2_mac(srh, srl, f2_bcast(f.x), f2_bcast(f.y), h0, h1);
                }
                f = fn;
                h0 = n0; h1 = n1; h2 = n2; h3 = n3;
            }
            if (!kin) continue;
            if constexpr (CPLX) {
                if (a.yinv) {
                    // (s_re + i s_im) (y_re + i y_im), float-float
                    const float4 y = yis[q * JM + mm];
                    f2x zrh = 0ull, zrl = 0ull, zih = 0ull, zil = 0ull;
                    ff2_mac(zrh, zrl, srh, srl, f2_bcast(y.x), f2_bcast(y.y));
                    ff2_mac(zrh, zrl, sih, sil, f2_bcast(-y.z), f2_bcast(-y.w));
                    ff2_mac(zih, zil, srh, srl, f2_bcast(y.z), f2_bcast(y.w));
                    ff2_mac(zih, zil, sih, sil, f2_bcast(y.x), f2_bcast(y.y));
                    srh = zrh; srl = zrl; sih = zih; sil = zil;
                }
                const float2 rh = f2_unpack(srh), rl = f2_unpack(srl), ih = f2_unpack(sih), il = f2_unpack(sil);
                const size_t r0 = (size_t)l * 2 * n + k, r1 = (size_t)(l + a.nqm) * 2 * n + k;
                if (a.J32) {
                    a.J32[r0] = -__fadd_rn(rh.x, rl.x);
                    a.J32[r1] = -__fadd_rn(ih.x, il.x);
                    a.J32[r0 + n] = -__fadd_rn(rh.y, rl.y);
                    a.J32[r1 + n] = -__fadd_rn(ih.y, il.y);
                } else {
                    a.J[r0] = -ff_to_double(rh.x, rl.x);
                    a.J[r1] = -ff_to_double(ih.x, il.x);
                    a.J[r0 + n] = -ff_to_double(rh.y, rl.y);
                    a.J[r1 + n] = -ff_to_double(ih.y, il.y);
                }
            } else {
                if (a.yinv) {
                    const float4 y = yis[q * JM + mm];
                    f2x zh = 0ull, zl = 0ull;
                    ff2_mac(zh, zl, srh, srl, f2_bcast(y.x), f2_bcast(y.y));
                    srh = zh; srl = zl;
                }
                const float2 rh = f2_unpack(srh), rl = f2_unpack(srl);
                if (a.J32) {
                    a.J32[(size_t)l * n + k] = -__fadd_rn(rh.x, rl.x);
                    a.J32[(size_t)(l + a.nqm) * n + k] = -__fadd_rn(rh.y, rl.y);
                } else {
                    a.J[(size_t)l * n + k] = -ff_to_double(rh.x, rl.x);
                    a.J[(size_t)(l + a.nqm) * n + k] = -ff_to_double(rh.y, rl.y);
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Nodal Jacobian (complex) on the tensor cores, FP64-level accuracy.
//
// Per node k the pair sums are one small matrix product: with the node's
// D neighbours, J_qm(k) = sum_i F_q(i) H_m(i), H_m(i) = sum_j W_k[i][j] G_m(j)
// (mua and kappa weights), i.e. (nq x D) times (D x nm), complex.  As a real
// product with K = 2D: rows (q, Re/Im) = [Fr, -Fi] / [Fi, Fr], columns
// (m, mua/kappa) = [Hr; Hi].
//
// Exact digit products (the splitting scheme of Ozaki et al.): every row of
// the left factor and every column of the right one is scaled by a power of
// two to |x| < 128 and cut into S = 7 balanced base-256 digits (integers in
// [-256, 256] when the hi and lo floats are cut separately and added), each
// exact in bf16 and pre-scaled by 256^-t.  A digit product is exact in FP32
// and so is a sum of products of one level t + u while it stays below 2^24
// units (K <= 64, at most four digit pairs per level): levels 0 to 3 have an
// accumulator each and are exact; levels 4 to 6 (relative weight 2^-32 and
// less) share one.  (One accumulator for levels 3 and up measured 1.3e-12
// instead of 4e-15: a sum of products of mixed levels is not exact.)  The
// five accumulators are summed in float-float on packed (mua, kappa) pairs,
// multiplied by 1/y in float-float and rounded once, scaled back by the
// exponents.  Against an FP64 Jacobian of the same fields: ~4e-15 in L2.
//
// CTA = (node, chunk of jmc detectors), 512 threads, two CTAs per SM;
// mma.sync m16n8k16 bf16 with m-tile = 8 sources x (Re, Im) rows and n-tile =
// 4 detectors x (mua, kappa), so each thread ends with the four J entries of
// one link.
// ---------------------------------------------------------------------------
struct JacOzArgs {
    MeshDev m;
    int nq, nm, nqm;
    const float4* F;              // float-float forward fields (re_hi, re_lo, im_hi, im_lo), node-major, ld nq
    const float4* G;              // float-float adjoint fields, node-major, ld nm
    const int* pairidx;           // nq*nm -> link index or -1
    const float4* yinv;           // per link 1/y as (re_hi, re_lo, im_hi, im_lo), or null
    double* J;                    // FP64 output, or
    float* J32;                   // FP32 output
    const float4* W;              // packed float-float weights (Wm_hi, Wk_hi, Wm_lo, Wk_lo), [tile][i][j][lane]
    int D;                        // weight slots per node (maximum degree)
    int jmc, nch;                 // detectors per CTA (a multiple of 4), chunks per node
};

// biased FP32 exponent of the largest |value| (bits of non-negative floats
// order as integers), clamped so that the scale 2^(133 - be) is a normal float
__device__ __forceinline__ int oz_be(unsigned maxbits)
{
    if (maxbits == 0u) return 133;
    const int be = (int)(maxbits >> 23);
    return be < 7 ? 7 : be;
}
// 2^(7 - E) with E = be - 126: values scaled by it lie in (-128, 128)
__device__ __forceinline__ float oz_scale(int be) { return __uint_as_float((unsigned)(260 - be) << 23); }

// balanced base-256 digits of (hi + lo) * sc: the digits of hi and of lo,
// added (|d| <= 256), digit t pre-scaled by 256^-t; every step is exact
template <int S>
__device__ __forceinline__ void oz_digits(float hi, float lo, float sc, float (&d)[S])
{
    float r = hi * sc, q = lo * sc, w = 1.0f;
#pragma unroll
    for (int t = 0; t < S; t++) {
        const float a = rintf(r), b = rintf(q);
        d[t] = (a + b) * w;
        r = (r - a) * 256.0f;
        q = (q - b) * 256.0f;
        w *= 0.00390625f;
    }
}

__device__ __forceinline__ unsigned oz_pack(float lo_half, float hi_half)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo_half, hi_half);  // .x in the low 16 bits
    unsigned u;
    memcpy(&u, &v, 4);
    return u;
}

// the Im row word {Fi, Fr} from the Re row word {Fr, -Fi}: swap, negate the low half
__device__ __forceinline__ unsigned oz_imword(unsigned w) { return ((w >> 16) | (w << 16)) ^ 0x00008000u; }

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// f * 2^e exactly as a double, built from the bits of f (normal floats and
// zero; the result stays in the normal double range)
__device__ __forceinline__ double oz_f2d(float f, int e)
{
    const unsigned u = __float_as_uint(f);
    const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned ex = (u >> 23) & 0xffu;
    if (ex == 0u) return __longlong_as_double((long long)s);
    return __longlong_as_double((long long)(s | ((unsigned long long)(ex + 896u + e) << 52) |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
}
// (h + l) * 2^e as a double: one FP64 addition, rounded once
__device__ __forceinline__ double oz_to_double(float h, float l, int e) { return oz_f2d(h, e) + oz_f2d(l, e); }

// AI: left-factor items per thread: NT / QR threads share a source row, AI * (NT / QR) >= deg
// (h, l) += x exactly, lane by lane on packed pairs (TwoSum)
__device__ __forceinline__ void oz_acc2(f2x& h, f2x& l, f2x x)
{
    const f2x s = f2_add(h, x), bp = f2_sub(s, h);
    l = f2_add(l, f2_add(f2_sub(h, f2_sub(s, bp)), f2_sub(x, bp)));
    h = s;
}

template <int S, int NG, int NT, int AI>
__global__ void __launch_bounds__(NT, 1024 / NT) jacobian_oz_kernel(JacOzArgs a)
{
    // accumulators: digit levels 0..3 apart (their sums are exact), 4..6
    // together (relative weight 2^-32 and less: FP32 rounding there stays
    // below the digit truncation)
    constexpr int NA = 5;
    extern __shared__ __align__(16) unsigned char jsm[];
    const MeshDev& m = a.m;
    const int k = blockIdx.x / a.nch, ch = blockIdx.x % a.nch;
    const int m0 = ch * a.jmc, jm = min(a.jmc, a.nm - m0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rb = m.jrowptr[k], deg = m.jrowptr[k + 1] - rb;
    const int KW = ((2 * deg + 15) / 16) * 8;       // words (bf16 pairs) per row: K = 2 deg padded to 16
    const int KWM = ((2 * a.D + 15) / 16) * 8;      // the same for the largest degree (layout)
    const int AST = KWM + 4;                        // row stride in words: fragment loads conflict-free
    const int QR = ((a.nq + 7) / 8) * 8;            // source rows, padded to m-tiles of 8 sources
    const int BC = 2 * a.jmc;                       // right-factor columns (detector x mua/kappa)
    int* nb = (int*)jsm;                            // [32] neighbours of k, natural order
    unsigned* ea = (unsigned*)(nb + 32);            // [QR] largest |value| (float bits) of each row
    unsigned* eb = ea + QR;                         // [BC] the same per column
    unsigned* Bw = eb + BC;                         // [S][BC][AST] right-factor digit words
    unsigned char* X = (unsigned char*)(Bw + (size_t)S * BC * AST);
    float4* Ws = (float4*)X;                        // [deg][deg] weights (phase 1)
    float4* Gs = Ws + deg * deg;                    // [deg][jmc] adjoint fields (phase 1)
    f2x* Hs = (f2x*)(Gs + (size_t)deg * a.jmc);     // [4 words][jmc][deg] H = W G (phase 1)
    unsigned* Aw = (unsigned*)X;                    // [S][QR][AST] left-factor digit words (phase 2)
    const size_t HW1 = (size_t)a.jmc * deg;

    for (int i = tid; i < deg; i += NT) nb[i] = m.jcolidx[rb + i];
    for (int i = tid; i < QR + BC; i += NT) ea[i] = 0u;  // ea and eb are adjacent
    __syncthreads();
    {
        const size_t tb = (size_t)(k / JKT) * a.D * a.D * JKT + (k % JKT);
        for (int e = tid; e < deg * deg; e += NT) {
            const int i = e / deg, j = e % deg;
            Ws[e] = a.W[tb + ((size_t)i * a.D + j) * JKT];
        }
        for (int e = tid; e < deg * jm; e += NT) {
            const int j = e / jm, mm = e % jm;
            Gs[j * a.jmc + mm] = a.G[(size_t)nb[j] * a.nm + m0 + mm];
        }
    }
    __syncthreads();
    // H[mm][i] = sum_j W[i][j] G[j][mm], packed (mua, kappa), float-float;
    // column maxima of the hi words
    for (int e = tid; e < jm * deg; e += NT) {
        const int i = e / jm, mm = e % jm;
        f2x rh = 0ull, rl = 0ull, ih = 0ull, il = 0ull;
        for (int j = 0; j < deg; j++) {
            const float4 w = Ws[i * deg + j];
            const f2x wh = f2_pack(w.x, w.y), wl = f2_pack(w.z, w.w);
            const float4 g = Gs[j * a.jmc + mm];
            ff2_mac(rh, rl, wh, wl, f2_bcast(g.x), f2_bcast(g.y));
            ff2_mac(ih, il, wh, wl, f2_bcast(g.z), f2_bcast(g.w));
        }
        const size_t o = (size_t)mm * deg + i;
        Hs[o] = rh;
        Hs[HW1 + o] = rl;
        Hs[2 * HW1 + o] = ih;
        Hs[3 * HW1 + o] = il;
        const float2 r = f2_unpack(rh), q = f2_unpack(ih);
        atomicMax(&eb[2 * mm], max(__float_as_uint(r.x) & 0x7fffffffu, __float_as_uint(q.x) & 0x7fffffffu));
        atomicMax(&eb[2 * mm + 1], max(__float_as_uint(r.y) & 0x7fffffffu, __float_as_uint(q.y) & 0x7fffffffu));
    }
    __syncthreads();
    // the forward fields of this thread's left-factor items (source q =
    // tid % QR, neighbours i = tid / QR + r * (NT / QR)), loaded together
    // (coalesced over q); their latency hides behind the right-factor digits
    const int QP = NT / QR, aq = tid % QR, ai0 = tid / QR;
    float4 fv[AI];
#pragma unroll
    for (int x = 0; x < AI; x++) {
        const int i = ai0 + x * QP;
        fv[x] = ai0 < QP && aq < a.nq && i < deg ? a.F[(size_t)nb[i] * a.nq + aq] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // right-factor digits: word (column c, i) = {Hr, Hi} of H[c/2][i], part
    // c&1; a warp per column, lane = word (KWM <= 32)
    for (int c = warp; c < BC; c += NT / 32) {
        const int i = lane, mm = c >> 1, p = c & 1;
        if (i >= KWM) continue;
        float dr[S], di[S];
        if (mm < jm && i < deg) {
            const float sc = oz_scale(oz_be(eb[c]));
            const size_t o = (size_t)mm * deg + i;
            const float2 xh = f2_unpack(Hs[o]), xl = f2_unpack(Hs[HW1 + o]);
            const float2 yh = f2_unpack(Hs[2 * HW1 + o]), yl = f2_unpack(Hs[3 * HW1 + o]);
            oz_digits<S>(p ? xh.y : xh.x, p ? xl.y : xl.x, sc, dr);
            oz_digits<S>(p ? yh.y : yh.x, p ? yl.y : yl.x, sc, di);
        } else {
#pragma unroll
            for (int t = 0; t < S; t++) dr[t] = di[t] = 0.0f;
        }
#pragma unroll
        for (int t = 0; t < S; t++) Bw[((size_t)t * BC + c) * AST + i] = oz_pack(dr[t], di[t]);
    }
    {
        unsigned mx = 0u;
#pragma unroll
        for (int x = 0; x < AI; x++)
            mx = max(mx, max(__float_as_uint(fv[x].x) & 0x7fffffffu, __float_as_uint(fv[x].z) & 0x7fffffffu));
        if (ai0 < QP && aq < a.nq) atomicMax(&ea[aq], mx);
    }
    __syncthreads();  // phase-1 buffers dead: Aw takes their place
    // left-factor digits: word (row q, i) = {Fr, -Fi} of F_q at neighbour i;
    // padding words (i >= deg, or a padding row) zero, a warp per row
    for (int q = warp; q < QR; q += NT / 32) {
        const int i = lane;
        if (i >= KWM || (q < a.nq && i < deg)) continue;
#pragma unroll
        for (int t = 0; t < S; t++) Aw[((size_t)t * QR + q) * AST + i] = 0u;
    }
    if (ai0 < QP && aq < a.nq) {
        const float sc = oz_scale(oz_be(ea[aq]));
#pragma unroll
        for (int x = 0; x < AI; x++) {
            const int i = ai0 + x * QP;
            if (i >= deg) break;
            float dr[S], di[S];
            oz_digits<S>(fv[x].x, fv[x].y, sc, dr);
            oz_digits<S>(fv[x].z, fv[x].w, sc, di);
#pragma unroll
            for (int t = 0; t < S; t++) Aw[((size_t)t * QR + aq) * AST + i] = oz_pack(dr[t], -di[t]);
        }
    }
    __syncthreads();
    // digit products: task = (m-tile of 8 sources, group of NG n-tiles)
    const int g = lane >> 2, c4 = lane & 3;
    const int QT = QR / 8, NTT = (2 * jm + 7) / 8, NGT = (NTT + NG - 1) / NG, KS = KW / 8;
    const int n = m.n;
    for (int task = warp; task < QT * NGT; task += NT / 32) {
        const int qt = task / NGT, ng = task % NGT;
        // this thread's links and their 1/y, loaded before the products
        // (their latency hides behind them)
        int lk[NG];
        float4 yk[NG];
#pragma unroll
        for (int nt = 0; nt < NG; nt++) {
            const int q = qt * 8 + g, mm = (ng * NG + nt) * 4 + c4;
            lk[nt] = q < a.nq && mm < jm ? a.pairidx[(size_t)q * a.nm + m0 + mm] : -1;
            yk[nt] = a.yinv && lk[nt] >= 0 ? a.yinv[lk[nt]] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        float acc[NG][NA][4];
#pragma unroll
        for (int x = 0; x < NG; x++)
#pragma unroll
            for (int y = 0; y < NA; y++)
#pragma unroll
                for (int z = 0; z < 4; z++) acc[x][y][z] = 0.0f;
        for (int ks = 0; ks < KS; ks++) {
            const int i0 = ks * 8;
            unsigned bf[S][NG][2];
#pragma unroll
            for (int u = 0; u < S; u++)
#pragma unroll
                for (int nt = 0; nt < NG; nt++) {
                    const int col = (ng * NG + nt) * 8 + g;
                    const unsigned* bp = Bw + ((size_t)u * BC + (col < BC ? col : 0)) * AST + i0 + c4;
                    bf[u][nt][0] = bp[0];
                    bf[u][nt][1] = bp[4];
                }
#pragma unroll
            for (int t = 0; t < S; t++) {
                unsigned af[4];
                const unsigned* ap = Aw + ((size_t)t * QR + qt * 8 + g) * AST + i0 + c4;
                af[0] = ap[0];
                af[2] = ap[4];
                af[1] = oz_imword(af[0]);
                af[3] = oz_imword(af[2]);
#pragma unroll
                for (int u = 0; u + t < S; u++) {
#pragma unroll
                    for (int nt = 0; nt < NG; nt++)
                        if (ng * NG + nt < NTT)
                            mma_bf16_16816(acc[nt][t + u < NA ? t + u : NA - 1], af, bf[u][nt][0], bf[u][nt][1]);
                }
            }
        }
        // epilogue: thread (g, c4) holds link (q, m) = (qt*8 + g, tile*4 + c4):
        // (Re mua, Re kappa, Im mua, Im kappa)
        const int q = qt * 8 + g;
#pragma unroll
        for (int nt = 0; nt < NG; nt++) {
            const int ntg = ng * NG + nt;
            const int mm = ntg * 4 + c4;
            const int l = lk[nt];
            if (ntg >= NTT || l < 0) continue;
            // the level sums, smallest first, in float-float; (Re mua, Re kappa)
            // and (Im mua, Im kappa) as packed pairs
            f2x srh = f2_pack(acc[nt][NA - 1][0], acc[nt][NA - 1][1]), srl = 0ull;
            f2x sih = f2_pack(acc[nt][NA - 1][2], acc[nt][NA - 1][3]), sil = 0ull;
#pragma unroll
            for (int y = NA - 2; y >= 0; y--) {
                oz_acc2(srh, srl, f2_pack(acc[nt][y][0], acc[nt][y][1]));
                oz_acc2(sih, sil, f2_pack(acc[nt][y][2], acc[nt][y][3]));
            }
            if (a.yinv) {
                const float4 y = yk[nt];
                f2x zrh = 0ull, zrl = 0ull, zih = 0ull, zil = 0ull;
                ff2_mac(zrh, zrl, srh, srl, f2_bcast(y.x), f2_bcast(y.y));
                ff2_mac(zrh, zrl, sih, sil, f2_bcast(-y.z), f2_bcast(-y.w));
                ff2_mac(zih, zil, srh, srl, f2_bcast(y.z), f2_bcast(y.w));
                ff2_mac(zih, zil, sih, sil, f2_bcast(y.x), f2_bcast(y.y));
                srh = zrh; srl = zrl; sih = zih; sil = zil;
            }
            // J = -PMDF: the float halves negated before the conversion
            const float2 rh = f2_unpack(f2_neg(srh)), rl = f2_unpack(f2_neg(srl));
            const float2 ih = f2_unpack(f2_neg(sih)), il = f2_unpack(f2_neg(sil));
            const int bq = oz_be(ea[q]);
            const int e0 = bq + oz_be(eb[2 * mm]) - 266, e1 = bq + oz_be(eb[2 * mm + 1]) - 266;
            const size_t r0 = (size_t)l * 2 * n + k, r1 = (size_t)(l + a.nqm) * 2 * n + k;
            const double jr0 = oz_to_double(rh.x, rl.x, e0), jr1 = oz_to_double(rh.y, rl.y, e1);
            const double ji0 = oz_to_double(ih.x, il.x, e0), ji1 = oz_to_double(ih.y, il.y, e1);
            if (a.J32) {
                a.J32[r0] = __double2float_rn(jr0);
                a.J32[r0 + n] = __double2float_rn(jr1);
                a.J32[r1] = __double2float_rn(ji0);
                a.J32[r1 + n] = __double2float_rn(ji1);
            } else {
                a.J[r0] = jr0;
                a.J[r0 + n] = jr1;
                a.J[r1] = ji0;
                a.J[r1 + n] = ji1;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The true residual's product A x of the mixed path in float-float
// arithmetic.  Each reliable update forms b - A x in FP64 for the columns
// waiting then; as FP64 arithmetic that product is bound by GB300's FP64 rate
// (about 350 us for 160 complex columns of the 30k cylinder).  Here A and x
// are (hi, lo) float pairs and every product and sum is compensated (the
// float-float arithmetic of the Jacobian), about 2^-46 of |A||x| per entry,
// far below what the stopping tests (backward error 1e-10, relative residual
// 1e-12) resolve; the result is rounded once to FP64.
// ---------------------------------------------------------------------------
// the waiting columns idx[0..kf) of the node-major FP64 block X (k columns) as
// float-float, node-major with kf columns
template <bool CPLX>
__global__ void gather_cols_ff_kernel(int n, int k, int kf, const int* __restrict__ idx, const double* __restrict__ X,
                                      void* __restrict__ out)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * kf) return;
    const size_t i = t / kf;
    const int c = idx[t % kf];
    if constexpr (CPLX) {
        const float2 r = ff_split(X[2 * (i * k + c)]), q = ff_split(X[2 * (i * k + c) + 1]);
        ((float4*)out)[t] = make_float4(r.x, r.y, q.x, q.y);
    } else {
        ((float2*)out)[t] = ff_split(X[i * k + c]);
    }
}

// Y = A X (FP64 out, node-major, kf columns): a warp per row, lane = column
template <bool CPLX, int NJ>
__global__ void __launch_bounds__(256) spmm_ff_kernel(int n, const int* __restrict__ rowptr,
                                                      const int* __restrict__ colidx, const void* __restrict__ Aff,
                                                      int kf, const void* __restrict__ Xff, double* __restrict__ Y)
{
    const int row = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (row >= n) return;
    const int b = rowptr[row], e = rowptr[row + 1];
    if constexpr (CPLX) {
        f2x h[NJ], l[NJ];  // packed (re, im)
#pragma unroll
        for (int j = 0; j < NJ; j++) h[j] = l[j] = 0ull;
        for (int p = b; p < e; p++) {
            const int col = colidx[p];
            const float4 a = ((const float4*)Aff)[p];  // (re_hi, re_lo, im_hi, im_lo)
            const f2x arh = f2_bcast(a.x), arl = f2_bcast(a.y);
            const f2x aih = f2_pack(-a.z, a.z), ail = f2_pack(-a.w, a.w);
#pragma unroll
            for (int j = 0; j < NJ; j++) {
                const int c = lane + 32 * j;
                if (c < kf) {
                    const float4 x = ((const float4*)Xff)[(size_t)col * kf + c];
                    ff2_mac(h[j], l[j], arh, arl, f2_pack(x.x, x.z), f2_pack(x.y, x.w));  // (ar xr, ar xi)
                    ff2_mac(h[j], l[j], aih, ail, f2_pack(x.z, x.x), f2_pack(x.w, x.y));  // (-ai xi, ai xr)
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NJ; j++) {
            const int c = lane + 32 * j;
            if (c < kf) {
                const float2 hh = f2_unpack(h[j]), ll = f2_unpack(l[j]);
                Y[2 * ((size_t)row * kf + c)] = oz_to_double(hh.x, ll.x, 0);
                Y[2 * ((size_t)row * kf + c) + 1] = oz_to_double(hh.y, ll.y, 0);
            }
        }
    } else {
        f2x h[NJ], l[NJ];  // the low half carries the column, the high half is unused
#pragma unroll
        for (int j = 0; j < NJ; j++) h[j] = l[j] = 0ull;
        for (int p = b; p < e; p++) {
            const int col = colidx[p];
            const float2 a = ((const float2*)Aff)[p];
            const f2x ah = f2_bcast(a.x), al = f2_bcast(a.y);
#pragma unroll
            for (int j = 0; j < NJ; j++) {
                const int c = lane + 32 * j;
                if (c < kf) {
                    const float2 x = ((const float2*)Xff)[(size_t)col * kf + c];
                    ff2_mac(h[j], l[j], ah, al, f2_bcast(x.x), f2_bcast(x.y));
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NJ; j++) {
            const int c = lane + 32 * j;
            if (c < kf) {
                const float2 hh = f2_unpack(h[j]), ll = f2_unpack(l[j]);
                Y[(size_t)row * kf + c] = oz_to_double(hh.x, ll.x, 0);
            }
        }
    }
}

// 1/y per link as float-float (re_hi, re_lo, im_hi, im_lo); real: (hi, lo, 0, 0)
template <class V>
__global__ void ff_recip_kernel(int cnt, const V* __restrict__ y, float4* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    const V r = vrecip(y[i]);
    const float2 a = ff_split(re(r)), b = ff_split(im(r));
    out[i] = make_float4(a.x, a.y, b.x, b.y);
}

}  // namespace tg
