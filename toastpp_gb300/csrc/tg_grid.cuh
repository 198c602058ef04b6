// tg_grid.cuh -- the grid-basis Jacobian of a pixel raster (basis = grid).
//
// Reference: GenerateJacobian_grid (src/libstoast/jacobian.cc:289-373,
// complex, projections given) and GenerateJacobian_cw_grid (516-712, real)
// with Raster_Pixel (raster_px.cc:10-48) whose basis equals its grid.
//
// Per request the fields are resampled at the solution points (the grid
// points inside the mesh) and at their grid neighbours, with central or
// one-sided differences as ImageGradient (jacobian.cc:944-1060) takes them,
// into planes P[(c * (1 + dim) + comp) * slen + s] (comp 0 the value, 1..dim
// the gradient), so that a thread per solution point reads every plane of a
// source or detector coalesced.  Then one thread per solution point and
// source walks the source's links and writes its column of every link row.
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

// f(g) = sum_j B(g, j) x[col j] (Map_MeshToGrid, raster.cc:188-199; complex:
// Ax_cplx, crmatrix_imp.hpp:1302-1327), x source-major natural
template <class V>
__device__ __forceinline__ V grid_value(const GridDev& G, const V* __restrict__ x, int g)
{
    V acc = vzero<V>();
    for (int j = G.rowptr[g]; j < G.rowptr[g + 1]; j++) acc = vadd(acc, vscale(x[G.col[j]], G.val[j]));
    return acc;
}

// one thread per (solution point, column); masked: the one-sided rules of
// ImageGradient with the element mask, else every grid point counts
template <class V, class OUT>
__global__ void grid_fields_kernel(GridDev G, int k, const V* __restrict__ src, int ld, int masked,
                                   OUT* __restrict__ planes)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (s >= G.slen || c >= k) return;
    const V* x = src + (size_t)c * ld;
    const int g = G.sol[s];
    const V v0 = grid_value(G, x, g);
    const int np = 1 + G.dim;
    OUT* out = planes + (size_t)c * np * G.slen + s;
    out[0] = vcast<OUT, V>(v0);
    const int x0 = g % G.nx, y0 = (g / G.nx) % G.ny, z0 = g / (G.nx * G.ny);
    const int co[3] = {x0, y0, z0}, len[3] = {G.nx, G.ny, G.nz}, st[3] = {1, G.nx, G.nx * G.ny};
    for (int d = 0; d < G.dim; d++) {
        const bool blo = co[d] > 0 && (!masked || G.elref[g - st[d]] >= 0);
        const bool bhi = co[d] < len[d] - 1 && (!masked || G.elref[g + st[d]] >= 0);
        // the point itself is a solution point, so inside the mask
        V gr = vzero<V>();
        using R = typename vt<V>::R;
        if (blo && bhi)
            gr = vscale(vsub(grid_value(G, x, g + st[d]), grid_value(G, x, g - st[d])), (R)(0.5 * G.ih[d]));
        else if (blo)
            gr = vscale(vsub(v0, grid_value(G, x, g - st[d])), (R)G.ih[d]);
        else if (bhi)
            gr = vscale(vsub(grid_value(G, x, g + st[d]), v0), (R)G.ih[d]);
        out[(size_t)(1 + d) * G.slen] = vcast<OUT, V>(gr);
    }
}

// Smith's complex division (Smith 1962), as the reference's complex
// division of the PMDF by the projection does
__device__ __forceinline__ cd cdiv_smith(cd a, cd b)
{
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, den = b.x + b.y * r;
        return cd{(a.x + a.y * r) / den, (a.y - a.x * r) / den};
    }
    const double r = b.x / b.y, den = b.x * r + b.y;
    return cd{(a.x * r + a.y) / den, (a.y * r - a.x) / den};
}
__device__ __forceinline__ cf cdiv_smith(cf a, cf b)
{
    const cd q = cdiv_smith(cd{a.x, a.y}, cd{b.x, b.y});
    return cf{(float)q.x, (float)q.y};
}

// One thread per (solution point, source): PMDF_mua = -(f a), PMDF_kap =
// -sum_d (grad_d f)(grad_d a) (jacobian.cc:58-72); complex LOG data divide
// by y (PMDF_log, 76-79) before the voxel scale; real LOG rows are scaled by
// 1/y after it (GenerateJacobian_cw, 178-193).  J rows: complex
// [Re mua | Re kap] at l and [Im mua | Im kap] at nQM + l (2 slen columns);
// real mua at l and kap at nQM + l (slen columns).
template <class V, class JT>
__global__ void grid_jacobian_kernel(int dim, int slen, int nq, int nqm, const V* __restrict__ Fp,
                                     const V* __restrict__ Ap, const int* __restrict__ link_ofs,
                                     const int* __restrict__ link_m, const V* __restrict__ y, int logscale, double sz,
                                     JT* __restrict__ J)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
    if (s >= slen || q >= nq) return;
    using R = typename vt<V>::R;
    const int np = 1 + dim;
    V f[4];
#pragma unroll
    for (int d = 0; d < 4; d++) f[d] = d < np ? Fp[((size_t)q * np + d) * slen + s] : vzero<V>();
    constexpr bool CPLX = vt<V>::cplx;
    const size_t cols = CPLX ? 2 * (size_t)slen : (size_t)slen;
    for (int l = link_ofs[q]; l < link_ofs[q + 1]; l++) {
        const int m = link_m[l];
        V a[4];
#pragma unroll
        for (int d = 0; d < 4; d++) a[d] = d < np ? Ap[((size_t)m * np + d) * slen + s] : vzero<V>();
        V pm = vsub(vzero<V>(), vmul(f[0], a[0]));
        V pk = vzero<V>();
#pragma unroll
        for (int d = 1; d < 4; d++)
            if (d < np) pk = vsub(pk, vmul(f[d], a[d]));
        JT* r0 = J + (size_t)l * cols;
        JT* r1 = J + (size_t)(l + nqm) * cols;
        if constexpr (CPLX) {
            if (logscale) {
                pm = cdiv_smith(pm, y[l]);
                pk = cdiv_smith(pk, y[l]);
            }
            r0[s] = (JT)(re(pm) * (R)sz);
            r1[s] = (JT)(im(pm) * (R)sz);
            r0[slen + s] = (JT)(re(pk) * (R)sz);
            r1[slen + s] = (JT)(im(pk) * (R)sz);
        } else {
            R vm = re(pm) * (R)sz, vk = re(pk) * (R)sz;
            if (logscale) {
                const R iy = (R)(1.0 / (double)re(y[l]));
                vm *= iy;
                vk *= iy;
            }
            r0[s] = (JT)vm;
            r1[s] = (JT)vk;
        }
    }
}

}  // namespace tg
