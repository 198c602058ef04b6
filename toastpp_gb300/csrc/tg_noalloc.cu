// tg_noalloc.cu -- ProjectAll for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs while a
// memory pool owned by another runtime holds the device, real-time loops that
// must not allocate after start-up, and plug-ins loaded into hosts that forbid
// allocation outside their own allocator.  tg_project_all_noalloc serves them:
// it takes the caller's device buffers for its inputs and outputs and keeps
// its scratch (support flags, the support list, the detector vectors
// compressed to their support and the link tables) in one fixed, file-scope
// device array instead of allocating it.
//
// The array is TG_NOALLOC_SCRATCH_BYTES (8 MiB) and is held by every GPU that
// loads the library until the process exits.  All calls share it and it keeps
// the last call's contents, so calls that overlap on the GPU (different
// streams, or different host threads) race; serialise them.  A call holds the
// solver's own lock, as the solver's other entry points do, and runs on the
// solver's device (the caller's current device is restored on return).
#include <cstdint>
#include <mutex>

#include "../../include/toastgpu.h"
#include "tg_jac.cuh"

extern "C" int tg_solver_internal(tg_solver s, int* n, int* cplx, cudaStream_t* stream, int* device, void** mu);

namespace tg {

static __device__ __align__(256) unsigned char g_noalloc_scratch[TG_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch, looked up once per device (the name is
// a host-side stand-in that must not be passed to a kernel).
static constexpr int kMaxDevices = 64;
static void* g_scratch_addr[kMaxDevices] = {};
static std::mutex g_scratch_mu;

static int scratch_address(void** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        set_error("tg_project_all_noalloc: no usable current device");
        return TG_ERR_CUDA;
    }
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            set_error("tg_project_all_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return TG_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return TG_OK;
}

// Same reduction as project_kernel, reading the fields source-major and
// finding the source of link l from the link offsets.
template <class V>
__global__ void project_srcmajor_kernel(const int* __restrict__ nsup_p, const int* __restrict__ sup,
                                        const V* __restrict__ phi, int n, const V* __restrict__ Msup, int nm,
                                        const int* __restrict__ link_ofs, int nq, const int* __restrict__ link_m,
                                        int nqm, V* __restrict__ lin, V* __restrict__ lg)
{
    int l = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x & 31;
    if (l >= nqm) return;
    int lo = 0, hi = nq - 1;  // largest q with link_ofs[q] <= l
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (link_ofs[mid] <= l) lo = mid; else hi = mid - 1;
    }
    int q = lo, m = link_m[l], nsup = *nsup_p;
    V s = vzero<V>();
    for (int t = lane; t < nsup; t += 32) s = vfma(s, phi[(size_t)q * n + sup[t]], Msup[(size_t)t * nm + m]);
    for (int o = 16; o; o >>= 1) {
        if constexpr (vt<V>::cplx) {
            s.x += __shfl_down_sync(0xffffffffu, s.x, o);
            s.y += __shfl_down_sync(0xffffffffu, s.y, o);
        } else {
            s += __shfl_down_sync(0xffffffffu, s, o);
        }
    }
    if (lane) return;
    if (lin) lin[l] = s;
    if (lg) {
        if constexpr (vt<V>::cplx) lg[l] = V{log(hypot(s.x, s.y)), atan2(s.y, s.x)};
        else lg[l] = log(s);
    }
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

template <class V>
static int run(cudaStream_t st, int n, int nq, const V* phi, int nm, const V* mvec, const int* link_ofs,
               const int* link_m, int nqm, int scale, V* proj, unsigned char* scratch)
{
    // scratch layout: flag[n] | sup[n] | nsup | link_ofs[nq+1] | link_m[nqm] | Msup[nsup*nm]
    size_t o_flag = 0, o_sup = align256((size_t)n * 4), o_ns = o_sup + align256((size_t)n * 4);
    size_t o_ofs = o_ns + 256, o_lm = o_ofs + align256((size_t)(nq + 1) * 4);
    size_t o_ms = o_lm + align256((size_t)nqm * 4);
    if (o_ms > TG_NOALLOC_SCRATCH_BYTES) {
        set_error("tg_project_all_noalloc: n=%d, nQM=%d need %zu bytes of scratch before the detector vectors; "
                  "the fixed scratch holds %d bytes (use tg_project_all)", n, nqm, o_ms, TG_NOALLOC_SCRATCH_BYTES);
        return TG_ERR_UNSUPPORTED;
    }
    int* flag = (int*)(scratch + o_flag);
    int* sup = (int*)(scratch + o_sup);
    int* nsup = (int*)(scratch + o_ns);
    int* d_ofs = (int*)(scratch + o_ofs);
    int* d_lm = (int*)(scratch + o_lm);
    V* Msup = (V*)(scratch + o_ms);
    if (cudaMemcpyAsync(d_ofs, link_ofs, (size_t)(nq + 1) * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(d_lm, link_m, (size_t)nqm * 4, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        set_error("tg_project_all_noalloc: copying the link list failed: %s", cudaGetErrorString(cudaGetLastError()));
        return TG_ERR_CUDA;
    }
    // every scratch region read below is written first in this call
    support_flag_kernel<V><<<(n + 255) / 256, 256, 0, st>>>(n, nm, mvec, flag);
    support_scan_kernel<<<1, 1024, 0, st>>>(n, flag, sup, nsup);
    int h_nsup = 0;
    if (cudaMemcpyAsync(&h_nsup, nsup, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("tg_project_all_noalloc: %s", cudaGetErrorString(cudaGetLastError()));
        return TG_ERR_CUDA;
    }
    size_t need = o_ms + (size_t)h_nsup * nm * sizeof(V);
    if (need > TG_NOALLOC_SCRATCH_BYTES) {
        set_error("tg_project_all_noalloc: %d support nodes x %d detectors need %zu bytes of scratch; the fixed "
                  "scratch holds %d bytes (use tg_project_all)", h_nsup, nm, need, TG_NOALLOC_SCRATCH_BYTES);
        return TG_ERR_UNSUPPORTED;
    }
    size_t g = (size_t)h_nsup * nm;
    if (g) support_gather_kernel<V><<<(unsigned)((g + 255) / 256), 256, 0, st>>>(n, nm, nsup, sup, mvec, Msup);
    project_srcmajor_kernel<V><<<(unsigned)(((size_t)nqm * 32 + 255) / 256), 256, 0, st>>>(
        nsup, sup, phi, n, Msup, nm, d_ofs, nq, d_lm, nqm, scale == TG_DATA_LIN ? proj : nullptr,
        scale == TG_DATA_LOG ? proj : nullptr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error("tg_project_all_noalloc: %s", cudaGetErrorString(e));
        return TG_ERR_CUDA;
    }
    return TG_OK;
}

}  // namespace tg

namespace {
// makes the solver's device current for the call and restores the caller's
struct DeviceScope {
    int prev = -1;
    bool ok = false;
    explicit DeviceScope(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) { cudaGetLastError(); prev = -1; }
        ok = cudaSetDevice(dev) == cudaSuccess;
        if (!ok) cudaGetLastError();
    }
    ~DeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};
}  // namespace

static int project_all_noalloc(tg_solver s, int nq, const double* phi, int nm, const double* mvec,
                               const int* link_ofs, const int* link_m, int scale, double* proj)
{
    using namespace tg;
    int n = 0, cplx = 0, device = 0;
    cudaStream_t st = 0;
    void* mu = nullptr;
    if (!s || !phi || !mvec || !link_ofs || !proj || nq <= 0 || nm <= 0) {
        set_error("tg_project_all_noalloc: invalid argument");
        return TG_ERR_ARG;
    }
    if (scale != TG_DATA_LIN && scale != TG_DATA_LOG) {
        set_error("tg_project_all_noalloc: scale must be TG_DATA_LIN or TG_DATA_LOG");
        return TG_ERR_ARG;
    }
    if (tg_solver_internal(s, &n, &cplx, &st, &device, &mu) != TG_OK) {
        set_error("tg_project_all_noalloc: invalid solver");
        return TG_ERR_ARG;
    }
    std::lock_guard<std::mutex> hold(*(std::mutex*)mu);
    DeviceScope ds(device);
    if (!ds.ok) {
        set_error("tg_project_all_noalloc: cannot make the solver's device %d current", device);
        return TG_ERR_CUDA;
    }
    if (link_ofs[0] != 0) { set_error("tg_project_all_noalloc: link_ofs must start at 0"); return TG_ERR_ARG; }
    for (int q = 0; q < nq; q++)
        if (link_ofs[q + 1] < link_ofs[q]) { set_error("tg_project_all_noalloc: link_ofs not ascending"); return TG_ERR_ARG; }
    int nqm = link_ofs[nq];
    if (nqm == 0) return TG_OK;
    if (!link_m) { set_error("tg_project_all_noalloc: link_m is NULL"); return TG_ERR_ARG; }
    for (int l = 0; l < nqm; l++)
        if (link_m[l] < 0 || link_m[l] >= nm) {
            set_error("tg_project_all_noalloc: link detector index out of range");
            return TG_ERR_ARG;
        }
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != TG_OK) return rc;
    if (cplx)
        return run<cd>(st, n, nq, (const cd*)phi, nm, (const cd*)mvec, link_ofs, link_m, nqm, scale, (cd*)proj,
                       (unsigned char*)scratch);
    return run<double>(st, n, nq, phi, nm, mvec, link_ofs, link_m, nqm, scale, proj, (unsigned char*)scratch);
}

extern "C" int tg_project_all_noalloc(tg_solver s, int nq, const double* phi, int nm, const double* mvec,
                                      const int* link_ofs, const int* link_m, int scale, double* proj)
{
    // no exception may cross the C boundary (a lock that cannot be taken
    // throws std::system_error)
    try {
        return project_all_noalloc(s, nq, phi, nm, mvec, link_ofs, link_m, scale, proj);
    } catch (...) {
        tg::set_error("tg_project_all_noalloc: internal error");
        return TG_ERR_CUDA;
    }
}
