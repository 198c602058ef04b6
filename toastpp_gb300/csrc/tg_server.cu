// tg_server.cu -- the request loop: whole forward-path requests (Reset,
// CalcFields of sources and detectors, ProjectAll, Jacobian) submitted from
// any host thread, admitted in arrival order while a slot is free and the
// requests on the device fit the HBM budget, run concurrently on per-slot
// CUDA streams, and completed with their latency recorded.
//
// The reference runs one request at a time per process (TFwdSolver::CalcFields
// keeps function-local static state, src/libstoast/fwdsolver.cc:658-731);
// the server is the GPU-side replacement for a loop of such calls.  Each slot
// keeps its solvers (system matrix, factor, work blocks) resident per mesh and
// settings, so a mesh that recurs pays no allocation.  Every kernel of the
// path has a fixed reduction order, so a request's result does not depend on
// which other requests share the device.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>
#include "../../include/toastgpu.h"

namespace {

using clk = std::chrono::steady_clock;

struct Ticket {
    tg_request req;
    long long id = 0;
    size_t bytes = 0;          // device working set estimate
    int state = TG_REQ_QUEUED;
    int status = TG_OK;
    std::string err;
    clk::time_point t_submit, t_start, t_done;
};

struct SolverKey {
    tg_mesh mesh;
    int cplx, method, precon, precision, maxit;
    double tol;
    bool operator<(const SolverKey& o) const
    {
        return std::memcmp(this, &o, sizeof(SolverKey)) < 0;
    }
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaStream_t copy = nullptr;              // the Jacobians' device-to-host copies
    std::map<SolverKey, tg_solver> solvers;   // resident per mesh and settings
    std::vector<SolverKey> lru;
    std::thread th;
    // requests whose compute is done and whose Jacobian copy is in flight,
    // completed in order by the slot's completion thread
    std::mutex pmu;
    std::condition_variable pcv;
    std::deque<std::pair<std::shared_ptr<Ticket>, cudaEvent_t>> pend;
    bool pstop = false;
    std::thread done_th;
};

}  // namespace

struct tg_server_s {
    int device = 0;
    size_t budget = 0;
    int max_cached = 4;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Ticket>> queue;           // arrival order
    std::map<long long, std::shared_ptr<Ticket>> all;    // every ticket not yet collected
    std::vector<std::shared_ptr<Ticket>> ready;          // admitted, waiting for a slot thread
    size_t inflight_bytes = 0;
    int inflight = 0, nslots = 0;
    int running = 0;          // requests computing in a slot (the rest of inflight: copies)
    long long next_id = 1;
    bool stop = false;
    std::vector<double> lat_ms;                          // completed requests
    long long completed = 0, failed = 0, solves = 0;
    clk::time_point t0 = clk::now();
    std::vector<std::unique_ptr<Slot>> slots;
    std::thread dispatcher;
};

namespace tg {
void set_error(const char* fmt, ...);
}

namespace {

int fail(int code, const std::string& msg)
{
    tg::set_error("%s", msg.c_str());
    return code;
}

size_t estimate_bytes(const tg_request& r)
{
    int n = 0, nnz = 0;
    tg_mesh_info(r.mesh, &n, nullptr, &nnz, nullptr, nullptr, nullptr);
    const size_t vb = r.is_complex ? 16 : 8;
    const size_t k = (size_t)r.nq + r.nm;
    // FP64 right-hand sides, solutions and Krylov block (about 12 n x k blocks)
    size_t b = (size_t)n * k * vb * 12;
    // FP32 inner block of the mixed path (about 10 more at half width)
    if (r.precision == TG_PREC_MIXED) b += (size_t)n * k * (vb / 2) * 10;
    // system matrix, factor, level layouts
    b += (size_t)nnz * (vb + 4) * 4;
    // Jacobian output block
    if (r.J) {
        int nqm = r.link_ofs[r.nq];
        b += (size_t)2 * nqm * (r.is_complex ? 2 : 1) * n * (r.j_fp32 ? 4 : 8);
    }
    return b;
}

// admission: strictly in arrival order, while a slot is free (not computing)
// and the working set of the requests in flight (computing, or copying their
// Jacobian out) fits the budget (a request larger than the budget runs alone)
void dispatch_loop(tg_server_s* S)
{
    std::unique_lock<std::mutex> g(S->mu);
    for (;;) {
        S->cv_work.wait(g, [&] {
            if (S->stop) return true;
            if (S->queue.empty() || S->running >= S->nslots) return false;
            const auto& h = S->queue.front();
            return S->inflight == 0 || S->inflight_bytes + h->bytes <= S->budget;
        });
        if (S->stop) return;
        auto t = S->queue.front();
        S->queue.pop_front();
        S->inflight++;
        S->running++;
        S->inflight_bytes += t->bytes;
        t->state = TG_REQ_RUNNING;
        S->ready.push_back(t);
        S->cv_work.notify_all();
    }
}

tg_solver get_solver(tg_server_s* S, Slot& sl, const tg_request& r)
{
    SolverKey key;
    std::memset(&key, 0, sizeof(key));
    key.mesh = r.mesh; key.cplx = r.is_complex != 0; key.method = r.method; key.precon = r.precon;
    key.precision = r.precision; key.maxit = r.maxit; key.tol = r.tol;
    auto it = sl.solvers.find(key);
    if (it != sl.solvers.end()) {
        sl.lru.erase(std::find_if(sl.lru.begin(), sl.lru.end(),
                                  [&](const SolverKey& k) { return !(k < key) && !(key < k); }));
        sl.lru.push_back(key);
        return it->second;
    }
    if ((int)sl.solvers.size() >= S->max_cached) {
        SolverKey old = sl.lru.front();
        sl.lru.erase(sl.lru.begin());
        tg_solver_destroy(sl.solvers[old]);
        sl.solvers.erase(old);
    }
    tg_solver s = nullptr;
    int rc = tg_solver_create(r.mesh, r.is_complex, r.method, r.precon, r.tol, r.maxit, r.precision, &s);
    if (rc != TG_OK) throw std::runtime_error(tg_last_error());
    tg_solver_set_stream(s, sl.stream);
    tg_solver_set_output_stream(s, sl.copy);
    sl.solvers[key] = s;
    sl.lru.push_back(key);
    return s;
}

// the bookkeeping of a finished request (its latency ends here)
void finish(tg_server_s* S, const std::shared_ptr<Ticket>& t, int rc, const std::string& msg)
{
    t->t_done = clk::now();
    const tg_request& r = t->req;
    {
        std::lock_guard<std::mutex> g(S->mu);
        t->status = rc;
        t->err = msg;
        t->state = rc == TG_OK ? TG_REQ_DONE : TG_REQ_FAILED;
        S->inflight--;
        S->inflight_bytes -= t->bytes;
        if (rc == TG_OK) {
            S->completed++;
            S->solves += (long long)r.nq + r.nm;
            S->lat_ms.push_back(std::chrono::duration<double, std::milli>(t->t_done - t->t_submit).count());
        } else {
            S->failed++;
        }
    }
    S->cv_work.notify_all();
    S->cv_done.notify_all();
}

// A slot runs one request at a time on its stream.  tg_forward_path returns
// once the compute is done and the Jacobian's copy is queued on the slot's
// copy stream, so the next request starts while that copy runs; the
// completion thread waits for each copy (an event) and completes the request.
void slot_loop(tg_server_s* S, Slot* sl)
{
    cudaSetDevice(S->device);
    for (;;) {
        std::shared_ptr<Ticket> t;
        {
            std::unique_lock<std::mutex> g(S->mu);
            S->cv_work.wait(g, [&] { return S->stop || !S->ready.empty(); });
            if (S->stop && S->ready.empty()) return;
            t = S->ready.front();
            S->ready.erase(S->ready.begin());
        }
        t->t_start = clk::now();
        const tg_request& r = t->req;
        int rc = TG_OK;
        std::string msg;
        cudaEvent_t ev = nullptr;
        try {
            tg_solver s = get_solver(S, *sl, r);
            rc = tg_forward_path(s, r.cmua, r.ckappa, r.c2a, r.omega, r.nq, r.qvec, r.nm, r.mvec, r.link_ofs,
                                 r.link_m, nullptr, nullptr, r.proj, r.logproj, r.J, r.j_fp32, TG_MEM_HOST, r.res);
            if (rc != TG_OK) msg = tg_last_error();
            else if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
                     cudaEventRecord(ev, sl->copy) != cudaSuccess) {
                rc = TG_ERR_CUDA;
                msg = "event record on the copy stream failed";
            }
        } catch (const std::exception& e) {
            rc = TG_ERR_ARG;
            msg = e.what();
        }
        {
            std::lock_guard<std::mutex> g(S->mu);
            S->running--;
        }
        S->cv_work.notify_all();
        if (rc != TG_OK) {
            if (ev) cudaEventDestroy(ev);
            finish(S, t, rc, msg);
            continue;
        }
        {
            std::lock_guard<std::mutex> g(sl->pmu);
            sl->pend.emplace_back(t, ev);
        }
        sl->pcv.notify_all();
    }
}

void done_loop(tg_server_s* S, Slot* sl)
{
    cudaSetDevice(S->device);
    for (;;) {
        std::pair<std::shared_ptr<Ticket>, cudaEvent_t> p;
        {
            std::unique_lock<std::mutex> g(sl->pmu);
            sl->pcv.wait(g, [&] { return sl->pstop || !sl->pend.empty(); });
            if (sl->pend.empty()) return;
            p = sl->pend.front();
            sl->pend.pop_front();
        }
        const cudaError_t e = cudaEventSynchronize(p.second);
        cudaEventDestroy(p.second);
        finish(S, p.first, e == cudaSuccess ? TG_OK : TG_ERR_CUDA,
               e == cudaSuccess ? std::string() : std::string("Jacobian copy failed: ") + cudaGetErrorString(e));
    }
}

double percentile(std::vector<double> v, double p)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    double x = p / 100.0 * (v.size() - 1);
    size_t i = (size_t)x;
    double f = x - i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int tg_server_create(int slots, double hbm_budget_gb, tg_server* out)
{
    if (!out || slots < 1 || slots > 64 || !(hbm_budget_gb > 0)) return fail(TG_ERR_ARG, "invalid argument");
    *out = nullptr;
    auto S = std::make_unique<tg_server_s>();
    if (cudaGetDevice(&S->device) != cudaSuccess) return fail(TG_ERR_CUDA, "no CUDA device");
    S->budget = (size_t)(hbm_budget_gb * 1e9);
    S->nslots = slots;
    for (int i = 0; i < slots; i++) {
        auto sl = std::make_unique<Slot>();
        if (cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&sl->copy, cudaStreamNonBlocking) != cudaSuccess)
            return fail(TG_ERR_CUDA, "stream creation failed");
        S->slots.push_back(std::move(sl));
    }
    tg_server_s* raw = S.get();
    for (auto& sl : S->slots) {
        sl->th = std::thread(slot_loop, raw, sl.get());
        sl->done_th = std::thread(done_loop, raw, sl.get());
    }
    S->dispatcher = std::thread(dispatch_loop, raw);
    *out = S.release();
    return TG_OK;
}

int tg_server_destroy(tg_server S)
{
    if (!S) return TG_OK;
    {
        std::unique_lock<std::mutex> g(S->mu);
        // finish what was submitted, then stop
        S->cv_done.wait(g, [&] { return S->queue.empty() && S->ready.empty() && S->inflight == 0; });
        S->stop = true;
    }
    S->cv_work.notify_all();
    S->dispatcher.join();
    for (auto& sl : S->slots) sl->th.join();
    for (auto& sl : S->slots) {
        {
            std::lock_guard<std::mutex> g(sl->pmu);
            sl->pstop = true;
        }
        sl->pcv.notify_all();
        sl->done_th.join();
    }
    for (auto& sl : S->slots) {
        for (auto& kv : sl->solvers) tg_solver_destroy(kv.second);
        cudaStreamDestroy(sl->stream);
        cudaStreamDestroy(sl->copy);
    }
    delete S;
    return TG_OK;
}

int tg_submit(tg_server S, const tg_request* r, long long* ticket)
{
    if (!S || !r || !ticket) return fail(TG_ERR_ARG, "NULL argument");
    if (!r->mesh || !r->cmua || !r->ckappa || !r->c2a || !r->qvec || !r->mvec || !r->link_ofs || !r->link_m ||
        r->nq <= 0 || r->nm <= 0)
        return fail(TG_ERR_ARG, "incomplete request");
    if (!r->is_complex && r->omega != 0.0) return fail(TG_ERR_ARG, "nonzero omega for a real request");
    auto t = std::make_shared<Ticket>();
    t->req = *r;
    t->bytes = estimate_bytes(*r);
    t->t_submit = clk::now();
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (S->stop) return fail(TG_ERR_STATE, "server is stopping");
        t->id = S->next_id++;
        S->queue.push_back(t);
        S->all[t->id] = t;
    }
    S->cv_work.notify_all();
    *ticket = t->id;
    return TG_OK;
}

int tg_poll(tg_server S, long long ticket, int* state)
{
    if (!S || !state) return fail(TG_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return fail(TG_ERR_ARG, "unknown ticket");
    *state = it->second->state;
    return TG_OK;
}

int tg_wait(tg_server S, long long ticket, double* latency_ms)
{
    if (!S) return fail(TG_ERR_ARG, "NULL argument");
    std::unique_lock<std::mutex> g(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return fail(TG_ERR_ARG, "unknown ticket");
    auto t = it->second;
    S->cv_done.wait(g, [&] { return t->state == TG_REQ_DONE || t->state == TG_REQ_FAILED; });
    S->all.erase(ticket);
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(t->t_done - t->t_submit).count();
    if (t->status != TG_OK) return fail(t->status, t->err);
    return TG_OK;
}

int tg_server_stats(tg_server S, long long* completed, long long* failed, long long* solves, double* p50_ms,
                    double* p99_ms, double* elapsed_s)
{
    if (!S) return fail(TG_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(S->mu);
    if (completed) *completed = S->completed;
    if (failed) *failed = S->failed;
    if (solves) *solves = S->solves;
    if (p50_ms) *p50_ms = percentile(S->lat_ms, 50);
    if (p99_ms) *p99_ms = percentile(S->lat_ms, 99);
    if (elapsed_s) *elapsed_s = std::chrono::duration<double>(clk::now() - S->t0).count();
    return TG_OK;
}

int tg_server_reset_stats(tg_server S)
{
    if (!S) return fail(TG_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(S->mu);
    S->lat_ms.clear();
    S->completed = S->failed = S->solves = 0;
    S->t0 = clk::now();
    return TG_OK;
}

}  // extern "C"
