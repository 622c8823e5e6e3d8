// host_pipe.cpp -- pcrp_solve_host: solves a batch held in HOST memory,
// streaming chunks of systems through the GPU so that the host<->device
// copies of one chunk overlap the solve of another.
//
// Two internal streams per device alternate over the chunks: chunk c is
// copied in, solved and copied out on stream c % 2, so while one stream runs
// its solve the copy engines serve the other.  Chunks grow: the first holds
// ceil(m/32) systems, so little copying precedes the first solve, and each
// next one three times as many, up to ceil(m/4), because a solve of few
// systems fills the GPU less well than a large one (measured on GB300, m=256
// n=65536: 0.102 ms per system at m=8, 0.088 at 32, 0.084 at 64).  The caller's stream is joined
// at both ends with events, so the call is asynchronous like the device
// entry points (the host arrays must stay valid until the stream reaches
// that point; page-locked host memory lets the copies run asynchronously).
#include <algorithm>
#include <mutex>

#include "pcrp_internal.h"

namespace pcrp {

pcrp_status get_workspace(const pcrp_opts* o, size_t bytes, cudaStream_t s, void** out);
pcrp_status f64_solve(const double* a, const double* b, const double* c, const double* d,
                      const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                      const pcrp_opts* o, cudaStream_t st, bool force_small, bool force_split,
                      const char* who);

namespace {
constexpr int kMaxDev = 64;
std::mutex g_mu;
cudaStream_t g_streams[kMaxDev][2] = {};
// One host thread at a time enqueues onto a device's internal streams: the
// solver scratch of each internal stream is a growing library buffer, and a
// growth started by one call between another call's lookup of that buffer
// and its launches would free memory those launches still use.
std::mutex g_enqueue_mu[kMaxDev];

pcrp_status dev_streams(int dev, cudaStream_t* s)
{
    if (dev < 0 || dev >= kMaxDev) return set_error(PCRP_ENOTSUP, "pcrp_solve_host: device %d", dev);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_streams[dev][0]) {
        for (int k = 0; k < 2; k++) {
            cudaError_t e = cudaStreamCreateWithFlags(&g_streams[dev][k], cudaStreamNonBlocking);
            if (e != cudaSuccess) return cuda_error(e, "cudaStreamCreate");
        }
    }
    s[0] = g_streams[dev][0]; s[1] = g_streams[dev][1];
    return PCRP_OK;
}

// The three join events of one call (caller -> internal streams, internal
// streams -> caller).  Each call owns its events: shared ones would let a
// concurrent call on another caller stream re-record the fork event between
// this call's record and its waits, so the internal streams would skip work
// the caller queued before the call.  An event may be destroyed as soon as
// its waits are enqueued (the runtime releases it once it completes).
struct CallEvents {
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    cudaError_t create() {
        for (auto& e : ev) {
            const cudaError_t rc = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            if (rc != cudaSuccess) return rc;
        }
        return cudaSuccess;
    }
    ~CallEvents() { for (auto e : ev) if (e) cudaEventDestroy(e); }
};

// copy systems [j0, j0+mc) of a host batch (layout) into / out of a device chunk
cudaError_t copy_chunk(double* dst, const double* src, int64_t j0, int64_t mc, int64_t m, int64_t n,
                       int32_t layout, bool to_device, cudaStream_t s)
{
    const cudaMemcpyKind kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    if (layout == PCRP_LAYOUT_CONTIGUOUS) {
        const size_t bytes = (size_t)mc * n * sizeof(double);
        return to_device ? cudaMemcpyAsync(dst, src + j0 * n, bytes, kind, s)
                         : cudaMemcpyAsync(dst + j0 * n, src, bytes, kind, s);
    }
    // interleaved: n rows of mc consecutive systems, host pitch m, chunk pitch mc
    const size_t w = (size_t)mc * sizeof(double);
    return to_device ? cudaMemcpy2DAsync(dst, w, src + j0, (size_t)m * sizeof(double), w, (size_t)n, kind, s)
                     : cudaMemcpy2DAsync(dst + j0, (size_t)m * sizeof(double), src, w, w, (size_t)n, kind, s);
}
}  // namespace

}  // namespace pcrp

using namespace pcrp;

extern "C" pcrp_status pcrp_solve_host(const double* a, const double* b, const double* c, const double* d,
                                       const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                                       int32_t precision, double tol, int32_t max_sweeps,
                                       const pcrp_opts* opts, pcrp_stream stream)
{
    const char* who = "pcrp_solve_host";
    NvtxRange nv(who);
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "%s: negative size", who);
    if (layout != PCRP_LAYOUT_CONTIGUOUS && layout != PCRP_LAYOUT_INTERLEAVED)
        return set_error(PCRP_EINVAL, "%s: bad layout %d", who, layout);
    if (precision != 0 && precision != 1) return set_error(PCRP_EINVAL, "%s: precision %d (0 FP64, 1 mixed)", who, precision);
    if (m == 0 || n == 0) return PCRP_OK;
    if (!b || !c || !d || !y) return set_error(PCRP_EINVAL, "%s: null array (only a and e may be null)", who);
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_error(ce, "cudaGetDevice");
    cudaStream_t S[2];
    pcrp_status rc = dev_streams(dev, S);
    if (rc != PCRP_OK) return rc;
    std::lock_guard<std::mutex> enqueue_lock(g_enqueue_mu[dev]);
    CallEvents CE;
    ce = CE.create();
    if (ce != cudaSuccess) return cuda_error(ce, "pcrp_solve_host: cudaEventCreate");
    cudaEvent_t* E = CE.ev;

    // chunk sizes: ceil(m/32) systems, then x3 per chunk up to ceil(m/4);
    // at most 2^26 unknowns each
    int64_t chunk = std::max<int64_t>(1, (m + 3) / 4);
    while (chunk > 1 && chunk * n > (int64_t(1) << 26)) chunk = (chunk + 1) / 2;
    const int64_t first = std::min(chunk, std::max<int64_t>(1, (m + 31) / 32));
    const size_t slot = (size_t)6 * chunk * n;
    void* ws = nullptr;
    rc = get_workspace(opts, 2 * slot * sizeof(double), st, &ws);
    if (rc != PCRP_OK) return rc;
    double* buf = static_cast<double*>(ws);
    // the solver's own scratch comes from the library cache of each internal stream
    pcrp_opts so{};
    if (opts && opts->size >= sizeof(pcrp_opts)) so = *opts;
    so.size = sizeof(pcrp_opts);
    so.workspace = nullptr; so.workspace_bytes = 0;

    const double* src[6] = {a, b, c, d, e, y};
    ce = cudaEventRecord(E[0], st);
    for (int k = 0; k < 2 && ce == cudaSuccess; k++) ce = cudaStreamWaitEvent(S[k], E[0], 0);
    if (ce != cudaSuccess) return cuda_error(ce, "pcrp_solve_host: stream join");
    pcrp_status failed = PCRP_OK;                 // the first error, after which nothing more is queued
    int64_t j0 = 0, next = first;
    for (int64_t q = 0; j0 < m; q++, j0 += next, next = std::min(3 * next, chunk)) {
        const int64_t mc = std::min(next, m - j0);
        cudaStream_t s = S[q & 1];
        double* base = buf + (q & 1) * slot;
        double* dv[6];
        // a null band stays null on the device (a zero band, not copied)
        for (int k = 0; k < 6; k++) dv[k] = src[k] ? base + (size_t)k * chunk * n : nullptr;
        for (int k = 0; k < 6 && ce == cudaSuccess; k++)
            if (src[k]) ce = copy_chunk(dv[k], src[k], j0, mc, m, n, layout, true, s);
        if (ce != cudaSuccess) { failed = cuda_error(ce, "pcrp_solve_host: copy in"); break; }
        rc = precision == 0
                 ? f64_solve(dv[0], dv[1], dv[2], dv[3], dv[4], dv[5], mc, n, layout, &so, s, false, false, who)
                 : pcrp_solve_mixed(dv[0], dv[1], dv[2], dv[3], dv[4], dv[5], mc, n, layout, tol, max_sweeps, &so,
                                    (pcrp_stream)s, nullptr);
        if (rc != PCRP_OK) { failed = rc; break; }
        ce = copy_chunk(y, dv[5], j0, mc, m, n, layout, false, s);
        if (ce != cudaSuccess) { failed = cuda_error(ce, "pcrp_solve_host: copy out"); break; }
    }
    // The caller's stream waits for the internal streams on every path, an
    // error included: copies from and to the caller's host arrays may already
    // be queued, and the caller must not reuse those arrays before they end.
    ce = cudaEventRecord(E[1], S[0]);
    if (ce == cudaSuccess) ce = cudaEventRecord(E[2], S[1]);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(st, E[1], 0);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(st, E[2], 0);
    if (failed != PCRP_OK) return failed;         // (its message stays the last error)
    return cuda_error(ce, "pcrp_solve_host: stream join");
}
