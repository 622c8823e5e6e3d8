// capi.cpp -- C ABI: argument checks, dispatch, scratch, error reporting.
//
// The dispatch mirrors the reference host code (main.cu:46-87): n <= 1024
// goes to the shared-memory path, larger n to global stride passes followed
// by a shared-memory finish.  Unlike the reference it validates arguments,
// returns a status instead of exiting (performanalysis.h:12-20), leaves the
// bands untouched and accepts any n >= 1.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "pcrp_internal.h"
#include "tuned_params.h"

namespace pcrp {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

void count_launch(int64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

pcrp_status set_error(pcrp_status st, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

pcrp_status cuda_error(cudaError_t e, const char* where)
{
    if (e == cudaSuccess) return PCRP_OK;
    if (e == cudaErrorMemoryAllocation)
        return set_error(PCRP_ENOMEM, "%s: %s", where, cudaGetErrorString(e));
    return set_error(PCRP_ECUDA, "%s: %s", where, cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// Library-owned scratch: one growing buffer per (device, stream).  Work on one
// stream is ordered, so reusing its buffer across calls is safe; calls on
// different streams get different buffers.
// ---------------------------------------------------------------------------
namespace {
std::mutex g_ws_mu;
std::map<std::pair<int, cudaStream_t>, std::pair<void*, size_t>> g_ws;
}  // namespace

pcrp_status get_workspace(const pcrp_opts* o, size_t bytes, cudaStream_t s, void** out)
{
    *out = nullptr;
    if (bytes == 0) return PCRP_OK;
    if (o && o->workspace) {
        if (o->workspace_bytes < bytes)
            return set_error(PCRP_ENOMEM, "workspace too small: %zu bytes given, %zu needed",
                             o->workspace_bytes, bytes);
        *out = o->workspace;
        return PCRP_OK;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_ws_mu);
    auto& slot = g_ws[{dev, s}];
    if (slot.second < bytes) {
        // growing means a stream synchronisation and a cudaMalloc, neither of
        // which a stream under capture allows
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
            return set_error(PCRP_ENOTSUP,
                             "the library workspace of this stream must grow to %zu bytes, which cannot happen "
                             "during stream capture: make one call of this size before capturing, or pass "
                             "opts->workspace", bytes);
        if (slot.first) {
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize (workspace growth)");
            cudaFree(slot.first);
            slot = {nullptr, 0};
        }
        e = cudaMalloc(&slot.first, bytes);
        if (e != cudaSuccess) { slot = {nullptr, 0}; cudaGetLastError(); return cuda_error(e, "cudaMalloc workspace"); }
        slot.second = bytes;
    }
    *out = slot.first;
    return PCRP_OK;
}

// ---------------------------------------------------------------------------
// Tuning and pass planning for the faithful FP64 path.
// ---------------------------------------------------------------------------
struct F64Plan {
    int smem_rows, fuse, tile_rows, threads;
};

F64Plan f64_plan(const pcrp_opts* o, int64_t n)
{
    // tuned defaults by system size (the last row covers everything larger)
    static const int64_t table[][5] = PCRP_TUNED_F64_TABLE;
    const int rows = (int)(sizeof(table) / sizeof(table[0]));
    int t = 0;
    while (t + 1 < rows && n > table[t][0]) t++;
    F64Plan p{(int)table[t][1], (int)table[t][2], (int)table[t][3], (int)table[t][4]};
    if (o && o->size >= sizeof(pcrp_opts)) {
        if (o->smem_rows > 0) p.smem_rows = o->smem_rows;
        if (o->fuse_strides > 0) p.fuse = o->fuse_strides;
        if (o->tile_rows > 0) p.tile_rows = o->tile_rows;
        if (o->threads > 0) p.threads = o->threads;
    }
    if (p.smem_rows > pcr_max_smem_rows()) p.smem_rows = pcr_max_smem_rows();
    if (p.smem_rows < 2) p.smem_rows = 2;
    if (p.fuse > 8) p.fuse = 8;
    if (p.threads > 256) p.threads = 256;
    return p;
}

static int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Strides done in global passes before the shared-memory finish.
static int split_strides(int64_t n, int smem_rows)
{
    const int ns = ref_strides(n);
    int s = 0;
    while (s < ns && ceil_div(n, int64_t(1) << s) > smem_rows) s++;
    return s;
}

size_t mixed_workspace_bytes(int64_t m, int64_t n, const pcrp_opts* o, int max_sweeps, bool info, int32_t layout);
size_t ragged_workspace_bytes(int64_t nsys, int64_t total_rows);
size_t ragged_mixed_workspace_bound(int64_t nsys, int64_t max_rows, const pcrp_opts* o);

// Whether a solve of n-row systems with these options runs global passes
// (and so needs split-path scratch); n <= the shared-memory tile needs none.
bool f64_needs_scratch(int64_t n, const pcrp_opts* o)
{
    return split_strides(n, f64_plan(o, n).smem_rows) > 0;
}

size_t f64_workspace_bytes(int64_t m, int64_t n, int32_t layout, const F64Plan& pl, bool split)
{
    (void)layout;
    if (!split) return 0;
    if (split_strides(n, pl.smem_rows) == 0) return 0;
    return 2 * (size_t)NSTATE * (size_t)m * (size_t)n * sizeof(double);
}

static bool valid_layout(int32_t l) { return l == PCRP_LAYOUT_CONTIGUOUS || l == PCRP_LAYOUT_INTERLEAVED; }

// Solves a uniform batch with the faithful PCR kernels.  `split` selects the
// global-pass path (n larger than the shared-memory tile).
pcrp_status f64_solve(const double* a, const double* b, const double* c, const double* d,
                      const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                      const pcrp_opts* o, cudaStream_t st, bool force_small, bool force_split,
                      const char* who)
{
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "%s: negative size (m=%lld n=%lld)", who, (long long)m, (long long)n);
    if (!valid_layout(layout)) return set_error(PCRP_EINVAL, "%s: bad layout %d", who, layout);
    if (force_small && n > 1024) return set_error(PCRP_EINVAL, "%s: n=%lld > 1024", who, (long long)n);
    if (force_split && n <= 1024 && n != 0) return set_error(PCRP_EINVAL, "%s: n=%lld <= 1024", who, (long long)n);
    if (m == 0 || n == 0) return PCRP_OK;
    if (!b || !c || !d || !y) return set_error(PCRP_EINVAL, "%s: null array (only a and e may be null)", who);
    if (n > (int64_t(1) << 31) || m > (int64_t(1) << 40))
        return set_error(PCRP_EINVAL, "%s: size out of range", who);
    if (m > (int64_t(1) << 52) / (2 * NSTATE * (int64_t)sizeof(double)) / n)
        return set_error(PCRP_EINVAL, "%s: m*n = %lld * %lld is too large for the split-path scratch", who,
                         (long long)m, (long long)n);

    // null a and e: a tridiagonal batch, both bands +0.0; the first pass
    // reads neither, and every pass runs the zero-state strides
    const bool tri = !a && !e;
    F64Plan pl = f64_plan(o, n);
    if (force_small && pl.smem_rows < n) pl.smem_rows = (int)n;         // the n <= 1024 path is one tile
    if (force_split && pl.smem_rows >= n) pl.smem_rows = 1024;         // the n > 1024 path splits
    const int ns = ref_strides(n);
    const int s1 = split_strides(n, pl.smem_rows);

    const int64_t ss = layout == PCRP_LAYOUT_CONTIGUOUS ? n : 1;
    const int64_t rs = layout == PCRP_LAYOUT_CONTIGUOUS ? 1 : m;

    PcrPassArgs p;
    std::memset(&p, 0, sizeof p);
    p.src[A_] = a; p.src[B_] = b; p.src[C_] = c; p.src[D_] = d; p.src[E_] = e; p.src[Y_] = y;
    p.src_ss = ss; p.src_rs = rs;
    p.n = n; p.m = m; p.G = 1;

    double* bufs[2][NSTATE] = {};
    if (s1 > 0) {
        void* ws = nullptr;
        const size_t need = 2 * (size_t)NSTATE * (size_t)m * (size_t)n * sizeof(double);
        pcrp_status rc = get_workspace(o, need, st, &ws);
        if (rc != PCRP_OK) return rc;
        if (!ws) return set_error(PCRP_ENOMEM, "%s: no scratch for the split path (%zu bytes)", who, need);
        double* base = static_cast<double*>(ws);
        for (int u = 0; u < 2; u++)
            for (int k = 0; k < NSTATE; k++) bufs[u][k] = base + ((size_t)u * NSTATE + k) * (size_t)(m * n);
    }

    // global passes: K strides each, windows of L rows plus 2*(2^K-1) halo rows.
    // The s1 strides are spread evenly over the ceil(s1/fuse) passes, the
    // longer passes last (2+2+3, not 3+3+1: a one-stride pass spreads a pass's
    // fixed costs over little work, and the later passes' shorter subsystems
    // fill their tiles better with the wider halo); a pass of fewer strides
    // turns the halo rows it does not need into tile rows.
    const int npass = s1 > 0 ? (s1 + pl.fuse - 1) / pl.fuse : 0;
    int cur = 0;
    for (int ip = 0; ip < npass; ip++) {
        const int K = s1 / npass + (ip >= npass - s1 % npass ? 1 : 0);
        const int H = 2 * ((1 << K) - 1);
        const int Hfuse = 2 * ((1 << std::min(pl.fuse, s1)) - 1);
        int L = (pl.tile_rows > 0 ? pl.tile_rows : 1024) + 2 * (Hfuse - H);
        if (L + 2 * H > pcr_max_smem_rows()) L = pcr_max_smem_rows() - 2 * H;
        if (L < 1) return set_error(PCRP_EINVAL, "%s: fuse_strides=%d leaves no tile rows", who, K);
        const int64_t nrmax = ceil_div(n, p.G);
        // windows of equal length (at most L): no nearly empty last window per
        // subsystem (results do not depend on where windows start)
        p.nwin = ceil_div(nrmax, L);
        L = (int)ceil_div(nrmax, p.nwin);
        p.K = K; p.H = H; p.L = L; p.final_step = 0;
        p.TRmax = (int)std::min<int64_t>(L + 2 * H, nrmax);
        for (int k = 0; k < NSTATE; k++) p.dst[k] = bufs[cur][k];
        p.dst_ss = n; p.dst_rs = 1;
        p.dst_sub = 1;                      // the next pass reads each subsystem in one run
        cudaError_t ce = launch_pcr_pass(p, pl.threads, st, tri);
        if (ce != cudaSuccess) return cuda_error(ce, "pcr global pass launch");
        for (int k = 0; k < NSTATE; k++) p.src[k] = bufs[cur][k];
        p.src_ss = n; p.src_rs = 1; p.src_sub = 1;
        cur ^= 1;
        p.G <<= K;
    }

    // shared-memory finish on whole subsystems of at most smem_rows rows
    const int64_t nrmax = ceil_div(n, p.G);
    p.K = ns - s1; p.H = 0; p.L = (int)nrmax; p.final_step = 1; p.nwin = 1;
    p.TRmax = (int)nrmax;
    // whole systems read straight from the caller's arrays: bulk-staged
    // tiles where every array row run is 16-byte aligned (contiguous layout,
    // even n, aligned arrays)
    if (s1 == 0 && layout == PCRP_LAYOUT_CONTIGUOUS && n % 2 == 0) {
        bool aligned = true;
        for (const double* q : {a, b, c, d, e, (const double*)y})
            if (q && (reinterpret_cast<uintptr_t>(q) & 15)) aligned = false;
        p.bulk = aligned ? 1 : 0;
    }
    p.x = y; p.dst_ss = ss; p.dst_rs = rs; p.dst_sub = 0;
    for (int k = 0; k < NSTATE; k++) p.dst[k] = nullptr;
    cudaError_t ce = launch_pcr_pass(p, pl.threads, st, tri);
    if (ce != cudaSuccess) return cuda_error(ce, "pcr shared-memory pass launch");
    return PCRP_OK;
}

}  // namespace pcrp

using namespace pcrp;

extern "C" {

pcrp_status pcrp_solve_f64(const double* a, const double* b, const double* c, const double* d,
                           const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                           const pcrp_opts* opts, pcrp_stream stream)
{
    NvtxRange nv("pcrp_solve_f64");
    return f64_solve(a, b, c, d, e, y, m, n, layout, opts, (cudaStream_t)stream, false, false, "pcrp_solve_f64");
}

pcrp_status pcrp_solve_f64_small(const double* a, const double* b, const double* c, const double* d,
                                 const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                                 const pcrp_opts* opts, pcrp_stream stream)
{
    NvtxRange nv("pcrp_solve_f64_small");
    return f64_solve(a, b, c, d, e, y, m, n, layout, opts, (cudaStream_t)stream, true, false, "pcrp_solve_f64_small");
}

pcrp_status pcrp_solve_f64_split(const double* a, const double* b, const double* c, const double* d,
                                 const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                                 const pcrp_opts* opts, pcrp_stream stream)
{
    NvtxRange nv("pcrp_solve_f64_split");
    return f64_solve(a, b, c, d, e, y, m, n, layout, opts, (cudaStream_t)stream, false, true, "pcrp_solve_f64_split");
}

pcrp_status pcrp_workspace_size(int64_t m, int64_t n, int32_t layout, int32_t which,
                                const pcrp_opts* opts, size_t* bytes)
{
    if (!bytes) return set_error(PCRP_EINVAL, "pcrp_workspace_size: null output");
    *bytes = 0;
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "pcrp_workspace_size: negative size");
    if (!valid_layout(layout)) return set_error(PCRP_EINVAL, "pcrp_workspace_size: bad layout %d", layout);
    // (no solver accepts a batch this large; the sizes below would wrap)
    if (n > 0 && m > (int64_t(1) << 52) / n) return set_error(PCRP_EINVAL, "pcrp_workspace_size: m*n too large");
    const F64Plan pl = f64_plan(opts, n);
    switch (which) {
    case 0: *bytes = f64_workspace_bytes(m, n, layout, pl, true); return PCRP_OK;
    case 1: *bytes = mixed_workspace_bytes(m, n, opts, 64, true, layout); return PCRP_OK;
    case 2:                                      // either mode of pcrp_solve_ragged: m systems of <= n rows
        *bytes = std::max(ragged_workspace_bytes(m, m * n), ragged_mixed_workspace_bound(m, n, opts));
        return PCRP_OK;
    default: return set_error(PCRP_EINVAL, "pcrp_workspace_size: unknown entry family %d", which);
    }
}

pcrp_status pcrp_release_workspace(void)
{
    std::lock_guard<std::mutex> lk(g_ws_mu);
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto& kv : g_ws) {
        if (kv.second.first) {
            cudaSetDevice(kv.first.first);
            cudaFree(kv.second.first);
        }
    }
    g_ws.clear();
    cudaSetDevice(cur);
    return PCRP_OK;
}

const char* pcrp_get_last_error_string(void) { return g_last_error.c_str(); }

int32_t pcrp_version(void) { return 100; }

int64_t pcrp_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
