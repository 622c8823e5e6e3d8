// noalloc.cu -- the FP64 PCR-Penta solve for callers that cannot allocate
// device memory.
//
// Some callers are not allowed to call cudaMalloc at all: code that runs
// inside a host callback or a driver/plugin hook where the CUDA allocator may
// not be entered, or real-time and embedded hosts whose device memory is
// budgeted once at start-up and must never grow afterwards.
// pcrp_solve_f64 would otherwise take its split-path scratch from a buffer it
// allocates on first use, so this file gives those callers a variant whose
// scratch is a fixed array compiled into the library instead.
//
// The array below is a file-scope __device__ object: every GPU that loads the
// library holds its kPcrpNoallocScratchBytes until the process exits.  In host
// code the symbol is only a host-side stand-in for that object, not a device
// address, so the host asks the runtime for the real address
// (cudaGetSymbolAddress) once per device, with that device current, and
// passes that pointer on.  The first call on a device does this set-up, so on
// each device make one call before any stream capture begins.
//
// All calls share the one array and it keeps whatever the last call left in
// it.  Two calls whose GPU work overlaps in time (different streams, or
// unordered host threads) therefore race on it and corrupt each other's
// results: issue such calls on a single stream.
#include <mutex>

#include "pcrp_internal.h"

namespace pcrp {

// Scratch of the split path: two ping-pong copies of the 8-array pass state
// (128 bytes per unknown), so this size limits one call of systems longer
// than the shared-memory tile (n > 512 with the tuned plan) to
// m*n <= 524288.  Shorter systems are solved whole in shared memory, need
// no scratch, and have no limit.
constexpr size_t kPcrpNoallocScratchBytes = size_t(64) << 20;   // 64 MiB
constexpr int64_t kPcrpNoallocMaxUnknowns = (int64_t)(kPcrpNoallocScratchBytes / (2 * NSTATE * sizeof(double)));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kPcrpNoallocScratchBytes];

pcrp_status f64_solve(const double* a, const double* b, const double* c, const double* d,
                      const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                      const pcrp_opts* o, cudaStream_t st, bool force_small, bool force_split,
                      const char* who);
bool f64_needs_scratch(int64_t n, const pcrp_opts* o);

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch on the current device (looked up once per device).
pcrp_status noalloc_scratch(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_solve_f64_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(PCRP_ENOTSUP, "pcrp_solve_f64_noalloc: device %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_error(e, "pcrp_solve_f64_noalloc: cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return PCRP_OK;
}
}  // namespace
}  // namespace pcrp

using namespace pcrp;

extern "C" pcrp_status pcrp_solve_f64_noalloc(const double* a, const double* b, const double* c,
                                              const double* d, const double* e, double* y,
                                              int64_t m, int64_t n, int32_t layout, pcrp_stream stream)
{
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "pcrp_solve_f64_noalloc: negative size");
    if (m == 0 || n == 0) return PCRP_OK;
    pcrp_opts o{};
    o.size = sizeof(pcrp_opts);
    // Systems that fit the shared-memory tile are solved whole and touch no
    // scratch, so only the split path has a size limit.  (Compared without
    // forming m*n, which could wrap for huge sizes.)
    if (f64_needs_scratch(n, &o) && m > kPcrpNoallocMaxUnknowns / n)
        return set_error(PCRP_EINVAL,
                         "pcrp_solve_f64_noalloc: m=%lld systems of n=%lld rows need %.0f bytes of scratch, "
                         "more than the library's fixed %zu bytes (m*n <= %lld for n above the "
                         "shared-memory tile); use pcrp_solve_f64 with a workspace",
                         (long long)m, (long long)n, 2.0 * NSTATE * sizeof(double) * (double)m * (double)n,
                         kPcrpNoallocScratchBytes, (long long)kPcrpNoallocMaxUnknowns);
    void* scratch = nullptr;
    pcrp_status rc = noalloc_scratch(&scratch);
    if (rc != PCRP_OK) return rc;
    // Every pass writes all the rows a later pass reads, so the scratch needs
    // no clearing; it keeps the previous call's contents.  A caller-provided
    // workspace is never grown, so nothing below can allocate.
    o.workspace = scratch;
    o.workspace_bytes = kPcrpNoallocScratchBytes;
    return f64_solve(a, b, c, d, e, y, m, n, layout, &o, (cudaStream_t)stream, false, false,
                     "pcrp_solve_f64_noalloc");
}
