// ragged_mixed.cu -- mixed-precision mode of pcrp_solve_ragged.
//
// Systems are binned by size into classes N a quarter of an octave apart
// (n in (2^k, 2^(k+1)] rounds up to a multiple of 2^(k-2): N/2^k is 5/4,
// 6/4, 7/4 or 2).  Each class runs the uniform mixed-precision solver (FP32
// block reduction + FP64 refinement, its sweep loop a while node that stops
// at convergence) as a batch of N-row systems that reads and writes the
// caller's arrays in place through a table of (first row, rows) per system:
// rows n..N-1 of a system are identity rows with zero right-hand side that
// exist only in the solver's own workspace, and the band slots that would
// couple the system to them (d_{n-1}, e_{n-2}, e_{n-1}) read as zero, so the
// padded solution restricted to the first n rows is the system's own.
// Padding adds at most a quarter and about an eighth of the rows on average
// to the solver's work, and nothing to the traffic on the caller's arrays.
// The classes are independent branches of one CUDA graph, captured once per
// (pointers, sizes) and replayed.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "mixed_internal.h"
#include "pcrp_internal.h"

namespace pcrp {

pcrp_status get_workspace(const pcrp_opts* o, size_t bytes, cudaStream_t s, void** out);
size_t mixed_workspace_bytes(int64_t m, int64_t n, const pcrp_opts* o, int max_sweeps, bool info, int32_t layout);

namespace {

// (first row, rows) of the systems of every class, class after class, from
// the offsets: the table the solver addresses the caller arrays through
__global__ void rgm_rows_kernel(const int64_t* __restrict__ offsets, const int64_t* __restrict__ sys, int64_t cnt,
                                longlong2* __restrict__ rows)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < cnt; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = sys[q];
        const int64_t o = offsets[k];
        rows[q] = make_longlong2(o, offsets[k + 1] - o);
    }
}

// systems of a class that did not converge (status 1: converged)
__global__ void rgm_count_kernel(const int* __restrict__ status, int64_t ms, int* __restrict__ unconverged)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ms; j += (int64_t)gridDim.x * blockDim.x)
        if (status[j] != 1) atomicAdd(unconverged, 1);
}

// The padded size of a system of n rows: n rounded up to a multiple of a
// quarter of its octave (2^(k-2) for n in (2^k, 2^(k+1)]), at least 2.
int64_t size_class(int64_t n)
{
    if (n <= 2) return 2;
    int k = 0;
    while ((int64_t(1) << (k + 1)) < n) k++;        // 2^k < n <= 2^(k+1)
    const int64_t step = int64_t(1) << std::max(k - 2, 0);
    return (n + step - 1) / step * step;
}

unsigned grid_for(int64_t total) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 16));
}

// A batch: its pointers, stream, sizes (hashed), solver settings and the
// tuning fields of its options (they shape the captured plan).
struct Key {
    int dev;
    cudaStream_t s;
    const void* p[7];
    int64_t nsys;
    uint64_t hash;
    double tol;
    int sweeps;
    int opt[6];
    bool operator<(const Key& o) const {
        if (dev != o.dev) return dev < o.dev;
        if (s != o.s) return s < o.s;
        for (int q = 0; q < 7; q++) if (p[q] != o.p[q]) return p[q] < o.p[q];
        if (nsys != o.nsys) return nsys < o.nsys;
        if (hash != o.hash) return hash < o.hash;
        if (tol != o.tol) return tol < o.tol;
        for (int q = 0; q < 6; q++) if (opt[q] != o.opt[q]) return opt[q] < o.opt[q];
        return sweeps < o.sweeps;
    }
};

// The batch's graph, the workspace it was captured on, and the device list
// of system indices (class after class) it reads; everything per call is in
// the graph, so a replay needs no upload.  The offsets it was built for are
// kept and compared on every hit (the key holds only their hash).
struct Entry {
    std::vector<int64_t> off;
    size_t total = 0;                 // workspace bytes
    void* ws = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;
    int64_t* d_sys = nullptr;
    uint64_t used = 0;
};
std::mutex g_mu;
std::map<Key, Entry> g_exec;
uint64_t g_clock = 0;
constexpr size_t kMaxEntries = 16;               // batches remembered (least recently used dropped)

}  // namespace

// An upper bound of the workspace of a mixed ragged batch of nsys systems
// of at most max_rows rows: every system padded to the largest class, the
// row table, and the 256-byte rounding of every array of every class (at
// most four classes per octave of sizes).
size_t ragged_mixed_workspace_bound(int64_t nsys, int64_t max_rows, const pcrp_opts* o)
{
    if (nsys <= 0 || max_rows <= 0) return 0;
    const int64_t N = size_class(max_rows);
    const size_t lists = ((size_t)nsys * sizeof(longlong2) + 255) / 256 * 256;
    const size_t classes = 4 * 64 + 2, arrays = 32;
    return lists + 256 + mixed_workspace_bytes(nsys, N, o, 64, false, PCRP_LAYOUT_CONTIGUOUS) +
           classes * arrays * 256;
}

pcrp_status ragged_mixed(const double* a, const double* b, const double* c, const double* d, const double* e,
                         double* y, const int64_t* offsets, int64_t nsys, int64_t max_rows, double tol,
                         int32_t max_sweeps, const pcrp_opts* o, cudaStream_t st)
{
    if (!(tol > 0.0)) tol = 1e-12;
    if (max_sweeps <= 0) max_sweeps = 8;
    if (max_sweeps > 64) max_sweeps = 64;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing(st, &cs);
    if (ce != cudaSuccess) return cuda_error(ce, "cudaStreamIsCapturing");
    if (cs != cudaStreamCaptureStatusNone)
        return set_error(PCRP_ENOTSUP, "pcrp_solve_ragged synchronises and cannot be captured; it replays its own graph");
    std::vector<int64_t> off((size_t)nsys + 1);
    ce = cudaMemcpyAsync(off.data(), offsets, (nsys + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_error(ce, "pcrp_solve_ragged: reading offsets");
    if (off[0] != 0) return set_error(PCRP_EINVAL, "pcrp_solve_ragged: offsets[0] = %lld, expected 0", (long long)off[0]);
    uint64_t h = 1469598103934665603ULL;
    for (int64_t k = 0; k < nsys; k++) {
        const int64_t n = off[k + 1] - off[k];
        if (n < 0 || n > max_rows)
            return set_error(PCRP_EINVAL, "pcrp_solve_ragged: system %lld has %lld rows (max_rows %lld)",
                             (long long)k, (long long)n, (long long)max_rows);
        h = (h ^ (uint64_t)n) * 1099511628211ULL;
    }

    int dev = 0;
    ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_error(ce, "cudaGetDevice");
    Key key{};
    key.dev = dev; key.s = st;
    const void* ptrs[7] = {a, b, c, d, e, y, offsets};
    for (int q = 0; q < 7; q++) key.p[q] = ptrs[q];
    key.nsys = nsys; key.hash = h; key.tol = tol; key.sweeps = max_sweeps;
    if (o && o->size >= sizeof(pcrp_opts)) {
        const int v[6] = {o->smem_rows, o->fuse_strides, o->tile_rows, o->threads, o->reserved0, o->window_levels};
        for (int q = 0; q < 6; q++) key.opt[q] = v[q];
    }

    // a batch seen before: its graph, if the workspace has not moved
    {
        size_t total = 0;
        {
            std::lock_guard<std::mutex> lk(g_mu);
            auto it = g_exec.find(key);
            if (it != g_exec.end() && it->second.exec && it->second.off == off) total = it->second.total;
        }
        if (total) {
            void* ws = nullptr;
            pcrp_status rc = get_workspace(o, total, st, &ws);
            if (rc != PCRP_OK) return rc;
            bool launched = false;
            int* d_unconv = reinterpret_cast<int*>(static_cast<char*>(ws) +
                                                   ((size_t)nsys * sizeof(longlong2) + 255) / 256 * 256);
            {
                // (launched under the lock: no other thread replaces the graph meanwhile)
                std::lock_guard<std::mutex> lk(g_mu);
                auto it = g_exec.find(key);
                if (it != g_exec.end() && it->second.exec && it->second.ws == ws && it->second.off == off) {
                    it->second.used = ++g_clock;
                    ce = cudaGraphLaunch(it->second.exec, st);
                    if (ce != cudaSuccess) return cuda_error(ce, "cudaGraphLaunch");
                    count_launch(it->second.kernels);
                    launched = true;
                }
            }
            if (launched) {
                int unconv = 0;
                ce = cudaMemcpyAsync(&unconv, d_unconv, sizeof(int), cudaMemcpyDeviceToHost, st);
                if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
                if (ce != cudaSuccess) return cuda_error(ce, "pcrp_solve_ragged");
                if (unconv)
                    return set_error(PCRP_ENOCONV, "pcrp_solve_ragged: %d systems did not reach tol=%g in %d sweeps",
                                     unconv, tol, max_sweeps);
                return PCRP_OK;
            }
        }
    }

    // size classes
    std::map<int64_t, std::vector<int64_t>> cls;
    for (int64_t k = 0; k < nsys; k++) {
        const int64_t n = off[k + 1] - off[k];
        if (n > 0) cls[size_class(n)].push_back(k);
    }
    if (cls.empty()) return PCRP_OK;                 // only empty systems
    // workspace: [row tables | counter | per class: mixed scratch]
    // (every class has its own, so that the classes run concurrently)
    auto r256 = [](size_t v) { return (v + 255) / 256 * 256; };
    std::vector<size_t> mix_off;
    size_t per_class = 0;
    for (auto& kv : cls) {
        const int64_t ms = (int64_t)kv.second.size(), N = kv.first;
        mix_off.push_back(per_class);
        per_class += r256(mixed_workspace_bytes(ms, N, o, max_sweeps, false, PCRP_LAYOUT_CONTIGUOUS));
    }
    const size_t lists = r256((size_t)nsys * sizeof(longlong2));
    const size_t total = lists + 256 + per_class;
    void* ws = nullptr;
    pcrp_status rc = get_workspace(o, total, st, &ws);
    if (rc != PCRP_OK) return rc;
    char* base = static_cast<char*>(ws);
    longlong2* d_rows = reinterpret_cast<longlong2*>(base);
    int* d_unconv = reinterpret_cast<int*>(base + lists);
    char* d_class = base + lists + 256;

    // system indices, class after class (the graph turns them into the row table)
    std::vector<int64_t> h_sys;
    h_sys.reserve(nsys);
    for (auto& kv : cls) h_sys.insert(h_sys.end(), kv.second.begin(), kv.second.end());
    const int64_t cnt = (int64_t)h_sys.size();
    int64_t* d_sys = nullptr;
    ce = cudaMalloc(&d_sys, cnt * sizeof(int64_t));
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(d_sys, h_sys.data(), cnt * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) {
        if (d_sys) cudaFree(d_sys);
        return cuda_error(ce, "pcrp_solve_ragged: system lists");
    }

    // One graph: the counter reset and the row table, then every size class
    // on its own branch (mixed solve with its device-side sweep loop, count
    // of the systems left unconverged), joined at the end.
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;
    {
        const size_t ncls = cls.size();
        cudaStream_t cst = nullptr;
        std::vector<cudaStream_t> bst(ncls, nullptr);
        std::vector<cudaEvent_t> bev(ncls + 1, nullptr);
        ce = cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking);
        for (size_t q = 0; q < ncls && ce == cudaSuccess; q++) ce = cudaStreamCreateWithFlags(&bst[q], cudaStreamNonBlocking);
        for (size_t q = 0; q <= ncls && ce == cudaSuccess; q++) ce = cudaEventCreateWithFlags(&bev[q], cudaEventDisableTiming);
        cudaGraph_t g = nullptr;
        pcrp_status prc = PCRP_OK;
        const int64_t before = pcrp_kernel_launches();
        if (ce == cudaSuccess) ce = cudaStreamBeginCapture(cst, cudaStreamCaptureModeRelaxed);
        if (ce == cudaSuccess) {
            cudaError_t le = cudaMemsetAsync(d_unconv, 0, sizeof(int), cst);
            if (le == cudaSuccess) {
                rgm_rows_kernel<<<grid_for(cnt), 256, 0, cst>>>(offsets, d_sys, cnt, d_rows);
                count_launch();
                le = cudaGetLastError();
            }
            if (le == cudaSuccess) le = cudaEventRecord(bev[ncls], cst);
            int64_t at = 0;
            size_t q = 0;
            for (auto& kv : cls) {
                if (le != cudaSuccess || prc != PCRP_OK) break;
                const int64_t ms = (int64_t)kv.second.size(), N = kv.first;
                const longlong2* rows = d_rows + at;
                at += ms;
                cudaStream_t bs = bst[q];
                void* d_mix = d_class + mix_off[q];
                le = cudaStreamWaitEvent(bs, bev[ncls], 0);
                if (le != cudaSuccess) break;
                MpArgs A{};
                prc = mixed_enqueue(a, b, c, d, e, y, ms, N, N, 1, tol, max_sweeps, o, false, d_mix, bs, &A,
                                    nullptr, nullptr, rows);
                if (prc != PCRP_OK) break;
                rgm_count_kernel<<<grid_for(ms), 256, 0, bs>>>(A.status, ms, d_unconv);
                count_launch();
                le = cudaGetLastError();
                if (le == cudaSuccess) le = cudaEventRecord(bev[q], bs);
                if (le == cudaSuccess) le = cudaStreamWaitEvent(cst, bev[q], 0);
                q++;
            }
            cudaError_t ee = cudaStreamEndCapture(cst, &g);
            if (ce == cudaSuccess) ce = le != cudaSuccess ? le : ee;
        }
        kernels = pcrp_kernel_launches() - before;
        count_launch(-kernels);              // counted when the graph runs, not when captured
        if (ce == cudaSuccess && prc == PCRP_OK) ce = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        for (auto ev : bev) if (ev) cudaEventDestroy(ev);
        for (auto bs : bst) if (bs) cudaStreamDestroy(bs);
        if (cst) cudaStreamDestroy(cst);
        if (prc != PCRP_OK || ce != cudaSuccess) {
            if (exec) cudaGraphExecDestroy(exec);
            cudaFree(d_sys);
            if (prc != PCRP_OK) return prc;
            return cuda_error(ce, "ragged mixed graph capture");
        }
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_exec.size() >= kMaxEntries && g_exec.find(key) == g_exec.end()) {
            auto old = g_exec.begin();
            for (auto jt = g_exec.begin(); jt != g_exec.end(); ++jt)
                if (jt->second.used < old->second.used) old = jt;
            if (old->second.exec) cudaGraphExecDestroy(old->second.exec);
            if (old->second.d_sys) cudaFree(old->second.d_sys);
            g_exec.erase(old);
        }
        Entry& E = g_exec[key];
        E.used = ++g_clock;
        if (E.exec) cudaGraphExecDestroy(E.exec);          // captured on a workspace that has moved
        if (E.d_sys) cudaFree(E.d_sys);
        E.off = off;
        E.total = total; E.ws = ws; E.exec = exec; E.kernels = kernels; E.d_sys = d_sys;
        ce = cudaGraphLaunch(exec, st);
        if (ce != cudaSuccess) return cuda_error(ce, "cudaGraphLaunch");
        count_launch(kernels);
    }
    int unconv = 0;
    ce = cudaMemcpyAsync(&unconv, d_unconv, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_error(ce, "pcrp_solve_ragged");
    if (unconv) return set_error(PCRP_ENOCONV, "pcrp_solve_ragged: %d systems did not reach tol=%g in %d sweeps",
                                 unconv, tol, max_sweeps);
    return PCRP_OK;
}

}  // namespace pcrp
