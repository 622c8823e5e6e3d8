// ragged_mixed.cu -- mixed-precision mode of pcrp_solve_ragged.
//
// Systems are binned by size into power-of-two classes N (n in (N/2, N]).
// Each class is gathered into a uniform padded batch (rows n..N-1 are
// identity rows with zero right-hand side, and the couplings that would reach
// them -- the out-of-range slots d_{n-1}, e_{n-2}, e_{n-1} -- are zeroed), so
// the padded solution restricted to the first n rows is the system's own.
// Each class runs the uniform mixed-precision solver (FP32 block reduction +
// FP64 refinement, its sweep loop a while node that stops at convergence),
// then the solutions are scattered back.  The classes are independent
// branches of one CUDA graph, captured once per (pointers, sizes) and
// replayed.
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

__global__ void rgm_gather_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                  const double* __restrict__ c, const double* __restrict__ d,
                                  const double* __restrict__ e, const double* __restrict__ y,
                                  const int64_t* __restrict__ offsets, const int64_t* __restrict__ sys,
                                  int64_t ms, int64_t N, double* __restrict__ out)
{
    const int64_t total = ms * N;
    double* pa = out; double* pb = pa + total; double* pc = pb + total;
    double* pd = pc + total; double* pe = pd + total; double* py = pe + total;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = q / N, i = q - s * N;
        const int64_t k = sys[s];
        const int64_t o = offsets[k], n = offsets[k + 1] - o;
        if (i < n) {
            pa[q] = (a && i >= 2) ? a[o + i] : 0.0;             // a null outer band is zero
            pb[q] = i >= 1 ? b[o + i] : 0.0;
            pc[q] = c[o + i];
            pd[q] = i + 1 < n ? d[o + i] : 0.0;
            pe[q] = (e && i + 2 < n) ? e[o + i] : 0.0;
            py[q] = y[o + i];
        } else {
            pa[q] = 0.0; pb[q] = 0.0; pc[q] = 1.0; pd[q] = 0.0; pe[q] = 0.0; py[q] = 0.0;
        }
    }
}

__global__ void rgm_scatter_kernel(const double* __restrict__ px, const int64_t* __restrict__ offsets,
                                   const int64_t* __restrict__ sys, int64_t ms, int64_t N, double* __restrict__ y,
                                   const int* __restrict__ status, int* __restrict__ unconverged)
{
    const int64_t total = ms * N;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = q / N, i = q - s * N;
        const int64_t k = sys[s];
        const int64_t o = offsets[k], n = offsets[k + 1] - o;
        if (i < n) y[o + i] = px[q];
        if (i == 0 && status[s] != 1) atomicAdd(unconverged, 1);
    }
}

unsigned grid_for(int64_t total) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 16));
}

struct Key {
    int dev;
    cudaStream_t s;
    const void* p[8];
    int64_t nsys;
    uint64_t hash;
    double tol;
    int sweeps;
    bool operator<(const Key& o) const {
        if (dev != o.dev) return dev < o.dev;
        if (s != o.s) return s < o.s;
        for (int q = 0; q < 8; q++) if (p[q] != o.p[q]) return p[q] < o.p[q];
        if (nsys != o.nsys) return nsys < o.nsys;
        if (hash != o.hash) return hash < o.hash;
        if (tol != o.tol) return tol < o.tol;
        return sweeps < o.sweeps;
    }
};
std::mutex g_mu;
std::map<Key, std::pair<cudaGraphExec_t, int64_t>> g_exec;   // graph and its kernel count

}  // namespace

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

    // size classes
    std::map<int64_t, std::vector<int64_t>> cls;
    uint64_t h = 1469598103934665603ULL;
    for (int64_t k = 0; k < nsys; k++) {
        const int64_t n = off[k + 1] - off[k];
        if (n < 0 || n > max_rows)
            return set_error(PCRP_EINVAL, "pcrp_solve_ragged: system %lld has %lld rows (max_rows %lld)",
                             (long long)k, (long long)n, (long long)max_rows);
        h = (h ^ (uint64_t)n) * 1099511628211ULL;
        if (n == 0) continue;
        int64_t N = 2;
        while (N < n) N <<= 1;
        cls[N].push_back(k);
    }
    // workspace: [system lists | counter | per class: padded batch, mixed scratch]
    // (every class has its own, so that the classes run concurrently)
    auto r256 = [](size_t v) { return (v + 255) / 256 * 256; };
    std::vector<size_t> pad_off, mix_off;
    size_t per_class = 0;
    for (auto& kv : cls) {
        const int64_t ms = (int64_t)kv.second.size(), N = kv.first;
        pad_off.push_back(per_class);
        per_class += r256((size_t)6 * ms * N * sizeof(double));
        mix_off.push_back(per_class);
        per_class += r256(mixed_workspace_bytes(ms, N, o, max_sweeps, false, PCRP_LAYOUT_CONTIGUOUS));
    }
    const size_t lists = r256((size_t)nsys * sizeof(int64_t));
    const size_t total = lists + 256 + per_class;
    void* ws = nullptr;
    pcrp_status rc = get_workspace(o, total, st, &ws);
    if (rc != PCRP_OK) return rc;
    char* base = static_cast<char*>(ws);
    int64_t* d_lists = reinterpret_cast<int64_t*>(base);
    int* d_unconv = reinterpret_cast<int*>(base + lists);
    char* d_class = base + lists + 256;

    std::vector<int64_t> h_lists;
    h_lists.reserve(nsys);
    for (auto& kv : cls) h_lists.insert(h_lists.end(), kv.second.begin(), kv.second.end());

    int dev = 0;
    ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_error(ce, "cudaGetDevice");
    Key key{};
    key.dev = dev; key.s = st;
    const void* ptrs[8] = {a, b, c, d, e, y, offsets, ws};
    for (int q = 0; q < 8; q++) key.p[q] = ptrs[q];
    key.nsys = nsys; key.hash = h; key.tol = tol; key.sweeps = max_sweeps;

    // the system lists are not graph nodes (they change with the offsets' content, which the key hashes)
    if (!h_lists.empty()) {
        ce = cudaMemcpyAsync(d_lists, h_lists.data(), h_lists.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) return cuda_error(ce, "pcrp_solve_ragged: system lists");
    }

    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_exec.find(key);
        if (it != g_exec.end()) { exec = it->second.first; kernels = it->second.second; }
    }
    if (!exec) {
        // One graph: the counter reset, then every size class on its own
        // branch (gather, mixed solve with its device-side sweep loop,
        // scatter), joined at the end.
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
            if (le == cudaSuccess) le = cudaEventRecord(bev[ncls], cst);
            int64_t at = 0;
            size_t q = 0;
            for (auto& kv : cls) {
                if (le != cudaSuccess || prc != PCRP_OK) break;
                const int64_t ms = (int64_t)kv.second.size(), N = kv.first;
                const int64_t* sys = d_lists + at;
                at += ms;
                cudaStream_t cs = bst[q];
                double* d_pad = reinterpret_cast<double*>(d_class + pad_off[q]);
                void* d_mix = d_class + mix_off[q];
                le = cudaStreamWaitEvent(cs, bev[ncls], 0);
                if (le != cudaSuccess) break;
                rgm_gather_kernel<<<grid_for(ms * N), 256, 0, cs>>>(a, b, c, d, e, y, offsets, sys, ms, N, d_pad);
                count_launch();
                const int64_t T = ms * N;
                MpArgs A{};
                prc = mixed_enqueue(d_pad, d_pad + T, d_pad + 2 * T, d_pad + 3 * T, d_pad + 4 * T, d_pad + 5 * T,
                                    ms, N, N, 1, tol, max_sweeps, o, false, d_mix, cs, &A);
                if (prc != PCRP_OK) break;
                rgm_scatter_kernel<<<grid_for(T), 256, 0, cs>>>(d_pad + 5 * T, offsets, sys, ms, N, y, A.status, d_unconv);
                count_launch();
                le = cudaGetLastError();
                if (le == cudaSuccess) le = cudaEventRecord(bev[q], cs);
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
        if (prc != PCRP_OK) return prc;
        if (ce != cudaSuccess) return cuda_error(ce, "ragged mixed graph capture");
        std::lock_guard<std::mutex> lk(g_mu);
        g_exec[key] = {exec, kernels};
    }
    ce = cudaGraphLaunch(exec, st);
    if (ce != cudaSuccess) return cuda_error(ce, "cudaGraphLaunch");
    count_launch(kernels);
    int unconv = 0;
    ce = cudaMemcpyAsync(&unconv, d_unconv, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_error(ce, "pcrp_solve_ragged");
    if (unconv) return set_error(PCRP_ENOCONV, "pcrp_solve_ragged: %d systems did not reach tol=%g in %d sweeps",
                                 unconv, tol, max_sweeps);
    return PCRP_OK;
}

}  // namespace pcrp
