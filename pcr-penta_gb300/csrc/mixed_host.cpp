// mixed_host.cpp -- host side of the mixed-precision solver: workspace
// layout, the FP32 pass plan and the refinement sweep loop.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "mixed_internal.h"
#include "pcrp_internal.h"
#include "tuned_params.h"

namespace pcrp {

pcrp_status get_workspace(const pcrp_opts* o, size_t bytes, cudaStream_t s, void** out);

namespace {

int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

struct MpPlan {
    int cap;        // block rows solved whole in shared memory
    int fuse;       // strides per global pass
    int s1;         // global strides in total
    int npass;
    int win;        // levels of the windowed cyclic-reduction pass (0: none)
};

MpPlan mp_plan(int64_t nb, const pcrp_opts* o)
{
    static const int64_t table[][3] = PCRP_TUNED_MP_TABLE;
    const int rows = (int)(sizeof(table) / sizeof(table[0]));
    int t = 0;
    while (t + 1 < rows && 2 * nb > table[t][0]) t++;
    MpPlan p{(int)table[t][1], (int)table[t][2], 0, 0, kMpTryLevels};
    // a system that fits one shared-memory tile is reduced whole (cyclic
    // reduction to the top, no global pass)
    if (nb <= kMpMaxRows) p.cap = kMpMaxRows;
    if (o && o->size >= sizeof(pcrp_opts)) {
        if (o->smem_rows > 0) p.cap = std::max(1, o->smem_rows / 2);
        if (o->fuse_strides > 0) p.fuse = o->fuse_strides;
        if (o->window_levels != 0) p.win = std::min(std::max(o->window_levels, 0), 7);   // halo 2^(K+1) < tile/2
    }
    p.cap = std::min(std::max(p.cap, 1), kMpMaxRows);
    p.fuse = std::min(std::max(p.fuse, 1), 9);
    while (cdiv(nb, int64_t(1) << p.s1) > p.cap) p.s1++;
    p.npass = (int)cdiv(p.s1, p.fuse);
    return p;
}

struct MpLayout {
    size_t S0, R, Mi, P0, P1, dx, X0, Yc, Xout, ctr, ndx, nx, fin, status, est, trunc, ndx_pre, live, fail, nfail, dnorm,
        err, rbuf, rn, total;
};

MpLayout mp_layout(int64_t m, int64_t n, int max_sweeps, const MpPlan& pl, bool info)
{
    const int64_t nb = (n + 1) / 2, T = m * nb;
    MpLayout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    L.S0 = take(2 * T * sizeof(float4));
    L.R = take(2 * T * sizeof(float2));
    L.Mi = take(T * sizeof(float4));
    L.P0 = pl.s1 > 0 ? take(2 * T * sizeof(float4) + T * sizeof(float2)) : 0;
    L.P1 = pl.npass > 1 ? take(2 * T * sizeof(float4) + T * sizeof(float2)) : 0;
    L.dx = take((size_t)m * n * sizeof(float));
    L.X0 = take((size_t)m * n * sizeof(double));
    L.Yc = take((size_t)m * n * sizeof(double));
    L.Xout = info ? take((size_t)m * n * sizeof(double)) : 0;
    L.ctr = take(sizeof(int));
    L.ndx = take((size_t)(max_sweeps + 1) * m * sizeof(unsigned));
    L.nx = take((size_t)(max_sweeps + 1) * m * sizeof(unsigned));
    L.fin = take(m * sizeof(int));
    L.status = take(m * sizeof(int));
    L.est = take(m * sizeof(float));
    L.trunc = take((size_t)kMpMaxPasses * m * sizeof(unsigned));
    L.ndx_pre = take((size_t)max_sweeps * kMpMaxPasses * m * sizeof(unsigned));
    L.live = take((size_t)(max_sweeps + 1) * sizeof(int));
    L.fail = take(m * sizeof(int));
    L.nfail = take(sizeof(int));
    L.dnorm = take(2 * (size_t)m * sizeof(unsigned));
    L.err = take(sizeof(int));
    L.rbuf = info ? take((size_t)m * n * sizeof(double)) : 0;
    L.rn = info ? take(3 * m * sizeof(unsigned)) : 0;
    L.total = off;
    return L;
}

bool valid_layout(int32_t l) { return l == PCRP_LAYOUT_CONTIGUOUS || l == PCRP_LAYOUT_INTERLEAVED; }

// Everything one sweep needs besides the argument block.
struct SweepPlan {
    MpPlan pl;
    MpWindows W;
    int64_t nb, T;
    bool windowed, cr_mode, fused;
    bool duo;                   // sweeps 0 and 1 of every system run first in mp_duo_kernel (mixed_duo.cu);
    DuoGeom D;                  // the general kernels then take only the systems it leaves
    float* P[2];                // ping-pong state of the block-PCR passes
};

// One sweep's kernels.  s >= 0: host-driven, the per-sweep fields are set
// here; s < 0: the body of the graph's while node, the kernels resolve them
// on the device from the sweep counter A.ctr.
pcrp_status enqueue_sweep(MpArgs A, const SweepPlan& S, int s, cudaStream_t st)
{
    const bool dev = s < 0;
    const int64_t m = A.m, n = A.n, nb = S.nb, T = S.T;
    const MpPlan& pl = S.pl;
    cudaError_t ce;
    if (!dev) {
        A.sweep = s;
        A.xsrc_rg = nullptr; A.xdst_rg = nullptr;
        if (s == 0) { A.xsrc = nullptr; A.xsrc_ss = 0; A.xsrc_rs = 0; }
        else if (s == 1) { A.xsrc = A.X0; A.xsrc_ss = n; A.xsrc_rs = 1; }
        else { A.xsrc = A.xout; A.xsrc_ss = A.oss; A.xsrc_rs = A.ors; A.xsrc_rg = A.rg; }
        if (s == 0 && A.max_sweeps >= 2) { A.xdst = A.X0; A.xdst_ss = n; A.xdst_rs = 1; }
        else { A.xdst = A.xout; A.xdst_ss = A.oss; A.xdst_rs = A.ors; A.xdst_rg = A.rg; }
    }

    // FP32 block solve of the normalised system with rhs R[s & 1]
    MpPassArgs p{};
    p.srcLU = A.S0;
    p.dx = A.dx; p.fin = A.fin; p.ndx = A.ndx;
    p.m = m; p.n = n; p.nb = nb; p.G = 1;
    if (dev) {
        p.ctr = A.ctr; p.live0 = A.live; p.R0 = A.R[0]; p.R1 = A.R[1]; p.pre0 = A.ndx_pre;
        p.X0 = A.X0; p.xout = A.xout; p.oss = A.oss; p.ors = A.ors; p.rg = A.rg; p.max_sweeps = A.max_sweeps;
    } else {
        p.sweep = s; p.srcY = A.R[s & 1]; p.live = A.live + s;
    }
    unsigned* pre = dev ? nullptr : A.ndx_pre + (size_t)s * kMpMaxPasses * m;
    if (S.cr_mode && (dev || !(S.fused && s == 0))) {
        // cyclic reduction of whole systems or of windows that decouple
        // within pl.win levels, with x_s = x_{s-1} + dx_s; the passes
        // below take the systems it leaves coupled
        MpPassArgs t = p;
        t.K = S.W.K; t.H = S.W.H; t.L = S.W.L; t.final_step = 0; t.nwin = S.W.nwin; t.TRmax = S.W.TRmax;
        t.fail = A.fail; t.nfail = A.nfail;
        if (dev) {
            t.pre0 = nullptr; t.level0 = 1; t.nx0 = A.nx; t.skip0 = S.fused;
        } else {
            t.xsrc = A.xsrc; t.xsrc_ss = A.xsrc_ss; t.xsrc_rs = A.xsrc_rs; t.xsrc_rg = A.xsrc_rg;
            t.xdst = A.xdst; t.xdst_ss = A.xdst_ss; t.xdst_rs = A.xdst_rs; t.xdst_rg = A.xdst_rg;
            t.nx = A.nx + (size_t)s * m;
        }
        ce = launch_mp_try(t, st);
        if (ce != cudaSuccess) return cuda_error(ce, "mixed cyclic-reduction launch");
    }
    if (S.cr_mode) { p.fail = A.fail; p.nfail = A.nfail; }
    int done = 0, pass = 0;
    while (done < pl.s1) {
        const int K = std::min(pl.fuse, pl.s1 - done);
        const int H = (1 << K) - 1;
        int Lw = std::max(1, pl.cap - 2 * H);
        const int64_t nrmax = cdiv(nb, p.G);
        char* D = reinterpret_cast<char*>(S.P[pass & 1]);
        p.dstLU = reinterpret_cast<float4*>(D);
        p.dstY = reinterpret_cast<float2*>(D + 2 * T * sizeof(float4));
        p.K = K; p.H = H; p.L = Lw; p.final_step = 0;
        p.nwin = cdiv(nrmax, Lw);
        p.TRmax = (int)std::min<int64_t>(Lw + 2 * H, nrmax);
        p.trunc_in = pass > 0 ? A.trunc + (pass - 1) * m : nullptr;
        p.trunc_out = A.trunc + pass * m;
        p.pass = pass; p.level0 = dev && pass == 0;
        if (!dev) {
            p.ndx_pre_in = pass > 0 ? pre + (pass - 1) * m : nullptr;
            p.ndx_pre_out = pre + pass * m;
        }
        ce = launch_mp_pass(p, st);
        if (ce != cudaSuccess) return cuda_error(ce, "mixed global pass launch");
        p.srcLU = p.dstLU; p.srcY = p.dstY;
        p.G <<= K; done += K; pass++;
    }
    if (!(S.cr_mode && pl.s1 == 0)) {            // whole systems never leave the cyclic-reduction pass
        const int64_t nrmax = cdiv(nb, p.G);
        int Kf = 0;
        while ((int64_t(1) << Kf) < nrmax) Kf++;
        p.K = Kf; p.H = 0; p.L = (int)nrmax; p.final_step = 1; p.nwin = 1; p.TRmax = (int)nrmax;
        p.trunc_in = pass > 0 ? A.trunc + (pass - 1) * m : nullptr;
        p.trunc_out = nullptr;
        p.pass = pass; p.level0 = dev && pass == 0;
        if (!dev) {
            p.ndx_pre_in = pass > 0 ? pre + (pass - 1) * m : nullptr;
            p.ndx_pre_out = nullptr;
        }
        ce = launch_mp_pass(p, st);
        if (ce != cudaSuccess) return cuda_error(ce, "mixed shared-memory pass launch");
        // x_s of the systems the passes solved
        ce = launch_mp_xupdate(A, st);
        if (ce != cudaSuccess) return cuda_error(ce, "mixed update launch");
    }
    // stopping decision, then the next rhs of the systems still running
    ce = launch_mp_decide(A, st);
    if (ce == cudaSuccess && (dev || s + 1 < A.max_sweeps)) ce = launch_mp_residual(A, st);
    if (ce != cudaSuccess) return cuda_error(ce, "mixed refinement launch");
    return PCRP_OK;
}

// ---------------------------------------------------------------------------
// Graph-driven sweeps: init and sweep 0's first kernel, then a while node
// whose body is one sweep ending in mp_advance_kernel, which stops the loop
// once every system has finished.  Sweeps after convergence cost nothing.
// One graph per argument set (pointers, sizes, tolerance, plan), built on
// the second call with that set and replayed afterwards.
// ---------------------------------------------------------------------------
struct GraphKey {
    int dev;
    const void* ptr[9];
    int64_t m, n, ss, rs;
    double tol;
    int max_sweeps, cap, fuse, win, duo, inject;
    bool operator<(const GraphKey& o) const { return std::memcmp(this, &o, sizeof(GraphKey)) < 0; }
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;             // kernels of the prefix and of one sweep
    bool failed = false;         // capture or instantiation refused: host-driven from now on
    uint64_t used = 0;
};

std::mutex g_graph_mu;
std::map<GraphKey, GraphEntry> g_graphs;
uint64_t g_graph_clock = 0;
constexpr size_t kMaxGraphs = 16;

// 0: host-driven sweeps; 1: replayed graph; 2: the caller is capturing `st`:
// the device-side loop goes into the caller's graph
int graph_mode(cudaStream_t st)
{
    if (std::getenv("PCRP_NO_GRAPH")) return 0;           // host-driven sweeps only (tests of both paths)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return 0;
    if (cs == cudaStreamCaptureStatusActive) return 2;
    return cs == cudaStreamCaptureStatusNone ? 1 : 0;
}

// Appends one solve to the capture in progress on `st`: init and sweep 0's
// first kernel, then a while node whose body (captured on a helper stream)
// is one sweep ending in mp_advance_kernel.  Returns false if this CUDA
// version or device refuses a step (the capture is then unusable).
bool capture_sweep_loop(const MpArgs& A, const SweepPlan& S, cudaStream_t st)
{
    cudaStreamCaptureStatus status;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaGraphConditionalHandle h = 0;
    // with the fused first sweeps, the loop runs only if the gate kernel
    // finds a system left; otherwise at least one sweep runs
    if (cudaStreamGetCaptureInfo(st, &status, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
        status != cudaStreamCaptureStatusActive ||
        cudaGraphConditionalHandleCreate(&h, g, S.duo ? 0 : 1, cudaGraphCondAssignDefault) != cudaSuccess)
        return false;
    if (launch_mp_init(A, st) != cudaSuccess) return false;
    if (S.duo && (launch_mp_duo(A, S.D, st) != cudaSuccess || launch_mp_duo_finish(A, st) != cudaSuccess))
        return false;
    if ((S.fused ? launch_mp_first(A, S.W, st) : launch_mp_prep(A, st)) != cudaSuccess) return false;
    if (S.duo && launch_mp_gate(A, h, st) != cudaSuccess) return false;
    if (cudaStreamGetCaptureInfo(st, &status, nullptr, &g, &deps, nullptr, &ndeps) != cudaSuccess ||
        status != cudaStreamCaptureStatusActive)
        return false;
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond = nullptr;
    if (cudaGraphAddNode(&cond, g, deps, nullptr, ndeps, &cp) != cudaSuccess ||
        cudaStreamUpdateCaptureDependencies(st, &cond, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
        return false;
    cudaStream_t bs = nullptr;
    if (cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking) != cudaSuccess) return false;
    bool ok = cudaStreamBeginCaptureToGraph(bs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                            cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (ok) {
        ok = enqueue_sweep(A, S, -1, bs) == PCRP_OK && launch_mp_advance(A, h, bs) == cudaSuccess;
        cudaGraph_t body = nullptr;
        ok = cudaStreamEndCapture(bs, &body) == cudaSuccess && ok;
    }
    cudaStreamDestroy(bs);
    return ok;
}

// Captures the graph of one solve; returns null (and clears the error) if
// this CUDA version or device refuses any step.
cudaGraphExec_t build_sweep_graph(const MpArgs& A, const SweepPlan& S, int* kernels)
{
    cudaStream_t cs = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int64_t before = pcrp_kernel_launches();
    bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (ok) {
        const bool body_ok = capture_sweep_loop(A, S, cs);
        const cudaError_t ee = cudaStreamEndCapture(cs, &graph);
        ok = body_ok && ee == cudaSuccess && graph != nullptr &&
             cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    }
    *kernels = (int)(pcrp_kernel_launches() - before);
    count_launch(-*kernels);                      // counted when the graph runs, not when captured
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamDestroy(cs);
    if (!ok) {
        if (exec) cudaGraphExecDestroy(exec);
        cudaGetLastError();                       // a refused capture is not the caller's error
        return nullptr;
    }
    return exec;
}

// PCRP_ENOTSUP: not (yet) graph-driven for this argument set; the caller
// enqueues host-driven sweeps.
pcrp_status launch_sweep_graph(const MpArgs& A, const SweepPlan& S, cudaStream_t st)
{
    GraphKey k;
    std::memset(&k, 0, sizeof k);
    if (cudaGetDevice(&k.dev) != cudaSuccess) return PCRP_ENOTSUP;
    const void* ptrs[9] = {A.a, A.b, A.c, A.d, A.e, A.y, A.S0, A.xout, A.rg};
    for (int i = 0; i < 9; i++) k.ptr[i] = ptrs[i];
    k.m = A.m; k.n = A.n; k.ss = A.ss; k.rs = A.rs; k.tol = A.tol; k.max_sweeps = A.max_sweeps;
    k.cap = S.pl.cap; k.fuse = S.pl.fuse; k.win = S.pl.win; k.duo = S.duo; k.inject = A.inject;
    std::lock_guard<std::mutex> lk(g_graph_mu);
    auto it = g_graphs.find(k);
    if (it == g_graphs.end()) {
        if (g_graphs.size() >= kMaxGraphs) {      // forget the least recently used
            auto old = g_graphs.begin();
            for (auto jt = g_graphs.begin(); jt != g_graphs.end(); ++jt)
                if (jt->second.used < old->second.used) old = jt;
            if (old->second.exec) cudaGraphExecDestroy(old->second.exec);
            g_graphs.erase(old);
        }
        g_graphs[k].used = ++g_graph_clock;       // first call: host-driven, remembered
        return PCRP_ENOTSUP;
    }
    GraphEntry& E = it->second;
    E.used = ++g_graph_clock;
    if (E.failed) return PCRP_ENOTSUP;
    if (!E.exec) {
        E.exec = build_sweep_graph(A, S, &E.kernels);
        if (!E.exec) { E.failed = true; return PCRP_ENOTSUP; }
    }
    const cudaError_t ce = cudaGraphLaunch(E.exec, st);
    if (ce != cudaSuccess) return cuda_error(ce, "mixed sweep graph launch");
    count_launch(E.kernels);                      // the prefix and the kernels of one sweep (the loop may repeat them)
    return PCRP_OK;
}

}  // namespace

// Contiguous copies of the six arrays for the layout adapter of an
// interleaved batch (m > 1), after the solver's own workspace.
static size_t adapter_array_bytes(int64_t m, int64_t n) { return ((size_t)m * n * sizeof(double) + 255) / 256 * 256; }
static bool adapts(int32_t layout, int64_t m) { return layout == PCRP_LAYOUT_INTERLEAVED && m > 1; }

size_t mixed_workspace_bytes(int64_t m, int64_t n, const pcrp_opts* o, int max_sweeps, bool info, int32_t layout)
{
    if (m <= 0 || n <= 0) return 0;
    const MpPlan pl = mp_plan((n + 1) / 2, o);
    return mp_layout(m, n, max_sweeps, pl, info).total + (adapts(layout, m) ? 6 * adapter_array_bytes(m, n) : 0);
}

// Enqueues prep + max_sweeps refinement sweeps of a uniform batch on `st`
// using the workspace `ws` (mixed_workspace_bytes(m, n, opts, max_sweeps, keep_x)
// bytes).  The bands and y use addressing (ss, rs).  Fills *out with the
// kernel arguments (per-system status arrays live in the workspace).
pcrp_status mixed_enqueue(const double* a, const double* b, const double* c, const double* d, const double* e,
                          double* y, int64_t m, int64_t n, int64_t ss, int64_t rs, double tol, int max_sweeps,
                          const pcrp_opts* opts, bool keep_x, void* ws, cudaStream_t st, MpArgs* out,
                          const MixedDest* dest, bool* dest_written, const longlong2* rg)
{
    const char* who = "pcrp_solve_mixed";
    if (dest_written) *dest_written = false;
    const int64_t nb = (n + 1) / 2, T = m * nb;
    const MpPlan pl = mp_plan(nb, opts);
    if (pl.npass > kMpMaxPasses) return set_error(PCRP_EINVAL, "%s: n too large for the pass plan", who);
    const MpLayout WL = mp_layout(m, n, max_sweeps, pl, keep_x);
    char* base = static_cast<char*>(ws);
    auto F = [&](size_t off) { return reinterpret_cast<float*>(base + off); };
    auto U = [&](size_t off) { return reinterpret_cast<unsigned*>(base + off); };

    MpArgs A{};
    A.a = a; A.b = b; A.c = c; A.d = d; A.e = e; A.y = y;
    if (rg) {                                    // a ragged batch keeps no report and has no adapter
        if (keep_x || dest) return set_error(PCRP_EINVAL, "%s: internal: ragged batch with a report", who);
        ss = n; rs = 1;
    }
    A.m = m; A.n = n; A.ss = ss; A.rs = rs; A.rg = rg;
    A.S0 = reinterpret_cast<float4*>(base + WL.S0);
    A.R[0] = reinterpret_cast<float2*>(base + WL.R);
    A.R[1] = A.R[0] + T;
    A.Mi = reinterpret_cast<float4*>(base + WL.Mi);
    A.dx = F(WL.dx);
    A.X0 = reinterpret_cast<double*>(base + WL.X0);
    A.Yc = reinterpret_cast<double*>(base + WL.Yc);
    A.Xout = keep_x ? reinterpret_cast<double*>(base + WL.Xout) : nullptr;
    A.ndx = U(WL.ndx); A.nx = U(WL.nx);
    A.fin = reinterpret_cast<int*>(base + WL.fin);
    A.status = reinterpret_cast<int*>(base + WL.status);
    A.est = F(WL.est); A.trunc = U(WL.trunc);
    A.ndx_pre = U(WL.ndx_pre);
    A.live = reinterpret_cast<int*>(base + WL.live);
    A.fail = reinterpret_cast<int*>(base + WL.fail);
    A.nfail = reinterpret_cast<int*>(base + WL.nfail);
    A.dnorm = U(WL.dnorm);
    A.err = reinterpret_cast<int*>(base + WL.err);
    A.inject = (opts && opts->size >= sizeof(pcrp_opts) && opts->reserved0 == 0x7E57) ? 1 : 0;
    A.max_sweeps = max_sweeps; A.tol = (float)tol; A.keep_x = keep_x;
    {
        const void* ptrs[6] = {a, b, c, d, e, y};
        A.vec = 1;
        for (const void* q : ptrs) if (reinterpret_cast<uintptr_t>(q) & 15) A.vec = 0;
    }

    // Iterates: x_0 in X0 when more sweeps follow, every later x_s in the
    // output (y, or Xout when y must keep the rhs for the report).
    A.xout = keep_x ? A.Xout : y;
    A.oss = keep_x ? n : ss;
    A.ors = keep_x ? 1 : rs;

    // Systems that fit one shared-memory tile: every sweep of a system in one
    // CTA, the whole solve one launch (no sweep loop to drive)
    if (pl.s1 == 0) {
        A.err = nullptr;                          // (no fused pass, no status word)
        if (dest && !keep_x) {
            A.xout = dest->x; A.oss = dest->ss; A.ors = dest->rs;
            if (dest_written) *dest_written = true;
        }
        if (out) *out = A;
        const cudaError_t cs = launch_mp_small(A, st);
        return cs == cudaSuccess ? PCRP_OK : cuda_error(cs, "mixed small-system launch");
    }

    // Windows of the level-0 cyclic-reduction passes (2^(win+1) halo), or
    // block-PCR passes only (win = 0).
    SweepPlan S{};
    S.pl = pl; S.nb = nb; S.T = T;
    S.windowed = pl.win > 0;
    S.cr_mode = S.windowed;
    if (S.windowed) {
        S.W.H = 2 << pl.win; S.W.K = pl.win; S.W.L = kMpTryRows - 2 * S.W.H;
        S.W.nwin = cdiv(nb, S.W.L);
        S.W.TRmax = (int)std::min<int64_t>(S.W.L + 2 * S.W.H, nb);
    }
    // Sweep 0 fused into one kernel (prep, reduction, x_0, r_0) when the
    // level-0 pass is a cyclic-reduction one and a second sweep exists.
    S.fused = max_sweeps >= 2 && S.cr_mode;
    A.first_fused = S.fused;
    A.cr_mode = S.cr_mode;
    // Sweeps 0 and 1 in one pass over the inputs for every system whose
    // windows decouple (contiguous, even n, aligned arrays); mp_first and
    // the sweep loop then see only the systems it leaves.
    S.duo = S.fused && duo_plan(A, pl.win, &S.D);
    if (!S.duo) A.err = nullptr;                 // (the status word belongs to the fused pass)
    S.P[0] = pl.s1 > 0 ? F(WL.P0) : nullptr;
    S.P[1] = pl.npass > 1 ? F(WL.P1) : nullptr;
    A.ctr = reinterpret_cast<int*>(base + WL.ctr);

    cudaError_t ce;
    const int gm = keep_x ? 0 : graph_mode(st);
    if (gm == 1) {
        const pcrp_status grc = launch_sweep_graph(A, S, st);
        if (grc != PCRP_ENOTSUP) {
            if (out) *out = A;
            return grc;
        }
    } else if (gm == 2) {
        if (!capture_sweep_loop(A, S, st))
            return set_error(PCRP_ECUDA, "pcrp_solve_mixed: the sweep loop could not be added to the stream's capture");
        if (out) *out = A;
        return PCRP_OK;
    }
    // host-driven sweeps: every kernel of every sweep is enqueued here
    A.ctr = nullptr;
    ce = launch_mp_init(A, st);
    if (ce != cudaSuccess) return cuda_error(ce, "mixed init launch");
    if (S.duo) {
        ce = launch_mp_duo(A, S.D, st);
        if (ce == cudaSuccess) ce = launch_mp_duo_finish(A, st);
        if (ce != cudaSuccess) return cuda_error(ce, "mixed fused-sweeps launch");
    }
    ce = S.fused ? launch_mp_first(A, S.W, st) : launch_mp_prep(A, st);
    if (ce != cudaSuccess) return cuda_error(ce, S.fused ? "mixed first-sweep launch" : "mixed prep launch");
    for (int s = 0; s < max_sweeps; s++) {
        const pcrp_status rc = enqueue_sweep(A, S, s, st);
        if (rc != PCRP_OK) return rc;
    }
    if (out) *out = A;
    return PCRP_OK;
}

}  // namespace pcrp

using namespace pcrp;

extern "C" pcrp_status pcrp_solve_mixed(const double* a, const double* b, const double* c, const double* d,
                                        const double* e, double* y, int64_t m, int64_t n, int32_t layout,
                                        double tol, int32_t max_sweeps, const pcrp_opts* opts, pcrp_stream stream,
                                        pcrp_mixed_info* info)
{
    const char* who = "pcrp_solve_mixed";
    NvtxRange nv(who);
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "%s: negative size", who);
    if (!valid_layout(layout)) return set_error(PCRP_EINVAL, "%s: bad layout %d", who, layout);
    if (info) std::memset(info, 0, sizeof *info);
    if (m == 0 || n == 0) { if (info) info->converged = 1; return PCRP_OK; }
    if (!b || !c || !d || !y) return set_error(PCRP_EINVAL, "%s: null array (only a and e may be null)", who);
    if (n > (int64_t(1) << 31) || m > (int64_t(1) << 24))
        return set_error(PCRP_EINVAL, "%s: size out of range (m <= 2^24, n <= 2^31)", who);
    if (!(tol > 0.0)) tol = 1e-12;
    if (max_sweeps <= 0) max_sweeps = 8;
    if (max_sweeps > 64) max_sweeps = 64;
    cudaStream_t st = (cudaStream_t)stream;

    const int64_t nb = (n + 1) / 2;
    const MpPlan pl = mp_plan(nb, opts);
    if (pl.npass > kMpMaxPasses) return set_error(PCRP_EINVAL, "%s: n too large for the pass plan", who);
    const MpLayout WL = mp_layout(m, n, max_sweeps, pl, info != nullptr);
    // Layout adapter: the window kernels walk along a system, which in the
    // interleaved layout means loads m doubles apart.  An interleaved batch
    // (m > 1) is transposed into contiguous copies in the workspace, solved
    // there, and the solution transposed back into y.
    const bool adapt = adapts(layout, m);
    const size_t arr = adapter_array_bytes(m, n);
    void* ws = nullptr;
    pcrp_status rc = get_workspace(opts, WL.total + (adapt ? 6 * arr : 0), st, &ws);
    if (rc != PCRP_OK) return rc;
    char* base = static_cast<char*>(ws);
    auto U = [&](size_t off) { return reinterpret_cast<unsigned*>(base + off); };
    cudaError_t ce;
    const double* src[6] = {a, b, c, d, e, y};
    double* cpy[6] = {};
    int64_t ss = layout == PCRP_LAYOUT_CONTIGUOUS ? n : 1, rs = layout == PCRP_LAYOUT_CONTIGUOUS ? 1 : m;
    if (adapt) {
        for (int k = 0; k < 6; k++)
            if (src[k]) cpy[k] = reinterpret_cast<double*>(base + WL.total + k * arr);
        ce = launch_transpose(src, cpy, 6, n, m, st);
        if (ce != cudaSuccess) return cuda_error(ce, "layout adapter (interleaved -> contiguous)");
        a = cpy[0]; b = cpy[1]; c = cpy[2]; d = cpy[3]; e = cpy[4];
        ss = n; rs = 1;
    }
    double* ys = adapt ? cpy[5] : y;             // the solver's y: the copy, or y itself
    MpArgs A{};
    // whole systems scatter x into the interleaved y from their final copy
    const MixedDest yd{y, 1, m};
    bool y_written = false;
    rc = mixed_enqueue(a, b, c, d, e, ys, m, n, ss, rs, tol, max_sweeps, opts, info != nullptr, ws, st, &A,
                       adapt ? &yd : nullptr, &y_written);
    if (rc != PCRP_OK) return rc;
    auto adapt_out = [&]() -> pcrp_status {
        if (!adapt || y_written) return PCRP_OK;
        const double* from[1] = {ys};
        double* to[1] = {y};
        cudaError_t te = launch_transpose(from, to, 1, m, n, st);
        return te == cudaSuccess ? PCRP_OK : cuda_error(te, "layout adapter (contiguous -> interleaved)");
    };

    if (!info) return adapt_out();

    // report: y still holds the rhs (the iterate was kept in X); final
    // residual r = y - A X, its norms, then X -> y
    double* rb = reinterpret_cast<double*>(base + WL.rbuf);
    unsigned* rn = U(WL.rn);
    ce = cudaMemsetAsync(rn, 0, 3 * m * sizeof(unsigned), st);
    if (ce != cudaSuccess) return cuda_error(ce, "cudaMemsetAsync");
    ce = launch_residual(a, b, c, d, e, ys, A.Xout, rb, m, n, A.ss, A.rs, n, 1, st);
    if (ce == cudaSuccess) ce = launch_resid_norm(a, b, c, d, e, A.Xout, rb, m, n, A.ss, A.rs, rn, rn + m, rn + 2 * m, st);
    if (ce == cudaSuccess) ce = launch_copy_out(A.Xout, ys, m, n, A.ss, A.rs, st);
    if (ce != cudaSuccess) return cuda_error(ce, "mixed report launch");
    rc = adapt_out();
    if (rc != PCRP_OK) return rc;
    std::vector<unsigned> norms(3 * m);
    ce = cudaMemcpyAsync(norms.data(), rn, 3 * m * sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (ce != cudaSuccess) return cuda_error(ce, "mixed report copy");
    std::vector<int> conv(m), sw(m);
    std::vector<float> est(m);
    ce = cudaMemcpyAsync(conv.data(), A.status, m * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(sw.data(), A.fin, m * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(est.data(), A.est, m * sizeof(float), cudaMemcpyDeviceToHost, st);
    int waits_gave_up = 0;
    if (ce == cudaSuccess && A.err)
        ce = cudaMemcpyAsync(&waits_gave_up, A.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_error(ce, "mixed report");
    if (waits_gave_up)
        return set_error(PCRP_ETIMEOUT, "%s: a staging wait of the fused first sweeps gave up (time limit)", who);
    int all = 1, maxsw = 0;
    float maxest = 0.0f;
    for (int64_t j = 0; j < m; j++) {
        all &= conv[j] == 1;
        maxsw = std::max(maxsw, sw[j]);
        maxest = std::max(maxest, est[j]);
    }
    info->sweeps = maxsw;
    info->converged = all;
    info->fwd_err_est = maxest;
    double worst = 0.0;
    for (int64_t j = 0; j < m; j++) {
        float rj, aj, xj;
        std::memcpy(&rj, &norms[j], 4); std::memcpy(&aj, &norms[m + j], 4); std::memcpy(&xj, &norms[2 * m + j], 4);
        const double den = (double)aj * (double)xj;
        const double v = den > 0.0 ? rj / den : (rj > 0.0f ? 1.0 : 0.0);
        worst = std::max(worst, v);
    }
    info->resid = worst;
    if (!all) return set_error(PCRP_ENOCONV, "%s: not every system reached tol=%g in %d sweeps", who, tol, max_sweeps);
    return PCRP_OK;
}

extern "C" pcrp_status pcrp_residual_f64(const double* a, const double* b, const double* c, const double* d,
                                         const double* e, const double* y, const double* x, double* r,
                                         int64_t m, int64_t n, int32_t layout, pcrp_stream stream)
{
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "pcrp_residual_f64: negative size");
    if (!valid_layout(layout)) return set_error(PCRP_EINVAL, "pcrp_residual_f64: bad layout %d", layout);
    if (m == 0 || n == 0) return PCRP_OK;
    if (!b || !c || !d || !y || !x || !r)
        return set_error(PCRP_EINVAL, "pcrp_residual_f64: null array (only a and e may be null)");
    if (r == x) return set_error(PCRP_EINVAL, "pcrp_residual_f64: r may not alias x");
    const int64_t ss = layout == PCRP_LAYOUT_CONTIGUOUS ? n : 1, rs = layout == PCRP_LAYOUT_CONTIGUOUS ? 1 : m;
    return cuda_error(launch_residual(a, b, c, d, e, y, x, r, m, n, ss, rs, ss, rs, (cudaStream_t)stream),
                      "pcrp_residual_f64 launch");
}
