// mixed_internal.h -- argument blocks and launchers of the mixed-precision solver.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pcrp.h"

namespace pcrp {

constexpr int kMpTile = 512;       // rows per CTA of the refinement kernel (2 per thread)
constexpr int kMpMaxRows = 2048;   // block rows per CTA of the FP32 PCR kernel (40 bytes each)
constexpr int kMpMaxPasses = 24;   // global FP32 passes per solve
constexpr int kMpTryLevels = 5;    // levels of the windowed cyclic-reduction pass (halo 2^(K+1) rows)
constexpr int kMpTryRows = 1024;   // rows of one window tile of that pass

// Whole-batch arguments (prep and refinement kernels).
struct MpArgs {
    const double *a, *b, *c, *d, *e;   // caller bands, layout (ss, rs)
    double* y;                          // caller rhs in, solution out
    int64_t m, n, ss, rs;
    const longlong2* rg;                // ragged batch: system j is rows rg[j].x .. rg[j].x + rg[j].y - 1 of
                                        // the caller arrays (row stride 1) and rows rg[j].y .. n-1 are identity
                                        // padding (zero rhs, zero couplings) that is neither read nor written
                                        // there; null: uniform batch addressed by (ss, rs)
    float4* S0;                         // level-0 normalised L,U: [2*q] = L, [2*q+1] = U, q < m*nb
    float2* R[2];                       // normalised rhs Y of block row q: sweep s reads R[s & 1]
    float4* Mi;                         // inverse of the row-scaled FP32 diagonal block of block row q
    float* dx;                          // FP32 correction, m*n (contiguous)
    double* X0;                         // x_0, m*n contiguous (sweep 0 of a multi-sweep solve)
    double* Xout;                       // iterates when the caller asked for a report (keep_x), else y
    double* Yc;                         // copy of the rhs, m*n contiguous (y may hold the iterate)
    const double* xsrc;                 // this sweep's x_{s-1} (null in sweep 0) ...
    int64_t xsrc_ss, xsrc_rs;           //   ... and its system / row strides
    const longlong2* xsrc_rg;           //   ... or its ragged rows (rg, when xsrc is the output)
    double* xdst;                       // this sweep's x_s ...
    int64_t xdst_ss, xdst_rs;
    const longlong2* xdst_rg;
    double* xout;                       // the output iterate (y or Xout) and its strides: x_s of sweeps >= 1
    int64_t oss, ors;
    int* ctr;                           // device sweep counter (graph-driven sweeps), or null: `sweep` and the
                                        // per-sweep fields above are set by the host for each launch
    unsigned* ndx;                      // [(max_sweeps+1) x m] max |dx| per sweep (float bits)
    unsigned* nx;                       // [(max_sweeps+1) x m] max |x| per sweep
    int* fin;                           // per system: 0 running, else the sweep it finished in, plus 1
    int* status;                        // per system: 1 converged, 2 stopped at max_sweeps
    float* est;                         // per system: estimated relative forward error
    unsigned* trunc;                    // [kMpMaxPasses x m] max |L|,|U| after each global pass
    unsigned* ndx_pre;                  // [max_sweeps x kMpMaxPasses x m] max |dx| written early by a global pass
    int* live;                          // [max_sweeps + 1] systems still running at the start of each sweep
    int* fail;                          // [m] 1: the windowed cyclic-reduction pass leaves the system coupled
    int* nfail;                         // systems with fail set
    unsigned* dnorm;                    // [2 x m] fused first two sweeps: max |dx_0| (= max |x_0|), max |dx_1|
    int* err;                           // nonzero: a bounded wait of the fused kernel gave up (null: no fused pass)
    int inject;                         // test hook: the fused kernel never stages its first chunk
    int sweep, max_sweeps, keep_x;
    int vec;                            // 1: all six caller arrays are 16-byte aligned (paired loads allowed)
    int first_fused;                    // sweep 0 ran as mp_first_kernel (the refinement of sweep 0 only
                                        // takes the systems it left to the general passes)
    int cr_mode;                        // a cyclic-reduction pass updates x of the systems it solves
    float tol;
};

// One FP32 block-PCR pass.
struct MpPassArgs {
    const float4* srcLU;                // [2*q] = L, [2*q+1] = U of block row q
    const float2* srcY;
    float4* dstLU;
    float2* dstY;
    float* dx;
    const int* fin;                     // systems with fin != 0 are finished: skip them
    unsigned* ndx;                      // final pass: max |dx| of this sweep
    const unsigned* trunc_in;           // previous pass's max |L|,|U| (or null)
    unsigned* trunc_out;                // this pass's max |L|,|U| (non-final)
    const unsigned* ndx_pre_in;         // max |dx| the previous pass wrote for decoupled windows (or null)
    unsigned* ndx_pre_out;              // same, written by this pass (non-final)
    const int* live;                    // systems still running in this sweep (0: the kernel returns at once)
    int* fail;                          // per system: the windowed cyclic-reduction pass did not decouple it
                                        // (null: no such pass; general passes then run for every system)
    int* nfail;                         // number of systems with fail set
    const double* xsrc;                 // cyclic-reduction passes: x_{s-1} (null in sweep 0) ...
    int64_t xsrc_ss, xsrc_rs;
    const longlong2* xsrc_rg;
    double* xdst;                       //   ... and x_s = x_{s-1} + dx_s (null: write dx instead)
    int64_t xdst_ss, xdst_rs;
    const longlong2* xdst_rg;
    unsigned* nx;                       //   ... and max |x_s|
    // Graph-driven sweeps: the fields above that change from sweep to sweep
    // (sweep, live, srcY at level 0, ndx_pre_in/out, xsrc, xdst, nx) are
    // derived on the device from the sweep counter and these:
    const int* ctr;                     // device sweep counter, or null (host-set fields)
    const int* live0;
    const float2* R0;                   // level-0 passes: rhs of even / odd sweeps
    const float2* R1;
    unsigned* pre0;                     // ndx_pre base
    unsigned* nx0;                      // nx base (cyclic-reduction pass)
    const double* X0;
    double* xout;
    int64_t oss, ors;
    const longlong2* rg;                // ragged output rows (see MpArgs::rg)
    int pass, max_sweeps, level0, skip0;   // skip0: sweep 0 belongs to the fused kernel
    int64_t m, n, nb, G, nwin;
    int K, final_step, L, H, TRmax, sweep;
};

// Programmatic dependent launch: a kernel of the mixed solver may be
// launched while its predecessor in the stream is still running; it waits
// (griddepcontrol.wait) for the predecessor to complete and its writes to be
// visible before touching memory.  Hides the launch gap between the many
// short dependent kernels of a solve.
template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                             Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// Window geometry of the windowed passes (level 0).
struct MpWindows {
    int64_t nwin;                       // windows per system
    int L, H, K, TRmax;                 // core rows, halo rows each side, levels (31: whole system), tile rows
};

// Window geometry of the fused first two sweeps (mixed_duo.cu), in block
// rows: core windows of L rows; sweep 1 needs the level-0 rows within R of
// the core (R = 2^(K+1) - 2 for K truncation levels), hence x_0 within R + 1
// and so a tile halo of H >= 2R + 1 for sweep 0.
struct DuoGeom {
    int64_t nb, nwin;
    int L, H, R, K;
};

// Where a solve that runs as one whole-system launch writes x when that is
// not its y (the caller's interleaved y behind the layout adapter): the
// kernel's final copy scatters x there, which takes the place of the
// transpose back.
struct MixedDest {
    double* x;
    int64_t ss, rs;                     // system / row strides of x
};

// Enqueues a uniform batch on `st` (mixed_host.cpp).  With `dest`, a solve of
// whole systems that keeps no report writes x to *dest and sets
// *dest_written; any other solve ignores it.
// With `rg` (device array of m (offset, rows) pairs, every rows <= n), the
// batch is m ragged systems of the caller arrays solved as n-row systems
// (see MpArgs::rg); ss and rs are then ignored.
pcrp_status mixed_enqueue(const double* a, const double* b, const double* c, const double* d, const double* e,
                          double* y, int64_t m, int64_t n, int64_t ss, int64_t rs, double tol, int max_sweeps,
                          const pcrp_opts* opts, bool keep_x, void* ws, cudaStream_t st, MpArgs* out,
                          const MixedDest* dest = nullptr, bool* dest_written = nullptr,
                          const longlong2* rg = nullptr);

cudaError_t launch_mp_init(const MpArgs& p, cudaStream_t s);
cudaError_t launch_mp_first(const MpArgs& p, const MpWindows& g, cudaStream_t s);
cudaError_t launch_mp_prep(const MpArgs& p, cudaStream_t s);
cudaError_t launch_mp_pass(const MpPassArgs& p, cudaStream_t s);
cudaError_t launch_mp_small(const MpArgs& p, cudaStream_t s);   // whole systems, every sweep in one CTA
cudaError_t launch_mp_try(const MpPassArgs& p, cudaStream_t s);
cudaError_t launch_mp_xupdate(const MpArgs& p, cudaStream_t s);
cudaError_t launch_mp_decide(const MpArgs& p, cudaStream_t s);
cudaError_t launch_mp_residual(const MpArgs& p, cudaStream_t s);
cudaError_t launch_mp_advance(const MpArgs& p, cudaGraphConditionalHandle h, cudaStream_t s);
// Fused sweeps 0 and 1 (mixed_duo.cu): whether a batch qualifies and its
// window geometry, the kernel, the decide-and-copy kernel that finishes the
// systems it converged, and the gate that opens the general sweep loop
// (graph while node) only if some system is left.
bool duo_plan(const MpArgs& p, int levels, DuoGeom* g);
cudaError_t launch_mp_duo(const MpArgs& p, const DuoGeom& g, cudaStream_t s);
cudaError_t launch_mp_duo_finish(const MpArgs& p, cudaStream_t s);
cudaError_t launch_mp_gate(const MpArgs& p, cudaGraphConditionalHandle h, cudaStream_t s);
cudaError_t launch_residual(const double* a, const double* b, const double* c, const double* d, const double* e,
                            const double* y, const double* x, double* r, int64_t m, int64_t n, int64_t ss,
                            int64_t rs, int64_t xss, int64_t xrs, cudaStream_t s);
cudaError_t launch_copy_out(const double* X, double* y, int64_t m, int64_t n, int64_t ss, int64_t rs, cudaStream_t s);
cudaError_t launch_resid_norm(const double* a, const double* b, const double* c, const double* d, const double* e,
                              const double* X, const double* r, int64_t m, int64_t n, int64_t ss,
                              int64_t rs, unsigned* rn, unsigned* an, unsigned* xn, cudaStream_t s);

}  // namespace pcrp
