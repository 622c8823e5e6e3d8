// pcrp_internal.h -- shared host/device definitions of the pcrp library.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include "pcrp.h"

namespace pcrp {

// NVTX range around an entry point (visible in Nsight timelines; no cost when
// no tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Six band/state arrays of a pentadiagonal batch: a b c d e y.  The faithful
// PCR state adds the two per-row multipliers that persist across strides
// (the reference keeps them in per-thread registers, kernel.cu:60).
enum { A_ = 0, B_ = 1, C_ = 2, D_ = 3, E_ = 4, Y_ = 5, AL1_ = 6, AL2_ = 7, NSTATE = 8 };

// Strides the reference runs on a system of n rows (main.cu:38-39, see the
// oracle for the derivation): log2(n) for powers of two, ceil(log2 n)-1
// otherwise; then the final pairwise/single step at delta = 2^strides.
__host__ __device__ inline int ref_strides(int64_t n) {
    if (n <= 1) return 0;
    int lg = 0;
    while ((int64_t(1) << lg) < n) lg++;
    if ((int64_t(1) << lg) == n) return lg;
    return lg - 1;
}

// One faithful global/shared pass over (sub)systems at decoupled level G.
// Element (system j, subsystem r, local row t) of an array lives at
//   (offsets ? offsets[j] : j*ss) + (r + t*G) * rs
// with (ss, rs) = (n, 1) for the contiguous layout and (1, m) interleaved;
// or, in a subsystem-major array of a uniform batch (src_sub / dst_sub), at
//   j*ss + r*(n/g) + min(r, n%g) + t
// where g is the array's gather stride (G for src, G*2^K for dst): every
// subsystem contiguous, so a pass reads its subsystem's rows in one run
// instead of G*8 bytes apart.
struct PcrPassArgs {
    const double* src[NSTATE];   // state in (A_/E_/AL1_/AL2_ may be null: zeros)
    double* dst[NSTATE];         // state out (non-final passes)
    double* x;                   // solution out (final pass)
    const int64_t* offsets;      // ragged first rows (nullable); ragged data is contiguous
    int64_t src_ss, src_rs;      // addressing of src
    int64_t dst_ss, dst_rs;      // addressing of dst and x
    int64_t n;                   // rows of each full system (uniform batch)
    int64_t m;                   // systems
    int64_t G;                   // gather stride = 2^(strides already done)
    int64_t nwin;                // windows per subsystem
    int K;                       // strides run by this pass (local deltas 1..2^(K-1))
    int final_step;              // 1: whole subsystem per CTA, finish and write x
    int L;                       // rows written per window (local)
    int H;                       // halo rows on each side (local), 2*(2^K-1)
    int TRmax;                   // shared-memory rows per CTA (>= L + 2H, or whole subsystem)
    int src_sub;                 // 1: src is subsystem-major at stride G (uniform batches)
    int dst_sub;                 // 1: dst is subsystem-major at stride G*2^K (uniform batches)
    int bulk;                    // 1: whole systems (G = 1, one tile) of even n in contiguous, 16-byte aligned
                                 // arrays: the tile is staged by bulk asynchronous copies (one per array)
};

// Passes whose longest stride reaches kZeroStride rows vote on the zero
// state: the outer coefficients of diagonally dominant systems underflow at
// strides ~2^8-2^10, and the vote (~10% of a dense stride) pays once two or
// more strides of the pass run in that state.  Others run without it, unless
// the batch is tridiagonal (a = e = 0 on entry): then every stride of every
// pass is in that state and every pass votes.  (Same bits either way.)
constexpr int64_t kZeroStride = 1024;
__host__ __device__ inline bool pass_votes(const PcrPassArgs& p, bool tridiagonal)
{
    return tridiagonal || (p.K > 0 && (p.G << (p.K - 1)) >= kZeroStride);
}


// Host-side launchers (pcr_f64.cu).  `tridiagonal`: the batch entered with
// a = e = 0, so every pass compiles in the zero-state vote.
cudaError_t launch_pcr_pass(const PcrPassArgs& p, int threads, cudaStream_t s, bool tridiagonal = false);
// dst[k] (cols x rows) = transpose of src[k] (rows x cols), both row-major,
// for up to 6 arrays in one launch; pairs with a null pointer are skipped
// (layout.cu): interleaved n x m <-> contiguous m x n batches
cudaError_t launch_transpose(const double* const* src, double* const* dst, int narr, int64_t rows, int64_t cols,
                             cudaStream_t s);
size_t pcr_pass_smem_bytes(int TRmax);
int pcr_max_smem_rows();


// Launch counter (capi.cpp), bumped by every kernel launch of the library.
void count_launch(int64_t k = 1);

// Error bookkeeping (capi.cpp).
pcrp_status set_error(pcrp_status st, const char* fmt, ...);
pcrp_status cuda_error(cudaError_t e, const char* where);

}  // namespace pcrp
