/*
 * pcrp.h -- C ABI of the GB300 (sm_103a) batched pentadiagonal PCR solver.
 *
 * A batch holds m independent systems of n rows.  Row i of a system reads
 *
 *     a_i x_{i-2} + b_i x_{i-1} + c_i x_i + d_i x_{i+1} + e_i x_{i+2} = y_i
 *
 * (PCR-Penta kernel.cu:77-79; Annexure A p.1).  Out-of-range band slots
 * (a_0, a_1, b_0, d_{n-1}, e_{n-2}, e_{n-1}) are never read as coefficients,
 * whatever they hold.
 *
 * Batch layouts (pcrp_layout):
 *   PCRP_LAYOUT_CONTIGUOUS   element (system j, row i) at j*n + i -- the
 *                            reference's own layout (kernel.cu:43,187,354,551).
 *   PCRP_LAYOUT_INTERLEAVED  element (j, i) at i*m + j -- the interleaved batch
 *                            format of Annexure A p.2 (cuSPARSE gpsv style).
 *
 * Conventions shared by every solve entry point:
 *   - a, b, c, d, e, y are caller-owned DEVICE pointers of m*n doubles.
 *     The bands are const: unlike the reference, which overwrites all six
 *     arrays on its n > 1024 path (kernel.cu:516-518,649-651), nothing but y is
 *     written.  y holds the right-hand side on entry and the solution on return.
 *   - Work is enqueued on `stream` (NULL = legacy default stream) and the call
 *     returns without synchronising, except where a function says otherwise.
 *   - Scratch comes from opts->workspace when given (see pcrp_workspace_size),
 *     else from a library-owned, per-device cache that grows on demand.
 *   - Errors are returned as pcrp_status; the library never exits or aborts
 *     (the reference's checkCuda() calls exit(), performanalysis.h:12-20).
 *     pcrp_get_last_error_string() describes the last failure of the calling
 *     thread.
 *   - Any n >= 1 and any m >= 0 (m = 0 or n = 0 is a no-op); 64-bit indexing.
 */
#ifndef PCRP_H
#define PCRP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t (struct CUstream_st *); NULL is the default stream. */
struct CUstream_st;
typedef struct CUstream_st* pcrp_stream;

typedef enum pcrp_status {
    PCRP_OK = 0,
    PCRP_EINVAL = 1,   /* bad argument (null pointer, negative size, n outside the path's range, bad layout) */
    PCRP_ECUDA = 2,    /* a CUDA runtime call or kernel launch failed                                    */
    PCRP_ENOMEM = 3,   /* scratch allocation failed, or opts->workspace is smaller than required          */
    PCRP_ETIMEOUT = 4, /* a bounded device-side wait gave up (persistent ragged kernel, or a staging wait
                          of the mixed solver's fused first sweeps; that solve still completes)           */
    PCRP_ENOCONV = 5,  /* iterative refinement did not reach tol within max_sweeps                        */
    PCRP_ENOTSUP = 6   /* unsupported combination of options                                              */
} pcrp_status;

typedef enum pcrp_layout {
    PCRP_LAYOUT_CONTIGUOUS = 0,
    PCRP_LAYOUT_INTERLEAVED = 1
} pcrp_layout;

/* Options; pass NULL for all defaults.  `size` must be sizeof(pcrp_opts).
 * Zero in any tuning field means "use the autotuned default". */
typedef struct pcrp_opts {
    uint32_t size;
    int32_t  smem_rows;        /* largest (sub)system solved whole in shared memory        */
    int32_t  fuse_strides;     /* PCR strides fused per global-memory pass (n > smem_rows)   */
    int32_t  tile_rows;        /* rows written per CTA in a global pass                      */
    int32_t  threads;          /* threads per CTA                                            */
    int32_t  reserved0;        /* 0; 0x7E57 makes pcrp_solve_ragged's first dependency wait,
                                  and the first staging wait of pcrp_solve_mixed's fused
                                  first sweeps, unsatisfiable (bounded, ~4 ms) to test
                                  PCRP_ETIMEOUT                                              */
    void*    workspace;        /* caller-provided device scratch, or NULL                    */
    size_t   workspace_bytes;
    int32_t  window_levels;    /* pcrp_solve_mixed, systems larger than one shared-memory
                                  tile: cyclic-reduction levels of the windowed first pass
                                  (0: 5; negative: no windowed pass, block-PCR passes only) */
} pcrp_opts;

/* Per-call report of the mixed-precision solver (host memory). */
typedef struct pcrp_mixed_info {
    int32_t sweeps;       /* refinement sweeps run (max over systems)                        */
    int32_t converged;    /* 1 if every system met tol                                        */
    double  fwd_err_est;  /* max over systems of the estimated relative forward error         */
    double  resid;        /* max over systems of ||y - A x||_inf / (||A||_inf ||x||_inf)       */
} pcrp_mixed_info;

/* ------------------------------------------------------------------------ */
/* Plain FP64 PCR-Penta (the drop-in)                                       */
/* ------------------------------------------------------------------------ */

/* Solves the batch with the reference's PCR-Penta stride arithmetic in FP64:
 * log2(n) strides for power-of-two n (ceil(log2 n)-1 strides and a pairwise
 * 2x2 finish otherwise), then x = y/c.  Every product, sum and IEEE quotient
 * is the one the reference forms, in the same order, without FMA contraction,
 * so the result is bit-identical to the reference kernels built with
 * -fmad=false.  Takes the place of the reference host code's dispatch
 * (main.cu:46-87: n <= 1024 -> pcr_penta, otherwise the splitting kernels),
 * with the split point from the tuned plan instead of n = 1024: systems of
 * at most the plan's shared-memory rows (opts->smem_rows; 512 tuned on
 * GB300) are solved whole in shared memory, longer ones by global passes
 * and the shared-memory finish -- the same bits either way.
 * pcrp_solve_f64_small and pcrp_solve_f64_split keep the reference's own
 * n = 1024 split.
 * `a` and `e` may be NULL: that band is +0.0 and is not read; with both NULL
 * (a tridiagonal batch) every stride runs the kernels' zero-operand form, with
 * the bits of explicit +0.0 bands.  The same holds for the two paths below,
 * pcrp_solve_f64_noalloc and pcrp_solve_host.
 * Replaces: main.cu:46-87 (time_* dispatch around pcr_penta and the splitting
 * kernels), kernel prototypes performanalysis.h:53-59. */
pcrp_status pcrp_solve_f64(const double* a, const double* b, const double* c,
                           const double* d, const double* e, double* y,
                           int64_t m, int64_t n, int32_t layout,
                           const pcrp_opts* opts, pcrp_stream stream);

/* The n <= 1024 path: one system per CTA group, solved whole in shared memory.
 * Returns PCRP_EINVAL for n > 1024.
 * Replaces: pcr_penta, kernel.cu:32-154 (launch main.cu:49). */
pcrp_status pcrp_solve_f64_small(const double* a, const double* b, const double* c,
                                 const double* d, const double* e, double* y,
                                 int64_t m, int64_t n, int32_t layout,
                                 const pcrp_opts* opts, pcrp_stream stream);

/* The n > 1024 path: global-memory passes that fuse several PCR strides each
 * until every system has split into interleaved subsystems of at most
 * opts->smem_rows rows, then a shared-memory finish on those subsystems.
 * Returns PCRP_EINVAL for n <= 1024.
 * Replaces: the stage-1 splitting kernels kernel.cu:158-659 (launch
 * main.cu:60,136,208) and pcr_penta_splitting_2nd_stage kernel.cu:665-791
 * (launch main.cu:73,147,219). */
pcrp_status pcrp_solve_f64_split(const double* a, const double* b, const double* c,
                                 const double* d, const double* e, double* y,
                                 int64_t m, int64_t n, int32_t layout,
                                 const pcrp_opts* opts, pcrp_stream stream);

/* The pcrp_solve_f64 solve for callers that must not allocate device memory
 * (host callbacks and plugin hooks that may not enter the CUDA allocator,
 * hosts whose GPU memory is fixed at start-up).  Its scratch is a 64 MiB
 * array compiled into the library, which every GPU that loads the library
 * keeps until the process exits.  Systems that fit the shared-memory tile
 * (n <= 512 with the tuned plan) need no scratch and any batch of them is
 * accepted; longer systems need 128 bytes of scratch per unknown, so a call
 * of those accepts at most m*n <= 524288 unknowns and returns PCRP_EINVAL,
 * with the limit in the error text, for more.  It calls no allocator.  The first call on a device looks up
 * the array's device address, so make one call per device before any stream
 * capture.  Calls share the array: calls whose GPU work overlaps in time race
 * on it, so order them on one stream.  Results are bit-identical to
 * pcrp_solve_f64.  No counterpart in the reference. */
pcrp_status pcrp_solve_f64_noalloc(const double* a, const double* b, const double* c,
                                   const double* d, const double* e, double* y,
                                   int64_t m, int64_t n, int32_t layout, pcrp_stream stream);

/* ------------------------------------------------------------------------ */
/* Mixed precision: FP32 PCR + FP64 iterative refinement                    */
/* ------------------------------------------------------------------------ */

/* Row-scales every system by its main diagonal, solves it in FP32 by 2x2-
 * block reduction on the CUDA cores (cyclic reduction of whole systems or of
 * decoupling windows, block PCR otherwise), and refines in FP64: r = y - A x
 * (fused FP64 pentadiagonal matvec), solve for the correction in FP32,
 * x += dx in FP64, until the estimated relative forward error is <= tol or
 * max_sweeps sweeps have run (tol <= 0: 1e-12; max_sweeps <= 0: 8).  `a` and
 * `e` may be NULL: that band is zero and neither read nor multiplied (NULL for
 * both: a tridiagonal batch, a third less band traffic).  If `info` is
 * non-NULL the call synchronises `stream` and fills it; if `info` is NULL the
 * call is asynchronous and never reports PCRP_ENOCONV.  From the second
 * asynchronous call with the same arguments and workspace the sweeps run as
 * a CUDA graph whose while node stops at convergence (environment variable
 * PCRP_NO_GRAPH: always host-driven launches).  An interleaved batch of more
 * than one system is transposed into contiguous copies in the workspace,
 * solved there and transposed back (same result bits as the contiguous solve;
 * pcrp_workspace_size counts the copies).  Systems longer than one shared-
 * memory tile (n > 4096), of even n with 16-byte aligned arrays, can run
 * their first two sweeps in one fused pass over the inputs (windows with
 * halos, inputs staged by bulk asynchronous copies, the tile's factorisation
 * kept in tensor memory; environment variable PCRP_DUO=1, off by default);
 * systems that pass need no other kernel, the rest are solved from the start
 * by the general kernels.
 * No counterpart in the reference (new work named by the solver's design). */
pcrp_status pcrp_solve_mixed(const double* a, const double* b, const double* c,
                             const double* d, const double* e, double* y,
                             int64_t m, int64_t n, int32_t layout,
                             double tol, int32_t max_sweeps,
                             const pcrp_opts* opts, pcrp_stream stream,
                             pcrp_mixed_info* info);

/* r = y - A x in FP64 for every system (fused pentadiagonal matvec).  x, y and
 * r are device arrays of m*n doubles in `layout`; r may not alias x; `a` and
 * `e` may be NULL (zero bands).
 * No counterpart in the reference. */
pcrp_status pcrp_residual_f64(const double* a, const double* b, const double* c,
                              const double* d, const double* e, const double* y,
                              const double* x, double* r,
                              int64_t m, int64_t n, int32_t layout, pcrp_stream stream);

/* Solves a batch that lives in HOST memory: a..e and y are host arrays of
 * m*n doubles (page-locked memory lets the copies run asynchronously; a
 * NULL `a` or `e` is a zero band and is not copied).  The
 * systems are streamed through the GPU in chunks on two internal streams, so
 * the host<->device copies of one chunk overlap the solve of another; y
 * receives the solution.  precision 0 = pcrp_solve_f64 (bit-identical
 * results), 1 = pcrp_solve_mixed (tol, max_sweeps as there; no report).
 * Asynchronous on `stream`: the host arrays must stay valid until the stream
 * reaches the end of the call.  Chunks grow from ceil(m/32) systems threefold
 * up to ceil(m/4) (at most 2^26 unknowns).  opts->workspace, if given, holds
 * the staging chunks: 2 x 6 x (largest chunk) x n doubles.  No counterpart in the reference (its host
 * code never moves data; this is the path of a caller whose batch is on the host). */
pcrp_status pcrp_solve_host(const double* a, const double* b, const double* c,
                            const double* d, const double* e, double* y,
                            int64_t m, int64_t n, int32_t layout,
                            int32_t precision, double tol, int32_t max_sweeps,
                            const pcrp_opts* opts, pcrp_stream stream);

/* ------------------------------------------------------------------------ */
/* Ragged batches                                                           */
/* ------------------------------------------------------------------------ */

/* Solves nsys systems of uneven size in one persistent kernel.  System k
 * occupies rows offsets[k] .. offsets[k+1]-1 of the six arrays (contiguous);
 * `offsets` is a DEVICE array of nsys+1 int64 values with offsets[0] = 0.
 * `a` and `e` may be NULL (zero bands, not read).
 * mode 0 = FP64 PCR-Penta (bit-identical to pcrp_solve_f64 on each system):
 * a device-side work queue bins the systems; those of at most
 * opts->smem_rows rows are solved whole in shared memory, larger ones are
 * split by global-memory stride passes first.  mode 1 = mixed precision
 * (tol, max_sweeps as in pcrp_solve_mixed): systems are grouped into size
 * classes a quarter octave apart, each solved in place as a uniform batch
 * padded (in the workspace only) with identity rows; PCRP_ENOCONV if a
 * system misses tol.  Queue waits are bounded; a wait
 * that gives up makes the call return PCRP_ETIMEOUT (reported only when the
 * call synchronises, i.e. always for this entry point).  The launch sequence
 * has a fixed shape for a given (nsys, max rows) and is replayed from a cached
 * CUDA graph.  No counterpart in the reference. */
pcrp_status pcrp_solve_ragged(const double* a, const double* b, const double* c,
                              const double* d, const double* e, double* y,
                              const int64_t* offsets, int64_t nsys, int64_t max_rows,
                              int32_t mode, double tol, int32_t max_sweeps,
                              const pcrp_opts* opts, pcrp_stream stream);

/* ------------------------------------------------------------------------ */
/* Workspace, errors, version                                               */
/* ------------------------------------------------------------------------ */

/* which: 0 = pcrp_solve_f64 family, 1 = pcrp_solve_mixed, 2 = pcrp_solve_ragged
 * (n = max_rows, m = nsys, and `total_rows` is taken as m*n as an upper bound). */
pcrp_status pcrp_workspace_size(int64_t m, int64_t n, int32_t layout, int32_t which,
                                const pcrp_opts* opts, size_t* bytes);

/* Frees the library-owned scratch of every device (call with the GPU idle). */
pcrp_status pcrp_release_workspace(void);

/* Text of the last error raised on the calling thread ("" if none). */
const char* pcrp_get_last_error_string(void);

/* MAJOR*10000 + MINOR*100 + PATCH. */
int32_t pcrp_version(void);

/* Kernels this library has launched in the calling process (all devices);
 * a diagnostic for benchmarks.  No counterpart in the reference. */
int64_t pcrp_kernel_launches(void);

/* Measures this GPU's FP64 issue rates with two throughput kernels on
 * `stream` (synchronous, ~a millisecond): independent DFMA chains, and
 * independent IEEE divisions (__ddiv_rn).  Rates in operations per second.
 * The roofline of the bit-faithful FP64 path is its FP64 instruction count
 * over these rates; a diagnostic for benchmarks, no counterpart in the
 * reference. */
pcrp_status pcrp_measure_fp64(double* dfma_per_s, double* ddiv_per_s, pcrp_stream stream);

/* Pipe sharing on this GPU (synchronous, a few milliseconds): one launch of
 * four CTAs per SM whose even warps run FP64 FMA chains and odd warps FP32
 * FMA or integer chains, timed with CUDA events in five forms: ms[0] FP64
 * alone, ms[1] FP32 alone, ms[2] integer alone, ms[3] FP64 + FP32, ms[4]
 * FP64 + integer.  A pair that shares a pipe takes about the sum of its
 * parts, one that does not about the longer part.  A diagnostic behind the
 * design of the mixed-precision kernels; no counterpart in the reference. */
pcrp_status pcrp_measure_pipes(float* ms, pcrp_stream stream);

/* Checks the FP64 kernels' phase-B quotient (Markstein's correction from the
 * correctly rounded reciprocal, inside its exponent guard) against IEEE
 * division (__ddiv_rn) on `samples` seeded random operand pairs of class
 * `mode` (0: exponents within 2^+-32, 1: the guard's whole range, 2: mantissas
 * near all ones, 3: near powers of two, 4: any exponent, zeros, subnormals,
 * inf and NaN included).  Synchronous.  *mismatches counts results whose bits
 * differ (any NaN matches any NaN), *markstein the pairs inside the guard.  A
 * diagnostic; no counterpart in the reference. */
pcrp_status pcrp_check_quotients(int32_t mode, uint64_t seed, int64_t samples, uint64_t* mismatches,
                                 uint64_t* markstein, pcrp_stream stream);

/* ------------------------------------------------------------------------ */
/* Seeded input generators (host memory, threads over systems)              */
/* ------------------------------------------------------------------------ */

/* kind:
 *   PCRP_GEN_DOMINANT  off-diagonals U[-1,1], c = sum|off| + U[1,2], y U[-1,1]
 *   PCRP_GEN_ADI       (I - theta*dt*L) of a convection-diffusion operator on
 *                      S in [0,800]; v ~ U[0.01,1] per system, r=0.03,
 *                      dt=1e-3, theta=0.5; y = max(S-K,0), K ~ U[50,150]
 *   PCRP_GEN_WEAK      off-diagonals U[-1,1], c = +-1.05*sum|off| (random sign)
 *   PCRP_GEN_TOEPLITZ  the reference's fixture (kernel.cu:5-26): rows
 *                      (1,-4,6,-4,1), c_0 = c_{n-1} = 5, b_0 = d_{n-1} = 1, y = 1
 * Values are a pure function of (seed, kind, system, row), so any m/n slice
 * regenerates identically.  Out-of-range band slots are written as 0 (the
 * TOEPLITZ fixture keeps the reference's b_0 = d_{n-1} = 1).  nthreads <= 0
 * uses every host core. */
enum { PCRP_GEN_DOMINANT = 0, PCRP_GEN_ADI = 1, PCRP_GEN_WEAK = 2, PCRP_GEN_TOEPLITZ = 3 };

pcrp_status pcrp_generate(int32_t kind, uint64_t seed, int64_t m, int64_t n, int32_t layout,
                          double* a, double* b, double* c, double* d, double* e, double* y,
                          int32_t nthreads);

/* Same values written by a kernel into DEVICE arrays on `stream`. */
pcrp_status pcrp_generate_device(int32_t kind, uint64_t seed, int64_t m, int64_t n, int32_t layout,
                                 double* a, double* b, double* c, double* d, double* e, double* y,
                                 pcrp_stream stream);

/* Ragged generator: sizes_out[k] = round(nmin * (nmax/nmin)^u_k), u_k ~ U[0,1)
 * seeded; host memory. */
pcrp_status pcrp_ragged_sizes(uint64_t seed, int64_t nsys, int64_t nmin, int64_t nmax,
                              int64_t* sizes_out);

/* Fills ragged systems (contiguous at offsets[k], nsys+1 host offsets). */
pcrp_status pcrp_generate_ragged(int32_t kind, uint64_t seed, const int64_t* offsets, int64_t nsys,
                                 double* a, double* b, double* c, double* d, double* e, double* y,
                                 int32_t nthreads);

#ifdef __cplusplus
}
#endif

#endif /* PCRP_H */
