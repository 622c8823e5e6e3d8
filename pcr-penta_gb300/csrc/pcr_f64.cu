// pcr_f64.cu -- faithful FP64 PCR-Penta stride kernel for sm_103a.
//
// One kernel serves both reference paths:
//   * whole (sub)systems in shared memory, strides + final step, x written
//     (the reference's pcr_penta, kernel.cu:32-154, and its second stage
//     pcr_penta_splitting_2nd_stage, kernel.cu:665-791);
//   * windows with halos of a long system: K strides fused per global-memory
//     pass, state written to a scratch buffer (the reference's stage-1
//     splitting kernels, kernel.cu:158-659, which run one stride per tile
//     sweep and one CTA per system).
//
// After s strides the rows of a system that are congruent mod G = 2^s form
// independent subsystems (row i then couples i +- G, i +- 2G only), so every
// pass works on a subsystem: rows  base + r + t*G,  t = 0 .. n_r-1.  Stride
// tests such as "i - delta >= 0" are exact in local coordinates
// (t - delta' >= 0 with delta = G*delta'), so a pass at level G performs the
// same operations on the same values as the global stride would.
//
// Arithmetic.  Each stride forms the reference's Reductions I, II, III
// (kernel.cu:68-140) with every product, sum and IEEE quotient rounded on its
// own (__dmul_rn/__dadd_rn/__ddiv_rn: no FMA contraction), in the
// reference's order of evaluation.  The two neighbour combinations a row
// needs, R1(i) (rows i-2d, i-d, i) and R2(i) (rows i, i+d, i+2d), are the
// same combination T(m) centred on m = i-d and m = i+d, built from identical
// expressions (compare kernel.cu:77-79 with kernel.cu:103-105), so T(m) is
// formed once per row in phase A and shared through shared memory in
// phase B: 4 IEEE quotients per row and stride instead of the reference's 6,
// with bit-identical results.  The two of phase B divide by cT of the
// neighbours; phase A also stores cT's correctly rounded reciprocal
// (__drcp_rn), and phase B finishes each quotient with Markstein's
// correction (IBM J. Res. Dev. 34(1), 1990): q0 = RN(b r), the remainder
// b - cT q0 exact in one FMA, RN(q0 + rem r) = RN(b / cT) when no
// intermediate leaves the normal range, which an exponent guard ensures (other
// operands take the division).  A reciprocal and two corrections cost ~10.5
// DFMA slots against ~14.4 for two divisions; pcrp_check_quotients compares
// them with IEEE division on random operand classes.  The reference's multiplier registers, which
// outlive a stride and are reused when a Reduction-III pivot is exactly zero
// (kernel.cu:122,129), are kept per row in registers inside a pass and in
// two extra state arrays between passes.
//
// GB300 note: FP64 issues at ~0.5 lanes/clk per SM sub-partition on this
// part, so this kernel is bounded by the FP64 pipe, not HBM; the design goal
// is to keep that pipe busy (several CTAs per SM, 4 rows per thread for ILP)
// and to spend no FP64 operation beyond the reference's own arithmetic.
//
// Zero operands.  Operations whose result IEEE 754 fixes without rounding
// (a product with a zero factor: the zero of the factors' sign xor; a sum
// with a zero term: the other term, or -0 only if both are -0; a zero
// numerator over a finite nonzero divisor) are formed on the integer pipe,
// an FP64 operation costing ~40 integer operations of pipe time here and a
// division with a zero numerator ~2.6 normal ones.  They matter once the
// outer coefficients a, e of a diagonally dominant system have underflowed
// to zero (from stride ~2^8-2^10 on): in passes whose longest stride is at
// least 1024 rows a vote per stride tells whether every row of the tile is in
// that state (a = e = 0, the rest finite; passes of shorter strides are
// compiled without the vote and its cost); then phase
// A forms no FP64 value and phase B only its quotients and the products and
// sums whose operands are nonzero.  Same bits as the FP64 operations.
#include "pcr_tile.cuh"

namespace pcrp {
namespace {

// Three CTAs per SM where shared memory allows (tiles up to ~620 rows): the
// tile state fits 80 registers without spills up to 4 rows per thread, and
// the extra warps hide more of the FP64 latency; two for 8 rows per thread.
template <int RPT, bool kZero>
__global__ void __launch_bounds__(kMaxThreads, RPT >= 8 ? 2 : 3)
pcr_pass_kernel(const PcrPassArgs p)
{
    extern __shared__ double smem[];
    const int64_t blk  = blockIdx.x;
    const int64_t item = blk / p.nwin;
    const int64_t w    = blk - item * p.nwin;
    const int64_t j    = item / p.G;
    const int64_t r    = item - j * p.G;
    pcr_tile<RPT, false, kZero>(p, j, r, w, smem);
}


template <int RPT, bool kZero>
cudaError_t launch_rz(const PcrPassArgs& p, int threads, size_t smem, int64_t blocks, cudaStream_t s)
{
    // per-device attribute; cheap, and legal while a stream is being captured
    cudaError_t e = cudaFuncSetAttribute(pcr_pass_kernel<RPT, kZero>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         pcr_max_smem_rows() * kSmemArrays * (int)sizeof(double));
    if (e != cudaSuccess) return e;
    pcr_pass_kernel<RPT, kZero><<<(unsigned)blocks, threads, smem, s>>>(p);
    count_launch();
    return cudaGetLastError();
}

template <int RPT>
cudaError_t launch_rpt(const PcrPassArgs& p, bool tridiagonal, int threads, size_t smem, int64_t blocks,
                       cudaStream_t s)
{
    if (pass_votes(p, tridiagonal))
        return launch_rz<RPT, true>(p, threads, smem, blocks, s);
    return launch_rz<RPT, false>(p, threads, smem, blocks, s);
}

}  // namespace

int pcr_max_smem_rows() { return 1920; }   // 15 arrays * 1920 * 8 B = 225 KiB

size_t pcr_pass_smem_bytes(int TRmax) { return (size_t)TRmax * kSmemArrays * sizeof(double); }

cudaError_t launch_pcr_pass(const PcrPassArgs& p, int threads, cudaStream_t s, bool tridiagonal)
{
    if (threads <= 0 || threads > kMaxThreads) threads = kMaxThreads;
    threads = (threads + 31) / 32 * 32;
    if (p.TRmax < threads) threads = (p.TRmax + 31) / 32 * 32;   // small (sub)systems: no idle warps
    int rpt = (p.TRmax + threads - 1) / threads;
    while (rpt > 8 && threads < kMaxThreads) { threads += 32; rpt = (p.TRmax + threads - 1) / threads; }
    if (rpt > 8 || p.TRmax > pcr_max_smem_rows()) return cudaErrorInvalidValue;
    const int64_t blocks = p.m * p.G * p.nwin;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    const size_t smem = pcr_pass_smem_bytes(p.TRmax);
    if (rpt <= 1) return launch_rpt<1>(p, tridiagonal, threads, smem, blocks, s);
    if (rpt <= 2) return launch_rpt<2>(p, tridiagonal, threads, smem, blocks, s);
    if (rpt <= 4) return launch_rpt<4>(p, tridiagonal, threads, smem, blocks, s);
    return launch_rpt<8>(p, tridiagonal, threads, smem, blocks, s);
}

}  // namespace pcrp
