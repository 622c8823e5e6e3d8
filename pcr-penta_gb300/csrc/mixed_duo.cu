// mixed_duo.cu -- the first two refinement sweeps of the mixed-precision
// solver fused into one pass over the FP64 inputs, for systems longer than
// one shared-memory tile.
//
// Per window of L block rows (a tile of the window plus H block rows each
// side, 1024 block rows in all), one CTA:
//  1. stages the tile's FP64 bands and right-hand side in chunks through a
//     ring of shared-memory slots filled by bulk asynchronous copies
//     (cp.async.bulk, completion on an mbarrier), row-scales them by the
//     power of two of each main diagonal and forms the normalised FP32 2x2
//     block rows in the cyclic-reduction tile;
//  2. sweep 0: truncated block cyclic reduction and back substitution give
//     x_0 (= dx_0) on the window and R + 1 block rows either side.  The
//     reduction keeps, for every row it eliminates into (one per thread and
//     level), that row's couplings and the inverse of its new diagonal block
//     in tensor memory (TMEM, tcgen05.st): the factorisation of the tile;
//  3. reads the bands again, from L2 (the bulk copies asked L2 to keep them),
//     each thread its own rows with a chunk of loads in flight ahead, for the
//     rows within R of the window: r_0 = y - A x_0 in FP64 (5 DFMA per row),
//     row-scaled and normalised (by the row's part of the diagonal-block
//     inverse, also kept in TMEM) into the tile's rhs; further rows get a
//     zero rhs (no row of the window depends on them);
//  4. sweep 1 replays the factorisation on the rhs only (the right-hand-side
//     update of each level, from TMEM) and back-substitutes with the blocks
//     left in place by sweep 0: dx_1; x_1 = x_0 + dx_1 (FP64) is written to
//     the workspace copy X0.
// The ring holds only the first read: once a tile is staged, the copies of
// the next tile's first chunks are in flight while the CTA reduces.  The
// FP64 inputs cross HBM once (the second read hits L2) and the only other
// traffic is x_1 (8 B per row) and its copy into y by mp_duo_finish_kernel,
// for the systems whose stopping rule is met after sweep 1 -- every system
// of the diagonally dominant and weakly dominant batches.  A system whose
// windows do not decouple within K levels, or that needs more sweeps, is
// left (fin = 0) to the general kernels of mixed.cu, which solve it from the
// start.
//
// Why the halos: after l levels a reduced row depends on the level-0 rows
// within 2^(l+1) - 1 of it, so with the check region of cr_reduce the rows
// of a region are exact (up to the truncation) when the tile covers the
// region widened by R = 2^(K+1) - 2.  Sweep 1 needs r_0 on the window
// widened by R, r_0 needs x_0 one block row further, and x_0 is exact where
// sweep 0's check region (the window widened by R + 1) lies R inside the
// tile: H = 2R + 1 suffices; H = 2^(K+2) is used.
//
// FP32 conversion: the first read converts the bands and y with a
// truncating integer conversion (6 integer operations; values below FP32's
// normal range flush to zero, and a value whose scaled exponent overflows,
// possible only for rows that are not diagonally dominant or hold inf/NaN,
// becomes some finite value: the FP64 residual then carries the inf/NaN or
// the refinement does not converge, and the stopping rule reports it).  The
// residual's conversion rounds to nearest and keeps inf/NaN (d2f_scaled).
//
// TMEM: each CTA allocates 256 columns (two CTAs per SM hold all 512) at
// its start and frees them on every way out.  A warp reaches the 32 TMEM
// lanes of its quarter (warp % 4); warp groups w / 4 = 0..3 take disjoint
// column ranges sized by the levels their threads can eliminate into (a
// thread t does so at level l only if t < 512 >> l).
//
// Failure detection: every wait on a slot's mbarrier gives up after a time
// limit (2 s; 4 ms under the test hook that never stages the first chunk),
// sets p.err, waits (again bounded) for the copies still in flight, frees
// its TMEM and returns.  The finishing kernel then leaves every system to
// the general kernels, so the solve still completes, and pcrp_solve_mixed
// reports PCRP_ETIMEOUT when asked for a report.
#include <algorithm>
#include <cstdlib>

#include "pcrp_internal.h"
#include "mixed_internal.h"
#include "mixed_dev.cuh"
#include "tma.cuh"

namespace pcrp {
namespace {

using namespace tma;

constexpr int kDuoThreads = 512;                       // threads per CTA
constexpr int kDuoRows = 1024;                         // block rows of a tile (two per thread at level 0)
constexpr int kDuoChunk = kDuoThreads / 2;             // block rows per staged chunk (two threads per block row)
constexpr int kDuoSlots = 2;                           // staged chunks in flight
constexpr int kDuoArrays = 6;                          // a b c d e y
constexpr int kDuoSlotDoubles = kDuoArrays * 2 * kDuoChunk;
constexpr int kDuoMaxChunks = kDuoRows / kDuoChunk;
constexpr int kDuoMaxLevels = 6;
constexpr size_t kDuoSmem = (size_t)kDuoSlots * kDuoSlotDoubles * sizeof(double)   // staging ring
                            + (size_t)kDuoRows * sizeof(double2)                     // x_0
                            + (size_t)kDuoRows * (2 * sizeof(float4) + sizeof(float2));   // reduction tile
static_assert(kDuoRows % 8 == 0 && kDuoRows == 2 * kDuoThreads, "whole swizzle groups; one survivor per thread");

// TMEM columns: per warp group (warps 4g..4g+3) a region of 16-column
// factorisation entries, one per level its threads can reach (levels
// 0..5, 0..1, 0, 0), then 2 columns per chunk for the diagonal-block row.
constexpr uint32_t kTmemCols = 256;
__host__ __device__ constexpr uint32_t tmem_group_base(int g) { return g == 0 ? 0u : g == 1 ? 112u : g == 2 ? 160u : 192u; }
__host__ __device__ constexpr int tmem_group_levels(int g) { return g == 0 ? kDuoMaxLevels : g == 1 ? 2 : 1; }
static_assert(tmem_group_base(3) + 16 * tmem_group_levels(3) + 2 * kDuoMaxChunks <= kTmemCols, "TMEM columns");
static_assert(tmem_group_base(0) + 16 * tmem_group_levels(0) + 2 * kDuoMaxChunks <= tmem_group_base(1), "TMEM g0");
static_assert(tmem_group_base(1) + 16 * tmem_group_levels(1) + 2 * kDuoMaxChunks <= tmem_group_base(2), "TMEM g1");
static_assert(tmem_group_base(2) + 16 * tmem_group_levels(2) + 2 * kDuoMaxChunks <= tmem_group_base(3), "TMEM g2");
// (warp group g reaches level l only if 128 g < 512 >> l: g = 1 up to l = 1, g = 2, 3 only l = 0)

// ---------------------------------------------------------------------------
// tensor memory as per-thread scratch (inline PTX, tcgen05)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" :: "r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }

// (the loaded registers pass through the wait, so that no use of them can
// be scheduled before it)
__device__ __forceinline__ void tmem_wait_ld2(float& a, float& b)
{
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" : "+f"(a), "+f"(b) :: "memory");
}

__device__ __forceinline__ void tmem_wait_ld16(float (&v)[16])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;\n"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]),
                   "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]), "+f"(v[15])
                 :: "memory");
}

// Warp-wide: each lane stores / loads 16 (or 2) 32-bit words at consecutive
// columns of its own TMEM lane (the warp's quarter of the lanes).
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                 "%13, %14, %15, %16};\n"
                 :: "r"(taddr), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]),
                    "f"(v[8]), "f"(v[9]), "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                 "%14, %15}, [%16];\n"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
                   "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
                 : "r"(taddr) : "memory");
}

__device__ __forceinline__ void tmem_st2(uint32_t taddr, float a, float b)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};\n" :: "r"(taddr), "f"(a), "f"(b) : "memory");
}

__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float& a, float& b)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];\n" : "=f"(a), "=f"(b) : "r"(taddr) : "memory");
}

// ---------------------------------------------------------------------------
// tiles, walked without divisions
// ---------------------------------------------------------------------------
// A CTA takes items it = blockIdx.x, blockIdx.x + G, ... (G = gridDim.x,
// item = system * nwin + window); (system, window) advance by (G / nwin,
// G % nwin) with a carry.
struct TileWalk {
    int64_t it, j, w;
};

__device__ __forceinline__ TileWalk walk_start(const DuoGeom& g)
{
    TileWalk q;
    q.it = blockIdx.x;
    q.j = q.it / g.nwin;
    q.w = q.it - q.j * g.nwin;
    return q;
}

// (dj, dw) = (G / nwin, G % nwin), computed once per CTA
__device__ __forceinline__ void walk_next(TileWalk& q, const DuoGeom& g, int64_t dj, int64_t dw)
{
    q.it += gridDim.x;
    q.j += dj;
    q.w += dw;
    if (q.w >= g.nwin) { q.w -= g.nwin; q.j++; }
}

struct DuoTile {
    int64_t j, wlo, whi, t0, t1, rlo, rhi, clo, chi;   // block rows of system j
};

__device__ __forceinline__ DuoTile duo_tile(const DuoGeom& g, int64_t j, int64_t w)
{
    DuoTile t;
    t.j = j;
    t.wlo = w * (int64_t)g.L;
    t.whi = min(t.wlo + (int64_t)g.L, g.nb);
    t.t0 = max(t.wlo - (int64_t)g.H, (int64_t)0);
    t.t1 = min(t.whi + (int64_t)g.H, g.nb);
    t.rlo = max(t.wlo - (int64_t)g.R, (int64_t)0);         // sweep 1 reads level-0 rows and r_0 here
    t.rhi = min(t.whi + (int64_t)g.R, g.nb);
    t.clo = max(t.rlo - 1, (int64_t)0);                   // x_0 needed (sweep 0's check region)
    t.chi = min(t.rhi + 1, g.nb);
    return t;
}

// Chunks of a tile: tile rows [c*kDuoChunk, ...), the same split in both
// phases, so that a thread handles the same rows in both.
__device__ __forceinline__ int tile_chunks(int64_t t0, int64_t t1) { return (int)((t1 - t0 + kDuoChunk - 1) / kDuoChunk); }

// Staging of one chunk is split over six threads (lane 0 of warps 0..5),
// one array each: each arms the slot's mbarrier with its own byte count
// (the barrier expects six arrivals; a null outer band arrives with zero
// bytes) and issues its bulk copy.  Chunk c of the tile at block rows
// [t0, t1) of system j covers block rows t0 + c*kDuoChunk ...  The copies
// ask L2 to keep the lines: the residual phase of this tile and the
// neighbouring windows read them again.
__device__ __forceinline__ void stage_array(const MpArgs& p, int a, int64_t j, int64_t t0, int64_t t1, int c,
                                            double* slot_buf, uint64_t* bar)
{
    const double* src = a == 0 ? p.a : a == 1 ? p.b : a == 2 ? p.c : a == 3 ? p.d : a == 4 ? p.e : p.y;
    const int64_t k0 = t0 + (int64_t)c * kDuoChunk;
    const uint32_t bytes = src ? (uint32_t)(min((int64_t)kDuoChunk, t1 - k0) * 2 * sizeof(double)) : 0u;
    mbar_expect_tx(bar, bytes);
    if (src) bulk_g2s(slot_buf + a * 2 * kDuoChunk, src + j * p.n + 2 * k0, bytes, bar, policy_evict_last());
}

// Tile bounds [t0, t1) of window w.
__device__ __forceinline__ void tile_span(const DuoGeom& g, int64_t w, int64_t& t0, int64_t& t1)
{
    const int64_t wlo = w * (int64_t)g.L, whi = min(wlo + (int64_t)g.L, g.nb);
    t0 = max(wlo - (int64_t)g.H, (int64_t)0);
    t1 = min(whi + (int64_t)g.H, g.nb);
}

// Chunk cc counted from the start of tile (wn, [n0, n1)), resolved to the
// tile that holds it (the last window of a system can be a single chunk);
// wn.it >= items when the stream has ended.
__device__ __forceinline__ void chunk_ahead(const DuoGeom& g, int64_t items, int64_t dj, int64_t dw, TileWalk& wn,
                                            int64_t& n0, int64_t& n1, int& cc)
{
    for (int nch = tile_chunks(n0, n1); cc >= nch; nch = tile_chunks(n0, n1)) {
        cc -= nch;
        walk_next(wn, g, dj, dw);
        if (wn.it >= items) return;
        tile_span(g, wn.w, n0, n1);
    }
}

// ---------------------------------------------------------------------------
// conversions
// ---------------------------------------------------------------------------
// (float)(v * 2^-sh) with the mantissa truncated, for values whose scaled
// exponent is in FP32's normal range; smaller values (zero included) give a
// zero of v's sign.  kb = (sh + 896) << 20: the exponent rebias in the high
// word (896 = 1023 - 127).  An out-of-range large exponent gives some finite
// value (see the file comment).
__device__ __forceinline__ float d2f_trunc(double v, int kb)
{
    const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
    const int t = (int)(hi & 0x7FFFFFFFu) - kb;               // rebiased exponent field and 20 mantissa bits
    const unsigned u = __funnelshift_l(lo, (unsigned)t, 3);   // exponent, 23 mantissa bits
    return __uint_as_float((t >= (1 << 20) ? u : 0u) | (hi & 0x80000000u));
}

// ---------------------------------------------------------------------------
// normalised FP32 block rows (first read)
// ---------------------------------------------------------------------------
// Two threads per block row: thread 2r+h holds row i = 2kb+h (FP64 bands and
// rhs), row-scales and converts its six values, and the pair exchanges them
// by shuffles; each forms row h of Mi L, Mi U and Mi Y (Mi the inverse of
// the scaled diagonal block, same products as prep_row of mixed.cu) and
// writes its half of tile row k.  Returns row h of Mi (mA, mB), which
// normalises the row pair's residual later.  Every lane of the warp takes
// part (the shuffles); only `active` pairs write.
__device__ __forceinline__ void put_block_half(double a, double b, double c, double d, double e, double y,
                                               bool hasA, bool hasB, bool hasD, bool hasE, int h, bool active, int k,
                                               float4* sL, float4* sU, float2* sY, float& mA, float& mB)
{
    const int kb = (d_exponent(c) + 896) << 20;
    const float af = hasA ? d2f_trunc(a, kb) : 0.0f;
    const float bf = hasB ? d2f_trunc(b, kb) : 0.0f;
    const float cf = d2f_trunc(c, kb);
    const float df = hasD ? d2f_trunc(d, kb) : 0.0f;
    const float ef = hasE ? d2f_trunc(e, kb) : 0.0f;
    const float yf = d2f_trunc(y, kb);
    const unsigned full = 0xffffffffu;
    const float pa = __shfl_xor_sync(full, af, 1), pb = __shfl_xor_sync(full, bf, 1);
    const float pc = __shfl_xor_sync(full, cf, 1), pd = __shfl_xor_sync(full, df, 1);
    const float pe = __shfl_xor_sync(full, ef, 1), py = __shfl_xor_sync(full, yf, 1);
    const float a0 = h ? pa : af, b0 = h ? pb : bf, c0 = h ? pc : cf, d0 = h ? pd : df, e0 = h ? pe : ef;
    const float y0 = h ? py : yf;
    const float a1 = h ? af : pa, b1 = h ? bf : pb, c1 = h ? cf : pc, d1 = h ? df : pd, e1 = h ? ef : pe;
    const float y1 = h ? yf : py;
    // Mi = [[c1, -d0], [-b1, c0]] / det; row h of Mi L, Mi U, Mi Y with
    // L = [[a0, b0], [0, a1]], U = [[e0, 0], [d1, e1]]
    const float det = fmaf(c0, c1, -d0 * b1);
    const float rd = __fdividef(1.0f, det);
    mA = h ? -b1 * rd : c1 * rd;
    mB = h ? c0 * rd : -d0 * rd;
    if (!active) return;
    const int sk = swz(k);
    reinterpret_cast<float2*>(sL + sk)[h] = make_float2(mA * a0, fmaf(mA, b0, mB * a1));
    reinterpret_cast<float2*>(sU + sk)[h] = make_float2(fmaf(mA, e0, mB * d1), mB * e1);
    reinterpret_cast<float*>(sY + sk)[h] = fmaf(mA, y0, mB * y1);
}

// ---------------------------------------------------------------------------
// cyclic reduction keeping its factorisation, and its replay on a new rhs
// ---------------------------------------------------------------------------
// As cr_reduce (mixed_dev.cuh) for a tile of TR <= 2 * blockDim.x rows (one
// survivor per thread and level), and each survivor's couplings L_k, U_k
// before the level and the inverse Mi of its new diagonal block go to the
// thread's TMEM lane (tw + 16 l): the rhs update of that level is then
// Y_k <- Mi (Y_k - L_k Y_{k-d} - U_k Y_{k+d}).  Ends with a barrier.
__device__ __forceinline__ int cr_reduce_keep(float4* sL, float4* sU, float2* sY, int TR, int kmax, int clo, int chi,
                                              uint32_t tw)
{
    const int tid = threadIdx.x;
    int top = TR <= 1 ? 0 : -1;
    for (int l = 0; l < kmax && (1 << l) < TR; l++) {
        const int d = 1 << l, d2 = 2 * d;
        const int k = tid * d2;
        const bool act = k < TR;
        bool coupled = false;
        float v[16];
        if (act) {
            const int sk = swz(k), sm = swz(max(k - d, 0)), sp = swz(min(k + d, TR - 1));
            const M2 Lk = m2(sL[sk]), Uk = m2(sU[sk]), Lm = m2(sL[sm]), Um = m2(sU[sm]);
            const M2 Lp = m2(sL[sp]), Up = m2(sU[sp]);
            const float2 Yk = sY[sk], ym = sY[sm], yp = sY[sp];
            M2 Dn;
            Dn.m0 = fmaf(-Uk.m1, Lp.m2, fmaf(-Uk.m0, Lp.m0, fmaf(-Lk.m1, Um.m2, fmaf(-Lk.m0, Um.m0, 1.0f))));
            Dn.m1 = fmaf(-Uk.m1, Lp.m3, fmaf(-Uk.m0, Lp.m1, fmaf(-Lk.m1, Um.m3, -Lk.m0 * Um.m1)));
            Dn.m2 = fmaf(-Uk.m3, Lp.m2, fmaf(-Uk.m2, Lp.m0, fmaf(-Lk.m3, Um.m2, -Lk.m2 * Um.m0)));
            Dn.m3 = fmaf(-Uk.m3, Lp.m3, fmaf(-Uk.m2, Lp.m1, fmaf(-Lk.m3, Um.m3, fmaf(-Lk.m2, Um.m1, 1.0f))));
            const float y0 = fmaf(-Uk.m1, yp.y, fmaf(-Uk.m0, yp.x, fmaf(-Lk.m1, ym.y, fmaf(-Lk.m0, ym.x, Yk.x))));
            const float y1 = fmaf(-Uk.m3, yp.y, fmaf(-Uk.m2, yp.x, fmaf(-Lk.m3, ym.y, fmaf(-Lk.m2, ym.x, Yk.y))));
            const M2 LL = mmul(Lk, Lm), UU = mmul(Uk, Up);
            const M2 Mi = minv(Dn);
            const M2 Mn = {-Mi.m0, -Mi.m1, -Mi.m2, -Mi.m3};
            const M2 Lo = mmul(Mn, LL), Uo = mmul(Mn, UU);
            sL[sk] = f4(Lo);
            sU[sk] = f4(Uo);
            sY[sk] = make_float2(fmaf(Mi.m0, y0, Mi.m1 * y1), fmaf(Mi.m2, y0, Mi.m3 * y1));
            if (k >= clo - d2 + 1 && k < chi + d2 - 1) coupled = fmaxf(amaxm(Lo), amaxm(Uo)) >= kTrunc;
            v[0] = Lk.m0; v[1] = Lk.m1; v[2] = Lk.m2; v[3] = Lk.m3;
            v[4] = Uk.m0; v[5] = Uk.m1; v[6] = Uk.m2; v[7] = Uk.m3;
            v[8] = Mi.m0; v[9] = Mi.m1; v[10] = Mi.m2; v[11] = Mi.m3;
        } else {
#pragma unroll
            for (int q = 0; q < 12; q++) v[q] = 0.0f;
        }
        v[12] = v[13] = v[14] = v[15] = 0.0f;
        if (__any_sync(0xffffffffu, act)) tmem_st16(tw + 16u * l, v);   // (warp-uniform)
        if (!__syncthreads_or(coupled)) { top = l + 1; break; }
    }
    tmem_wait_st();
    return top;
}

// The rhs-only replay of cr_reduce_keep's first `top` levels.  Ends with a
// barrier.
__device__ __forceinline__ void cr_replay_rhs(float2* sY, int TR, int top, uint32_t tw)
{
    const int tid = threadIdx.x;
    for (int l = 0; l < top; l++) {
        const int d = 1 << l, d2 = 2 * d;
        const int k = tid * d2;
        const bool act = k < TR;
        if (__any_sync(0xffffffffu, act)) {
            float v[16];
            tmem_ld16(tw + 16u * l, v);
            tmem_wait_ld16(v);
            if (act) {
                const int sk = swz(k), sm = swz(max(k - d, 0)), sp = swz(min(k + d, TR - 1));
                const float2 Yk = sY[sk], ym = sY[sm], yp = sY[sp];
                const float y0 = fmaf(-v[5], yp.y, fmaf(-v[4], yp.x, fmaf(-v[1], ym.y, fmaf(-v[0], ym.x, Yk.x))));
                const float y1 = fmaf(-v[7], yp.y, fmaf(-v[6], yp.x, fmaf(-v[3], ym.y, fmaf(-v[2], ym.x, Yk.y))));
                sY[sk] = make_float2(fmaf(v[8], y0, v[9] * y1), fmaf(v[10], y0, v[11] * y1));
            }
        }
        __syncthreads();
    }
}

// The six FP64 values of row g (second read, from L2; streaming).
struct Row6 { double a, b, c, d, e, y; };

__device__ __forceinline__ Row6 load_row6(const MpArgs& p, int64_t g, bool on)
{
    Row6 v{0.0, 0.0, 1.0, 0.0, 0.0, 0.0};
    if (on) {
        v.a = p.a ? __ldcs(p.a + g) : 0.0;
        v.b = __ldcs(p.b + g);
        v.c = __ldcs(p.c + g);
        v.d = __ldcs(p.d + g);
        v.e = p.e ? __ldcs(p.e + g) : 0.0;
        v.y = __ldcs(p.y + g);
    }
    return v;
}

// Maximum of |v| as a bit pattern: non-negative floats order like their
// bits and a NaN (any payload, sign cleared) lies above inf, so a NaN in the
// solution poisons the norm and the stopping rule never accepts it.
__device__ __forceinline__ unsigned abs_bits(float v) { return __float_as_uint(v) & 0x7FFFFFFFu; }

// CTA-wide maximum of such bit patterns into *dst (atomic).
__device__ __forceinline__ void cta_max_bits_to(unsigned* dst, unsigned v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v) atomicMax(dst, v);
}

// Persistent CTAs (two per SM) over the windows of all systems.
__global__ void __launch_bounds__(kDuoThreads, 2)
mp_duo_kernel(MpArgs p, DuoGeom g)
{
    extern __shared__ __align__(128) unsigned char duo_smem[];
    double* ring = reinterpret_cast<double*>(duo_smem);
    double2* sX0 = reinterpret_cast<double2*>(duo_smem + (size_t)kDuoSlots * kDuoSlotDoubles * sizeof(double));
    float4* sL = reinterpret_cast<float4*>(sX0 + kDuoRows);
    float4* sU = sL + kDuoRows;
    float2* sY = reinterpret_cast<float2*>(sU + kDuoRows);
    __shared__ __align__(8) uint64_t bars[kDuoSlots];
    __shared__ uint32_t tmem_base;
    __shared__ int64_t walk_dj, walk_dw;

    const int tid = threadIdx.x, bd = blockDim.x, h = tid & 1, r = tid >> 1, warp = tid >> 5;
    if (tid == 0) {
        for (int s = 0; s < kDuoSlots; s++) mbar_init(&bars[s], kDuoArrays);
        fence_mbarrier_init();
        walk_dj = (int64_t)gridDim.x / g.nwin;
        walk_dw = (int64_t)gridDim.x - walk_dj * g.nwin;
    }
    if (warp == 0) tmem_alloc(&tmem_base, kTmemCols);
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    // this warp's TMEM lane quarter and its group's columns
    const uint32_t tw = tmem_base + ((uint32_t)(32 * (warp & 3)) << 16) + tmem_group_base(warp >> 2);
    const uint32_t tmab = tw + 16u * tmem_group_levels(warp >> 2);   // 2 columns per chunk
    pdl_wait();
    pdl_release();                                 // one wave of persistent CTAs: the successor may queue now

    const int64_t items = p.m * g.nwin, n = p.n;
    const uint64_t limit = p.inject ? 4000000ull : 2000000000ull;   // ns
    const int64_t dj = walk_dj, dw = walk_dw;
    // the stagers: lane 0 of warps 0..kDuoArrays-1, array `warp` each
    const bool stager = (tid & 31) == 0 && warp < kDuoArrays;
    uint32_t issued = 0, used = 0;                 // chunks staged / consumed by this CTA
    // the stream's first chunks
    for (int s = 0; s < kDuoSlots; s++) {
        TileWalk wn = walk_start(g);
        if (wn.it >= items) break;
        int64_t n0, n1;
        tile_span(g, wn.w, n0, n1);
        int cc = s;
        chunk_ahead(g, items, dj, dw, wn, n0, n1, cc);
        if (wn.it >= items) break;
        if (stager && !(p.inject && issued == 0))
            stage_array(p, warp, wn.j, n0, n1, cc, ring + s * kDuoSlotDoubles, &bars[s]);
        issued++;
    }
    bool gave_up = false;

    for (TileWalk wk = walk_start(g); wk.it < items; walk_next(wk, g, dj, dw)) {
        const DuoTile t = duo_tile(g, wk.j, wk.w);
        const int TR = (int)(t.t1 - t.t0);
        const bool whole = t.t0 == 0 && t.t1 == g.nb;
        const int nch = tile_chunks(t.t0, t.t1);
        // Band slots outside the system (n even): row i = 2kb+h has a_i, b_i
        // unless kb = 0 (b_1 exists), d_i, e_i unless kb = nb-1 (d of the
        // block row's first row exists); tile-local tests.
        const bool sys_first = t.t0 == 0, sys_last = t.t1 == g.nb;
        // phase 0: the staged tile -> level-0 blocks with rhs y
        for (int c = 0; c < nch; c++, used++) {
            const int slot = (int)(used % kDuoSlots);
            const bool got = mbar_wait_bounded(&bars[slot], (used / kDuoSlots) & 1u, limit);
            if (__syncthreads_or(!got)) { gave_up = true; break; }
            const int k = c * kDuoChunk + r;
            const bool active = k < TR;
            const bool at0 = sys_first && k == 0, atN = sys_last && k == TR - 1;
            const double* st = ring + slot * kDuoSlotDoubles + 2 * r + h;
            double a = 0.0, b = 0.0, cc = 1.0, d = 0.0, e = 0.0, y = 0.0;
            if (active) {
                a = p.a ? st[0 * 2 * kDuoChunk] : 0.0;
                b = st[1 * 2 * kDuoChunk];
                cc = st[2 * 2 * kDuoChunk];
                d = st[3 * 2 * kDuoChunk];
                e = p.e ? st[4 * 2 * kDuoChunk] : 0.0;
                y = st[5 * 2 * kDuoChunk];
            }
            float mA, mB;
            put_block_half(a, b, cc, d, e, y, !at0, !(at0 && h == 0), !(atN && h == 1), !atN, h, active, k, sL, sU, sY,
                           mA, mB);
            tmem_st2(tmab + 2u * c, mA, mB);        // (warp-uniform)
            __syncthreads();                       // the slot's data is consumed
            // refill the slot with the chunk kDuoSlots ahead in the stream
            {
                TileWalk wn = wk;
                int64_t n0 = t.t0, n1 = t.t1;
                int cc = c + kDuoSlots;
                chunk_ahead(g, items, dj, dw, wn, n0, n1, cc);
                if (wn.it < items) {
                    if (stager) {
                        fence_proxy_async();
                        stage_array(p, warp, wn.j, n0, n1, cc, ring + slot * kDuoSlotDoubles, &bars[slot]);
                    }
                    issued++;
                }
            }
        }
        if (gave_up) break;
        tmem_wait_st();
        // sweep 0: reduce the tile, keeping the factorisation; x_0 exact on
        // [clo, chi).  (A tile never holds a whole system here, and no more
        // levels than TMEM keeps are reduced: deeper coupling leaves the
        // system to the general kernels.)
        const int klo0 = (int)(t.clo - t.t0), khi0 = (int)(t.chi - t.t0);
        const int top0 = cr_reduce_keep(sL, sU, sY, TR, min(whole ? 31 : g.K, kDuoMaxLevels), klo0, khi0, tw);
        if (top0 < 0) {
            if (tid == 0 && atomicOr(&p.fail[t.j], 1) == 0) atomicAdd(p.nfail, 1);
            continue;                              // (cr_reduce_keep ended with a barrier)
        }
        cr_substitute(sL, sU, sY, TR, top0);       // (ends with a barrier)
        // x_0 (FP64) on the check region; max |x_0| over the window
        const int klo = (int)(t.wlo - t.t0), khi = (int)(t.whi - t.t0);
        unsigned xm = 0u;
        for (int k = klo0 + tid; k < khi0; k += bd) {
            const float2 v = sY[swz(k)];
            sX0[k] = make_double2(f2d(v.x), f2d(v.y));
            if (k >= klo && k < khi) xm = max(xm, max(abs_bits(v.x), abs_bits(v.y)));
        }
        cta_max_bits_to(&p.dnorm[t.j], xm);
        __syncthreads();                           // x_0 complete before the residual reads neighbours
        // phase 1: r_0 = y - A x_0 (FP64) on [rlo, rhi), row-scaled and
        // normalised by the diagonal-block row kept in TMEM -> the rhs; a zero
        // rhs elsewhere.  The six values come from L2, one chunk loaded ahead.
        const int krl = (int)(t.rlo - t.t0), krh = (int)(t.rhi - t.t0);
        const int64_t rowbase = t.j * n + 2 * t.t0 + h;
        Row6 cur = load_row6(p, rowbase + 2 * r, r >= krl && r < krh);
        for (int c = 0; c < nch; c++) {
            const int k = c * kDuoChunk + r;
            const bool active = k < TR, resid = k >= krl && k < krh;
            const int kn = k + kDuoChunk;
            const Row6 nxt = load_row6(p, rowbase + 2 * kn, c + 1 < nch && kn >= krl && kn < krh);
            float mA, mB;
            tmem_ld2(tmab + 2u * c, mA, mB);
            float rf = 0.0f;
            if (resid) {
                const bool at0 = sys_first && k == 0, atN = sys_last && k == TR - 1;
                // x_0 of rows i-2 .. i+2: tile rows k-1, k, k+1
                const double2 xc = sX0[k];
                const double2 xl = !at0 ? sX0[k - 1] : make_double2(0.0, 0.0);
                const double2 xr = !atN ? sX0[k + 1] : make_double2(0.0, 0.0);
                const double xa = h ? xl.y : xl.x, xb = h ? xc.x : xl.y, xi = h ? xc.y : xc.x;
                const double xd = h ? xr.x : xc.y, xe = h ? xr.y : xr.x;
                // same FMA order as the refinement kernel of mixed.cu
                double rhs = fma(-cur.c, xi, cur.y);
                if (p.a && !at0) rhs = fma(-cur.a, xa, rhs);
                if (!(at0 && h == 0)) rhs = fma(-cur.b, xb, rhs);
                if (!(atN && h == 1)) rhs = fma(-cur.d, xd, rhs);
                if (p.e && !atN) rhs = fma(-cur.e, xe, rhs);
                rf = d2f_scaled(rhs, d_exponent(cur.c));
            }
            const float pf = __shfl_xor_sync(0xffffffffu, rf, 1);
            tmem_wait_ld2(mA, mB);
            if (active) reinterpret_cast<float*>(sY + swz(k))[h] = fmaf(mA, h ? pf : rf, mB * (h ? rf : pf));
            cur = nxt;
        }
        __syncthreads();
        // sweep 1: the factorisation replayed on the new rhs, back substitution
        // with the blocks sweep 0 left in place
        cr_replay_rhs(sY, TR, top0, tw);
        cr_substitute(sL, sU, sY, TR, top0);
        // x_1 = x_0 + dx_1 on the window -> X0; max |dx_1|
        unsigned dm = 0u;
        double2* X = reinterpret_cast<double2*>(p.X0 + t.j * n);
        for (int k = klo + tid; k < khi; k += bd) {
            const float2 v = sY[swz(k)];
            const double2 x0 = sX0[k];
            X[t.t0 + k] = make_double2(__dadd_rn(x0.x, f2d(v.x)), __dadd_rn(x0.y, f2d(v.y)));
            dm = max(dm, max(abs_bits(v.x), abs_bits(v.y)));
        }
        cta_max_bits_to(&p.dnorm[p.m + t.j], dm);
        __syncthreads();                           // the tile is reused by the next window
    }

    if (gave_up && tid == 0) {
        atomicOr(p.err, 1);
        // wait (bounded) for the copies still in flight into the ring
        for (; used < issued; used++)
            mbar_wait_bounded(&bars[used % kDuoSlots], (used / kDuoSlots) & 1u, limit);
    }
    // every way out: free the TMEM columns once all their accesses are done
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0) tmem_dealloc(tmem_base, kTmemCols);
}

// Systems the fused kernel solved: the stopping rule after sweep 1 from its
// norms; a system that is done (or out of sweeps) gets x_1 copied from X0 to
// the output and is finished (fin = 2).  Others (windows that stayed
// coupled, or more sweeps needed) keep fin = 0 for the general kernels.
constexpr int kFinThreads = 256;
constexpr int kFinRows = 8 * kFinThreads;        // rows per CTA item (a double2 per thread, 4 per thread)

__global__ void __launch_bounds__(kFinThreads)
mp_duo_finish_kernel(MpArgs p)
{
    pdl_wait();
    pdl_release();
    // a CTA of the fused kernel gave up a wait: its windows are missing, so
    // every system goes to the general kernels (the call reports the timeout)
    if (__ldg(p.err)) return;
    const int64_t n = p.n, chunks = (n + kFinRows - 1) / kFinRows;
    for (int64_t blk = blockIdx.x; blk < p.m * chunks; blk += gridDim.x) {
        const int64_t j = blk / chunks, c = blk - j * chunks;
        if (__ldg(p.fail + j)) continue;
        const float nd0 = __uint_as_float(__ldg(p.dnorm + j)), nd1 = __uint_as_float(__ldg(p.dnorm + p.m + j));
        const UpDecision D = stop_rule(1, nd1, nd0, nd0, p.tol, p.max_sweeps);
        if (!D.last) continue;
        const int64_t i0 = c * kFinRows, i1 = min(i0 + kFinRows, n);
        const double2* __restrict__ src = reinterpret_cast<const double2*>(p.X0 + j * n);
        double2* __restrict__ dst = reinterpret_cast<double2*>(p.xout + j * p.oss);
#pragma unroll 4
        for (int64_t q = i0 / 2 + threadIdx.x; q < i1 / 2; q += kFinThreads) __stcs(dst + q, __ldcs(src + q));
        if (c == 0 && threadIdx.x == 0) {
            p.fin[j] = 2;
            p.status[j] = D.done ? 1 : 2;
            p.est[j] = D.est;
            for (int s = 0; s <= p.max_sweeps; s++) atomicSub(&p.live[s], 1);
        }
    }
}

// Graph-driven solves: opens the general sweep loop (while node) only if a
// system is left after the fused sweeps.
__global__ void mp_gate_kernel(MpArgs p, cudaGraphConditionalHandle h)
{
    pdl_wait();
    cudaGraphSetConditional(h, p.live[0] > 0 ? 1u : 0u);
}

}  // namespace

bool duo_plan(const MpArgs& p, int levels, DuoGeom* g)
{
    // contiguous systems of even n, 16-byte aligned arrays (whole 16-byte
    // row pairs for the bulk copies), at least two sweeps, and windows that
    // leave a core
    if (levels < 1 || levels > kDuoMaxLevels || p.max_sweeps < 2 || !p.vec || p.rg) return false;
    if (p.rs != 1 || p.ss != p.n || (p.n & 1) || p.xout == nullptr || p.ors != 1 || p.oss != p.n) return false;
    if (reinterpret_cast<uintptr_t>(p.X0) & 15 || reinterpret_cast<uintptr_t>(p.xout) & 15) return false;
    // Opt-in (PCRP_DUO=1) while the fused pass is slower than the general
    // kernels on GB300: it moves fewer bytes but issues more instructions
    // per unknown (see the design notes); PCRP_NO_DUO forces it off.
    if (!std::getenv("PCRP_DUO") || std::getenv("PCRP_NO_DUO")) return false;
    const int R = (2 << levels) - 2;
    const int H = 4 << levels;
    const int L = kDuoRows - 2 * H;
    if (L < 64) return false;
    g->nb = p.n / 2;
    if (g->nb <= kDuoRows) return false;                     // whole systems have their own kernel
    g->K = levels; g->R = R; g->H = H; g->L = L;
    g->nwin = (g->nb + L - 1) / L;
    return true;
}

cudaError_t launch_mp_duo(const MpArgs& p, const DuoGeom& g, cudaStream_t s)
{
    const int64_t items = p.m * g.nwin;
    if (items <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(mp_duo_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDuoSmem);
    if (e != cudaSuccess) return e;
    // Two CTAs per SM: registers (64 x 512) and shared memory allow two, and
    // their TMEM (256 columns each) fills the SM's 512.  (The occupancy
    // query answers one for a kernel that allocates TMEM.)  A CTA that
    // found no free columns would wait in tcgen05.alloc for the resident
    // ones, which finish without waiting on it.
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int64_t blocks = std::min<int64_t>(items, 2 * (int64_t)sms);
    e = launch_dependent(mp_duo_kernel, (unsigned)blocks, kDuoThreads, kDuoSmem, s, p, g);
    count_launch();
    return e;
}

cudaError_t launch_mp_duo_finish(const MpArgs& p, cudaStream_t s)
{
    const int64_t chunks = (p.n + kFinRows - 1) / kFinRows;
    const int64_t blocks = std::min<int64_t>(p.m * chunks, mp_grid_cap((const void*)mp_duo_finish_kernel, kFinThreads, 0));
    const cudaError_t e = launch_dependent(mp_duo_finish_kernel, (unsigned)std::max<int64_t>(blocks, 1), kFinThreads, 0,
                                           s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_gate(const MpArgs& p, cudaGraphConditionalHandle h, cudaStream_t s)
{
    const cudaError_t e = launch_dependent(mp_gate_kernel, 1u, 1u, 0, s, p, h);
    count_launch();
    return e;
}

}  // namespace pcrp
