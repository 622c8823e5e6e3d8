// mixed.cu -- mixed-precision solve: FP32 2x2-block PCR + FP64 iterative
// refinement, and the fused FP64 pentadiagonal residual.
//
// Why blocks.  The reference's scalar PCR-Penta eliminates with off-diagonal
// pivots (alpha = -a[i]/b[i-2d], kernel.cu:73), which amplifies rounding by
// 1/|pivot|: in FP32 it loses 3-4 digits on diagonally dominant inputs, and
// an exactly zero off-diagonal breaks it outright.  Grouping rows in pairs
// turns the pentadiagonal matrix into a block-tridiagonal one with 2x2
// blocks; block PCR then pivots on the 2x2 diagonal blocks, which stay
// well conditioned for dominant systems (block cyclic reduction preserves
// block dominance and squares the coupling every stride), so the FP32 solve
// keeps ~7 digits and one refinement sweep usually reaches 1e-13.
//
// Block row k holds rows 2k, 2k+1 and reads L_k X_{k-d} + X_k + U_k X_{k+d}
// = Y_k after normalisation by its diagonal block (D = I).  One stride:
//     D' = I - L_k U_{k-d} - U_k L_{k+d},  L' = -L_k L_{k-d},
//     U' = -U_k U_{k+d},  Y' = Y_k - L_k Y_{k-d} - U_k Y_{k+d},
// then L, U, Y <- D'^{-1} (L', U', Y').  Strides stop early once every
// |L|,|U| entry of a system is below kTrunc (the couplings then change X by
// less than kTrunc*|X|, far below FP32 resolution) -- truncated PCR.
//
// FP64 budget.  GB300 issues FP64 at ~1/64 of the FP32 rate, so FP64 is kept
// to the residual (5 DFMA per row) and the correction (1 DADD per row).  Row
// scaling by the main diagonal is done by powers of two in the integer
// pipe, and every FP64<->FP32 conversion here is integer bit arithmetic
// (no F2F instructions, which also issue on the FP64 pipe).
//
// Stopping rule.  With dx_s the correction of sweep s, a system is done when
// |dx_s| <= tol/2 |x| (the correction bounds what it leaves), or when the
// corrections contract (rho = |dx_s|/|dx_{s-1}| < 0.5) and twice the
// geometric tail rho/(1-rho)|dx_s| is <= tol |x|.
// Each kernel reads the per-system norms left by the previous kernel, so the
// decision needs no host round trip; finished systems skip all later work.
#include <algorithm>
#include <cfloat>
#include <cstring>

#include "pcrp_internal.h"
#include "mixed_internal.h"
#include "mixed_dev.cuh"
#include "tma.cuh"

namespace pcrp {
namespace {

constexpr int kMpThreads = 256;
constexpr int kMpTryThreads = 256;
static_assert(kMpTile % kMpThreads == 0 && kMpThreads % 2 == 0, "refinement tiles: whole rows per thread, pairs in adjacent lanes");

// Row i of system j of an iterate: at j*ss + i*rs, or (ragged output, rg
// non-null) at rg[j].x + i for i < rg[j].y; padding rows read as zero and
// are not stored.
__device__ __forceinline__ double x_read(const double* __restrict__ x, int64_t ss, int64_t rs,
                                         const longlong2* __restrict__ rg, int64_t j, int64_t i)
{
    if (!rg) return x[j * ss + i * rs];
    const longlong2 g = __ldg(rg + j);
    return i < g.y ? x[g.x + i] : 0.0;
}

__device__ __forceinline__ void x_write(double* __restrict__ x, int64_t ss, int64_t rs,
                                        const longlong2* __restrict__ rg, int64_t j, int64_t i, double v)
{
    if (!rg) { x[j * ss + i * rs] = v; return; }
    const longlong2 g = __ldg(rg + j);
    if (i < g.y) x[g.x + i] = v;
}

// x_s of row i of system j (FP32 correction d), with the maxima of |dx| and
// |x| folded into dmax and xbits.
__device__ __forceinline__ double x_update(const double* __restrict__ xsrc, int64_t xss, int64_t xrs,
                                           const longlong2* srg, double* __restrict__ xdst, int64_t dss, int64_t drs,
                                           const longlong2* drg, int64_t j, int64_t i, float d, float& dmax,
                                           unsigned long long& xbits)
{
    const double dd = f2d(d);
    const double x = xsrc ? __dadd_rn(x_read(xsrc, xss, xrs, srg, j, i), dd) : dd;
    x_write(xdst, dss, drs, drg, j, i, x);
    dmax = fmaxf(dmax, fabsf(d));
    xbits = max(xbits, absbits(x));
    return x;
}

// Rows i0 (even) and i0 + 1 < n of system j: as two x_update calls, with
// one 16-byte load and store when both iterates are contiguous there and
// 16-byte aligned (same values).
__device__ __forceinline__ void x_update_pair(const double* __restrict__ xsrc, int64_t xss, int64_t xrs,
                                              const longlong2* srg, double* __restrict__ xdst, int64_t dss,
                                              int64_t drs, const longlong2* drg, int64_t j, int64_t i0, float2 d,
                                              float& dmax, unsigned long long& xbits)
{
    if (!srg && !drg && xrs == 1 && drs == 1) {
        const double* s = xsrc ? xsrc + j * xss + i0 : nullptr;
        double* t = xdst + j * dss + i0;
        if (((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(t)) & 15) == 0) {
            const double2 dd = make_double2(f2d(d.x), f2d(d.y));
            double2 x = dd;
            if (s) {
                const double2 xs = *reinterpret_cast<const double2*>(s);
                x = make_double2(__dadd_rn(xs.x, dd.x), __dadd_rn(xs.y, dd.y));
            }
            *reinterpret_cast<double2*>(t) = x;
            dmax = fmaxf(dmax, fmaxf(fabsf(d.x), fabsf(d.y)));
            xbits = max(xbits, max(absbits(x.x), absbits(x.y)));
            return;
        }
    }
    x_update(xsrc, xss, xrs, srg, xdst, dss, drs, drg, j, i0, d.x, dmax, xbits);
    x_update(xsrc, xss, xrs, srg, xdst, dss, drs, drg, j, i0 + 1, d.y, dmax, xbits);
}

// Iterates of sweep s: x_0 in X0 when more sweeps follow, every later x_s in
// the output; x_{s-1} is read from where sweep s-1 wrote it.
// The output of a ragged batch is addressed through rg.
struct XView { const double* src; int64_t sss, srs; const longlong2* srg; double* dst; int64_t dss, drs; const longlong2* drg; };

__device__ __forceinline__ XView x_view(int s, int max_sweeps, const double* X0, double* xout, int64_t n,
                                        int64_t oss, int64_t ors, const longlong2* rg)
{
    XView v;
    v.srg = nullptr; v.drg = nullptr;
    if (s == 0) { v.src = nullptr; v.sss = 0; v.srs = 0; }
    else if (s == 1) { v.src = X0; v.sss = n; v.srs = 1; }
    else { v.src = xout; v.sss = oss; v.srs = ors; v.srg = rg; }
    if (s == 0 && max_sweeps >= 2) { v.dst = const_cast<double*>(X0); v.dss = n; v.drs = 1; }
    else { v.dst = xout; v.dss = oss; v.drs = ors; v.drg = rg; }
    return v;
}

// Graph-driven sweeps: the per-sweep fields from the device sweep counter
// (written by the previous sweep's last kernel, complete before this one
// starts).  No-ops for host-driven launches.
__device__ __forceinline__ void mp_resolve(MpArgs& p)
{
    if (!p.ctr) return;
    p.sweep = *p.ctr;
    const XView v = x_view(p.sweep, p.max_sweeps, p.X0, p.xout, p.n, p.oss, p.ors, p.rg);
    p.xsrc = v.src; p.xsrc_ss = v.sss; p.xsrc_rs = v.srs; p.xsrc_rg = v.srg;
    p.xdst = v.dst; p.xdst_ss = v.dss; p.xdst_rs = v.drs; p.xdst_rg = v.drg;
}

__device__ __forceinline__ void mp_resolve(MpPassArgs& p)
{
    if (!p.ctr) return;
    const int s = *p.ctr;
    p.sweep = s;
    p.live = p.live0 + s;
    if (p.level0) p.srcY = (s & 1) ? p.R1 : p.R0;
    if (p.pre0) {
        unsigned* pre = p.pre0 + (size_t)s * kMpMaxPasses * p.m;
        p.ndx_pre_in = p.pass > 0 ? pre + (size_t)(p.pass - 1) * p.m : nullptr;
        p.ndx_pre_out = p.final_step ? nullptr : pre + (size_t)p.pass * p.m;
    }
    if (p.nx0) {
        p.nx = p.nx0 + (size_t)s * p.m;
        const XView v = x_view(s, p.max_sweeps, p.X0, p.xout, p.n, p.oss, p.ors, p.rg);
        p.xsrc = v.src; p.xsrc_ss = v.sss; p.xsrc_rs = v.srs; p.xsrc_rg = v.srg;
        p.xdst = v.dst; p.xdst_ss = v.dss; p.xdst_rs = v.drs; p.xdst_rg = v.drg;
    }
}

// The six FP64 values of rows i0 = 2k and i1 = 2k+1 of system j (i1 may be
// the dummy row n of an odd system).  Contiguous pairs at an even element
// offset are read as one 16-byte load per array.  A null outer band (a or e)
// is zero and not read.  In a ragged batch the rows past the system's own
// are identity rows, and the band slots of its last rows that would couple
// to them read as zero (the caller's values there are not part of the
// system).
struct PairRow { double a0, a1, b0, b1, c0, c1, d0, d1, e0, e1, y0, y1; };

// L2 residency of the band loads of sweep 0: the prep loads a tile's bands
// to keep (the residual of the same tile reads them again once its cyclic
// reduction is done), the residual loads them for the last time.
enum class Keep { normal, last, first };

__device__ __forceinline__ double2 ldg2_policy(const double* q, uint64_t pol)
{
    double2 v;
    asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(q), "l"(pol));
    return v;
}

__device__ __forceinline__ double2 ldg2(const double* q, Keep keep, uint64_t pol)
{
    return keep == Keep::normal ? *reinterpret_cast<const double2*>(q) : ldg2_policy(q, pol);
}

// RG: the batch is ragged (p.rg non-null); the uniform kernels are compiled
// without the ragged addressing.
template <bool RG>
__device__ __forceinline__ PairRow load_pair(const MpArgs& p, int64_t j, int64_t i0, Keep keep = Keep::normal)
{
    PairRow P;
    int64_t n = p.n, rs = p.rs, base = j * p.ss;
    if (RG) {
        const longlong2 g = __ldg(p.rg + j);
        base = g.x; n = g.y; rs = 1;
        if (i0 >= n) {
            P = {0.0, 0.0, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            return P;
        }
    }
    const int64_t g0 = base + i0 * rs;
    const double2 z = make_double2(0.0, 0.0);
    if (p.vec && rs == 1 && ((g0 & 1) == 0) && i0 + 1 < n) {
        const uint64_t pol = keep == Keep::last ? tma::policy_evict_last()
                             : keep == Keep::first ? tma::policy_evict_first() : 0;
        const double2 a = p.a ? ldg2(p.a + g0, keep, pol) : z;
        const double2 b = ldg2(p.b + g0, keep, pol);
        const double2 c = ldg2(p.c + g0, keep, pol);
        const double2 d = ldg2(p.d + g0, keep, pol);
        const double2 e = p.e ? ldg2(p.e + g0, keep, pol) : z;
        const double2 y = ldg2(p.y + g0, keep, pol);
        P = {a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x, e.y, y.x, y.y};
    } else {
        P.a0 = p.a ? p.a[g0] : 0.0; P.b0 = p.b[g0]; P.c0 = p.c[g0]; P.d0 = p.d[g0];
        P.e0 = p.e ? p.e[g0] : 0.0; P.y0 = p.y[g0];
        if (i0 + 1 < n) {
            const int64_t g1 = g0 + rs;
            P.a1 = p.a ? p.a[g1] : 0.0; P.b1 = p.b[g1]; P.c1 = p.c[g1]; P.d1 = p.d[g1];
            P.e1 = p.e ? p.e[g1] : 0.0; P.y1 = p.y[g1];
        } else {
            P.a1 = 0.0; P.b1 = 0.0; P.c1 = 1.0; P.d1 = 0.0; P.e1 = 0.0; P.y1 = 0.0;
        }
    }
    if (RG) {
        if (i0 + 1 >= n) P.d0 = 0.0;
        if (i0 + 2 >= n) { P.e0 = 0.0; P.d1 = 0.0; }
        if (i0 + 3 >= n) P.e1 = 0.0;
    }
    return P;
}

// The FP32 row-scaled diagonal block and couplings of block row k (rows
// i0 = 2k, i1 = 2k+1) of a system with n rows.  Row i1 = n (odd n) is a
// dummy identity row.  Out-of-range band slots are never read as values.
struct BlockRow { M2 D, L, U; int sh0, sh1; };

__device__ __forceinline__ BlockRow block_of(const PairRow& P, int64_t i0, int64_t n)
{
    BlockRow B;
    const int64_t i1 = i0 + 1;
    B.sh0 = d_exponent(P.c0);
    const float a0 = i0 >= 2 ? d2f_scaled(P.a0, B.sh0) : 0.0f;
    const float b0 = i0 >= 1 ? d2f_scaled(P.b0, B.sh0) : 0.0f;
    const float d0 = i0 + 1 < n ? d2f_scaled(P.d0, B.sh0) : 0.0f;
    const float e0 = i0 + 2 < n ? d2f_scaled(P.e0, B.sh0) : 0.0f;
    const float cf0 = d2f_scaled(P.c0, B.sh0);
    float a1 = 0.0f, b1 = 0.0f, cf1 = 1.0f, d1 = 0.0f, e1 = 0.0f;
    B.sh1 = 0;
    if (i1 < n) {
        B.sh1 = d_exponent(P.c1);
        a1 = i1 >= 2 ? d2f_scaled(P.a1, B.sh1) : 0.0f;
        b1 = d2f_scaled(P.b1, B.sh1);
        cf1 = d2f_scaled(P.c1, B.sh1);
        d1 = i1 + 1 < n ? d2f_scaled(P.d1, B.sh1) : 0.0f;
        e1 = i1 + 2 < n ? d2f_scaled(P.e1, B.sh1) : 0.0f;
    }
    B.D = {cf0, d0, b1, cf1};
    B.L = {a0, b0, 0.0f, a1};
    B.U = {e0, 0.0f, d1, e1};
    return B;
}

// ---------------------------------------------------------------------------
// prep: level-0 normalised block state and the first right-hand side
// ---------------------------------------------------------------------------
// One block row of the prep work: row scaling, FP32 blocks, diagonal inverse,
// the normalised couplings and rhs.
struct PrepRow { M2 L, U, Mi; float2 Y; double2 y; };   // y: the two FP64 rhs values (0 past the system)

template <bool RG>
__device__ __forceinline__ PrepRow prep_row(const MpArgs& p, int64_t j, int64_t k, Keep keep = Keep::normal)
{
    const PairRow P = load_pair<RG>(p, j, 2 * k, keep);
    const BlockRow B = block_of(P, 2 * k, p.n);
    PrepRow r;
    r.Mi = minv(B.D);
    r.L = mmul(r.Mi, B.L);
    r.U = mmul(r.Mi, B.U);
    const float y0 = d2f_scaled(P.y0, B.sh0);
    const float y1 = 2 * k + 1 < p.n ? d2f_scaled(P.y1, B.sh1) : 0.0f;
    r.Y = make_float2(fmaf(r.Mi.m0, y0, r.Mi.m1 * y1), fmaf(r.Mi.m2, y0, r.Mi.m3 * y1));
    r.y = make_double2(P.y0, 2 * k + 1 < p.n ? P.y1 : 0.0);
    return r;
}

// Rows i0 = 2k, i0 + 1 of the rhs of system j (loaded by prep_row) -> the
// contiguous copy Yc, one 16-byte store where the pair is aligned.
__device__ __forceinline__ void store_rhs_pair(const MpArgs& p, int64_t j, int64_t i0, double2 y)
{
    const int64_t q = j * p.n + i0;
    if (i0 + 1 < p.n) {
        if ((q & 1) == 0) *reinterpret_cast<double2*>(p.Yc + q) = y;   // (Yc is 256-byte aligned)
        else { p.Yc[q] = y.x; p.Yc[q + 1] = y.y; }
    } else {
        p.Yc[q] = y.x;
    }
}

__device__ __forceinline__ void prep_store(const MpArgs& p, int64_t q, const PrepRow& r)
{
    // (the rhs copy Yc is written by the callers, which have y in hand)
    p.S0[2 * q] = make_float4(r.L.m0, r.L.m1, r.L.m2, r.L.m3);
    p.S0[2 * q + 1] = make_float4(r.U.m0, r.U.m1, r.U.m2, r.U.m3);
    p.Mi[q] = make_float4(r.Mi.m0, r.Mi.m1, r.Mi.m2, r.Mi.m3);
    p.R[0][q] = r.Y;
}

// per-system flags and norms of a solve
__global__ void __launch_bounds__(kMpThreads)
mp_init_kernel(MpArgs p)
{
    pdl_wait();
    pdl_release();
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, st = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = t0; j < p.m; j += st) { p.fin[j] = 0; p.status[j] = 0; p.est[j] = 0.0f; p.fail[j] = 0; }
    for (int64_t q = t0; q < (int64_t)kMpMaxPasses * p.m; q += st) p.trunc[q] = 0u;
    for (int64_t q = t0; q < (int64_t)(p.max_sweeps + 1) * p.m; q += st) { p.ndx[q] = 0u; p.nx[q] = 0u; }
    for (int64_t q = t0; q < (int64_t)p.max_sweeps * kMpMaxPasses * p.m; q += st) p.ndx_pre[q] = 0u;
    if (t0 == 0) { *p.nfail = 0; if (p.ctr) *p.ctr = 0; }
    for (int64_t q = t0; q <= p.max_sweeps; q += st) p.live[q] = (int)p.m;
    for (int64_t q = t0; q < 2 * p.m; q += st) p.dnorm[q] = 0u;
    if (t0 == 0 && p.err) *p.err = 0;
}

template <bool RG>
__global__ void __launch_bounds__(kMpThreads)
mp_prep_kernel(MpArgs p)
{
    pdl_wait();
    const int64_t nb = (p.n + 1) / 2;
    const int64_t total = p.m * nb;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = q / nb, k = q - j * nb;
        const PrepRow r = prep_row<RG>(p, j, k);
        prep_store(p, q, r);
        store_rhs_pair(p, j, 2 * k, r.y);
    }
    pdl_release();                                // (multi-wave grid: release once this CTA is done)
}

// ---------------------------------------------------------------------------
// FP32 block PCR pass (windows + halos at block level G, or whole subsystems)
// ---------------------------------------------------------------------------
// One window of a global FP32 block-PCR pass (K strides at level G, halo H).
// Each thread keeps the rows it owns (k = tid + q*blockDim) in registers;
// shared memory holds one copy of the level's rows (L and U as float4 arrays,
// Y as float2), read for the two neighbours of a row and rewritten after
// every stride: 80 bytes read and 40 written per row and stride.
template <int RPT>
__device__ __forceinline__ void mp_pass_item(const MpPassArgs& p, int64_t j, int64_t r, int64_t w,
                                             float4* sL, float4* sU, float2* sY, unsigned* s_max)
{
    const int64_t nb = p.nb;
    if (r >= nb) return;
    const int64_t nr = (nb - 1 - r) / p.G + 1;
    const int64_t wlo = w * (int64_t)p.L;
    if (wlo >= nr) return;
    const int64_t whi = min(wlo + (int64_t)p.L, nr);
    const int64_t t0 = max(wlo - (int64_t)p.H, (int64_t)0);
    const int64_t t1 = min(whi + (int64_t)p.H, nr);
    const int TR = (int)(t1 - t0);
    const int tid = threadIdx.x, bd = blockDim.x;
    const int64_t g0 = j * nb + r;                 // block row of local t = 0
    const int K = p.K;

    M2 Lr[RPT], Ur[RPT];
    float2 Yr[RPT];
#pragma unroll
    for (int q = 0; q < RPT; q++) {
        const int k = tid + q * bd;
        Lr[q] = {0.0f, 0.0f, 0.0f, 0.0f}; Ur[q] = Lr[q]; Yr[q] = make_float2(0.0f, 0.0f);
        if (k < TR) {
            const int64_t gi = g0 + (t0 + k) * p.G;
            const float4 lv = p.srcLU[2 * gi], uv = p.srcLU[2 * gi + 1];
            const float2 yv = p.srcY[gi];
            sL[k] = lv; sU[k] = uv; sY[k] = yv;
            Lr[q] = m2(lv); Ur[q] = m2(uv); Yr[q] = yv;
        }
    }
    if (tid == 0) s_max[0] = 0u;
    __syncthreads();

    for (int st = 0; st < K; st++) {
        const int dl = 1 << st;
        // rows this stride must produce: the window widened by the halo the
        // remaining strides of the pass still consume
        const int64_t rem = (int64_t(1) << K) - (int64_t(2) << st);   // block halo = 2^K - 1
        const int klo = (int)(max(wlo - rem, (int64_t)0) - t0);
        const int khi = (int)(min(whi + rem, nr) - t0);
        // A row without a neighbour at distance dl has exactly zero coupling
        // towards it (the boundary blocks are zero at level 0 and stay zero),
        // so the neighbour index is clamped into the tile instead of
        // branching: the clamped row is finite and enters multiplied by zero.
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            if (k >= klo && k < khi) {
                const int km = max(k - dl, 0), kp = min(k + dl, TR - 1);
                reduce_row(Lr[q], Ur[q], Yr[q], m2(sL[km]), m2(sU[km]), sY[km], m2(sL[kp]), m2(sU[kp]), sY[kp],
                           Lr[q], Ur[q], Yr[q]);
            }
        }
        __syncthreads();                                   // every read of this stride is done
        if (st == K - 1) break;
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            if (k >= klo && k < khi) { sL[k] = f4(Lr[q]); sU[k] = f4(Ur[q]); sY[k] = Yr[q]; }
        }
        __syncthreads();
    }

    float lmax = 0.0f;
#pragma unroll
    for (int q = 0; q < RPT; q++) {
        const int k = tid + q * bd;
        const int64_t t = t0 + k;
        if (k < TR && t >= wlo && t < whi) {
            const int64_t gi = g0 + t * p.G;
            p.dstLU[2 * gi] = f4(Lr[q]);
            p.dstLU[2 * gi + 1] = f4(Ur[q]);
            p.dstY[gi] = Yr[q];
            lmax = fmaxf(lmax, fmaxf(amaxm(Lr[q]), amaxm(Ur[q])));
        }
    }
    lmax = warp_max(lmax);
    if ((tid & 31) == 0) {
        atomic_max_pos(&p.trunc_out[j], lmax);
        atomic_max_pos(&s_max[0], lmax);
    }
    __syncthreads();
    // A window whose couplings all vanished is decoupled: its rows already
    // hold X = Y.  Write them now; if every window of the system is
    // decoupled the later passes of this sweep skip the system.
    if (__uint_as_float(s_max[0]) < kTrunc) {
        float xm = 0.0f;
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            const int64_t t = t0 + k;
            if (k < TR && t >= wlo && t < whi) {
                const int64_t i0 = 2 * (r + t * p.G);
                p.dx[j * p.n + i0] = Yr[q].x;
                xm = fmaxf(xm, fabsf(Yr[q].x));
                if (i0 + 1 < p.n) { p.dx[j * p.n + i0 + 1] = Yr[q].y; xm = fmaxf(xm, fabsf(Yr[q].y)); }
            }
        }
        xm = warp_max(xm);
        if ((tid & 31) == 0) atomic_max_pos(&p.ndx_pre_out[j], xm);
    }
}

// Loads rows [t0, t0 + TR) of subsystem r (level G) of system j into the
// swizzled tile.
__device__ __forceinline__ void cr_load(const MpPassArgs& p, int64_t j, int64_t r, int64_t t0, int TR,
                                        float4* sL, float4* sU, float2* sY)
{
    const int64_t g0 = j * p.nb + r;
    for (int k = threadIdx.x; k < TR; k += blockDim.x) {
        const int64_t gi = g0 + (t0 + k) * p.G;
        const int s = swz(k);
        sL[s] = p.srcLU[2 * gi]; sU[s] = p.srcLU[2 * gi + 1]; sY[s] = p.srcY[gi];
    }
    __syncthreads();
}

// dx rows of tile rows [klo, khi) (tile row k = subsystem row t0 + k of
// subsystem r at level G) and their |dx| maximum into *norm.
__device__ __forceinline__ void cr_store(const MpPassArgs& p, int64_t j, int64_t r, int64_t t0, int klo, int khi,
                                         const float2* sY, unsigned* norm)
{
    float xmx = 0.0f;
    for (int k = klo + threadIdx.x; k < khi; k += blockDim.x) {
        const int64_t i0 = 2 * (r + (t0 + k) * p.G);      // first row of the block row
        const float2 xv = sY[swz(k)];
        p.dx[j * p.n + i0] = xv.x;
        xmx = fmaxf(xmx, fabsf(xv.x));
        if (i0 + 1 < p.n) { p.dx[j * p.n + i0 + 1] = xv.y; xmx = fmaxf(xmx, fabsf(xv.y)); }
    }
    xmx = warp_max(xmx);
    if ((threadIdx.x & 31) == 0) atomic_max_pos(norm, xmx);
}

// A whole subsystem (nr <= TRmax rows at level G) by block cyclic reduction
// to the top (or until truncation) and back substitution: about 2 row
// updates per row instead of log2(nr).
__device__ __forceinline__ void mp_final_item(const MpPassArgs& p, int64_t j, int64_t r,
                                              float4* sL, float4* sU, float2* sY)
{
    if (r >= p.nb) return;
    const int nr = (int)((p.nb - 1 - r) / p.G + 1);
    cr_load(p, j, r, 0, nr, sL, sU, sY);
    const int top = cr_reduce(sL, sU, sY, nr, 31, 0, nr);   // never -1 on a whole subsystem
    cr_substitute(sL, sU, sY, nr, top);
    cr_store(p, j, r, 0, 0, nr, sY, &p.ndx[(int64_t)p.sweep * p.m + j]);
}

// Windowed truncated cyclic reduction at level 0 (the first pass of a large
// system): window [wlo, wlo + L) with a halo of H = 2^(K+1) rows each side.
// After l <= K levels the reduced rows the window depends on lie within
// 2^l - 1 rows of it and are exact when their own dependence (2^l - 1 rows
// further) is inside the tile; if they are decoupled, back substitution
// gives the window's dx with no other window involved.  Otherwise the system
// is marked for the general passes (block PCR windows + shared-memory
// finish) and the window writes nothing.
struct TryTile {
    int64_t j, wlo, whi, t0;
    int TR;
    bool whole;                                   // the tile holds the whole system
};

__device__ __forceinline__ TryTile try_tile(const MpPassArgs& p, int64_t item)
{
    TryTile t;
    t.j = item / p.nwin;
    const int64_t w = item - t.j * p.nwin;
    t.wlo = w * (int64_t)p.L;
    t.whi = min(t.wlo + (int64_t)p.L, p.nb);
    t.t0 = max(t.wlo - (int64_t)p.H, (int64_t)0);
    const int64_t t1 = min(t.whi + (int64_t)p.H, p.nb);
    t.TR = (int)(t1 - t.t0);
    t.whole = t.t0 == 0 && t1 == p.nb;
    return t;
}

// next item of this CTA with work: running system, window inside it, and
// (after sweep 0) a system the windowed pass solves
__device__ __forceinline__ int64_t try_next(const MpPassArgs& p, int64_t item, int64_t items)
{
    for (; item < items; item += gridDim.x) {
        const int64_t j = item / p.nwin;
        if (__ldg(p.fin + j)) continue;
        if (p.sweep > 0 && __ldg(p.fail + j)) continue;
        if ((item - j * p.nwin) * (int64_t)p.L >= p.nb) continue;
        break;
    }
    return item;
}

__device__ __forceinline__ void try_solve(const MpPassArgs& p, const TryTile& t, float4* sL, float4* sU, float2* sY)
{
    cr_load(p, t.j, 0, t.t0, t.TR, sL, sU, sY);
    // a tile holding the whole system needs no truncation: reduce to the top
    const int kmax = t.whole ? 31 : p.K;
    const int top = cr_reduce(sL, sU, sY, t.TR, kmax, (int)(t.wlo - t.t0), (int)(t.whi - t.t0));
    if (top < 0) {
        if (threadIdx.x == 0 && atomicOr(&p.fail[t.j], 1) == 0) atomicAdd(p.nfail, 1);
        return;
    }
    cr_substitute(sL, sU, sY, t.TR, top);
    // x_s = x_{s-1} + dx_s on the window's rows, straight from the tile.  The
    // norms go straight into the sweep's: if another window of the system
    // fails, the general passes redo these rows with values equal to within
    // the truncation, so the maxima stand either way.
    const int klo = (int)(t.wlo - t.t0), khi = (int)(t.whi - t.t0);
    float dmax = 0.0f;
    unsigned long long xbits = 0ull;
    for (int k = klo + threadIdx.x; k < khi; k += blockDim.x) {
        const int64_t i0 = 2 * (t.t0 + k);
        const float2 v = sY[swz(k)];
        if (i0 + 1 < p.n) {
            x_update_pair(p.xsrc, p.xsrc_ss, p.xsrc_rs, p.xsrc_rg, p.xdst, p.xdst_ss, p.xdst_rs, p.xdst_rg, t.j, i0,
                          v, dmax, xbits);
        } else {
            x_update(p.xsrc, p.xsrc_ss, p.xsrc_rs, p.xsrc_rg, p.xdst, p.xdst_ss, p.xdst_rs, p.xdst_rg, t.j, i0, v.x,
                     dmax, xbits);
        }
    }
    dmax = warp_max(dmax);
    const float xmax = warp_max(d2f_scaled(__longlong_as_double((long long)xbits), 0));
    if ((threadIdx.x & 31) == 0) {
        atomic_max_pos(&p.ndx[(int64_t)p.sweep * p.m + t.j], dmax);
        atomic_max_pos(&p.nx[t.j], xmax);
    }
}

// Persistent CTAs over the windows, 4 per SM (40 KB tiles of 1024 rows, at
// most 64 registers): the reduction levels are short dependent chains
// separated by barriers, so several tiles per SM keep it busy (5 per SM at
// 48 registers measured 1 % slower on GB300, 6 at 40 no faster).
__global__ void __launch_bounds__(kMpTryThreads, 4)
mp_try_kernel(MpPassArgs p)
{
    extern __shared__ float4 fsm[];
    pdl_wait();
    pdl_release();                                // one wave of persistent CTAs: the successor may queue now
    mp_resolve(p);
    if (p.skip0 && p.sweep == 0) return;          // sweep 0 ran in the fused kernel
    if (__ldg(p.live) == 0) return;               // every system finished in an earlier sweep
    const int TRs = mp_pass_rows(p.TRmax);
    float4* sL = fsm;
    float4* sU = fsm + TRs;
    float2* sY = reinterpret_cast<float2*>(fsm + 2 * TRs);
    const int64_t items = p.m * p.nwin;
    for (int64_t it = try_next(p, blockIdx.x, items); it < items; it = try_next(p, it + gridDim.x, items)) {
        try_solve(p, try_tile(p, it), sL, sU, sY);
        __syncthreads();
    }
}

// Sweep 0 fused (prep, windowed cyclic reduction and the first refinement),
// for windows that decouple (or hold the whole system).  Per window tile:
//  1. FP64 bands and y of the tile's block rows -> row-scaled, normalised FP32
//     blocks in shared memory; the window's own rows also go to S0, Mi and
//     R[0] for the later sweeps and the general passes;
//  2. cyclic reduction and back substitution (as mp_try_item): dx_0;
//  3. x_0 = dx_0 on the window's rows and one block row each side (exact
//     there: the valid region of the tile reaches 2 block rows beyond the
//     window), written to X[0]; norms of dx_0 and x_0;
//  4. r_0 = y - A x_0 in FP64 for the window's rows (bands and y read again,
//     from L2), row-scaled and normalised -> R[1].
// No decision is needed in sweep 0, so nothing waits for other windows.  A
// window whose system stays coupled marks it and stops after step 1; the
// general passes and the refinement kernel then take the whole system.
template <bool RG>
__device__ __forceinline__ void first_item(const MpArgs& p, const MpWindows& g, int64_t item,
                                           float4* sL, float4* sU, float2* sY)
{
    const int tid = threadIdx.x, bd = blockDim.x;
    const int64_t n = p.n, nb = (n + 1) / 2;
    const int64_t j = item / g.nwin, w = item - j * g.nwin;
    const int64_t wlo = w * (int64_t)g.L, whi = min(wlo + (int64_t)g.L, nb);
    const int64_t t0 = max(wlo - (int64_t)g.H, (int64_t)0), t1 = min(whi + (int64_t)g.H, nb);
    const int TR = (int)(t1 - t0);
    const bool whole = t0 == 0 && t1 == nb;

    for (int k = tid; k < TR; k += bd) {
        const int64_t kb = t0 + k;
        const PrepRow r = prep_row<RG>(p, j, kb, Keep::last);
        const int sk = swz(k);
        sL[sk] = f4(r.L); sU[sk] = f4(r.U); sY[sk] = r.Y;
        if (kb >= wlo && kb < whi) {
            prep_store(p, j * nb + kb, r);
            store_rhs_pair(p, j, 2 * kb, r.y);
        }
    }
    __syncthreads();
    const int klo = (int)(wlo - t0), khi = (int)(whi - t0);
    const int top = cr_reduce(sL, sU, sY, TR, whole ? 31 : g.K, klo, khi);
    if (top < 0) {
        if (tid == 0 && atomicOr(&p.fail[j], 1) == 0) atomicAdd(p.nfail, 1);
        return;
    }
    cr_substitute(sL, sU, sY, TR, top);           // ends with a barrier: the L slots are free

    // x_0 pairs, kept as double2 in the L slots for the residual's neighbours
    double2* sX = reinterpret_cast<double2*>(sL);
    const int xlo = max(klo - 1, 0), xhi = min(khi + 1, TR);
    float dmax = 0.0f;
    unsigned long long xbits = 0ull;
    for (int k = xlo + tid; k < xhi; k += bd) {
        const float2 v = sY[swz(k)];
        const double2 x = make_double2(f2d(v.x), f2d(v.y));
        sX[swz(k)] = x;
        if (k >= klo && k < khi) {
            const int64_t i0 = 2 * (t0 + k), q = j * n + i0;
            dmax = fmaxf(dmax, fabsf(v.x));
            xbits = max(xbits, (unsigned long long)__double_as_longlong(x.x) & 0x7FFFFFFFFFFFFFFFull);
            if (i0 + 1 < n) {
                if ((q & 1) == 0) *reinterpret_cast<double2*>(p.X0 + q) = x;   // (X0 is 256-byte aligned)
                else { p.X0[q] = x.x; p.X0[q + 1] = x.y; }
                dmax = fmaxf(dmax, fabsf(v.y));
                xbits = max(xbits, (unsigned long long)__double_as_longlong(x.y) & 0x7FFFFFFFFFFFFFFFull);
            } else {
                p.X0[q] = x.x;
            }
        }
    }
    dmax = warp_max(dmax);
    float xmax = warp_max(d2f_scaled(__longlong_as_double((long long)xbits), 0));
    if ((tid & 31) == 0) {
        atomic_max_pos(&p.ndx[j], dmax);
        atomic_max_pos(&p.nx[j], xmax);
    }
    __syncthreads();

    // r_0 = y - A x_0 on the window's block rows (FP64, same FMA order as the
    // refinement kernel), row-scaled and normalised -> the rhs of sweep 1
    for (int k = klo + tid; k < khi; k += bd) {
        const int64_t kb = t0 + k, i0 = 2 * kb;
        const PairRow P = load_pair<RG>(p, j, i0, Keep::first);
        const double2 xm = k > 0 ? sX[swz(k - 1)] : make_double2(0.0, 0.0);
        const double2 xc = sX[swz(k)];
        const double2 xp = k + 1 < TR ? sX[swz(k + 1)] : make_double2(0.0, 0.0);
        double r0 = P.y0;                          // row i0: x_{i0-2..i0+2} = xm.x xm.y xc.x xc.y xp.x
        r0 = fma(-P.c0, xc.x, r0);
        if (p.a && i0 >= 2) r0 = fma(-P.a0, xm.x, r0);
        if (i0 >= 1) r0 = fma(-P.b0, xm.y, r0);
        if (i0 + 1 < n) r0 = fma(-P.d0, xc.y, r0);
        if (p.e && i0 + 2 < n) r0 = fma(-P.e0, xp.x, r0);
        float rf1 = 0.0f;                          // row i0+1 (the identity row of an odd system: 0)
        if (i0 + 1 < n) {
            const int64_t i1 = i0 + 1;             // x_{i1-2..i1+2} = xm.y xc.x xc.y xp.x xp.y
            double r1 = P.y1;
            r1 = fma(-P.c1, xc.y, r1);
            if (p.a && i1 >= 2) r1 = fma(-P.a1, xm.y, r1);
            r1 = fma(-P.b1, xc.x, r1);
            if (i1 + 1 < n) r1 = fma(-P.d1, xp.x, r1);
            if (p.e && i1 + 2 < n) r1 = fma(-P.e1, xp.y, r1);
            rf1 = d2f_scaled(r1, d_exponent(P.c1));
        }
        const float rf0 = d2f_scaled(r0, d_exponent(P.c0));
        const float4 Mi = p.Mi[j * nb + kb];
        p.R[1][j * nb + kb] = make_float2(fmaf(Mi.x, rf0, Mi.y * rf1), fmaf(Mi.z, rf0, Mi.w * rf1));
    }
}

// Persistent CTAs over the windows of all systems (40 KB tiles of 1024
// block rows, or whole systems of up to 2048), 4 per SM at most.
template <bool RG>
__global__ void __launch_bounds__(kMpTryThreads, 4)
mp_first_kernel(MpArgs p, MpWindows g)
{
    extern __shared__ float4 fsm[];
    pdl_wait();
    pdl_release();                                // one wave of persistent CTAs: the successor may queue now
    const int TRs = mp_pass_rows(g.TRmax);
    float4* sL = fsm;
    float4* sU = fsm + TRs;
    float2* sY = reinterpret_cast<float2*>(fsm + 2 * TRs);
    if (__ldg(p.live) == 0) return;               // the fused first sweeps finished every system
    const int64_t items = p.m * g.nwin;
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        if (__ldg(p.fin + it / g.nwin)) continue;   // finished by the fused first sweeps
        first_item<RG>(p, g, it, sL, sU, sY);
        __syncthreads();
    }
}

// 4 CTAs per SM up to 4 rows per thread (64 registers, 40 KB of shared
// memory each at 1024 block rows), 2 beyond
template <int RPT>
__global__ void __launch_bounds__(kMpThreads, RPT >= 8 ? 2 : 4)
mp_pass_kernel(MpPassArgs p)
{
    extern __shared__ float4 fsm[];
    __shared__ unsigned s_max[1];
    pdl_wait();
    pdl_release();                                // one wave of persistent CTAs: the successor may queue now
    mp_resolve(p);
    // the flags read here were written by earlier kernels: read-only cache
    if (__ldg(p.live) == 0) return;               // every system finished in an earlier sweep
    if (p.fail && __ldg(p.nfail) == 0) return;    // the windowed pass solved every system
    const int TRs = mp_pass_rows(p.TRmax);
    float4* sL = fsm;
    float4* sU = fsm + TRs;
    float2* sY = reinterpret_cast<float2*>(fsm + 2 * TRs);
    // grid-stride over the items (about one wave of CTAs)
    const int64_t items = p.m * p.G * p.nwin;
    for (int64_t blk = blockIdx.x; blk < items; blk += gridDim.x) {
        const int64_t item = blk / p.nwin;
        const int64_t w = blk - item * p.nwin;
        const int64_t j = item / p.G;
        const int64_t r = item - j * p.G;
        if (__ldg(p.fin + j)) continue;
        if (p.fail && !__ldg(p.fail + j)) continue;   // solved by the windowed cyclic-reduction pass
        if (p.trunc_in && __uint_as_float(__ldg(p.trunc_in + j)) < kTrunc) {
            // Every window of the previous pass found itself decoupled and
            // wrote its rows of dx (X = Y): item (0, 0) carries the |dx|
            // maximum they left into the sweep's norm, the rest is skipped.
            if (r == 0 && w == 0 && threadIdx.x == 0)
                atomicMax(&p.ndx[(int64_t)p.sweep * p.m + j], p.ndx_pre_in[j]);
            continue;
        }
        if (p.final_step) mp_final_item(p, j, r, sL, sU, sY);
        else mp_pass_item<RPT>(p, j, r, w, sL, sU, sY, s_max);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// refinement: x_s = x_{s-1} + dx_s (FP64), decide, r_s = y - A x_s
// ---------------------------------------------------------------------------
// Iterates: sweep 0 writes x_0 to X0 (workspace), every later sweep reads
// x_{s-1} and writes x_s in the output (the caller's y, or Xout when the
// report keeps y): a system that finishes in sweep s already holds its
// answer there, and the rhs is read from the copy Yc.  The host passes each
// sweep's source and destination (xsrc, xdst with their strides).

// Systems whose dx came from the general passes (all of them when no cyclic-
// reduction pass ran): x_s = x_{s-1} + dx_s and max |x_s|.
__global__ void __launch_bounds__(kMpThreads)
mp_xupdate_kernel(MpArgs p)
{
    __shared__ float s_red[kMpThreads / 32];
    pdl_wait();
    pdl_release();                                // one wave of persistent CTAs: the successor may queue now
    mp_resolve(p);
    const int s = p.sweep;
    if (__ldg(p.live + s) == 0) return;           // every system finished in an earlier sweep
    if (p.cr_mode && __ldg(p.nfail) == 0) return; // the cyclic-reduction passes updated every system
    constexpr int XT = 4 * kMpThreads;            // rows per tile
    const int64_t n = p.n, tiles = (n + XT - 1) / XT;
    for (int64_t blk = blockIdx.x; blk < p.m * tiles; blk += gridDim.x) {
        const int64_t j = blk / tiles, t0 = (blk - j * tiles) * XT;
        if (__ldg(p.fin + j) != 0) continue;
        if (p.cr_mode && !__ldg(p.fail + j)) continue;
        float dmax = 0.0f;
        unsigned long long xbits = 0ull;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t i = t0 + threadIdx.x + u * kMpThreads;
            if (i < n) x_update(p.xsrc, p.xsrc_ss, p.xsrc_rs, p.xsrc_rg, p.xdst, p.xdst_ss, p.xdst_rs, p.xdst_rg, j,
                                i, p.dx[j * n + i], dmax, xbits);
        }
        float xmax = warp_max(d2f_scaled(__longlong_as_double((long long)xbits), 0));
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = xmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            float v = 0.0f;
            for (int w = 0; w < kMpThreads / 32; w++) v = fmaxf(v, s_red[w]);
            atomic_max_pos(&p.nx[(int64_t)s * p.m + j], v);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ UpDecision up_decide(const MpArgs& p, int64_t j)
{
    const int s = p.sweep;
    if (s < 1) return stop_rule(s, 0.0f, 0.0f, 0.0f, p.tol, p.max_sweeps);
    return stop_rule(s, __uint_as_float(p.ndx[(int64_t)s * p.m + j]),
                     __uint_as_float(p.ndx[(int64_t)(s - 1) * p.m + j]),
                     __uint_as_float(p.nx[(int64_t)(s - 1) * p.m + j]), p.tol, p.max_sweeps);
}

// One thread per system: a system that is done (or out of sweeps) finishes in
// sweep s; its answer is already in the output.
__global__ void __launch_bounds__(kMpThreads)
mp_decide_kernel(MpArgs p)
{
    pdl_wait();
    pdl_release();
    mp_resolve(p);
    const int s = p.sweep;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool finish = false;
    if (j < p.m && p.fin[j] == 0) {
        const UpDecision D = up_decide(p, j);
        if (D.last) {
            p.est[j] = D.est;
            p.status[j] = D.done ? 1 : 2;         // 2: stopped at max_sweeps
            p.fin[j] = s + 1;
            finish = true;
        }
    }
    const int cnt = __syncthreads_count(finish);
    if (threadIdx.x == 0 && cnt > 0)
        for (int s2 = s + 1; s2 <= p.max_sweeps; s2++) atomicSub(&p.live[s2], cnt);
}

// Systems that fit one shared-memory tile (every block row of a system in
// one CTA): all sweeps of a system run inside its CTA, so nothing waits for
// the rest of the batch between sweeps and the whole solve is one launch.
// Per system:
//  1. FP64 bands and y -> row-scaled, normalised FP32 blocks (prep_row): in
//     shared memory for the first solve, and in S0, Mi for the later ones;
//  2. per sweep: cyclic reduction to the top and back substitution (dx_s),
//     x_s = x_{s-1} + dx_s in FP64 (X0, contiguous), the maxima of |dx_s| and
//     |x_s| over the CTA, the stopping rule; if another sweep follows,
//     r_s = y - A x_s in FP64, row-scaled and normalised into the tile's rhs,
//     and the level-0 blocks back from S0 (the reduction overwrote them);
//  3. x -> the output, status, sweeps and estimate.
// y keeps the rhs until the final copy, so no copy of it is needed.
__device__ __forceinline__ void block_max(unsigned& dmb, unsigned long long& xb, unsigned* red_d,
                                          unsigned long long* red_x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dmb = max(dmb, __shfl_xor_sync(0xffffffffu, dmb, o));
        xb = max(xb, __shfl_xor_sync(0xffffffffu, xb, o));
    }
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) { red_d[w] = dmb; red_x[w] = xb; }
    __syncthreads();
    dmb = 0u; xb = 0ull;
    for (int k = 0; k < nw; k++) { dmb = max(dmb, red_d[k]); xb = max(xb, red_x[k]); }
    __syncthreads();                              // the scratch is reused by the next call
}

constexpr int kMpSmallThreadsMax = 512;          // systems of >= 1024 block rows: 512 threads

template <bool RG>
__global__ void __launch_bounds__(kMpSmallThreadsMax, 2)
mp_small_kernel(MpArgs p)
{
    extern __shared__ float4 fsm[];
    __shared__ unsigned red_d[kMpSmallThreadsMax / 32];
    __shared__ unsigned long long red_x[kMpSmallThreadsMax / 32];
    pdl_wait();
    pdl_release();
    const int64_t n = p.n, nb = (n + 1) / 2;
    const int TR = (int)nb, TRs = mp_pass_rows(TR);
    float4* sL = fsm;
    float4* sU = fsm + TRs;
    float2* sY = reinterpret_cast<float2*>(fsm + 2 * TRs);
    const int tid = threadIdx.x, bd = blockDim.x;
    for (int64_t j = blockIdx.x; j < p.m; j += gridDim.x) {
        double* __restrict__ X = p.X0 + j * n;
        for (int k = tid; k < TR; k += bd) {
            const PrepRow r = prep_row<RG>(p, j, k);
            const int64_t q = j * nb + k;
            p.S0[2 * q] = f4(r.L);
            p.S0[2 * q + 1] = f4(r.U);
            p.Mi[q] = f4(r.Mi);
            const int sk = swz(k);
            sL[sk] = f4(r.L); sU[sk] = f4(r.U); sY[sk] = r.Y;
        }
        __syncthreads();
        float ndp = 0.0f, nxp = 0.0f;
        UpDecision D{false, false, 0.0f};
        int s = 0;
        for (;; s++) {
            const int top = cr_reduce(sL, sU, sY, TR, 31, 0, TR);   // a whole system: never -1
            cr_substitute(sL, sU, sY, TR, top);
            unsigned dmb = 0u;
            unsigned long long xb = 0ull;
            for (int k = tid; k < TR; k += bd) {
                const float2 v = sY[swz(k)];
                const int64_t i0 = 2 * (int64_t)k;
                const double x0 = s ? __dadd_rn(X[i0], f2d(v.x)) : f2d(v.x);
                X[i0] = x0;
                dmb = max(dmb, __float_as_uint(fabsf(v.x)));
                xb = max(xb, absbits(x0));
                if (i0 + 1 < n) {
                    const double x1 = s ? __dadd_rn(X[i0 + 1], f2d(v.y)) : f2d(v.y);
                    X[i0 + 1] = x1;
                    dmb = max(dmb, __float_as_uint(fabsf(v.y)));
                    xb = max(xb, absbits(x1));
                }
            }
            block_max(dmb, xb, red_d, red_x);     // (its barriers also publish X to the CTA)
            // non-negative floats order like their bits, a nan above everything
            const float nd = __uint_as_float(dmb);
            const float nx = d2f_scaled(__longlong_as_double((long long)xb), 0);
            D = stop_rule(s, nd, ndp, nxp, p.tol, p.max_sweeps);
            if (D.last) break;
            ndp = nd; nxp = nx;
            for (int k = tid; k < TR; k += bd) {
                const int64_t i0 = 2 * (int64_t)k, q = j * nb + k;
                const PairRow P = load_pair<RG>(p, j, i0);
                const double xm2 = i0 >= 2 ? X[i0 - 2] : 0.0, xm1 = i0 >= 1 ? X[i0 - 1] : 0.0, x0 = X[i0];
                const double x1 = i0 + 1 < n ? X[i0 + 1] : 0.0, x2 = i0 + 2 < n ? X[i0 + 2] : 0.0;
                const double x3 = i0 + 3 < n ? X[i0 + 3] : 0.0;
                double r0 = fma(-P.c0, x0, P.y0);
                if (p.a && i0 >= 2) r0 = fma(-P.a0, xm2, r0);
                if (i0 >= 1) r0 = fma(-P.b0, xm1, r0);
                if (i0 + 1 < n) r0 = fma(-P.d0, x1, r0);
                if (p.e && i0 + 2 < n) r0 = fma(-P.e0, x2, r0);
                const float rf0 = d2f_scaled(r0, d_exponent(P.c0));
                float rf1 = 0.0f;                 // the identity row of an odd system's last block row
                if (i0 + 1 < n) {
                    double r1 = fma(-P.c1, x1, P.y1);
                    if (p.a && i0 >= 1) r1 = fma(-P.a1, xm1, r1);
                    r1 = fma(-P.b1, x0, r1);
                    if (i0 + 2 < n) r1 = fma(-P.d1, x2, r1);
                    if (p.e && i0 + 3 < n) r1 = fma(-P.e1, x3, r1);
                    rf1 = d2f_scaled(r1, d_exponent(P.c1));
                }
                const float4 Mi = p.Mi[q];
                const int sk = swz(k);
                sY[sk] = make_float2(fmaf(Mi.x, rf0, Mi.y * rf1), fmaf(Mi.z, rf0, Mi.w * rf1));
                sL[sk] = p.S0[2 * q];
                sU[sk] = p.S0[2 * q + 1];
            }
            __syncthreads();
        }
        for (int64_t i = tid; i < n; i += bd) x_write(p.xout, p.oss, p.ors, RG ? p.rg : nullptr, j, i, X[i]);
        if (tid == 0) { p.fin[j] = s + 1; p.status[j] = D.done ? 1 : 2; p.est[j] = D.est; }
        __syncthreads();                          // the next system reuses the tile
    }
}

// r_s = y - A x_s (FP64, FMA chain) for the systems still running, row-scaled
// to FP32 by the power of two of the main diagonal; the odd row of a block
// row reaches the even lane by a shuffle, which normalises the pair by the
// block's diagonal inverse -> R[(s+1) & 1], the rhs of sweep s+1.
template <bool RG>
__device__ __forceinline__ void residual_tile(const MpArgs& p, int s, const double* __restrict__ x, int64_t xss,
                                              int64_t xrs, const longlong2* xrg, int64_t j, int64_t tile, double* sx)
{
    const int tid = threadIdx.x;
    const int64_t n = p.n;
    constexpr int XR = kMpTile / kMpThreads;             // rows per thread
    const int64_t t0 = tile * kMpTile, t1 = min(t0 + kMpTile, n);
    const int64_t ih = tid < 2 ? t0 - 2 + tid : t1 + tid - 2;          // halo row of threads 0-3
    const bool halo = tid < 4 && ih >= 0 && ih < n;
    // the system's rows in the caller arrays (a ragged system ends at nj <= n:
    // identity rows beyond, and its slots coupling to them are zero)
    int64_t base = j * p.ss, rs = p.rs, nj = n;
    if (RG) { const longlong2 g = __ldg(p.rg + j); base = g.x; rs = 1; nj = g.y; }
    else xrg = nullptr;
    double ba[XR], bb[XR], bc[XR], bd[XR], be[XR], by[XR];
#pragma unroll
    for (int u = 0; u < XR; u++) {
        const int64_t i = t0 + tid + u * kMpThreads;
        ba[u] = 0.0; bb[u] = 0.0; bc[u] = 1.0; bd[u] = 0.0; be[u] = 0.0; by[u] = 0.0;
        if (i < t1) {
            if (i < nj) {
                const int64_t g = base + i * rs;
                ba[u] = p.a ? p.a[g] : 0.0; bb[u] = p.b[g]; bc[u] = p.c[g];
                if (i + 1 < nj) bd[u] = p.d[g];
                if (p.e && i + 2 < nj) be[u] = p.e[g];
            }
            by[u] = p.Yc[j * n + i];
            sx[tid + u * kMpThreads + 2] = x_read(x, xss, xrs, xrg, j, i);
        }
    }
    if (halo) sx[ih - t0 + 2] = x_read(x, xss, xrs, xrg, j, ih);
    __syncthreads();

    const int64_t nb = (n + 1) / 2;
    const bool interior = t0 >= 2 && t1 + 2 <= n;          // no band slot of the tile falls outside the system
#pragma unroll
    for (int u = 0; u < XR; u++) {
        const int r0 = tid + u * kMpThreads;               // row within the tile (even lanes: first row of a block row)
        const int64_t i = t0 + r0;
        const bool even = (r0 & 1) == 0;
        float4 Mi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (even && i < t1) Mi = p.Mi[j * nb + (i >> 1)];
        float rf = 0.0f;
        if (i < t1) {
            const int li = r0 + 2;
            double r = by[u];
            r = fma(-bc[u], sx[li], r);
            if (interior) {
                if (p.a) r = fma(-ba[u], sx[li - 2], r);
                r = fma(-bb[u], sx[li - 1], r);
                r = fma(-bd[u], sx[li + 1], r);
                if (p.e) r = fma(-be[u], sx[li + 2], r);
            } else {
                if (p.a && i >= 2) r = fma(-ba[u], sx[li - 2], r);
                if (i >= 1) r = fma(-bb[u], sx[li - 1], r);
                if (i + 1 < n) r = fma(-bd[u], sx[li + 1], r);
                if (p.e && i + 2 < n) r = fma(-be[u], sx[li + 2], r);
            }
            rf = d2f_scaled(r, d_exponent(bc[u]));
        }
        // (the partner of row n-1 of an odd system is the identity row of the
        // padded block, r = 0: its lane lies past t1 and keeps rf = 0)
        const float rf1 = __shfl_xor_sync(0xffffffffu, rf, 1);
        if (even && i < t1)
            p.R[(s + 1) & 1][j * nb + (i >> 1)] = make_float2(fmaf(Mi.x, rf, Mi.y * rf1), fmaf(Mi.z, rf, Mi.w * rf1));
    }
}

// 5 CTAs per SM (at most 51 registers)
template <bool RG>
__global__ void __launch_bounds__(kMpThreads, 5)
mp_residual_kernel(MpArgs p)
{
    __shared__ double sx[kMpTile + 4];
    pdl_wait();
    pdl_release();                                // one wave of persistent CTAs: the successor may queue now
    // (resolved into locals: the argument block itself stays read-only)
    const int s = p.ctr ? *p.ctr : p.sweep;
    const double* x = p.xdst;
    int64_t xss = p.xdst_ss, xrs = p.xdst_rs;
    const longlong2* xrg = p.xdst_rg;
    if (p.ctr) {
        const XView v = x_view(s, p.max_sweeps, p.X0, p.xout, p.n, p.oss, p.ors, p.rg);
        x = v.dst; xss = v.dss; xrs = v.drs; xrg = v.drg;
    }
    if (__ldg(p.live + s + 1) == 0) return;       // every system has finished
    const bool fused0 = p.first_fused && s == 0;  // the fused sweep 0 formed r_0 of the systems it solved
    if (fused0 && __ldg(p.nfail) == 0) return;
    const int64_t tiles = (p.n + kMpTile - 1) / kMpTile;
    for (int64_t blk = blockIdx.x; blk < p.m * tiles; blk += gridDim.x) {
        const int64_t j = blk / tiles;
        if (__ldg(p.fin + j) != 0) continue;
        if (fused0 && !__ldg(p.fail + j)) continue;
        residual_tile<RG>(p, s, x, xss, xrs, xrg, j, blk - j * tiles, sx);
        __syncthreads();
    }
}

// End of a graph-driven sweep: advance the counter and tell the enclosing
// while node whether another sweep runs (a sweep remains and a system is
// still running).
__global__ void mp_advance_kernel(MpArgs p, cudaGraphConditionalHandle h)
{
    pdl_wait();
    const int s = *p.ctr + 1;
    *p.ctr = s;
    cudaGraphSetConditional(h, (s < p.max_sweeps && p.live[s] > 0) ? 1u : 0u);
}

// r = y - A x (FP64 FMA chain; a null outer band is zero).  Bands and y use the caller's layout (ss, rs);
// x and r use (xss, xrs).
__global__ void __launch_bounds__(kMpThreads)
residual_kernel(const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                const double* __restrict__ d, const double* __restrict__ e, const double* __restrict__ y,
                const double* __restrict__ x, double* __restrict__ r, int64_t m, int64_t n, int64_t ss, int64_t rs,
                int64_t xss, int64_t xrs)
{
    const int64_t total = m * n;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        int64_t j, i;
        if (rs == 1) { j = q / n; i = q - j * n; } else { i = q / m; j = q - i * m; }
        const int64_t g = j * ss + i * rs;
        const int64_t gx = j * xss + i * xrs;
        double v = y[g];
        v = fma(-c[g], x[gx], v);
        if (a && i >= 2) v = fma(-a[g], x[gx - 2 * xrs], v);
        if (i >= 1) v = fma(-b[g], x[gx - xrs], v);
        if (i + 1 < n) v = fma(-d[g], x[gx + xrs], v);
        if (e && i + 2 < n) v = fma(-e[g], x[gx + 2 * xrs], v);
        r[gx] = v;
    }
}

// x (workspace, contiguous) -> y (caller layout)
__global__ void copy_out_kernel(const double* __restrict__ X, double* __restrict__ y, int64_t m, int64_t n,
                                int64_t ss, int64_t rs)
{
    const int64_t total = m * n;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = q / n, i = q - j * n;
        y[j * ss + i * rs] = X[q];
    }
}

// Per system: max |r_i|, max_i sum_k |A_ik| and max |x_i| (float bit patterns).
// X and r are contiguous; the bands use the caller's layout.
__global__ void __launch_bounds__(kMpThreads)
resid_norm_kernel(const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                  const double* __restrict__ d, const double* __restrict__ e,
                  const double* __restrict__ X, const double* __restrict__ r, int64_t m, int64_t n,
                  int64_t ss, int64_t rs, unsigned* __restrict__ rn, unsigned* __restrict__ an,
                  unsigned* __restrict__ xn)
{
    const int64_t tiles = (n + 1023) / 1024;
    const int64_t j = blockIdx.x / tiles, tile = blockIdx.x - j * tiles;
    float rm = 0.0f, am = 0.0f, xm = 0.0f;
    const int64_t iend = min((tile + 1) * 1024, n);
    for (int64_t i = tile * 1024 + threadIdx.x; i < iend; i += blockDim.x) {
        const int64_t g = j * ss + i * rs;
        double rowsum = fabs(c[g]);
        if (a && i >= 2) rowsum += fabs(a[g]);
        if (i >= 1) rowsum += fabs(b[g]);
        if (i + 1 < n) rowsum += fabs(d[g]);
        if (e && i + 2 < n) rowsum += fabs(e[g]);
        rm = fmaxf(rm, (float)fabs(r[j * n + i]));
        am = fmaxf(am, (float)rowsum);
        xm = fmaxf(xm, (float)fabs(X[j * n + i]));
    }
    rm = warp_max(rm); am = warp_max(am); xm = warp_max(xm);
    if ((threadIdx.x & 31) == 0) {
        atomic_max_pos(&rn[j], rm); atomic_max_pos(&an[j], am); atomic_max_pos(&xn[j], xm);
    }
}

// shared memory of the pass kernel: L, U (float4) and Y (float2) per block row
size_t mp_pass_smem(int rows) { return (size_t)mp_pass_rows(rows) * (2 * sizeof(float4) + sizeof(float2)); }

template <int RPT>
cudaError_t launch_mp_pass_rpt(const MpPassArgs& p, int threads, int64_t blocks, cudaStream_t s)
{
    const size_t smem = mp_pass_smem(p.TRmax);
    cudaError_t e = cudaFuncSetAttribute(mp_pass_kernel<RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mp_pass_smem(kMpMaxRows));
    if (e != cudaSuccess) return e;
    blocks = std::min<int64_t>(blocks, mp_grid_cap((const void*)mp_pass_kernel<RPT>, threads, smem));
    e = launch_dependent(mp_pass_kernel<RPT>, (unsigned)blocks, threads, smem, s, p);
    count_launch();
    return e;
}

}  // namespace

cudaError_t launch_mp_init(const MpArgs& p, cudaStream_t s)
{
    const cudaError_t e = launch_dependent(mp_init_kernel, 152u * 2, kMpThreads, 0, s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_first(const MpArgs& p, const MpWindows& g, cudaStream_t s)
{
    if (g.TRmax > kMpMaxRows) return cudaErrorInvalidValue;
    const int64_t items = p.m * g.nwin;
    if (items <= 0) return cudaSuccess;
    const size_t smem = mp_pass_smem(g.TRmax);
    auto kern = p.rg ? mp_first_kernel<true> : mp_first_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mp_pass_smem(kMpMaxRows));
    if (e != cudaSuccess) return e;
    const int64_t blocks = std::min<int64_t>(items, mp_grid_cap((const void*)kern, kMpTryThreads, smem));
    e = launch_dependent(kern, (unsigned)blocks, kMpTryThreads, smem, s, p, g);
    count_launch();
    return e;
}

cudaError_t launch_mp_prep(const MpArgs& p, cudaStream_t s)
{
    const int64_t nb = (p.n + 1) / 2;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((p.m * nb + kMpThreads - 1) / kMpThreads, 152 * 16));
    const cudaError_t e = launch_dependent(p.rg ? mp_prep_kernel<true> : mp_prep_kernel<false>, (unsigned)blocks,
                                           kMpThreads, 0, s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_pass(const MpPassArgs& p, cudaStream_t s)
{
    if (p.TRmax > kMpMaxRows) return cudaErrorInvalidValue;
    int threads = kMpThreads;
    if (p.TRmax < threads) threads = std::max(32, (p.TRmax + 31) / 32 * 32);
    const int rpt = (p.TRmax + threads - 1) / threads;
    const int64_t items = p.m * p.G * p.nwin;
    if (items <= 0) return cudaSuccess;
    const int64_t blocks = items;
    if (rpt <= 1) return launch_mp_pass_rpt<1>(p, threads, blocks, s);
    if (rpt <= 2) return launch_mp_pass_rpt<2>(p, threads, blocks, s);
    if (rpt <= 4) return launch_mp_pass_rpt<4>(p, threads, blocks, s);
    if (rpt <= 8) return launch_mp_pass_rpt<8>(p, threads, blocks, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_mp_try(const MpPassArgs& p, cudaStream_t s)
{
    if (p.TRmax > kMpMaxRows) return cudaErrorInvalidValue;
    const int64_t items = p.m * p.nwin;
    if (items <= 0) return cudaSuccess;
    const size_t smem = mp_pass_smem(p.TRmax);
    cudaError_t e = cudaFuncSetAttribute(mp_try_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mp_pass_smem(kMpMaxRows));
    if (e != cudaSuccess) return e;
    const int64_t blocks = std::min<int64_t>(items, mp_grid_cap((const void*)mp_try_kernel, kMpTryThreads, smem));
    e = launch_dependent(mp_try_kernel, (unsigned)blocks, kMpTryThreads, smem, s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_small(const MpArgs& p, cudaStream_t s)
{
    const int64_t nb = (p.n + 1) / 2;
    if (nb > kMpMaxRows) return cudaErrorInvalidValue;
    if (p.m <= 0) return cudaSuccess;
    const size_t smem = mp_pass_smem((int)nb);
    auto kern = p.rg ? mp_small_kernel<true> : mp_small_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mp_pass_smem(kMpMaxRows));
    if (e != cudaSuccess) return e;
    // large tiles hold two CTAs per SM (shared memory): twice the threads per
    // CTA keep as many warps resident as four CTAs of small tiles; systems of
    // fewer than 256 block rows get one thread per block row (whole warps),
    // so small systems fill the SM with more CTAs instead of idle threads
    const int threads = nb >= 1024 ? kMpSmallThreadsMax
                        : nb >= kMpThreads ? kMpThreads : (int)std::max<int64_t>(32, (nb + 31) / 32 * 32);
    const int64_t blocks = std::min<int64_t>(p.m, mp_grid_cap((const void*)kern, threads, smem));
    e = launch_dependent(kern, (unsigned)blocks, threads, smem, s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_xupdate(const MpArgs& p, cudaStream_t s)
{
    const int64_t tiles = (p.n + 4 * kMpThreads - 1) / (4 * kMpThreads);
    const int64_t blocks = std::min<int64_t>(p.m * tiles, mp_grid_cap((const void*)mp_xupdate_kernel, kMpThreads, 0));
    const cudaError_t e = launch_dependent(mp_xupdate_kernel, (unsigned)blocks, kMpThreads, 0, s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_decide(const MpArgs& p, cudaStream_t s)
{
    const int64_t blocks = (p.m + kMpThreads - 1) / kMpThreads;
    const cudaError_t e = launch_dependent(mp_decide_kernel, (unsigned)blocks, kMpThreads, 0, s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_residual(const MpArgs& p, cudaStream_t s)
{
    // one wave of CTAs striding over the tiles: a sweep after which every
    // system has finished returns at once through the live count
    const int64_t tiles = (p.n + kMpTile - 1) / kMpTile;
    auto kern = p.rg ? mp_residual_kernel<true> : mp_residual_kernel<false>;
    const int64_t blocks = std::min<int64_t>(p.m * tiles, mp_grid_cap((const void*)kern, kMpThreads, 0));
    const cudaError_t e = launch_dependent(kern, (unsigned)blocks, kMpThreads, 0, s, p);
    count_launch();
    return e;
}

cudaError_t launch_mp_advance(const MpArgs& p, cudaGraphConditionalHandle h, cudaStream_t s)
{
    const cudaError_t e = launch_dependent(mp_advance_kernel, 1u, 1u, 0, s, p, h);
    count_launch();
    return e;
}

cudaError_t launch_residual(const double* a, const double* b, const double* c, const double* d, const double* e,
                            const double* y, const double* x, double* r, int64_t m, int64_t n, int64_t ss,
                            int64_t rs, int64_t xss, int64_t xrs, cudaStream_t s)
{
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((m * n + kMpThreads - 1) / kMpThreads, 152 * 16));
    residual_kernel<<<(unsigned)blocks, kMpThreads, 0, s>>>(a, b, c, d, e, y, x, r, m, n, ss, rs, xss, xrs);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_copy_out(const double* X, double* y, int64_t m, int64_t n, int64_t ss, int64_t rs, cudaStream_t s)
{
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((m * n + kMpThreads - 1) / kMpThreads, 152 * 16));
    copy_out_kernel<<<(unsigned)blocks, kMpThreads, 0, s>>>(X, y, m, n, ss, rs);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_resid_norm(const double* a, const double* b, const double* c, const double* d, const double* e,
                              const double* X, const double* r, int64_t m, int64_t n, int64_t ss,
                              int64_t rs, unsigned* rn, unsigned* an, unsigned* xn, cudaStream_t s)
{
    const int64_t blocks = m * ((n + 1023) / 1024);
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    resid_norm_kernel<<<(unsigned)blocks, kMpThreads, 0, s>>>(a, b, c, d, e, X, r, m, n, ss, rs, rn, an, xn);
    count_launch();
    return cudaGetLastError();
}

}  // namespace pcrp
