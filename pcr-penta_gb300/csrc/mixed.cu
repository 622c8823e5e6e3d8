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

namespace pcrp {
namespace {

constexpr float kTrunc = 1e-10f;
constexpr int kMpThreads = 256;
static_assert(kMpTile % kMpThreads == 0 && kMpThreads % 2 == 0, "refinement tiles: whole rows per thread, pairs in adjacent lanes");
// CTAs of one wave of a kernel (the pass kernel strides over its items with
// one wave, so that sweeps of mostly finished systems stay cheap)
int mp_grid_cap(const void* kernel, int threads, size_t smem)
{
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152 * 2;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 152 * 2;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1) per = 1;
    return sms * per;
}

// ---------------------------------------------------------------------------
// integer-pipe conversions
// ---------------------------------------------------------------------------

// Exponent e of |v| in [2^e, 2^(e+1)); 0 for zero, subnormal, inf, nan.
__device__ __forceinline__ int d_exponent(double v) {
    const int E = (int)((__double_as_longlong(v) >> 52) & 0x7FF);
    return (E == 0 || E == 0x7FF) ? 0 : E - 1023;
}

// (float)(v * 2^-sh), rounded to nearest (ties away), flushing results below
// FLT_MIN to zero and saturating to inf; integer arithmetic only.
__device__ __forceinline__ float d2f_scaled(double v, int sh) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(bits >> 63) << 31;
    const int E = (int)((bits >> 52) & 0x7FF);
    if (E == 0) return __uint_as_float(sign);                      // zero / subnormal
    if (E == 0x7FF) {                                               // inf / nan
        const unsigned nan = (bits & 0xFFFFFFFFFFFFFULL) ? 0x400000u : 0u;
        return __uint_as_float(sign | 0x7F800000u | nan);
    }
    const int F = E - sh - 1023 + 127;
    if (F <= 0) return __uint_as_float(sign);
    if (F >= 255) return __uint_as_float(sign | 0x7F800000u);
    const unsigned long long mant = bits & 0xFFFFFFFFFFFFFULL;
    unsigned u = ((unsigned)F << 23) + (unsigned)(mant >> 29) + (unsigned)((mant >> 28) & 1);
    if (u >= 0x7F800000u) u = 0x7F800000u;
    return __uint_as_float(sign | u);
}

// Exact (double)f for normal floats; subnormals flush to zero.
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned E = (u >> 23) & 0xFF;
    if (E == 0) return __longlong_as_double((long long)sign);
    if (E == 0xFF) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ULL |
                                                           ((unsigned long long)(u & 0x7FFFFF) << 29)));
    return __longlong_as_double((long long)(sign | ((unsigned long long)(E - 127 + 1023) << 52) |
                                            ((unsigned long long)(u & 0x7FFFFF) << 29)));
}

__device__ __forceinline__ void atomic_max_pos(unsigned* addr, float v) {
    // non-negative floats order like their bit patterns
    if (v > 0.0f) atomicMax(addr, __float_as_uint(v));
    else if (!(v >= 0.0f)) atomicMax(addr, 0x7FC00000u);   // nan poisons the norm
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ---------------------------------------------------------------------------
// 2x2 helpers (row-major m[0] m[1] / m[2] m[3])
// ---------------------------------------------------------------------------
struct M2 { float m0, m1, m2, m3; };

__device__ __forceinline__ M2 mmul(const M2& A, const M2& B) {
    return {fmaf(A.m0, B.m0, A.m1 * B.m2), fmaf(A.m0, B.m1, A.m1 * B.m3),
            fmaf(A.m2, B.m0, A.m3 * B.m2), fmaf(A.m2, B.m1, A.m3 * B.m3)};
}

__device__ __forceinline__ M2 minv(const M2& D) {
    const float det = fmaf(D.m0, D.m3, -D.m1 * D.m2);
    const float r = __fdividef(1.0f, det);
    return {D.m3 * r, -D.m1 * r, -D.m2 * r, D.m0 * r};
}

// The six FP64 values of rows i0 = 2k and i1 = 2k+1 of one system (i1 may be
// the dummy row n of an odd system).  Contiguous pairs at an even element
// offset are read as one 16-byte load per array.
struct PairRow { double a0, a1, b0, b1, c0, c1, d0, d1, e0, e1, y0, y1; };

__device__ __forceinline__ PairRow load_pair(const MpArgs& p, int64_t base, int64_t i0)
{
    PairRow P;
    const int64_t n = p.n, rs = p.rs;
    const int64_t g0 = base + i0 * rs;
    if (p.vec && rs == 1 && ((g0 & 1) == 0) && i0 + 1 < n) {
        const double2 a = *reinterpret_cast<const double2*>(p.a + g0);
        const double2 b = *reinterpret_cast<const double2*>(p.b + g0);
        const double2 c = *reinterpret_cast<const double2*>(p.c + g0);
        const double2 d = *reinterpret_cast<const double2*>(p.d + g0);
        const double2 e = *reinterpret_cast<const double2*>(p.e + g0);
        const double2 y = *reinterpret_cast<const double2*>(p.y + g0);
        P = {a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x, e.y, y.x, y.y};
    } else {
        P.a0 = p.a[g0]; P.b0 = p.b[g0]; P.c0 = p.c[g0]; P.d0 = p.d[g0]; P.e0 = p.e[g0]; P.y0 = p.y[g0];
        if (i0 + 1 < n) {
            const int64_t g1 = g0 + rs;
            P.a1 = p.a[g1]; P.b1 = p.b[g1]; P.c1 = p.c[g1]; P.d1 = p.d[g1]; P.e1 = p.e[g1]; P.y1 = p.y[g1];
        } else {
            P.a1 = 0.0; P.b1 = 0.0; P.c1 = 1.0; P.d1 = 0.0; P.e1 = 0.0; P.y1 = 0.0;
        }
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
__global__ void __launch_bounds__(kMpThreads)
mp_prep_kernel(MpArgs p)
{
    const int64_t nb = (p.n + 1) / 2;
    const int64_t total = p.m * nb;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = q / nb, k = q - j * nb;
        const int64_t base = j * p.ss;
        const PairRow P = load_pair(p, base, 2 * k);
        const BlockRow B = block_of(P, 2 * k, p.n);
        const M2 Mi = minv(B.D);
        const M2 L = mmul(Mi, B.L), U = mmul(Mi, B.U);
        const float y0 = d2f_scaled(P.y0, B.sh0);
        const float y1 = 2 * k + 1 < p.n ? d2f_scaled(P.y1, B.sh1) : 0.0f;
        p.S0[2 * q] = make_float4(L.m0, L.m1, L.m2, L.m3);
        p.S0[2 * q + 1] = make_float4(U.m0, U.m1, U.m2, U.m3);
        p.R[q] = make_float2(fmaf(Mi.m0, y0, Mi.m1 * y1), fmaf(Mi.m2, y0, Mi.m3 * y1));
    }
    if (blockIdx.x == 0) {
        for (int64_t j = threadIdx.x; j < p.m; j += blockDim.x) {
            p.fin[j] = 0; p.status[j] = 0; p.est[j] = 0.0f;
        }
        for (int64_t q = threadIdx.x; q < (int64_t)kMpMaxPasses * p.m; q += blockDim.x) p.trunc[q] = 0u;
        for (int64_t q = threadIdx.x; q < (int64_t)(p.max_sweeps + 1) * p.m; q += blockDim.x) {
            p.ndx[q] = 0u; p.nx[q] = 0u;
        }
        for (int64_t q = threadIdx.x; q < (int64_t)p.max_sweeps * kMpMaxPasses * p.m; q += blockDim.x)
            p.ndx_pre[q] = 0u;
        for (int q = threadIdx.x; q <= p.max_sweeps; q += blockDim.x) p.live[q] = (int)p.m;
    }
}

// ---------------------------------------------------------------------------
// FP32 block PCR pass (windows + halos at block level G, or whole subsystems)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float amaxm(const M2& a) {
    return fmaxf(fmaxf(fabsf(a.m0), fabsf(a.m1)), fmaxf(fabsf(a.m2), fabsf(a.m3)));
}
__device__ __forceinline__ M2 m2(const float4& v) { return {v.x, v.y, v.z, v.w}; }
__device__ __forceinline__ float4 f4(const M2& a) { return make_float4(a.m0, a.m1, a.m2, a.m3); }

// One window (or whole subsystem) of one FP32 block-PCR pass.  Each thread
// keeps the rows it owns (k = tid + q*blockDim) in registers; shared memory
// holds one copy of the level's rows (L and U as float4 arrays, Y as float2),
// read for the two neighbours of a row and rewritten after every stride:
// 80 bytes read and 40 written per row and stride, conflict-free.
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
    if (tid == 0) { s_max[0] = 0u; s_max[1] = 0u; s_max[2] = 0u; }
    __syncthreads();

    for (int st = 0; st < K; st++) {
        const int dl = 1 << st;
        int64_t rlo, rhi;
        if (p.final_step) { rlo = 0; rhi = nr; }
        else {
            const int64_t rem = (int64_t(1) << p.K) - (int64_t(2) << st);   // block halo = 2^K - 1
            rlo = max(wlo - rem, (int64_t)0); rhi = min(whi + rem, nr);
        }
        // Rows [klo, khi) (local k = t - t0) are computed.  A row without a
        // neighbour at distance dl has exactly zero coupling towards it (the
        // boundary blocks are zero at level 0 and stay zero), so the
        // neighbour index is clamped into the tile instead of branching: the
        // clamped row is finite and enters multiplied by zero.
        const int klo = (int)(rlo - t0), khi = (int)(rhi - t0);
        float lmax = 0.0f;
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            if (k >= klo && k < khi) {
                const M2 Lk = Lr[q], Uk = Ur[q];
                const int km = max(k - dl, 0), kp = min(k + dl, TR - 1);
                const M2 Lm = m2(sL[km]), Um = m2(sU[km]), Lp = m2(sL[kp]), Up = m2(sU[kp]);
                const float2 ym = sY[km], yp = sY[kp];
                // D' = I - L_k U_{k-d} - U_k L_{k+d}
                M2 Dn;
                Dn.m0 = fmaf(-Uk.m1, Lp.m2, fmaf(-Uk.m0, Lp.m0, fmaf(-Lk.m1, Um.m2, fmaf(-Lk.m0, Um.m0, 1.0f))));
                Dn.m1 = fmaf(-Uk.m1, Lp.m3, fmaf(-Uk.m0, Lp.m1, fmaf(-Lk.m1, Um.m3, -Lk.m0 * Um.m1)));
                Dn.m2 = fmaf(-Uk.m3, Lp.m2, fmaf(-Uk.m2, Lp.m0, fmaf(-Lk.m3, Um.m2, -Lk.m2 * Um.m0)));
                Dn.m3 = fmaf(-Uk.m3, Lp.m3, fmaf(-Uk.m2, Lp.m1, fmaf(-Lk.m3, Um.m3, fmaf(-Lk.m2, Um.m1, 1.0f))));
                // Y' = Y_k - L_k Y_{k-d} - U_k Y_{k+d}
                const float y0 = fmaf(-Uk.m1, yp.y, fmaf(-Uk.m0, yp.x, fmaf(-Lk.m1, ym.y, fmaf(-Lk.m0, ym.x, Yr[q].x))));
                const float y1 = fmaf(-Uk.m3, yp.y, fmaf(-Uk.m2, yp.x, fmaf(-Lk.m3, ym.y, fmaf(-Lk.m2, ym.x, Yr[q].y))));
                const M2 LL = mmul(Lk, Lm), UU = mmul(Uk, Up);
                // L' = -D'^-1 L_k L_{k-d},  U' = -D'^-1 U_k U_{k+d},  Y' <- D'^-1 Y'
                const M2 Mi = minv(Dn);
                const M2 Mn = {-Mi.m0, -Mi.m1, -Mi.m2, -Mi.m3};
                Lr[q] = mmul(Mn, LL);
                Ur[q] = mmul(Mn, UU);
                Yr[q] = make_float2(fmaf(Mi.m0, y0, Mi.m1 * y1), fmaf(Mi.m2, y0, Mi.m3 * y1));
                if (p.final_step) lmax = fmaxf(lmax, fmaxf(amaxm(Lr[q]), amaxm(Ur[q])));
            }
        }
        if (p.final_step) {
            lmax = warp_max(lmax);
            if ((tid & 31) == 0) atomicMax(&s_max[st & 1], __float_as_uint(lmax));
        }
        __syncthreads();                                   // every read of this stride is done
        bool stop = st == K - 1;
        if (p.final_step) {
            // truncation test over the whole subsystem
            const float smax = __uint_as_float(s_max[st & 1]);
            if (tid == 0) s_max[(st + 1) & 1] = 0u;
            if (!(smax >= kTrunc)) stop = true;            // (nan also stops: the refinement will report it)
        }
        if (stop) break;
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            if (k >= klo && k < khi) { sL[k] = f4(Lr[q]); sU[k] = f4(Ur[q]); sY[k] = Yr[q]; }
        }
        __syncthreads();
    }

    if (p.final_step) {
        // X = Y: write the correction rows and the system's |dx| maximum
        float lmax = 0.0f;
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            if (k < TR) {
                const int64_t i0 = 2 * (r + k * p.G);       // first row of the block row
                p.dx[j * p.n + i0] = Yr[q].x;
                lmax = fmaxf(lmax, fabsf(Yr[q].x));
                if (i0 + 1 < p.n) { p.dx[j * p.n + i0 + 1] = Yr[q].y; lmax = fmaxf(lmax, fabsf(Yr[q].y)); }
            }
        }
        lmax = warp_max(lmax);
        if ((tid & 31) == 0) atomic_max_pos(&p.ndx[(int64_t)p.sweep * p.m + j], lmax);
    } else {
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
            atomic_max_pos(&s_max[2], lmax);
        }
        __syncthreads();
        // A window whose couplings all vanished is decoupled: its rows already
        // hold X = Y.  Write them now; if every window of the system is
        // decoupled the later passes of this sweep skip the system.
        if (__uint_as_float(s_max[2]) < kTrunc) {
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
}

// 4 CTAs per SM up to 4 rows per thread (64 registers, 40 KB of shared
// memory each at 1024 block rows), 2 beyond
template <int RPT>
__global__ void __launch_bounds__(kMpThreads, RPT >= 8 ? 2 : 4)
mp_pass_kernel(MpPassArgs p)
{
    extern __shared__ float4 fsm[];
    __shared__ unsigned s_max[3];
    // the flags read here were written by earlier kernels: read-only cache
    if (__ldg(p.live) == 0) return;               // every system finished in an earlier sweep
    float4* sL = fsm;
    float4* sU = fsm + p.TRmax;
    float2* sY = reinterpret_cast<float2*>(fsm + 2 * p.TRmax);
    // grid-stride over the items (about one wave of CTAs)
    const int64_t items = p.m * p.G * p.nwin;
    for (int64_t blk = blockIdx.x; blk < items; blk += gridDim.x) {
        const int64_t item = blk / p.nwin;
        const int64_t w = blk - item * p.nwin;
        const int64_t j = item / p.G;
        const int64_t r = item - j * p.G;
        if (__ldg(p.fin + j)) continue;
        if (p.trunc_in && __uint_as_float(__ldg(p.trunc_in + j)) < kTrunc) {
            // Every window of the previous pass found itself decoupled and
            // wrote its rows of dx (X = Y): item (0, 0) carries the |dx|
            // maximum they left into the sweep's norm, the rest is skipped.
            if (r == 0 && w == 0 && threadIdx.x == 0)
                atomicMax(&p.ndx[(int64_t)p.sweep * p.m + j], p.ndx_pre_in[j]);
            continue;
        }
        mp_pass_item<RPT>(p, j, r, w, sL, sU, sY, s_max);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// refinement: x += dx (FP64), decide, and r = y - A x for the next sweep
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mp_update_tile(const MpArgs& p, int64_t j, int64_t tile, double* sx, float* s_red)
{
    const int s = p.sweep;
    const int tid = threadIdx.x;
    const int64_t n = p.n;
    constexpr int XR = kMpTile / kMpThreads;             // rows per thread

    // Rows t0 + tid + u*kMpThreads of the tile [t0, t1); threads 0-3 also take
    // the halo rows t0-2, t0-1, t1, t1+1 of x, recomputed bit-identically by
    // the neighbouring tiles.  The x loads go first, then the norms the
    // decision needs, then the bands: one memory round trip in sweep 0 (no
    // decision to wait for) and in a last sweep (no bands to read).
    const int64_t t0 = tile * kMpTile;
    const int64_t t1 = min(t0 + kMpTile, n);
    const int64_t ih = tid < 2 ? t0 - 2 + tid : t1 + tid - 2;          // halo row of threads 0-3
    const bool halo = tid < 4 && ih >= 0 && ih < n;
    // x_{s-1} comes from the other ping-pong buffer: neighbouring tiles read
    // their halo rows from it while this tile writes x_s
    const double* __restrict__ xprev = p.X[(s + 1) & 1] + j * n;
    const float* __restrict__ dxs = p.dx + j * n;
    float dv[XR], dvh = 0.0f;
    double xv[XR], xvh = 0.0;
#pragma unroll
    for (int u = 0; u < XR; u++) {
        const int64_t i = t0 + tid + u * kMpThreads;
        dv[u] = 0.0f; xv[u] = 0.0;
        if (i < t1) { dv[u] = dxs[i]; if (s > 0) xv[u] = xprev[i]; }
    }
    if (halo) { dvh = dxs[ih]; if (s > 0) xvh = xprev[ih]; }

    // per-system decision from the norms the previous kernels left behind
    bool done = false;
    float est = 0.0f;
    if (s >= 1) {
        const float nd = __uint_as_float(p.ndx[(int64_t)s * p.m + j]);
        const float ndp = __uint_as_float(p.ndx[(int64_t)(s - 1) * p.m + j]);
        const float nxp = __uint_as_float(p.nx[(int64_t)(s - 1) * p.m + j]);
        if (nd == 0.0f) { done = true; est = 0.0f; }
        else if (ndp > 0.0f) {
            // Two ways to be done.  (1) The correction itself is below tol/2:
            // x_{s-1} was off by about |dx_s|, and applying dx_s leaves at most
            // that much (this also ends refinement that has reached the FP64
            // rounding floor, where dx is noise and no longer contracts).
            // (2) The corrections contract (rho < 0.5): the error left after
            // dx_s is ~ sum_k rho^k |dx_s| = rho/(1-rho)|dx_s|, doubled for the
            // drift of rho between sweeps.
            const float rel = nd / fmaxf(nxp, FLT_MIN);
            const float rho = nd / ndp;
            const float contr = rho < 0.5f ? 2.0f * rho / (1.0f - rho) * rel : rel;
            est = fminf(rel, contr);
            done = rel <= 0.5f * p.tol || (rho < 0.5f && contr <= p.tol);
        }
    }
    const bool last = done || s == p.max_sweeps - 1;
    const bool to_user = last && !p.keep_x;

    // bands and y of this thread's rows, for the residual (not read in a last sweep)
    const int64_t ybase = j * p.ss;
    double ba[XR], bb[XR], bc[XR], bd[XR], be[XR], by[XR];
#pragma unroll
    for (int u = 0; u < XR; u++) {
        const int64_t i = t0 + tid + u * kMpThreads;
        ba[u] = 0.0; bb[u] = 0.0; bc[u] = 1.0; bd[u] = 0.0; be[u] = 0.0; by[u] = 0.0;
        if (!last && i < t1) {
            const int64_t g = ybase + i * p.rs;
            ba[u] = p.a[g]; bb[u] = p.b[g]; bc[u] = p.c[g]; bd[u] = p.d[g]; be[u] = p.e[g]; by[u] = p.y[g];
        }
    }

    float xmax = 0.0f;
#pragma unroll
    for (int u = 0; u < XR; u++) {
        const int64_t i = t0 + tid + u * kMpThreads;
        if (i < t1) {
            const double xi = s == 0 ? f2d(dv[u]) : __dadd_rn(xv[u], f2d(dv[u]));
            sx[tid + u * kMpThreads + 2] = xi;
            if (to_user) p.y[ybase + i * p.rs] = xi;
            else if (last) p.Xout[j * n + i] = xi;
            else p.X[s & 1][j * n + i] = xi;
            xmax = fmaxf(xmax, fabsf(d2f_scaled(xi, 0)));     // |x| in FP32: it only feeds the estimate
        }
    }
    if (halo) sx[ih - t0 + 2] = s == 0 ? f2d(dvh) : __dadd_rn(xvh, f2d(dvh));
    xmax = warp_max(xmax);
    if ((tid & 31) == 0) s_red[tid >> 5] = xmax;
    __syncthreads();
    if (tid == 0) {
        float v = 0.0f;
        for (int w = 0; w < (int)(blockDim.x / 32); w++) v = fmaxf(v, s_red[w]);
        atomic_max_pos(&p.nx[(int64_t)s * p.m + j], v);
        if (tile == 0 && last) {
            p.est[j] = est;
            p.status[j] = done ? 1 : 2;      // 2: stopped at max_sweeps
            p.fin[j] = s + 1;
            for (int s2 = s + 1; s2 <= p.max_sweeps; s2++) atomicSub(&p.live[s2], 1);
        }
    }
    if (last) return;

    // residual r = y - A x (FP64, FMA chain), row-scaled to FP32; the two rows
    // of a block row sit in lanes 2k, 2k+1 and meet by a shuffle, and the even
    // lane normalises by the block's diagonal inverse -> the next FP32 rhs
    const int64_t nb = (n + 1) / 2;
#pragma unroll
    for (int u = 0; u < XR; u++) {
        const int64_t i = t0 + tid + u * kMpThreads;
        float rf = 0.0f, cs = 1.0f, os = 0.0f;             // r, c and the off-diagonal entry of D, scaled
        if (i < t1) {
            const int li = tid + u * kMpThreads + 2;
            double r = by[u];
            r = fma(-bc[u], sx[li], r);
            if (i >= 2) r = fma(-ba[u], sx[li - 2], r);
            if (i >= 1) r = fma(-bb[u], sx[li - 1], r);
            if (i + 1 < n) r = fma(-bd[u], sx[li + 1], r);
            if (i + 2 < n) r = fma(-be[u], sx[li + 2], r);
            const int sh = d_exponent(bc[u]);
            rf = d2f_scaled(r, sh);
            cs = d2f_scaled(bc[u], sh);
            // D = {c0, d0; b1, c1}: the even row contributes d, the odd row b
            if ((i & 1) == 0) os = i + 1 < n ? d2f_scaled(bd[u], sh) : 0.0f;
            else os = d2f_scaled(bb[u], sh);
        }
        const float rf1 = __shfl_xor_sync(0xffffffffu, rf, 1);
        const float cs1 = __shfl_xor_sync(0xffffffffu, cs, 1);
        const float os1 = __shfl_xor_sync(0xffffffffu, os, 1);
        if (i < t1 && (i & 1) == 0) {
            // the odd partner of row n-1 (odd n) is the identity row: c 1, b 0, r 0
            const bool dummy = i + 1 >= n;
            const M2 Mi = minv({cs, os, dummy ? 0.0f : os1, dummy ? 1.0f : cs1});
            const float r1 = dummy ? 0.0f : rf1;
            p.R[j * nb + (i >> 1)] = make_float2(fmaf(Mi.m0, rf, Mi.m1 * r1), fmaf(Mi.m2, rf, Mi.m3 * r1));
        }
    }
}

// 3 CTAs per SM (at most 85 registers): 3072 rows in flight per SM
__global__ void __launch_bounds__(kMpThreads, 3)
mp_update_kernel(MpArgs p)
{
    __shared__ double sx[kMpTile + 4];
    __shared__ float s_red[kMpThreads / 32];
    if (__ldg(p.live + p.sweep) == 0) return;      // every system finished in an earlier sweep
    const int64_t tiles = (p.n + kMpTile - 1) / kMpTile;
    for (int64_t blk = blockIdx.x; blk < p.m * tiles; blk += gridDim.x) {
        const int64_t j = blk / tiles;
        const int64_t tile = blk - j * tiles;
        // finished in an earlier sweep?  (fin is written during this kernel by
        // the tile-0 CTA for the current sweep; the other tiles must still run)
        const int f = p.fin[j];
        if (f == 0 || f > p.sweep) mp_update_tile(p, j, tile, sx, s_red);
        __syncthreads();
    }
}

// r = y - A x (FP64 FMA chain).  Bands and y use the caller's layout (ss, rs);
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
        if (i >= 2) v = fma(-a[g], x[gx - 2 * xrs], v);
        if (i >= 1) v = fma(-b[g], x[gx - xrs], v);
        if (i + 1 < n) v = fma(-d[g], x[gx + xrs], v);
        if (i + 2 < n) v = fma(-e[g], x[gx + 2 * xrs], v);
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
        if (i >= 2) rowsum += fabs(a[g]);
        if (i >= 1) rowsum += fabs(b[g]);
        if (i + 1 < n) rowsum += fabs(d[g]);
        if (i + 2 < n) rowsum += fabs(e[g]);
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
size_t mp_pass_smem(int rows) { return (size_t)rows * (2 * sizeof(float4) + sizeof(float2)); }

template <int RPT>
cudaError_t launch_mp_pass_rpt(const MpPassArgs& p, int threads, int64_t blocks, cudaStream_t s)
{
    const size_t smem = mp_pass_smem(p.TRmax);
    cudaError_t e = cudaFuncSetAttribute(mp_pass_kernel<RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mp_pass_smem(kMpMaxRows));
    if (e != cudaSuccess) return e;
    blocks = std::min<int64_t>(blocks, mp_grid_cap((const void*)mp_pass_kernel<RPT>, threads, smem));
    mp_pass_kernel<RPT><<<(unsigned)blocks, threads, smem, s>>>(p);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_mp_prep(const MpArgs& p, cudaStream_t s)
{
    const int64_t nb = (p.n + 1) / 2;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((p.m * nb + kMpThreads - 1) / kMpThreads, 152 * 16));
    mp_prep_kernel<<<(unsigned)blocks, kMpThreads, 0, s>>>(p);
    count_launch();
    return cudaGetLastError();
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

cudaError_t launch_mp_update(const MpArgs& p, cudaStream_t s)
{
    // one CTA per tile: the tiles of a sweep are latency-bound FP64 and HBM
    // work that needs every resident CTA; a sweep with nothing left returns
    // at once through the live count
    const int64_t tiles = (p.n + kMpTile - 1) / kMpTile;
    const int64_t blocks = std::min<int64_t>(p.m * tiles, 0x7fffffffLL);
    mp_update_kernel<<<(unsigned)blocks, kMpThreads, 0, s>>>(p);
    count_launch();
    return cudaGetLastError();
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
