// mixed_dev.cuh -- device helpers shared by the kernels of the mixed-precision
// solver (mixed.cu, mixed_duo.cu): integer-pipe FP64<->FP32 conversions, 2x2
// block arithmetic, the block reduction step, block cyclic reduction in a
// shared-memory tile, and the refinement stopping rule.  Everything lives in
// an anonymous namespace: each translation unit gets its own copy.
#pragma once
#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "mixed_internal.h"

namespace pcrp {
namespace {

constexpr float kTrunc = 1e-10f;

// rows allocated per shared-memory array of the pass kernel (whole groups of
// 8, the span of the swizzle of the whole-subsystem pass)
__host__ __device__ __forceinline__ int mp_pass_rows(int rows) { return (rows + 7) & ~7; }

// CTAs of one wave of a kernel (the pass kernel strides over its items with
// one wave, so that sweeps of mostly finished systems stay cheap)
inline int mp_grid_cap(const void* kernel, int threads, size_t smem)
{
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152 * 2;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 152 * 2;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1) per = 1;
    return sms * per;
}

// Programmatic dependent launch (see launch_dependent): wait for the
// predecessor kernel's completion and memory before touching memory; allow
// the successor to be launched (it waits in turn).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// integer-pipe conversions
// ---------------------------------------------------------------------------

// Exponent e of |v| in [2^e, 2^(e+1)); 0 for zero, subnormal, inf, nan.
__device__ __forceinline__ int d_exponent(double v) {
    const int E = (int)((__double_as_longlong(v) >> 52) & 0x7FF);
    return (E == 0 || E == 0x7FF) ? 0 : E - 1023;
}

// (float)(v * 2^-sh), rounded to nearest (ties away), flushing results below
// FLT_MIN to zero and saturating to inf; integer arithmetic only, branch-free
// (the special cases are selects).
__device__ __forceinline__ float d2f_scaled(double v, int sh) {
    const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
    const unsigned sign = hi & 0x80000000u;
    const int E = (int)((hi >> 20) & 0x7FF);
    const int F = E - sh - (1023 - 127);                        // biased FP32 exponent of the result
    if ((unsigned)(F - 1) < 254u && (unsigned)(E - 1) < 0x7FEu) {
        // normal input and result (the common case): rebias the exponent in
        // place and round the mantissa; a rounding carry into exponent 255
        // gives inf
        const unsigned u = ((((hi & 0x800FFFFFu) | ((unsigned)F << 20)) << 3) | (lo >> 29)) + ((lo >> 28) & 1u);
        return __uint_as_float((u & 0x7FFFFFFFu) | sign);
    }
    const unsigned mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);   // top 23 bits of the mantissa
    unsigned u = ((unsigned)F << 23) + mant + ((lo >> 28) & 1u);
    u = min(u, 0x7F800000u);                                     // rounded past the largest float: inf
    u = F <= 0 ? 0u : u;
    u = F >= 255 ? 0x7F800000u : u;
    u = E == 0 ? 0u : u;                                         // zero and subnormal
    u = E == 0x7FF ? (0x7F800000u | ((((hi & 0xFFFFFu) | lo) != 0u) ? 0x400000u : 0u)) : u;
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

// max |x| as the largest bit pattern with the sign cleared (non-negative
// doubles order like their bits; a nan wins and poisons the norm)
__device__ __forceinline__ unsigned long long absbits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
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

__device__ __forceinline__ float amaxm(const M2& a) {
    return fmaxf(fmaxf(fabsf(a.m0), fabsf(a.m1)), fmaxf(fabsf(a.m2), fabsf(a.m3)));
}
__device__ __forceinline__ M2 m2(const float4& v) { return {v.x, v.y, v.z, v.w}; }
__device__ __forceinline__ float4 f4(const M2& a) { return make_float4(a.m0, a.m1, a.m2, a.m3); }

// One block reduction step of a normalised row k (D = I) with its neighbours
// m = k-d and p = k+d (PCR stride and cyclic-reduction level alike):
//     D' = I - L_k U_m - U_k L_p,  L' = -D'^-1 L_k L_m,  U' = -D'^-1 U_k U_p,
//     Y' = D'^-1 (Y_k - L_k Y_m - U_k Y_p).
__device__ __forceinline__ void reduce_row(const M2& Lk, const M2& Uk, float2 Yk,
                                           const M2& Lm, const M2& Um, float2 ym,
                                           const M2& Lp, const M2& Up, float2 yp,
                                           M2& Lo, M2& Uo, float2& Yo)
{
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
    Lo = mmul(Mn, LL);
    Uo = mmul(Mn, UU);
    Yo = make_float2(fmaf(Mi.m0, y0, Mi.m1 * y1), fmaf(Mi.m2, y0, Mi.m3 * y1));
}

// Shared-memory position of row k of a cyclic-reduction tile: an XOR swizzle
// inside each aligned group of 8 rows, so that the power-of-two strides of
// cyclic reduction hit distinct banks (16-byte slots) for 8 consecutive
// lanes.  The arrays are allocated for whole groups of 8 rows (mp_pass_rows).
__device__ __forceinline__ int swz(int k) { return k ^ (((k >> 3) ^ (k >> 6) ^ (k >> 9)) & 7); }

// Forward block cyclic reduction of the TR rows held (swizzled) in shared
// memory: level l turns the rows k = 0 mod 2^(l+1) into the reduced system
// at stride 2^(l+1), while the other rows keep their level-l equations.
// Survivors are rewritten in place (their neighbours at a level are rows that
// level does not write); a neighbour beyond the tile is clamped to an edge
// row, exact at a system boundary (the coupling towards it is exactly zero)
// and otherwise confined to rows whose results are not used.  Stops when the
// reduced rows that rows [clo, chi) depend on are decoupled (|L|,|U| <
// kTrunc, truncated reduction) and returns the number of levels; returns -1
// if they are still coupled after kmax levels.  A barrier must separate the
// loads from the call.
__device__ __forceinline__ int cr_reduce(float4* sL, float4* sU, float2* sY, int TR, int kmax, int clo, int chi)
{
    const int tid = threadIdx.x, bd = blockDim.x;
    for (int l = 0; l < kmax && (1 << l) < TR; l++) {
        const int d = 1 << l, d2 = 2 * d;
        const int lo = clo - d2 + 1, hi = chi + d2 - 1;
        bool coupled = false;
        for (int k = tid * d2; k < TR; k += bd * d2) {
            const int sk = swz(k), sm = swz(max(k - d, 0)), sp = swz(min(k + d, TR - 1));
            M2 Lo, Uo;
            float2 Yo;
            reduce_row(m2(sL[sk]), m2(sU[sk]), sY[sk], m2(sL[sm]), m2(sU[sm]), sY[sm], m2(sL[sp]), m2(sU[sp]), sY[sp],
                       Lo, Uo, Yo);
            sL[sk] = f4(Lo); sU[sk] = f4(Uo); sY[sk] = Yo;
            if (k >= lo && k < hi) coupled |= fmaxf(amaxm(Lo), amaxm(Uo)) >= kTrunc;
        }
        // the barrier reduces the test: (nan entries do not count; a nan
        // solution is reported by the refinement)
        if (!__syncthreads_or(coupled)) return l + 1;
    }
    return TR <= 1 ? 0 : -1;
}

// Back substitution after cr_reduce: the rows left at level `top` hold
// x = Y; x_k = Y_k - L_k x_{k-d} - U_k x_{k+d} level by level downwards,
// written over Y.
__device__ __forceinline__ void cr_substitute(const float4* sL, const float4* sU, float2* sY, int TR, int top)
{
    const int tid = threadIdx.x, bd = blockDim.x;
    for (int l = top - 1; l >= 0; l--) {
        const int d = 1 << l;
        for (int k = d + tid * 2 * d; k < TR; k += bd * 2 * d) {
            const int sk = swz(k), sm = swz(k - d), sp = swz(min(k + d, TR - 1));
            const M2 Lk = m2(sL[sk]), Uk = m2(sU[sk]);
            const float2 xm = sY[sm], xp = sY[sp], yk = sY[sk];
            sY[sk] = make_float2(fmaf(-Uk.m1, xp.y, fmaf(-Uk.m0, xp.x, fmaf(-Lk.m1, xm.y, fmaf(-Lk.m0, xm.x, yk.x)))),
                                 fmaf(-Uk.m3, xp.y, fmaf(-Uk.m2, xp.x, fmaf(-Lk.m3, xm.y, fmaf(-Lk.m2, xm.x, yk.y)))));
        }
        __syncthreads();
    }
}

// Per-system decision after sweep s from the norms of this sweep and the last.
struct UpDecision { bool done, last; float est; };

// The stopping rule after sweep s from the sweep's max |dx_s| (nd) and the
// previous sweep's max |dx_{s-1}| (ndp) and max |x_{s-1}| (nxp).
__device__ __forceinline__ UpDecision stop_rule(int s, float nd, float ndp, float nxp, float tol, int max_sweeps)
{
    UpDecision D{false, false, 0.0f};
    if (s >= 1) {
        if (nd == 0.0f) D.done = true;
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
            D.est = fminf(rel, contr);
            D.done = rel <= 0.5f * tol || (rho < 0.5f && contr <= tol);
        }
    }
    D.last = D.done || s == max_sweeps - 1;
    return D;
}

}  // namespace
}  // namespace pcrp
