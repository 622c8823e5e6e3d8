// diag.cu -- FP64 throughput probe (pcrp_measure_fp64): the denominator of
// the FP64-pipe roofline of the bit-faithful path; the FP64 / FP32 / integer
// pipe-sharing probe (pcrp_measure_pipes); the quotient check of the FP64
// kernels (pcrp_check_quotients).
#include <cuda_runtime.h>

#include "pcr_tile.cuh"
#include "pcrp_internal.h"

namespace pcrp {
namespace {

constexpr int kChains = 8;        // independent dependency chains per thread
constexpr int kProbeThreads = 256;

// kChains independent FMA chains x <- x*a + b per thread; |a| < 1 keeps the
// values bounded and normal
__global__ void __launch_bounds__(kProbeThreads) fma_probe(double* out, int iters, double a, double b)
{
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) x[k] = fma(x[k], a, b);
    }
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++) acc += x[k];
    if (acc == 1234.5) out[0] = acc;               // keeps the chains alive; never true for these inputs
}

// kChains independent division chains x <- x / a per thread, a slightly
// above 1 so that the values stay normal over the run
__global__ void __launch_bounds__(kProbeThreads) div_probe(double* out, int iters, double a)
{
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) x[k] = __ddiv_rn(x[k], a);
    }
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++) acc += x[k];
    if (acc == 1234.5) out[0] = acc;
}

template <typename Launch>
cudaError_t time_ms(Launch launch, cudaStream_t s, float* ms)
{
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        launch();                                   // warm-up
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) launch();
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
        cudaEventDestroy(e1);
    }
    cudaEventDestroy(e0);
    return e;
}

// Pipe sharing: FP64 FMA chains on the even warps of every CTA, and FP32 FMA
// or integer (xor-shift-add) chains on the odd warps; which of the three run
// is selected by `mode` (bit 0 FP64, bit 1 FP32, bit 2 integer).  Timing the
// parts alone and together shows whether the SM runs them side by side.
__global__ void __launch_bounds__(kProbeThreads) pipe_probe(double* out, int it64, int it32, int itint, int mode)
{
    const int w = threadIdx.x >> 5;
    if ((mode & 1) && !(w & 1)) {
        double x[4];
#pragma unroll
        for (int k = 0; k < 4; k++) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
        for (int i = 0; i < it64; i++) {
#pragma unroll
            for (int k = 0; k < 4; k++) x[k] = fma(x[k], 0.999999, 1e-6);
        }
        if (x[0] + x[1] + x[2] + x[3] == 1234.5) out[0] = x[0];   // keeps the chains alive; never true
    }
    if ((mode & 2) && (w & 1)) {
        float f[8];
#pragma unroll
        for (int k = 0; k < 8; k++) f[k] = 1.0f + 1e-3f * (threadIdx.x + k);
        for (int i = 0; i < it32; i++) {
#pragma unroll
            for (int k = 0; k < 8; k++) f[k] = fmaf(f[k], 0.999999f, 1e-6f);
        }
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; k++) acc += f[k];
        if (acc == 1234.5f) out[0] = acc;
    }
    if ((mode & 4) && (w & 1)) {
        unsigned u[8];
#pragma unroll
        for (int k = 0; k < 8; k++) u[k] = threadIdx.x * 2654435761u + k;
        for (int i = 0; i < itint; i++) {
#pragma unroll
            for (int k = 0; k < 8; k++) u[k] = (u[k] ^ (u[k] >> 7)) + 0x9E3779B9u;
        }
        unsigned acc = 0u;
#pragma unroll
        for (int k = 0; k < 8; k++) acc ^= u[k];
        if (acc == 0x12345678u) out[0] = acc;
    }
}

}  // namespace
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// A double of operand class `mode` from 64 random bits: 0 exponents within
// 2^+-32, 1 every exponent the quotient's guard admits, 2 mantissas near all
// ones, 3 mantissas near a power of two, 4 any finite or infinite exponent
// (zeros, subnormals and the guard's excluded ranges included).
__device__ __forceinline__ double operand(uint64_t r, int mode)
{
    uint64_t mant = r & 0xFFFFFFFFFFFFFull;
    int e;
    switch (mode) {
    case 0: e = 1023 + (int)((r >> 52) % 64) - 32; break;
    case 1: e = 100 + (int)((r >> 52) % 1847); break;
    case 2: e = 1023 + (int)((r >> 52) % 16) - 8; mant |= 0xFFFFFFFFFFF00ull; break;
    case 3: e = 1023 + (int)((r >> 52) % 16) - 8; mant &= 0xFFull; break;
    default: e = (int)((r >> 52) % 2048); break;
    }
    return __longlong_as_double((long long)(((r >> 63) << 63) | ((uint64_t)e << 52) | mant));
}

// The phase-B quotient of the FP64 kernels (mdiv: Markstein's correction
// from the correctly rounded reciprocal) against __ddiv_rn on random pairs.
__global__ void __launch_bounds__(kProbeThreads)
quotient_check(int mode, uint64_t seed, int64_t per_thread, unsigned long long* bad, unsigned long long* fast)
{
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    unsigned long long nb = 0, nf = 0;
    for (int64_t i = 0; i < per_thread; i++) {
        const uint64_t r1 = mix64(seed ^ (t * 0x100000001B3ull + (uint64_t)i * 2));
        const uint64_t r2 = mix64(seed + t * 0x9E37ull + (uint64_t)i * 2 + 1);
        const double a = operand(r1, mode), b = operand(r2, (r2 & 1) ? 4 : mode);
        if (!nz(b)) continue;                     // the kernels never divide by zero
        const double q = mdiv(a, b, __drcp_rn(b)), ref = __ddiv_rn(a, b);
        const bool same = __double_as_longlong(q) == __double_as_longlong(ref) || (q != q && ref != ref);
        nb += !same;
        const int ea = (int)((hiw(a) >> 20) & 0x7FFu), eb = (int)((hiw(b) >> 20) & 0x7FFu);
        nf += (unsigned)(ea - 100) <= 1846u && (unsigned)(eb - 100) <= 1846u && (unsigned)(ea - eb + 900) <= 1800u;
    }
    atomicAdd(bad, nb);
    atomicAdd(fast, nf);
}

}  // namespace
}  // namespace pcrp

using namespace pcrp;

extern "C" pcrp_status pcrp_check_quotients(int32_t mode, uint64_t seed, int64_t samples, uint64_t* mismatches,
                                            uint64_t* markstein, pcrp_stream stream)
{
    if (!mismatches || !markstein || samples < 0 || mode < 0 || mode > 4)
        return set_error(PCRP_EINVAL, "pcrp_check_quotients: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_check_quotients");
    unsigned long long* cnt = nullptr;
    e = cudaMallocAsync(reinterpret_cast<void**>(&cnt), 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_check_quotients allocation");
    const unsigned grid = (unsigned)sms * 8;
    const int64_t threads = (int64_t)grid * kProbeThreads;
    const int64_t per = (samples + threads - 1) / threads;
    unsigned long long host[2] = {0, 0};
    e = cudaMemsetAsync(cnt, 0, sizeof host, s);
    if (e == cudaSuccess) {
        quotient_check<<<grid, kProbeThreads, 0, s>>>(mode, seed, per, cnt, cnt + 1);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, cnt, sizeof host, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(cnt, s);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_check_quotients");
    *mismatches = host[0];
    *markstein = host[1];
    return PCRP_OK;
}

extern "C" pcrp_status pcrp_measure_fp64(double* dfma_per_s, double* ddiv_per_s, pcrp_stream stream)
{
    if (!dfma_per_s || !ddiv_per_s) return set_error(PCRP_EINVAL, "pcrp_measure_fp64: null output");
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_measure_fp64");
    double* out = nullptr;
    e = cudaMallocAsync(reinterpret_cast<void**>(&out), sizeof(double), s);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_measure_fp64 allocation");
    const unsigned grid = (unsigned)sms * 8;
    const int fma_iters = 2048, div_iters = 256;
    float ms_fma = 0.0f, ms_div = 0.0f;
    e = time_ms([&] { fma_probe<<<grid, kProbeThreads, 0, s>>>(out, fma_iters, 0.999999, 1e-6); count_launch(); },
                s, &ms_fma);
    if (e == cudaSuccess)
        e = time_ms([&] { div_probe<<<grid, kProbeThreads, 0, s>>>(out, div_iters, 1.0000001); count_launch(); },
                    s, &ms_div);
    cudaFreeAsync(out, s);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_measure_fp64");
    const double lanes = (double)grid * kProbeThreads * kChains;
    *dfma_per_s = lanes * fma_iters / (ms_fma * 1e-3);
    *ddiv_per_s = lanes * div_iters / (ms_div * 1e-3);
    return PCRP_OK;
}

extern "C" pcrp_status pcrp_measure_pipes(float* ms, pcrp_stream stream)
{
    if (!ms) return set_error(PCRP_EINVAL, "pcrp_measure_pipes: null output");
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_measure_pipes");
    double* out = nullptr;
    e = cudaMallocAsync(reinterpret_cast<void**>(&out), sizeof(double), s);
    if (e != cudaSuccess) return cuda_error(e, "pcrp_measure_pipes allocation");
    // four CTAs per SM; loop counts that give each part alone about a millisecond on GB300
    const unsigned grid = (unsigned)sms * 4;
    const int modes[5] = {1, 2, 4, 3, 5};
    for (int q = 0; q < 5 && e == cudaSuccess; q++)
        e = time_ms([&] { pipe_probe<<<grid, kProbeThreads, 0, s>>>(out, 2000, 40000, 10000, modes[q]); count_launch(); },
                    s, &ms[q]);
    cudaFreeAsync(out, s);
    return e == cudaSuccess ? PCRP_OK : cuda_error(e, "pcrp_measure_pipes");
}
