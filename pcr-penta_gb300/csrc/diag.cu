// diag.cu -- FP64 throughput probe (pcrp_measure_fp64): the denominator of
// the FP64-pipe roofline of the bit-faithful path.
#include <cuda_runtime.h>

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

}  // namespace
}  // namespace pcrp

using namespace pcrp;

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
