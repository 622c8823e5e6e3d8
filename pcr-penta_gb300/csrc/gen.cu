// gen.cu -- seeded input generators (host threads and a device kernel).
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "gen.cuh"
#include "pcrp_internal.h"

namespace pcrp {
namespace {

__global__ void gen_kernel(int kind, uint64_t seed, int64_t m, int64_t n, int layout,
                           double* a, double* b, double* c, double* d, double* e, double* y)
{
    const int64_t total = m * n;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int64_t j, i;
        if (layout == PCRP_LAYOUT_CONTIGUOUS) { j = idx / n; i = idx - j * n; }
        else { i = idx / m; j = idx - i * m; }
        const gen::Row R = gen::row(kind, seed, (uint64_t)j, i, n);
        a[idx] = R.a; b[idx] = R.b; c[idx] = R.c; d[idx] = R.d; e[idx] = R.e; y[idx] = R.y;
    }
}

int host_threads(int32_t nthreads) {
    if (nthreads > 0) return nthreads;
    unsigned hc = std::thread::hardware_concurrency();
    return hc ? (int)hc : 1;
}

template <class F>
void parallel_for(int64_t count, int nthreads, F f) {
    nthreads = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads, count));
    if (nthreads == 1) { f(0, count); return; }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([=] { f(count * t / nthreads, count * (t + 1) / nthreads); });
    for (auto& x : th) x.join();
}

bool kind_ok(int32_t kind) { return kind >= PCRP_GEN_DOMINANT && kind <= PCRP_GEN_TOEPLITZ; }

}  // namespace
}  // namespace pcrp

using namespace pcrp;

extern "C" pcrp_status pcrp_generate(int32_t kind, uint64_t seed, int64_t m, int64_t n, int32_t layout,
                                     double* a, double* b, double* c, double* d, double* e, double* y,
                                     int32_t nthreads)
{
    if (!kind_ok(kind)) return set_error(PCRP_EINVAL, "pcrp_generate: unknown kind %d", kind);
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "pcrp_generate: negative size");
    if (layout != PCRP_LAYOUT_CONTIGUOUS && layout != PCRP_LAYOUT_INTERLEAVED)
        return set_error(PCRP_EINVAL, "pcrp_generate: bad layout %d", layout);
    if (m == 0 || n == 0) return PCRP_OK;
    if (!a || !b || !c || !d || !e || !y) return set_error(PCRP_EINVAL, "pcrp_generate: null array");
    parallel_for(m, host_threads(nthreads), [&](int64_t j0, int64_t j1) {
        for (int64_t j = j0; j < j1; j++)
            for (int64_t i = 0; i < n; i++) {
                const int64_t idx = layout == PCRP_LAYOUT_CONTIGUOUS ? j * n + i : i * m + j;
                const gen::Row R = gen::row(kind, seed, (uint64_t)j, i, n);
                a[idx] = R.a; b[idx] = R.b; c[idx] = R.c; d[idx] = R.d; e[idx] = R.e; y[idx] = R.y;
            }
    });
    return PCRP_OK;
}

extern "C" pcrp_status pcrp_generate_device(int32_t kind, uint64_t seed, int64_t m, int64_t n, int32_t layout,
                                            double* a, double* b, double* c, double* d, double* e, double* y,
                                            pcrp_stream stream)
{
    if (!kind_ok(kind)) return set_error(PCRP_EINVAL, "pcrp_generate_device: unknown kind %d", kind);
    if (m < 0 || n < 0) return set_error(PCRP_EINVAL, "pcrp_generate_device: negative size");
    if (layout != PCRP_LAYOUT_CONTIGUOUS && layout != PCRP_LAYOUT_INTERLEAVED)
        return set_error(PCRP_EINVAL, "pcrp_generate_device: bad layout %d", layout);
    if (m == 0 || n == 0) return PCRP_OK;
    if (!a || !b || !c || !d || !e || !y) return set_error(PCRP_EINVAL, "pcrp_generate_device: null array");
    const int64_t total = m * n;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 16);
    gen_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(kind, seed, m, n, layout, a, b, c, d, e, y);
    count_launch();
    return cuda_error(cudaGetLastError(), "pcrp_generate_device");
}

extern "C" pcrp_status pcrp_ragged_sizes(uint64_t seed, int64_t nsys, int64_t nmin, int64_t nmax,
                                         int64_t* sizes_out)
{
    if (nsys < 0 || nmin < 1 || nmax < nmin) return set_error(PCRP_EINVAL, "pcrp_ragged_sizes: bad range");
    if (nsys > 0 && !sizes_out) return set_error(PCRP_EINVAL, "pcrp_ragged_sizes: null output");
    const double lr = std::log((double)nmax / (double)nmin);
    for (int64_t k = 0; k < nsys; k++) {
        const double u = gen::unit(seed, gen::S_P1, (uint64_t)k, 0x7A66ED);
        int64_t v = (int64_t)std::floor((double)nmin * std::exp(u * lr) + 0.5);
        sizes_out[k] = std::min(std::max(v, nmin), nmax);
    }
    return PCRP_OK;
}

extern "C" pcrp_status pcrp_generate_ragged(int32_t kind, uint64_t seed, const int64_t* offsets, int64_t nsys,
                                            double* a, double* b, double* c, double* d, double* e, double* y,
                                            int32_t nthreads)
{
    if (!kind_ok(kind)) return set_error(PCRP_EINVAL, "pcrp_generate_ragged: unknown kind %d", kind);
    if (nsys < 0 || (nsys > 0 && !offsets)) return set_error(PCRP_EINVAL, "pcrp_generate_ragged: bad offsets");
    if (nsys == 0) return PCRP_OK;
    if (!a || !b || !c || !d || !e || !y) return set_error(PCRP_EINVAL, "pcrp_generate_ragged: null array");
    for (int64_t k = 0; k < nsys; k++)
        if (offsets[k + 1] < offsets[k]) return set_error(PCRP_EINVAL, "pcrp_generate_ragged: offsets decrease at %lld", (long long)k);
    parallel_for(nsys, host_threads(nthreads), [&](int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; k++) {
            const int64_t o = offsets[k], n = offsets[k + 1] - offsets[k];
            for (int64_t i = 0; i < n; i++) {
                const gen::Row R = gen::row(kind, seed, (uint64_t)k, i, n);
                a[o + i] = R.a; b[o + i] = R.b; c[o + i] = R.c; d[o + i] = R.d; e[o + i] = R.e; y[o + i] = R.y;
            }
        }
    });
    return PCRP_OK;
}
