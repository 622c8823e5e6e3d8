// layout.cu -- batch layout adapter: transposes between the interleaved
// layout (element (system j, row i) at i*m + j) and the contiguous one
// (j*n + i).  An interleaved batch is an n x m row-major matrix and its
// contiguous form the m x n transpose, so one tiled transpose converts either
// way.  Used by the mixed solver, whose window kernels walk along a system:
// in the interleaved layout those walks are 8-byte loads m doubles apart,
// while two transposes cost 2 x 16 B per unknown and array of coalesced
// traffic.
#include <algorithm>

#include "pcrp_internal.h"

namespace pcrp {
namespace {

constexpr int kTile = 32;           // 32 x 32 doubles per tile, 8 KB of shared memory
constexpr int kRowsPerPass = 8;     // 32 x 8 threads

// Up to six arrays per launch (null entries are skipped).
struct TransposeSet {
    const double* src[6];
    double* dst[6];
};

// dst[k] (cols x rows, row-major) = transpose of src[k] (rows x cols,
// row-major) for every array k of the set, in one launch.  Persistent over
// (array, tile) pairs; loads and stores move 32 consecutive doubles per warp
// row; the 33-double pitch staggers the banks of the transposed reads.
__global__ void __launch_bounds__(kTile * kRowsPerPass)
transpose_kernel(const __grid_constant__ TransposeSet set, int narr, int64_t rows, int64_t cols)
{
    __shared__ double tile[kTile][kTile + 1];
    const int64_t tiles_c = (cols + kTile - 1) / kTile;
    const int64_t tiles = ((rows + kTile - 1) / kTile) * tiles_c;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int64_t u = blockIdx.x; u < tiles * narr; u += gridDim.x) {
        const int k = (int)(u / tiles);
        const int64_t t = u - (int64_t)k * tiles;
        const double* __restrict__ src = set.src[k];
        double* __restrict__ dst = set.dst[k];
        const int64_t r0 = (t / tiles_c) * kTile, c0 = (t % tiles_c) * kTile;
#pragma unroll
        for (int q = ty; q < kTile; q += kRowsPerPass) {
            const int64_t r = r0 + q, c = c0 + tx;
            if (r < rows && c < cols) tile[q][tx] = src[r * cols + c];
        }
        __syncthreads();
#pragma unroll
        for (int q = ty; q < kTile; q += kRowsPerPass) {
            const int64_t c = c0 + q, r = r0 + tx;
            if (c < cols && r < rows) dst[c * rows + r] = tile[tx][q];
        }
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_transpose(const double* const* src, double* const* dst, int narr, int64_t rows, int64_t cols,
                             cudaStream_t s)
{
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    TransposeSet set{};
    int k = 0;
    for (int i = 0; i < narr && i < 6; i++) {
        if (!src[i] || !dst[i]) continue;
        set.src[k] = src[i]; set.dst[k] = dst[i]; k++;
    }
    if (k == 0) return cudaSuccess;
    const int64_t tiles = ((rows + kTile - 1) / kTile) * ((cols + kTile - 1) / kTile) * k;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t blocks = std::min<int64_t>(tiles, (int64_t)std::max(sms, 1) * 16);
    transpose_kernel<<<(unsigned)blocks, dim3(kTile, kRowsPerPass), 0, s>>>(set, k, rows, cols);
    count_launch();
    return cudaGetLastError();
}

}  // namespace pcrp
