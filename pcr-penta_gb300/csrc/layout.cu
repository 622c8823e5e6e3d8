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

// The same for narrow sources (cols < 32, an interleaved batch of few
// systems): a tile holds TR whole rows (TR x cols elements, one contiguous
// run of src), loaded with consecutive lanes on consecutive elements and
// stored as cols runs of TR consecutive elements.
constexpr int kNarrowElems = 1024;

__global__ void __launch_bounds__(kTile * kRowsPerPass)
transpose_narrow_kernel(const __grid_constant__ TransposeSet set, int narr, int64_t rows, int cols)
{
    __shared__ double tile[2 * kNarrowElems];             // TR * (cols + 1) <= 1024 + 1024 / cols
    const int TR = kNarrowElems / cols / 32 * 32;         // rows per tile (>= 32), a multiple of 32
    const int pitch = cols + 1;                           // staggers the banks of the column reads
    const int64_t tiles = (rows + TR - 1) / TR;
    const int tid = threadIdx.y * kTile + threadIdx.x, nt = kTile * kRowsPerPass;
    for (int64_t u = blockIdx.x; u < tiles * narr; u += gridDim.x) {
        const int k = (int)(u / tiles);
        const int64_t r0 = (u - (int64_t)k * tiles) * TR;
        const int nr = (int)min((int64_t)TR, rows - r0);
        const double* __restrict__ src = set.src[k] + r0 * cols;
        double* __restrict__ dst = set.dst[k];
        for (int e = tid; e < nr * cols; e += nt) {
            const int r = e / cols, c = e - r * cols;
            tile[r * pitch + c] = src[e];
        }
        __syncthreads();
        for (int e = tid; e < nr * cols; e += nt) {
            const int c = e / nr, r = e - c * nr;
            dst[(int64_t)c * rows + r0 + r] = tile[r * pitch + c];
        }
        __syncthreads();
    }
}

// Narrow destinations (rows < 32: back into an interleaved batch of few
// systems): a tile is TC source columns, i.e. TC x rows elements of dst, one
// contiguous run, stored with consecutive lanes on consecutive elements.
__global__ void __launch_bounds__(kTile * kRowsPerPass)
transpose_narrow_dst_kernel(const __grid_constant__ TransposeSet set, int narr, int rows, int64_t cols)
{
    __shared__ double tile[2 * kNarrowElems];             // TC * (rows + 1) <= 1024 + 1024 / rows
    const int TC = kNarrowElems / rows / 32 * 32;         // source columns per tile (>= 32)
    const int pitch = rows + 1;
    const int64_t tiles = (cols + TC - 1) / TC;
    const int tid = threadIdx.y * kTile + threadIdx.x, nt = kTile * kRowsPerPass;
    for (int64_t u = blockIdx.x; u < tiles * narr; u += gridDim.x) {
        const int k = (int)(u / tiles);
        const int64_t c0 = (u - (int64_t)k * tiles) * TC;
        const int nc = (int)min((int64_t)TC, cols - c0);
        const double* __restrict__ src = set.src[k];
        double* __restrict__ dst = set.dst[k] + c0 * rows;
        for (int e = tid; e < rows * nc; e += nt) {
            const int r = e / nc, c = e - r * nc;
            tile[c * pitch + r] = src[(int64_t)r * cols + c0 + c];
        }
        __syncthreads();
        for (int e = tid; e < nc * rows; e += nt) {
            const int c = e / rows, r = e - c * rows;
            dst[e] = tile[c * pitch + r];
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
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t cap = (int64_t)std::max(sms, 1) * 16;
    if (rows < kTile && cols >= kTile) {
        const int TC = kNarrowElems / (int)rows / 32 * 32;
        const int64_t tiles = (cols + TC - 1) / TC * k;
        transpose_narrow_dst_kernel<<<(unsigned)std::min<int64_t>(tiles, cap), dim3(kTile, kRowsPerPass), 0, s>>>(
            set, k, (int)rows, cols);
    } else if (cols < kTile) {
        const int TR = kNarrowElems / (int)cols / 32 * 32;
        const int64_t tiles = (rows + TR - 1) / TR * k;
        transpose_narrow_kernel<<<(unsigned)std::min<int64_t>(tiles, cap), dim3(kTile, kRowsPerPass), 0, s>>>(
            set, k, rows, (int)cols);
    } else {
        const int64_t tiles = ((rows + kTile - 1) / kTile) * ((cols + kTile - 1) / kTile) * k;
        transpose_kernel<<<(unsigned)std::min<int64_t>(tiles, cap), dim3(kTile, kRowsPerPass), 0, s>>>(set, k, rows,
                                                                                                     cols);
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace pcrp
