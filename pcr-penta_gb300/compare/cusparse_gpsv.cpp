// cusparse_gpsv.cpp -- timed comparison point: cuSPARSE's batched
// pentadiagonal solver (cusparseDgpsvInterleavedBatch, QR with Householder
// reflections), called as a library on the same interleaved FP64 batch the
// pcrp solvers take.  Not part of libpcrp; built beside it for the benchmark
// and its test.  Note that gpsv overwrites the five band arrays.
#include <cuda_runtime.h>
#include <cusparse.h>

#include <cstddef>

namespace {
thread_local cusparseHandle_t g_handle = nullptr;

int handle(cudaStream_t s) {
    if (!g_handle && cusparseCreate(&g_handle) != CUSPARSE_STATUS_SUCCESS) return -1;
    return cusparseSetStream(g_handle, s) == CUSPARSE_STATUS_SUCCESS ? 0 : -2;
}
}  // namespace

extern "C" int cmp_gpsv_buffer_size(const double* ds, const double* dl, const double* d, const double* du,
                                    const double* dw, const double* x, int n, int batch, size_t* bytes)
{
    if (handle(nullptr)) return -1;
    return (int)cusparseDgpsvInterleavedBatch_bufferSizeExt(g_handle, 0, n, ds, dl, d, du, dw, x, batch, bytes);
}

extern "C" int cmp_gpsv_solve(double* ds, double* dl, double* d, double* du, double* dw, double* x, int n,
                              int batch, void* buffer, void* stream)
{
    if (handle((cudaStream_t)stream)) return -1;
    return (int)cusparseDgpsvInterleavedBatch(g_handle, 0, n, ds, dl, d, du, dw, x, batch, buffer);
}
