/*
 * refrun.c -- runs the reference's OWN kernels (PCR-Penta kernel.cu, compiled
 * unmodified to PTX by build_ref.sh) on the GPU through the CUDA driver API,
 * with the launch geometry of the reference host code (main.cu:16-22,38-39,
 * 46-87).  TEST INFRASTRUCTURE ONLY: it produces the reference's own outputs
 * that pin the CPU oracle; the product never loads it.
 *
 * variant 0: pcr_penta (n <= 1024), main.cu:49
 * variant 2: global_cached_shared_tile_splitting + pcr_penta_splitting_2nd_stage, main.cu:136,147
 * variant 3: global_cached_global_tile_splitting + pcr_penta_splitting_2nd_stage, main.cu:208,219
 * (variant 1, shared_cached_shared_tile_splitting, has a shared-memory race
 *  between kernel.cu:201-228 and kernel.cu:309-314 and is not run.)
 * The reference's kernels are valid for power-of-two n > 1024 only up to
 * n = 2^19 (their stage-1 tiles look back one 512-row tile); larger or
 * non-power-of-two n above 1024 are refused here.  Registers are capped at
 * 64 (JIT option) so the 1024-thread launches fit the register file.
 */
#include <cuda.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static char g_err[512];
const char* refrun_last_error(void) { return g_err; }

#define CK(call) do { CUresult r_ = (call); if (r_ != CUDA_SUCCESS) { const char* s_ = 0; \
    cuGetErrorString(r_, &s_); snprintf(g_err, sizeof g_err, "%s failed: %s (line %d)", #call, s_ ? s_ : "?", __LINE__); \
    rc = -(int)r_; goto done; } } while (0)

static char* read_file(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    char* buf = (char*)malloc((size_t)sz + 1);
    if (buf && fread(buf, 1, (size_t)sz, f) != (size_t)sz) { free(buf); buf = NULL; }
    if (buf) buf[sz] = 0;
    fclose(f);
    return buf;
}

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* The reference host code's launches for one solve (main.cu:39,49 for
 * n <= 1024; main.cu:95-99,115,136-156 (variant 2) and
 * main.cu:168-172,188,208-228 (variant 3) above). */
static CUresult launch_ref(CUmodule mod, int variant, CUdeviceptr* dp, int m, int n)
{
    CUresult r;
    if (n <= 1024) {
        int k2 = (int)ceil((float)log((double)n) / log(2.0));
        CUfunction f;
        if ((r = cuModuleGetFunction(&f, mod, "_Z9pcr_pentaPdS_S_S_S_S_ii")) != CUDA_SUCCESS) return r;
        void* args[8] = {&dp[0], &dp[1], &dp[2], &dp[3], &dp[4], &dp[5], &k2, &n};
        return cuLaunchKernel(f, (unsigned)m, 1, 1, (unsigned)n, 1, 1, (unsigned)(6 * n * sizeof(double)), NULL, args,
                              NULL);
    }
    int tile_size = 512;
    int num_tile = (int)ceil((float)n / tile_size);
    int gen_sys_size = 1024;
    int num_gen_sys = (int)ceil((float)n / gen_sys_size);
    int num_split = (int)(log((double)num_gen_sys) / log(2.0));
    int k1 = (int)ceil((float)log((double)gen_sys_size) / log(2.0));
    CUfunction f1, f2;
    if ((r = cuModuleGetFunction(&f1, mod, variant == 2 ? "_Z35global_cached_shared_tile_splittingPdS_S_S_S_S_iiii"
                                                        : "_Z35global_cached_global_tile_splittingPdS_S_S_S_S_iiii"))
        != CUDA_SUCCESS) return r;
    if ((r = cuModuleGetFunction(&f2, mod, "_Z29pcr_penta_splitting_2nd_stagePdS_S_S_S_S_iiii")) != CUDA_SUCCESS)
        return r;
    void* args1[10] = {&dp[0], &dp[1], &dp[2], &dp[3], &dp[4], &dp[5], &num_split, &num_tile, &tile_size, &n};
    unsigned smem1 = variant == 2 ? (unsigned)(6 * tile_size * sizeof(double)) : 0u;
    if ((r = cuLaunchKernel(f1, (unsigned)m, 1, 1, (unsigned)tile_size, 1, 1, smem1, NULL, args1, NULL))
        != CUDA_SUCCESS) return r;
    void* args2[10] = {&dp[0], &dp[1], &dp[2], &dp[3], &dp[4], &dp[5], &k1, &num_gen_sys, &gen_sys_size, &n};
    return cuLaunchKernel(f2, (unsigned)(m * num_gen_sys), 1, 1, (unsigned)gen_sys_size, 1, 1,
                          (unsigned)(6 * gen_sys_size * sizeof(double)), NULL, args2, NULL);
}

static int check_args(int variant, int m, int n)
{
    if (m <= 0 || n <= 0 || (long long)m * n >= (1LL << 31)) { snprintf(g_err, sizeof g_err, "bad size"); return -1000; }
    if (n > 1024 && (!is_pow2(n) || n > (1 << 19))) { snprintf(g_err, sizeof g_err, "reference kernels invalid for n=%d", n); return -1001; }
    if (n > 1024 && variant != 2 && variant != 3) { snprintf(g_err, sizeof g_err, "variant %d is not a split variant", variant); return -1002; }
    return 0;
}

/* Host arrays in, solution out (contiguous layout, m systems of n rows).
 * With reps > 0 (refrun_time) the solve is also timed: after the first
 * solve, `reps` more run with the inputs restored from a pristine device
 * copy before each (the split kernels overwrite the bands), CUDA events
 * around each solve's launches only; *ms receives the mean. */
static int run(const char* ptx_path, int variant, const double* const* host, double* x, int m, int n, int reps,
               float* ms)
{
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = NULL;
    CUmodule mod = NULL;
    CUdeviceptr dp[6] = {0, 0, 0, 0, 0, 0}, keep[6] = {0, 0, 0, 0, 0, 0};
    CUevent e0 = NULL, e1 = NULL;
    char* ptx = NULL;
    g_err[0] = 0;
    if ((rc = check_args(variant, m, n)) != 0) return rc;
    ptx = read_file(ptx_path);
    if (!ptx) { snprintf(g_err, sizeof g_err, "cannot read %s", ptx_path); return -1003; }

    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxPushCurrent(ctx));
    {
        CUjit_option opt[1] = {CU_JIT_MAX_REGISTERS};
        void* val[1] = {(void*)(size_t)64};
        CK(cuModuleLoadDataEx(&mod, ptx, 1, opt, val));
    }
    const size_t bytes = (size_t)m * (size_t)n * sizeof(double);
    for (int k = 0; k < 6; k++) {
        CK(cuMemAlloc(&dp[k], bytes));
        CK(cuMemcpyHtoD(dp[k], host[k], bytes));
        if (reps > 0) { CK(cuMemAlloc(&keep[k], bytes)); CK(cuMemcpyDtoD(keep[k], dp[k], bytes)); }
    }
    CK(launch_ref(mod, variant, dp, m, n));
    CK(cuCtxSynchronize());
    if (x) CK(cuMemcpyDtoH(x, dp[5], bytes));
    if (reps > 0) {
        float total = 0.0f;
        CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
        CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
        for (int r = 0; r < reps; r++) {
            for (int k = 0; k < 6; k++) CK(cuMemcpyDtoD(dp[k], keep[k], bytes));
            CK(cuCtxSynchronize());
            CK(cuEventRecord(e0, NULL));
            CK(launch_ref(mod, variant, dp, m, n));
            CK(cuEventRecord(e1, NULL));
            CK(cuEventSynchronize(e1));
            float t = 0.0f;
            CK(cuEventElapsedTime(&t, e0, e1));
            total += t;
        }
        *ms = total / (float)reps;
    }
done:
    if (e0) cuEventDestroy(e0);
    if (e1) cuEventDestroy(e1);
    for (int k = 0; k < 6; k++) { if (dp[k]) cuMemFree(dp[k]); if (keep[k]) cuMemFree(keep[k]); }
    if (mod) cuModuleUnload(mod);
    if (ctx) { CUcontext tmp; cuCtxPopCurrent(&tmp); cuDevicePrimaryCtxRelease(dev); }
    free(ptx);
    return rc;
}

int refrun_solve(const char* ptx_path, int variant, const double* a, const double* b, const double* c,
                 const double* d, const double* e, const double* y, double* x, int m, int n)
{
    const double* host[6] = {a, b, c, d, e, y};
    return run(ptx_path, variant, host, x, m, n, 0, NULL);
}

int refrun_time(const char* ptx_path, int variant, const double* a, const double* b, const double* c,
                const double* d, const double* e, const double* y, double* x, int m, int n, int reps, float* ms)
{
    const double* host[6] = {a, b, c, d, e, y};
    if (reps < 1 || !ms) { snprintf(g_err, sizeof g_err, "refrun_time: reps >= 1 and ms needed"); return -1004; }
    return run(ptx_path, variant, host, x, m, n, reps, ms);
}
