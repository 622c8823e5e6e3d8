/*
 * pcrp_oracle.c -- CPU oracle for the batched pentadiagonal solve.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file.  It is the checker that tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py compare the CUDA path against.
 *
 * Two solvers live here:
 *
 *  1. oracle_pcr_*  -- a plain-C restatement of the reference's PCR-Penta
 *     algorithm (AbhijitGhosh0007/PCR-Penta, kernel.cu:32-154, whose stride
 *     arithmetic is repeated in kernel.cu:158-791 for the n>1024 path).  One
 *     stride maps every row i to a new row that couples i-4d, i-2d, i, i+2d,
 *     i+4d (Reductions I, II, III).  Each stride is Jacobi style: all new rows
 *     are formed from the old state, then the state is replaced, exactly as
 *     the two __syncthreads() of kernel.cu:135,142 order it.  The number of
 *     strides follows the host code main.cu:38-39 (see oracle_ref_strides),
 *     the final pairwise 2x2 / single x=y/c step follows kernel.cu:145-153.
 *     Zero-divisor guards follow kernel.cu:72-75,85-86,98-101,111-112 and the
 *     Reduction-III fallback (kernel.cu:122,129: a zero pivot keeps the
 *     multiplier of the last assignment) is kept, with the multipliers of each
 *     row persisting across strides like the per-thread registers they are in
 *     the reference.  The reference leaves them uninitialised; here they start
 *     at 0.
 *
 *  2. oracle_ge_*   -- FP64 banded Gaussian elimination without pivoting
 *     (pentadiagonal LU), the ground truth for diagonally dominant inputs.
 *     It has no counterpart in the reference.
 *
 * Band convention (reference Annexure A p.1, kernel.cu:77-79): row i reads
 *     a_i x_{i-2} + b_i x_{i-1} + c_i x_i + d_i x_{i+1} + e_i x_{i+2} = y_i.
 * Out-of-range slots (a_0, a_1, b_0, d_{n-1}, e_{n-2}, e_{n-1}) are never read
 * as coefficients by either solver, whatever they hold.
 *
 * Batch addressing: element (system j, row i) lives at  j*sys_stride +
 * i*row_stride.  Contiguous layout (the reference's, kernel.cu:43) is
 * (sys_stride=n, row_stride=1); interleaved (Annexure A p.2) is (1, m).
 *
 * Build with -ffp-contract=off so x86 and aarch64 hosts round identically.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------ */
/* stride count                                                        */
/* ------------------------------------------------------------------ */

/* Number of PCR strides the reference runs on a system of n rows.
 * main.cu:39 computes k2 = ceil((float)log(n)/log(2)) and pcr_penta loops
 * k2-1 times (kernel.cu:63).  Because (float)ln(2^k) rounds up, k2 is
 * log2(n)+1 for every power of two up to 1024, so a power-of-two system gets
 * log2(n) strides and finishes with x = y/c; any other n gets ceil(log2 n)-1
 * strides and finishes with the pairwise 2x2 solve.  For n > 1024 the
 * reference (main.cu:17-20,38,73) runs log2(n/1024) splitting strides plus
 * k1-1 = 10 second-stage strides: log2(n) again.  The same rule is applied
 * to every n here (the reference itself accepts only powers of two above
 * 1024, main.cu:9-10). */
int oracle_ref_strides(int64_t n)
{
    if (n <= 1) return 0;
    int lg = 0;
    while (((int64_t)1 << lg) < n) lg++;          /* lg = ceil(log2 n) */
    if (((int64_t)1 << lg) == n) return lg;        /* power of two       */
    return lg - 1;
}

/* ------------------------------------------------------------------ */
/* PCR-Penta restatement, one system                                   */
/* ------------------------------------------------------------------ */

/* work must hold 14*n doubles.  x may alias nothing else.  Inputs are read
 * through (base + i*rs). */
static void pcr_one(const double* ga, const double* gb, const double* gc,
                    const double* gd, const double* ge, const double* gy,
                    double* gx, int64_t n, int64_t rs, double* work)
{
    double *a = work, *b = a + n, *c = b + n, *d = c + n, *e = d + n, *x = e + n;
    double *na = x + n, *nb = na + n, *nc = nb + n, *nd = nc + n, *ne = nd + n, *nx = ne + n;
    double *al1 = nx + n, *al2 = al1 + n;          /* persistent multipliers */
    for (int64_t i = 0; i < n; i++) {
        a[i] = ga[i * rs]; b[i] = gb[i * rs]; c[i] = gc[i * rs];
        d[i] = gd[i * rs]; e[i] = ge[i * rs]; x[i] = gy[i * rs];
        al1[i] = 0.0; al2[i] = 0.0;
    }
    const int ns = oracle_ref_strides(n);
    int64_t delta = 1;
    for (int l = 0; l < ns; l++) {
        for (int64_t id = 0; id < n; id++) {
            const int64_t p1 = id - delta, p2 = id - 2 * delta;
            const int64_t q1 = id + delta, q2 = id + 2 * delta;
            double alfa1 = al1[id], alfa2 = al2[id];
            double a1 = 0, b1 = 0, c1 = 0, d1 = 0, e1 = 0, k1 = 0;
            double a2 = 0, b2 = 0, c2 = 0, d2 = 0, e2 = 0, k2 = 0;
            /* Reduction-I: rows p2, p1, id (kernel.cu:69-91) */
            if (p2 >= 0) {
                alfa1 = 0.0; alfa2 = 0.0;
                if (id - 3 * delta >= 0 && b[p2] != 0.0) alfa1 = -a[p1] / b[p2];
                if (q1 <= n - 1 && d[id] != 0.0) alfa2 = -e[p1] / d[id];
                a1 = alfa1 * a[p2];
                b1 = alfa1 * c[p2] + b[p1] + alfa2 * a[id];
                c1 = alfa1 * d[p2] + c[p1] + alfa2 * b[id];
                d1 = alfa1 * e[p2] + d[p1] + alfa2 * c[id];
                e1 = alfa2 * e[id];
                k1 = alfa1 * x[p2] + x[p1] + alfa2 * x[id];
            }
            if (p1 >= 0 && p2 < 0) {
                alfa2 = 0.0;
                if (q1 <= n - 1 && d[id] != 0.0) alfa2 = -e[p1] / d[id];
                a1 = 0.0; b1 = 0.0;
                c1 = c[p1] + alfa2 * b[id];
                d1 = d[p1] + alfa2 * c[id];
                e1 = alfa2 * e[id];
                k1 = x[p1] + alfa2 * x[id];
            }
            /* Reduction-II: rows id, q1, q2 (kernel.cu:94-117) */
            if (q2 <= n - 1) {
                alfa1 = 0.0; alfa2 = 0.0;
                if (p1 >= 0 && b[id] != 0.0) alfa1 = -a[q1] / b[id];
                if (id + 3 * delta <= n - 1 && d[q2] != 0.0) alfa2 = -e[q1] / d[q2];
                a2 = alfa1 * a[id];
                b2 = alfa1 * c[id] + b[q1] + alfa2 * a[q2];
                c2 = alfa1 * d[id] + c[q1] + alfa2 * b[q2];
                d2 = alfa1 * e[id] + d[q1] + alfa2 * c[q2];
                e2 = alfa2 * e[q2];
                k2 = alfa1 * x[id] + x[q1] + alfa2 * x[q2];
            }
            if (q1 <= n - 1 && q2 > n - 1) {
                alfa1 = 0.0;
                if (p1 >= 0 && b[id] != 0.0) alfa1 = -a[q1] / b[id];
                a2 = alfa1 * a[id];
                b2 = alfa1 * c[id] + b[q1];
                c2 = alfa1 * d[id] + c[q1];
                d2 = 0.0; e2 = 0.0;
                k2 = alfa1 * x[id] + x[q1];
            }
            /* Reduction-III (kernel.cu:120-132) */
            if (p1 >= 0) {
                if (c1 != 0.0) alfa1 = b[id] / c1;
                a1 = alfa1 * a1; b1 = alfa1 * b1; c1 = alfa1 * d1; d1 = alfa1 * e1; k1 = alfa1 * k1;
            } else { a1 = 0.0; b1 = 0.0; c1 = 0.0; d1 = 0.0; k1 = 0.0; }
            if (q1 <= n - 1) {
                if (c2 != 0.0) alfa2 = d[id] / c2;
                c2 = alfa2 * b2; b2 = alfa2 * a2; d2 = alfa2 * d2; e2 = alfa2 * e2; k2 = alfa2 * k2;
            } else { b2 = 0.0; c2 = 0.0; d2 = 0.0; e2 = 0.0; k2 = 0.0; }
            /* new row (kernel.cu:138-140) */
            nb[id] = b1 - a[id] + b2;
            nc[id] = c1 - c[id] + c2;
            nd[id] = d1 - e[id] + d2;
            nx[id] = k1 - x[id] + k2;
            na[id] = a1;
            ne[id] = e2;
            al1[id] = alfa1; al2[id] = alfa2;
        }
        memcpy(a, na, n * sizeof(double)); memcpy(b, nb, n * sizeof(double));
        memcpy(c, nc, n * sizeof(double)); memcpy(d, nd, n * sizeof(double));
        memcpy(e, ne, n * sizeof(double)); memcpy(x, nx, n * sizeof(double));
        delta *= 2;
    }
    /* final pairwise / single solve (kernel.cu:145-153) */
    for (int64_t id = 0; id < n; id++) {
        if (id < n - delta) {
            const int64_t iid = id + delta;
            const double deno = c[id] * c[iid] - b[iid] * d[id];
            gx[id * rs] = (c[iid] * x[id] - d[id] * x[iid]) / deno;
            gx[iid * rs] = (c[id] * x[iid] - b[iid] * x[id]) / deno;
        }
        if (id >= n - delta && id < delta) gx[id * rs] = x[id] / c[id];
    }
}

/* ------------------------------------------------------------------ */
/* Banded Gaussian elimination, one system                             */
/* ------------------------------------------------------------------ */

/* work must hold 3*n doubles.  Out-of-range band slots are skipped. */
static void ge_one(const double* a, const double* b, const double* c,
                   const double* d, const double* e, const double* y,
                   double* x, int64_t n, int64_t rs, double* work)
{
    double *p = work, *q = p + n, *z = q + n;   /* U row i: x_i + p_i x_{i+1} + q_i x_{i+2} = z_i */
    for (int64_t i = 0; i < n; i++) {
        double bb = (i >= 1) ? b[i * rs] : 0.0;
        double cc = c[i * rs];
        double dd = (i + 1 < n) ? d[i * rs] : 0.0;
        double ee = (i + 2 < n) ? e[i * rs] : 0.0;
        double zz = y[i * rs];
        if (i >= 2) {
            const double aa = a[i * rs];
            bb -= aa * p[i - 2];
            cc -= aa * q[i - 2];
            zz -= aa * z[i - 2];
        }
        if (i >= 1) {
            cc -= bb * p[i - 1];
            dd -= bb * q[i - 1];
            zz -= bb * z[i - 1];
        }
        p[i] = dd / cc;
        q[i] = ee / cc;
        z[i] = zz / cc;
    }
    for (int64_t i = n - 1; i >= 0; i--) {
        double v = z[i];
        if (i + 1 < n) v -= p[i] * x[(i + 1) * rs];
        if (i + 2 < n) v -= q[i] * x[(i + 2) * rs];
        x[i * rs] = v;
    }
}

/* ------------------------------------------------------------------ */
/* batch drivers (threads over systems)                                */
/* ------------------------------------------------------------------ */

typedef struct {
    const double *a, *b, *c, *d, *e, *y;
    double* x;
    const int64_t* offs;     /* ragged: first row of each system (contiguous), or NULL */
    const int64_t* sizes;    /* ragged: rows of each system, or NULL                    */
    int64_t m, n, ss, rs;
    int kind;                /* 0 = pcr, 1 = ge */
    int64_t j0, j1;
    int rc;
} job_t;

static void* job_run(void* arg)
{
    job_t* jb = (job_t*)arg;
    int64_t nmax = jb->n;
    if (jb->sizes) {
        nmax = 1;
        for (int64_t j = jb->j0; j < jb->j1; j++) if (jb->sizes[j] > nmax) nmax = jb->sizes[j];
    }
    double* w = (double*)malloc(sizeof(double) * (size_t)(nmax > 0 ? nmax : 1) * (jb->kind == 0 ? 14 : 3));
    if (!w) { jb->rc = -1; return NULL; }
    for (int64_t j = jb->j0; j < jb->j1; j++) {
        int64_t o = jb->offs ? jb->offs[j] : j * jb->ss;
        int64_t n = jb->sizes ? jb->sizes[j] : jb->n;
        if (jb->kind == 0)
            pcr_one(jb->a + o, jb->b + o, jb->c + o, jb->d + o, jb->e + o, jb->y + o, jb->x + o, n, jb->rs, w);
        else
            ge_one(jb->a + o, jb->b + o, jb->c + o, jb->d + o, jb->e + o, jb->y + o, jb->x + o, n, jb->rs, w);
    }
    free(w);
    jb->rc = 0;
    return NULL;
}

static int run_batch(job_t base, int nthreads)
{
    if (base.m <= 0) return 0;
    if (nthreads <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        nthreads = c > 0 ? (int)c : 1;
    }
    if (nthreads > base.m) nthreads = (int)base.m;
    job_t* jobs = (job_t*)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return -1; }
    int rc = 0;
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = base;
        jobs[t].j0 = base.m * t / nthreads;
        jobs[t].j1 = base.m * (t + 1) / nthreads;
        if (nthreads == 1) job_run(&jobs[t]);
        else if (pthread_create(&th[t], NULL, job_run, &jobs[t]) != 0) { job_run(&jobs[t]); th[t] = 0; }
    }
    for (int t = 0; t < nthreads; t++) {
        if (nthreads > 1 && th[t]) pthread_join(th[t], NULL);
        if (jobs[t].rc) rc = jobs[t].rc;
    }
    free(jobs); free(th);
    return rc;
}

/* layout: 0 contiguous (j*n+i), 1 interleaved (i*m+j).  nthreads<=0: all cores.
 * Returns 0 on success. */
int oracle_pcr_batch(const double* a, const double* b, const double* c, const double* d,
                     const double* e, const double* y, double* x, int64_t m, int64_t n,
                     int layout, int nthreads)
{
    job_t jb; memset(&jb, 0, sizeof jb);
    jb.a = a; jb.b = b; jb.c = c; jb.d = d; jb.e = e; jb.y = y; jb.x = x;
    jb.m = m; jb.n = n; jb.kind = 0;
    jb.ss = layout ? 1 : n; jb.rs = layout ? m : 1;
    return run_batch(jb, nthreads);
}

int oracle_ge_batch(const double* a, const double* b, const double* c, const double* d,
                    const double* e, const double* y, double* x, int64_t m, int64_t n,
                    int layout, int nthreads)
{
    job_t jb; memset(&jb, 0, sizeof jb);
    jb.a = a; jb.b = b; jb.c = c; jb.d = d; jb.e = e; jb.y = y; jb.x = x;
    jb.m = m; jb.n = n; jb.kind = 1;
    jb.ss = layout ? 1 : n; jb.rs = layout ? m : 1;
    return run_batch(jb, nthreads);
}

/* Ragged batch: system j occupies rows offs[j] .. offs[j]+sizes[j]-1, contiguous. */
int oracle_ragged_batch(const double* a, const double* b, const double* c, const double* d,
                        const double* e, const double* y, double* x, const int64_t* offs,
                        const int64_t* sizes, int64_t nsys, int kind, int nthreads)
{
    job_t jb; memset(&jb, 0, sizeof jb);
    jb.a = a; jb.b = b; jb.c = c; jb.d = d; jb.e = e; jb.y = y; jb.x = x;
    jb.m = nsys; jb.n = 0; jb.kind = kind; jb.offs = offs; jb.sizes = sizes;
    jb.ss = 0; jb.rs = 1;
    return run_batch(jb, nthreads);
}

/* r = y - A x for every system (contiguous or interleaved), FP64 with the
 * products summed in long double to keep the residual itself accurate. */
int oracle_residual_batch(const double* a, const double* b, const double* c, const double* d,
                          const double* e, const double* y, const double* x, double* r,
                          int64_t m, int64_t n, int layout)
{
    const int64_t ss = layout ? 1 : n, rs = layout ? m : 1;
    for (int64_t j = 0; j < m; j++) {
        const int64_t o = j * ss;
        for (int64_t i = 0; i < n; i++) {
            const int64_t k = o + i * rs;
            long double s = (long double)y[k] - (long double)c[k] * x[k];
            if (i >= 2) s -= (long double)a[k] * x[k - 2 * rs];
            if (i >= 1) s -= (long double)b[k] * x[k - rs];
            if (i + 1 < n) s -= (long double)d[k] * x[k + rs];
            if (i + 2 < n) s -= (long double)e[k] * x[k + 2 * rs];
            r[k] = (double)s;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* seeded inputs                                                       */
/* ------------------------------------------------------------------ */

/* The benchmark inputs, restated here so that the CPU leg of the benchmark
 * (and the reference arm, which times this file's PCR restatement) never
 * loads the product library.  Same definition as the library's generator:
 * every value is a pure function of (seed, kind, system j, row i, n), drawn
 * from SplitMix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number
 * generators", OOPSLA 2014) of a counter packing (stream, system, row).
 * tests/test_oracle.py checks the two bit for bit.  kind: 0 dominant
 * (a,b,d,e ~ U[-1,1], c = sum|off| + U[1,2]), 1 ADI convection-diffusion
 * (M = I - theta dt L, theta = 0.5, dt = 1e-3, r = 0.03 on S in [0, 800]),
 * 2 weakly dominant (c = +-1.05 sum|off|), 3 the reference's Toeplitz
 * fixture (kernel.cu:19-24).  y ~ U[-1,1], or the payoff max(S-K, 0). */
static uint64_t sm64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double g_unit(uint64_t seed, int stream, uint64_t j, uint64_t i)
{
    const uint64_t ctr = ((uint64_t)stream << 56) | ((j & 0xFFFFFFULL) << 32) | (i & 0xFFFFFFFFULL);
    const uint64_t z = sm64(sm64(seed) + ctr * 0xD1B54A32D192ED03ULL);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

static double g_uniform(uint64_t seed, int stream, uint64_t j, uint64_t i, double lo, double hi)
{
    return lo + (hi - lo) * g_unit(seed, stream, j, i);
}

static void g_row(int kind, uint64_t seed, uint64_t j, int64_t i, int64_t n, double* v)
{
    const int hasA = i >= 2, hasB = i >= 1, hasD = i + 1 < n, hasE = i + 2 < n;
    double a, b, c, d, e, y;
    if (kind == 0 || kind == 2) {
        a = hasA ? g_uniform(seed, 0, j, (uint64_t)i, -1.0, 1.0) : 0.0;
        b = hasB ? g_uniform(seed, 1, j, (uint64_t)i, -1.0, 1.0) : 0.0;
        d = hasD ? g_uniform(seed, 3, j, (uint64_t)i, -1.0, 1.0) : 0.0;
        e = hasE ? g_uniform(seed, 4, j, (uint64_t)i, -1.0, 1.0) : 0.0;
        const double off = ((fabs(a) + fabs(b)) + fabs(d)) + fabs(e);
        if (kind == 0) {
            c = off + g_uniform(seed, 2, j, (uint64_t)i, 1.0, 2.0);
        } else {
            const double sgn = (sm64(seed ^ 0x5EED5EED5EEDULL ^ (j << 32) ^ (uint64_t)i) >> 63) ? -1.0 : 1.0;
            c = off != 0.0 ? sgn * (1.05 * off) : sgn;
        }
        y = g_uniform(seed, 5, j, (uint64_t)i, -1.0, 1.0);
    } else if (kind == 1) {
        const double vv = g_uniform(seed, 6, j, 0, 0.01, 1.0);
        const double K = g_uniform(seed, 7, j, 0, 50.0, 150.0);
        const double rr = 0.03, tdt = 0.5 * 1e-3;
        const double h = n > 1 ? 800.0 / (double)(n - 1) : 800.0;
        const double S = (double)i * h;
        const double diff = ((0.5 * vv) * (S * S)) / (h * h);
        const double conv = (rr * S) / (2.0 * h);
        a = 0.0;
        b = hasB ? -(tdt * diff) : 0.0;
        c = 1.0 + tdt * (((2.0 * diff) + (3.0 * conv)) + rr);
        d = hasD ? -(tdt * (diff + 4.0 * conv)) : 0.0;
        e = hasE ? tdt * conv : 0.0;
        const double pay = S - K;
        y = pay > 0.0 ? pay : 0.0;
    } else {
        a = 1.0; b = -4.0; c = 6.0; d = -4.0; e = 1.0; y = 1.0;
        if (i == 0) { a = 0.0; b = 1.0; c = 5.0; }
        if (i == 1) a = 0.0;
        if (i == n - 2) e = 0.0;
        if (i == n - 1) { c = 5.0; d = 1.0; e = 0.0; }
    }
    v[0] = a; v[1] = b; v[2] = c; v[3] = d; v[4] = e; v[5] = y;
}

typedef struct {
    int kind, layout;
    uint64_t seed;
    int64_t m, n, j0, j1;
    double *a, *b, *c, *d, *e, *y;
} gen_job_t;

static void* gen_run(void* arg)
{
    const gen_job_t* g = (const gen_job_t*)arg;
    for (int64_t j = g->j0; j < g->j1; j++)
        for (int64_t i = 0; i < g->n; i++) {
            double v[6];
            const int64_t k = g->layout ? i * g->m + j : j * g->n + i;
            g_row(g->kind, g->seed, (uint64_t)j, i, g->n, v);
            g->a[k] = v[0]; g->b[k] = v[1]; g->c[k] = v[2]; g->d[k] = v[3]; g->e[k] = v[4]; g->y[k] = v[5];
        }
    return NULL;
}

/* Fills the six arrays of a batch (layout 0 contiguous, 1 interleaved),
 * systems split over nthreads threads (<= 0: all cores). */
int oracle_generate(int kind, uint64_t seed, int64_t m, int64_t n, int layout,
                    double* a, double* b, double* c, double* d, double* e, double* y, int nthreads)
{
    if (kind < 0 || kind > 3 || m < 0 || n < 0) return -1;
    if (nthreads <= 0) {
        long cpus = sysconf(_SC_NPROCESSORS_ONLN);
        nthreads = cpus > 0 ? (int)cpus : 1;
    }
    if (nthreads > m) nthreads = m > 0 ? (int)m : 1;
    gen_job_t jobs[256];
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    for (int t = 0; t < nthreads; t++) {
        gen_job_t g = {kind, layout, seed, m, n, m * t / nthreads, m * (t + 1) / nthreads, a, b, c, d, e, y};
        jobs[t] = g;
        if (nthreads == 1 || pthread_create(&th[t], NULL, gen_run, &jobs[t]) != 0) {
            gen_run(&jobs[t]);
            th[t] = 0;
        }
    }
    for (int t = 0; t < nthreads; t++)
        if (nthreads > 1 && th[t]) pthread_join(th[t], NULL);
    return 0;
}
