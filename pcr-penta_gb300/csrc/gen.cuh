// gen.cuh -- seeded, counter-based band generators shared by host and device.
//
// Every value is a pure function of (seed, kind, system j, row i, n), so the
// host threads and the device kernel produce bit-identical batches and any
// slice of a batch regenerates identically.  Arithmetic goes through the
// explicitly rounded helpers below (no FMA contraction on either side).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define PCRP_HD __host__ __device__ __forceinline__
#else
#define PCRP_HD inline
#endif

namespace pcrp {
namespace gen {

PCRP_HD uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

#if defined(__CUDA_ARCH__)
PCRP_HD double gmul(double x, double y) { return __dmul_rn(x, y); }
PCRP_HD double gadd(double x, double y) { return __dadd_rn(x, y); }
PCRP_HD double gsub(double x, double y) { return __dsub_rn(x, y); }
PCRP_HD double gdiv(double x, double y) { return __ddiv_rn(x, y); }
#else
// host side: the library is compiled with -ffp-contract=off
PCRP_HD double gmul(double x, double y) { return x * y; }
PCRP_HD double gadd(double x, double y) { return x + y; }
PCRP_HD double gsub(double x, double y) { return x - y; }
PCRP_HD double gdiv(double x, double y) { return x / y; }
#endif
PCRP_HD double gabs(double x) { return x < 0.0 ? -x : x; }

// Stream ids of the counter.
enum { S_A = 0, S_B = 1, S_C = 2, S_D = 3, S_E = 4, S_Y = 5, S_P1 = 6, S_P2 = 7 };

// u in [0,1): 53 random bits of splitmix64(splitmix64(seed) + counter) where the
// counter packs (stream << 56) | (system << 32) | row  (system < 2^24, row < 2^32).
PCRP_HD double unit(uint64_t seed, int stream, uint64_t j, uint64_t i) {
    const uint64_t ctr = ((uint64_t)stream << 56) | ((j & 0xFFFFFFULL) << 32) | (i & 0xFFFFFFFFULL);
    const uint64_t z = splitmix64(splitmix64(seed) + ctr * 0xD1B54A32D192ED03ULL);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

PCRP_HD double uniform(uint64_t seed, int stream, uint64_t j, uint64_t i, double lo, double hi) {
    return gadd(lo, gmul(gsub(hi, lo), unit(seed, stream, j, i)));
}

struct Row { double a, b, c, d, e, y; };

// kind: 0 dominant, 1 ADI convection-diffusion, 2 weakly dominant, 3 Toeplitz fixture.
PCRP_HD Row row(int kind, uint64_t seed, uint64_t j, int64_t i, int64_t n) {
    Row R;
    const bool hasA = i >= 2, hasB = i >= 1, hasD = i + 1 < n, hasE = i + 2 < n;
    if (kind == 0 || kind == 2) {
        R.a = hasA ? uniform(seed, S_A, j, i, -1.0, 1.0) : 0.0;
        R.b = hasB ? uniform(seed, S_B, j, i, -1.0, 1.0) : 0.0;
        R.d = hasD ? uniform(seed, S_D, j, i, -1.0, 1.0) : 0.0;
        R.e = hasE ? uniform(seed, S_E, j, i, -1.0, 1.0) : 0.0;
        const double off = gadd(gadd(gadd(gabs(R.a), gabs(R.b)), gabs(R.d)), gabs(R.e));
        if (kind == 0) {
            R.c = gadd(off, uniform(seed, S_C, j, i, 1.0, 2.0));
        } else {
            const double sgn = (splitmix64(seed ^ 0x5EED5EED5EEDULL ^ ((uint64_t)j << 32) ^ (uint64_t)i) >> 63) ? -1.0 : 1.0;
            R.c = off != 0.0 ? gmul(sgn, gmul(1.05, off)) : sgn;
        }
        R.y = uniform(seed, S_Y, j, i, -1.0, 1.0);
    } else if (kind == 1) {
        // M = I - theta*dt*L on S_i = i*h, h = 800/(n-1);
        // L = 0.5 v S^2 (1,-2,1)/h^2 + r S (-3,4,-1)/(2h) on offsets (0,+1,+2) - r.
        const double v = uniform(seed, S_P1, j, 0, 0.01, 1.0);
        const double K = uniform(seed, S_P2, j, 0, 50.0, 150.0);
        const double rr = 0.03, tdt = gmul(0.5, 1e-3);
        const double h = n > 1 ? gdiv(800.0, (double)(n - 1)) : 800.0;
        const double S = gmul((double)i, h);
        const double diff = gdiv(gmul(gmul(0.5, v), gmul(S, S)), gmul(h, h));
        const double conv = gdiv(gmul(rr, S), gmul(2.0, h));
        R.a = 0.0;
        R.b = hasB ? -gmul(tdt, diff) : 0.0;
        R.c = gadd(1.0, gmul(tdt, gadd(gadd(gmul(2.0, diff), gmul(3.0, conv)), rr)));
        R.d = hasD ? -gmul(tdt, gadd(diff, gmul(4.0, conv))) : 0.0;
        R.e = hasE ? gmul(tdt, conv) : 0.0;
        const double pay = gsub(S, K);
        R.y = pay > 0.0 ? pay : 0.0;
    } else {
        // the reference's initialize kernel (kernel.cu:19-24), same order of overrides
        R.a = 1.0; R.b = -4.0; R.c = 6.0; R.d = -4.0; R.e = 1.0; R.y = 1.0;
        if (i == 0) { R.a = 0.0; R.b = 1.0; R.c = 5.0; }
        if (i == 1) R.a = 0.0;
        if (i == n - 2) R.e = 0.0;
        if (i == n - 1) { R.c = 5.0; R.d = 1.0; R.e = 0.0; }
    }
    return R;
}

}  // namespace gen
}  // namespace pcrp
