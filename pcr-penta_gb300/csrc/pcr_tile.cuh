// pcr_tile.cuh -- the faithful FP64 PCR-Penta work of one CTA (shared by the
// uniform-batch kernels of pcr_f64.cu and the persistent ragged kernel).
// The arithmetic and its correspondence with the reference are described at
// the top of pcr_f64.cu.
#pragma once
#include "pcrp_internal.h"
#include "tma.cuh"

namespace pcrp {

__device__ __forceinline__ double mul(double x, double y) { return __dmul_rn(x, y); }
__device__ __forceinline__ double add(double x, double y) { return __dadd_rn(x, y); }
__device__ __forceinline__ double sub(double x, double y) { return __dsub_rn(x, y); }
// Bits of x other than the sign, OR-folded into one word: zero exactly for
// +-0.  Written in PTX on the two 32-bit halves so that it stays on the
// integer pipe (the equivalent C bit test can be turned into an FP64 compare,
// which here takes a slot of the FP64 pipe).
__device__ __forceinline__ unsigned magbits(double x) {
    unsigned r;
    asm("{\n\t.reg .b32 lo, hi;\n\tmov.b64 {lo, hi}, %1;\n\tshl.b32 hi, hi, 1;\n\tor.b32 %0, hi, lo;\n\t}"
        : "=r"(r) : "d"(x));
    return r;
}
// x != 0.0 (false for +-0, true for everything else including NaN)
__device__ __forceinline__ bool nz(double x) { return magbits(x) != 0u; }
// x / y, IEEE round-to-nearest.  A zero x over a nonzero finite y is the
// signed zero IEEE 754 prescribes (sign of x xor sign of y), formed on the
// integer pipe: the FP64 division takes ~2.6x its normal time for a zero
// numerator, and from stride ~2^9 on the outer coefficients of a diagonally
// dominant system are zero, so half of the divisions of the late strides
// have one.  Every other operand pair goes to the division.
__device__ __forceinline__ double dvd(double x, double y) {
    const unsigned yh = (unsigned)__double2hiint(y);
    if (magbits(x) == 0u && magbits(y) != 0u && (yh & 0x7FF00000u) != 0x7FF00000u)
        return __hiloint2double((int)((((unsigned)__double2hiint(x)) ^ yh) & 0x80000000u), 0);
    return __ddiv_rn(x, y);
}
// -x by flipping the sign bit on the integer pipe (bit-identical to unary
// minus), in PTX for the same reason as magbits
__device__ __forceinline__ double neg(double x) {
    double r;
    asm("{\n\t.reg .b32 lo, hi;\n\tmov.b64 {lo, hi}, %1;\n\txor.b32 hi, hi, 0x80000000;\n\tmov.b64 %0, {lo, hi};\n\t}"
        : "=d"(r) : "d"(x));
    return r;
}

// Exact IEEE results of operations with a zero operand, formed on the
// integer pipe (an FP64 operation costs ~40 integer operations of pipe time
// here), for the strides after the outer coefficients have decayed to zero.
__device__ __forceinline__ unsigned hiw(double x) { return (unsigned)__double2hiint(x); }
// the zero whose sign is bit 31 of s
__device__ __forceinline__ double szero(unsigned s) { return __hiloint2double((int)(s & 0x80000000u), 0); }
// x + z for a zero z with sign bit zs, x not NaN: x itself, unless x is a
// zero too (then -0 only if both are -0: round-to-nearest)
__device__ __forceinline__ double add_z(double x, unsigned zs) { return nz(x) ? x : szero(hiw(x) & zs); }
// x / y from y's correctly rounded reciprocal r = RN(1/y) (__drcp_rn):
// Markstein's correction (IBM J. Res. Dev. 1990): q0 = RN(x r) is within an
// ulp of x/y, the remainder x - y q0 is exact in one FMA, and RN(q0 + rem r)
// = RN(x / y) while no intermediate leaves the normal range, which the
// exponent guard ensures; other operands take the division.
__device__ __forceinline__ double mdiv(double x, double y, double r) {
    const int ex = (int)((hiw(x) >> 20) & 0x7FFu), ey = (int)((hiw(y) >> 20) & 0x7FFu);
    if ((unsigned)(ex - 100) <= 1846u && (unsigned)(ey - 100) <= 1846u && (unsigned)(ex - ey + 900) <= 1800u) {
        const double q0 = __dmul_rn(x, r);
        const double rem = __fma_rn(-y, q0, x);
        return __fma_rn(rem, r, q0);
    }
    return dvd(x, y);
}
__device__ __forceinline__ bool finite4(double p, double q, double r, double s) {
    return max(max(hiw(p) & 0x7FF00000u, hiw(q) & 0x7FF00000u), max(hiw(r) & 0x7FF00000u, hiw(s) & 0x7FF00000u))
           < 0x7FF00000u;
}
// "zero state" of a row: outer coefficients a, e zero, the others finite.
// While every row a stride reads is in it, both multipliers of phase A are
// zeros, every product with them is a zero and phase A forms no FP64 value.
__device__ __forceinline__ bool zero_state(double a, double b, double c, double d, double e, double y) {
    return !nz(a) && !nz(e) && finite4(b, c, d, y);
}

constexpr int kMaxThreads = 256;
constexpr int kSmemArrays = 15;   // 6 state + 6 T coefficients + 2 T multipliers + 1/cT

// Global loads of the state; kL2Only reads through L2 only (ld.global.cg), for
// persistent kernels that read data other CTAs wrote earlier in the same launch.
template <bool kL2Only>
__device__ __forceinline__ double gload(const double* p) {
    if (kL2Only) return __ldcg(p);
    return *p;
}

// One CTA's work: window w of subsystem r of system j (whole subsystem when
// p.final_step).  Every thread of the CTA must call it with the same (j, r, w).
// kZero compiles the zero-state vote and its integer-pipe strides in; without
// it every stride takes the FP64 operations (passes of short strides, where
// the outer coefficients have not underflowed yet, skip the vote's cost).
template <int RPT, bool kL2Only = false, bool kZero = true>
__device__ __forceinline__ void pcr_tile(const PcrPassArgs& p, int64_t j, int64_t r, int64_t w, double* smem)
{
    const int TRm = p.TRmax;
    double* sa = smem;            double* sb = sa + TRm;  double* sc = sb + TRm;
    double* sd = sc + TRm;        double* se = sd + TRm;  double* sy = se + TRm;
    double* Ta = sy + TRm;        double* Tb = Ta + TRm;  double* Tc = Tb + TRm;
    double* Td = Tc + TRm;        double* Te = Td + TRm;  double* Tk = Te + TRm;
    double* T1 = Tk + TRm;        double* T2 = T1 + TRm;  double* Tr = T2 + TRm;

    const int64_t sbase = p.offsets ? p.offsets[j] : j * p.src_ss;
    const int64_t dbase = p.offsets ? p.offsets[j] : j * p.dst_ss;
    const int64_t nsys = p.offsets ? (p.offsets[j + 1] - p.offsets[j]) : p.n;
    if (r >= nsys) return;
    const int64_t nr  = (nsys - 1 - r) / p.G + 1;           // rows of subsystem r
    const int64_t wlo = w * (int64_t)p.L;
    if (wlo >= nr) return;
    const int64_t whi = min(wlo + (int64_t)p.L, nr);
    const int64_t t0  = max(wlo - (int64_t)p.H, (int64_t)0);
    const int64_t t1  = min(whi + (int64_t)p.H, nr);
    const int TR = (int)(t1 - t0);
    const int tid = threadIdx.x, bd = blockDim.x;
    // distance of local rows t, t+1 and local row 0 of the source
    const int64_t sstep = p.src_sub ? 1 : p.G * p.src_rs;
    const int64_t soff = p.src_sub ? sbase + r * (nsys / p.G) + min(r, nsys % p.G) : sbase + r * p.src_rs;
    const int64_t dstep = p.G * p.dst_rs;
    const int64_t doff = dbase + r * p.dst_rs;
    // a null outer band (a tridiagonal batch, first pass only) is +0.0
    const bool has_a = p.src[A_] != nullptr, has_e = p.src[E_] != nullptr;
    const double* __restrict__ ga = has_a ? p.src[A_] + soff : nullptr;
    const double* __restrict__ gb = p.src[B_] + soff;
    const double* __restrict__ gc = p.src[C_] + soff;
    const double* __restrict__ gd = p.src[D_] + soff;
    const double* __restrict__ ge = has_e ? p.src[E_] + soff : nullptr;
    const double* __restrict__ gy = p.src[Y_] + soff;

    double al1p[RPT], al2p[RPT];
    bool zrow = true;           // every row this thread holds in the zero state
    bool zdrow = true;          // ... with d = 0 as well
    if (p.bulk) {
        // The whole system is the tile (t0 = 0, TR = n, even): thread 0
        // stages each array with one bulk asynchronous copy straight into its
        // shared-memory row array (16-byte aligned: contiguous layout, even
        // n, aligned arrays -- the host checks), completing on an mbarrier.
        // A wait that gives up (2 s; copies do not take that long) leaves
        // x = NaN for this system, so the failure shows in the result.
        __shared__ __align__(8) uint64_t bulk_bar;
        if (tid == 0) {
            tma::mbar_init(&bulk_bar, 1);
            tma::fence_mbarrier_init();
        }
        __syncthreads();
        if (tid == 0) {
            const uint32_t bytes = (uint32_t)TR * (uint32_t)sizeof(double);
            const uint64_t pol = tma::policy_evict_first();
            tma::mbar_expect_tx(&bulk_bar, (4u + (has_a ? 1u : 0u) + (has_e ? 1u : 0u)) * bytes);
            if (has_a) tma::bulk_g2s(sa, ga, bytes, &bulk_bar, pol);
            tma::bulk_g2s(sb, gb, bytes, &bulk_bar, pol);
            tma::bulk_g2s(sc, gc, bytes, &bulk_bar, pol);
            tma::bulk_g2s(sd, gd, bytes, &bulk_bar, pol);
            if (has_e) tma::bulk_g2s(se, ge, bytes, &bulk_bar, pol);
            tma::bulk_g2s(sy, gy, bytes, &bulk_bar, pol);
        }
        const bool got = tma::mbar_wait_bounded(&bulk_bar, 0, 2000000000ull);
        if (__syncthreads_or(!got)) {
            if (tid == 0) tma::mbar_wait_bounded(&bulk_bar, 0, 2000000000ull);   // (copies in flight)
            __syncthreads();
            double* __restrict__ gx = p.x + doff;
            for (int k = tid; k < TR; k += bd) gx[k * dstep] = __longlong_as_double(0x7FF8000000000000LL);
            return;
        }
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            al1p[q] = 0.0; al2p[q] = 0.0;
            if (k < TR) {
                if (!has_a) sa[k] = 0.0;
                if (!has_e) se[k] = 0.0;
                if constexpr (kZero) {
                    const bool z = zero_state(sa[k], sb[k], sc[k], sd[k], se[k], sy[k]);
                    zrow = zrow && z; zdrow = zdrow && z && !nz(sd[k]);
                }
            }
        }
    } else {
    #pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            al1p[q] = 0.0; al2p[q] = 0.0;
            if (k < TR) {
                const int64_t gi = (t0 + k) * sstep;
                const double a = has_a ? gload<kL2Only>(ga + gi) : 0.0;
                const double e = has_e ? gload<kL2Only>(ge + gi) : 0.0;
                const double b = gload<kL2Only>(gb + gi), c = gload<kL2Only>(gc + gi);
                const double d = gload<kL2Only>(gd + gi), y = gload<kL2Only>(gy + gi);
                sa[k] = a; sb[k] = b; sc[k] = c; sd[k] = d; se[k] = e; sy[k] = y;
                if constexpr (kZero) {
                    const bool z = zero_state(a, b, c, d, e, y);
                    zrow = zrow && z; zdrow = zdrow && z && !nz(d);
                }
                if (p.src[AL1_]) {
                    al1p[q] = gload<kL2Only>(p.src[AL1_] + soff + gi);
                    al2p[q] = gload<kL2Only>(p.src[AL2_] + soff + gi);
                }
            }
        }
    }
    // rows read by a stride are the rows the previous stride wrote (all
    // loaded rows for the first): votes per stride tell whether the whole
    // tile is in the zero state, and in it with d = 0 too
    int ztile = 0, zdtile = 0;
    if constexpr (kZero) { ztile = __syncthreads_and(zrow); zdtile = __syncthreads_and(zdrow); }
    else __syncthreads();

    for (int s = 0; s < p.K; s++) {
        const int dl = 1 << s;
        // rows this stride must produce: the window widened by the halo the
        // remaining strides of the pass still consume (everything if final).
        int64_t rlo, rhi;
        if (p.final_step) { rlo = 0; rhi = nr; }
        else {
            const int64_t rem = 2 * ((int64_t(1) << p.K) - (int64_t(2) << s));
            rlo = max(wlo - rem, (int64_t)0); rhi = min(whi + rem, nr);
        }
        const int64_t Tlo = max(rlo - dl, (int64_t)0), Thi = min(rhi + dl, nr);

        // ---- phase A: T(m) = a1*row(m-d) + row(m) + a2*row(m+d) ----------
        if (kZero && ztile) {
            // a1 = -a(m)/b(m-d) and a2 = -e(m)/d(m+d) are zeros (b, d finite):
            // only their signs are formed; every product with them is the
            // zero of sign xor, every sum row m's value (kernel.cu:63-117)
#pragma unroll
            for (int q = 0; q < RPT; q++) {
                const int k = tid + q * bd;
                const int64_t t = t0 + k;
                if (k < TR && t >= Tlo && t < Thi) {
                    const bool hasL = t - dl >= 0, hasR = t + dl <= nr - 1;
                    if (hasL || hasR) {
                        const double bm = sb[k], cm = sc[k], dm = sd[k], ym = sy[k];
                        unsigned s1 = 0u, s2 = 0u;
                        if (hasL && t - 2 * dl >= 0) {
                            const double bL = sb[k - dl];
                            if (nz(bL)) s1 = (hiw(sa[k]) ^ hiw(bL)) ^ 0x80000000u;
                        }
                        if (hasR && t + 2 * dl <= nr - 1) {
                            const double dR = sd[k + dl];
                            if (nz(dR)) s2 = (hiw(se[k]) ^ hiw(dR)) ^ 0x80000000u;
                        }
                        // sign bits of the products a1*row(m-d) and a2*row(m+d)
                        // (+0 for a missing neighbour: adding +0 keeps -0 out)
                        unsigned La = 0u, Lc = 0u, Ld = 0u, Le = 0u, Ly = 0u;
                        unsigned Ra = 0u, Rb = 0u, Rc = 0u, Re = 0u, Ry = 0u;
                        if (hasL) {
                            La = s1 ^ hiw(sa[k - dl]); Lc = s1 ^ hiw(sc[k - dl]); Ld = s1 ^ hiw(sd[k - dl]);
                            Le = s1 ^ hiw(se[k - dl]); Ly = s1 ^ hiw(sy[k - dl]);
                        }
                        if (hasR) {
                            Ra = s2 ^ hiw(sa[k + dl]); Rb = s2 ^ hiw(sb[k + dl]); Rc = s2 ^ hiw(sc[k + dl]);
                            Re = s2 ^ hiw(se[k + dl]); Ry = s2 ^ hiw(sy[k + dl]);
                        }
                        if (hasL && hasR) {
                            Ta[k] = szero(La);
                            Tb[k] = add_z(bm, Lc & Ra); Tc[k] = add_z(cm, Ld & Rb);
                            Td[k] = add_z(dm, Le & Rc); Te[k] = szero(Re);
                            Tk[k] = add_z(ym, Ly & Ry);
                        } else if (hasR) {     // kernel.cu:82-91: aT = bT = 0
                            Ta[k] = 0.0; Tb[k] = 0.0;
                            Tc[k] = add_z(cm, Rb); Td[k] = add_z(dm, Rc); Te[k] = szero(Re);
                            Tk[k] = add_z(ym, Ry);
                        } else {               // kernel.cu:108-117: dT = eT = 0
                            Ta[k] = szero(La); Tb[k] = add_z(bm, Lc); Tc[k] = add_z(cm, Ld);
                            Td[k] = 0.0; Te[k] = 0.0;
                            Tk[k] = add_z(ym, Ly);
                        }
                        T1[k] = szero(s1); T2[k] = szero(s2);
                    }
                }
            }
        } else {
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            const int64_t t = t0 + k;
            if (k < TR && t >= Tlo && t < Thi) {
                const bool hasL = t - dl >= 0, hasR = t + dl <= nr - 1;
                if (hasL || hasR) {
                    const double am = sa[k], bm = sb[k], cm = sc[k], dm = sd[k], em = se[k], ym = sy[k];
                    double al1 = 0.0, al2 = 0.0;
                    double aT, bT, cT, dT, eT, kT;
                    if (hasL && hasR) {
                        const double aL = sa[k - dl], bL = sb[k - dl], cL = sc[k - dl], dL = sd[k - dl],
                                     eL = se[k - dl], yL = sy[k - dl];
                        const double aR = sa[k + dl], bR = sb[k + dl], cR = sc[k + dl], dR = sd[k + dl],
                                     eR = se[k + dl], yR = sy[k + dl];
                        if (t - 2 * dl >= 0 && nz(bL)) al1 = dvd(neg(am), bL);
                        if (t + 2 * dl <= nr - 1 && nz(dR)) al2 = dvd(neg(em), dR);
                        aT = mul(al1, aL);
                        bT = add(add(mul(al1, cL), bm), mul(al2, aR));
                        cT = add(add(mul(al1, dL), cm), mul(al2, bR));
                        dT = add(add(mul(al1, eL), dm), mul(al2, cR));
                        eT = mul(al2, eR);
                        kT = add(add(mul(al1, yL), ym), mul(al2, yR));
                    } else if (hasR) {     // row m-d outside: kernel.cu:82-91
                        const double aR = sa[k + dl], bR = sb[k + dl], cR = sc[k + dl], dR = sd[k + dl],
                                     eR = se[k + dl], yR = sy[k + dl];
                        (void)aR;
                        if (t + 2 * dl <= nr - 1 && nz(dR)) al2 = dvd(neg(em), dR);
                        aT = 0.0; bT = 0.0;
                        cT = add(cm, mul(al2, bR));
                        dT = add(dm, mul(al2, cR));
                        eT = mul(al2, eR);
                        kT = add(ym, mul(al2, yR));
                    } else {               // row m+d outside: kernel.cu:108-117
                        const double aL = sa[k - dl], bL = sb[k - dl], cL = sc[k - dl], dL = sd[k - dl],
                                     yL = sy[k - dl];
                        if (t - 2 * dl >= 0 && nz(bL)) al1 = dvd(neg(am), bL);
                        aT = mul(al1, aL);
                        bT = add(mul(al1, cL), bm);
                        cT = add(mul(al1, dL), cm);
                        dT = 0.0; eT = 0.0;
                        kT = add(mul(al1, yL), ym);
                        (void)em;
                    }
                    Ta[k] = aT; Tb[k] = bT; Tc[k] = cT; Td[k] = dT; Te[k] = eT; Tk[k] = kT;
                    T1[k] = al1; T2[k] = al2;
                    Tr[k] = __drcp_rn(cT);
                }
            }
        }
        }
        __syncthreads();

        // ---- phase B: new row = b/cT(i-d)*T(i-d) - row(i) + d/cT(i+d)*T(i+d)
        zrow = true; zdrow = true;
        // the reference's update of row i (kernel.cu:120-140, in place: phase
        // B reads no other row's state); folds the row's zero state into zrow
        auto row_b = [&](int q, int k, bool hasL, bool hasR, double a1pre, double a2pre, bool rcp) {
            const double ai = sa[k], bi = sb[k], ci = sc[k], di = sd[k], ei = se[k], yi = sy[k];
            double a1 = 0.0, b1 = 0.0, c1 = 0.0, d1 = 0.0, k1 = 0.0, f1 = a1pre;
            double b2 = 0.0, c2 = 0.0, d2 = 0.0, e2 = 0.0, k2 = 0.0, f2 = a2pre;
            if (hasL) {                    // kernel.cu:120-125
                const double cTL = Tc[k - dl];
                if (nz(cTL)) f1 = rcp ? mdiv(bi, cTL, Tr[k - dl]) : dvd(bi, cTL);
                a1 = mul(f1, Ta[k - dl]); b1 = mul(f1, Tb[k - dl]); c1 = mul(f1, Td[k - dl]);
                d1 = mul(f1, Te[k - dl]); k1 = mul(f1, Tk[k - dl]);
            }
            if (hasR) {                    // kernel.cu:127-132
                const double cTR = Tc[k + dl];
                if (nz(cTR)) f2 = rcp ? mdiv(di, cTR, Tr[k + dl]) : dvd(di, cTR);
                c2 = mul(f2, Tb[k + dl]); b2 = mul(f2, Ta[k + dl]); d2 = mul(f2, Td[k + dl]);
                e2 = mul(f2, Te[k + dl]); k2 = mul(f2, Tk[k + dl]);
            }
            const double nb = add(sub(b1, ai), b2), nc = add(sub(c1, ci), c2);   // kernel.cu:138-140
            const double nd = add(sub(d1, ei), d2), ny = add(sub(k1, yi), k2);
            sb[k] = nb; sc[k] = nc; sd[k] = nd; sy[k] = ny;
            sa[k] = a1; se[k] = e2;
            al1p[q] = f1; al2p[q] = f2;
            if constexpr (kZero) {
                const bool z = zero_state(a1, nb, nc, nd, e2, ny);
                zrow = zrow && z; zdrow = zdrow && z && !nz(nd);
            }
        };
        if (kZero && zdtile) {
            // zero state with d = 0: f2 = d(i)/cT(i+d) is a zero, and so is
            // every product with it; dT of the neighbours is zero, so c1 is
            // too: besides the quotient f1 only b1, k1 and k1 - y(i) are FP64
#pragma unroll
            for (int q = 0; q < RPT; q++) {
                const int k = tid + q * bd;
                const int64_t t = t0 + k;
                if (k < TR && t >= rlo && t < rhi) {
                    const bool hasL = t - dl >= 0, hasR = t + dl <= nr - 1;
                    // multipliers last assigned before Reduction-III (kernel.cu:96-112)
                    const double a1pre = hasR ? T1[k + dl] : ((t - 2 * dl >= 0) ? T1[k - dl] : al1p[q]);
                    const double a2pre = (t + 2 * dl <= nr - 1) ? T2[k + dl] : (hasL ? T2[k - dl] : al2p[q]);
                    double f1 = a1pre, f2 = a2pre;
                    if (hasL) { const double cTL = Tc[k - dl]; if (nz(cTL)) f1 = dvd(sb[k], cTL); }
                    if (hasR) { const double cTR = Tc[k + dl]; if (nz(cTR)) f2 = dvd(sd[k], cTR); }
                    // f2 is the stored multiplier where cT(i+d) = 0: then the row
                    // takes the reference's operations
                    if (finite4(hasL ? f1 : 0.0, 0.0, 0.0, 0.0) && (!hasR || !nz(f2))) {
                        const double ai = sa[k], ci = sc[k], ei = se[k], yi = sy[k];
                        const unsigned s1 = hiw(f1), s2 = hiw(f2);
                        unsigned a1s = 0u, c1s = 0u, d1s = 0u, b2s = 0u, c2s = 0u, d2s = 0u, e2s = 0u, k2s = 0u;
                        double b1 = 0.0, k1 = 0.0;
                        if (hasL) {
                            a1s = s1 ^ hiw(Ta[k - dl]); c1s = s1 ^ hiw(Td[k - dl]); d1s = s1 ^ hiw(Te[k - dl]);
                            b1 = mul(f1, Tb[k - dl]); k1 = mul(f1, Tk[k - dl]);
                        }
                        if (hasR) {
                            b2s = s2 ^ hiw(Ta[k + dl]); c2s = s2 ^ hiw(Tb[k + dl]); d2s = s2 ^ hiw(Td[k + dl]);
                            e2s = s2 ^ hiw(Te[k + dl]); k2s = s2 ^ hiw(Tk[k + dl]);
                        }
                        // (b1 - ai) + b2, (c1 - ci) + c2, (d1 - ei) + d2, (k1 - yi) + k2
                        // with zeros ai, b2, c1, c2, d1, ei, d2, k2
                        const double nb = add_z(add_z(b1, hiw(ai) ^ 0x80000000u), b2s);
                        const double nc = add_z(add_z(neg(ci), c1s), c2s);
                        const double nd = szero(d1s & (hiw(ei) ^ 0x80000000u) & d2s);
                        const double ny = add_z(sub(k1, yi), k2s);
                        sb[k] = nb; sc[k] = nc; sd[k] = nd; sy[k] = ny;
                        sa[k] = szero(a1s); se[k] = szero(e2s);
                        al1p[q] = f1; al2p[q] = f2;
                        const bool z = finite4(nb, nc, nd, ny);
                        zrow = zrow && z; zdrow = zdrow && z;
                    } else {
                        row_b(q, k, hasL, hasR, a1pre, a2pre, false);
                    }
                }
            }
        } else if (kZero && ztile) {
            // zero state: aT, eT of both neighbours and a, e of row i are
            // zeros, so are a1, d1, b2, e2 (for finite f1, f2), and the b and
            // d sums reduce to one term
#pragma unroll
            for (int q = 0; q < RPT; q++) {
                const int k = tid + q * bd;
                const int64_t t = t0 + k;
                if (k < TR && t >= rlo && t < rhi) {
                    const bool hasL = t - dl >= 0, hasR = t + dl <= nr - 1;
                    // multipliers last assigned before Reduction-III (kernel.cu:96-112)
                    const double a1pre = hasR ? T1[k + dl] : ((t - 2 * dl >= 0) ? T1[k - dl] : al1p[q]);
                    const double a2pre = (t + 2 * dl <= nr - 1) ? T2[k + dl] : (hasL ? T2[k - dl] : al2p[q]);
                    double f1 = a1pre, f2 = a2pre;
                    if (hasL) { const double cTL = Tc[k - dl]; if (nz(cTL)) f1 = dvd(sb[k], cTL); }
                    if (hasR) { const double cTR = Tc[k + dl]; if (nz(cTR)) f2 = dvd(sd[k], cTR); }
                    if (finite4(hasL ? f1 : 0.0, hasR ? f2 : 0.0, 0.0, 0.0)) {
                        const double ai = sa[k], ci = sc[k], ei = se[k], yi = sy[k];
                        const unsigned s1 = hiw(f1), s2 = hiw(f2);
                        unsigned a1s = 0u, d1s = 0u, b2s = 0u, e2s = 0u;
                        double b1 = 0.0, c1 = 0.0, k1 = 0.0, c2 = 0.0, d2 = 0.0, k2 = 0.0;
                        if (hasL) {
                            a1s = s1 ^ hiw(Ta[k - dl]); d1s = s1 ^ hiw(Te[k - dl]);
                            b1 = mul(f1, Tb[k - dl]); c1 = mul(f1, Td[k - dl]); k1 = mul(f1, Tk[k - dl]);
                        }
                        if (hasR) {
                            b2s = s2 ^ hiw(Ta[k + dl]); e2s = s2 ^ hiw(Te[k + dl]);
                            c2 = mul(f2, Tb[k + dl]); d2 = mul(f2, Td[k + dl]); k2 = mul(f2, Tk[k + dl]);
                        }
                        // b1 - ai + b2 with ai, b2 zeros; d1 - ei + d2 with d1, ei zeros
                        const double nb = add_z(add_z(b1, hiw(ai) ^ 0x80000000u), b2s);
                        const double nc = add(sub(c1, ci), c2);
                        const double nd = add_z(d2, d1s & (hiw(ei) ^ 0x80000000u));
                        const double ny = add(sub(k1, yi), k2);
                        sb[k] = nb; sc[k] = nc; sd[k] = nd; sy[k] = ny;
                        sa[k] = szero(a1s); se[k] = szero(e2s);
                        al1p[q] = f1; al2p[q] = f2;
                        const bool z = finite4(nb, nc, nd, ny);
                        zrow = zrow && z; zdrow = zdrow && z && !nz(nd);
                    } else {
                        row_b(q, k, hasL, hasR, a1pre, a2pre, false);
                    }
                }
            }
        } else {
#pragma unroll
            for (int q = 0; q < RPT; q++) {
                const int k = tid + q * bd;
                const int64_t t = t0 + k;
                if (k < TR && t >= rlo && t < rhi) {
                    const bool hasL = t - dl >= 0, hasR = t + dl <= nr - 1;
                    // multipliers last assigned before Reduction-III (kernel.cu:96-112)
                    const double a1pre = hasR ? T1[k + dl] : ((t - 2 * dl >= 0) ? T1[k - dl] : al1p[q]);
                    const double a2pre = (t + 2 * dl <= nr - 1) ? T2[k + dl] : (hasL ? T2[k - dl] : al2p[q]);
                    row_b(q, k, hasL, hasR, a1pre, a2pre, true);
                }
            }
        }
        if constexpr (kZero) { ztile = __syncthreads_and(zrow); zdtile = __syncthreads_and(zdrow); }
        else __syncthreads();
    }

    if (p.final_step) {
        // kernel.cu:145-153: pairs (i, i+delta) by Cramer's rule, singles x = y/c
        const int64_t df = int64_t(1) << p.K;
        double* __restrict__ gx = p.x + doff;
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            if (k < TR) {
                const int64_t t = k;       // whole subsystem: t0 == 0
                if (t < nr - df) {
                    const int kk = k + (int)df;
                    const double deno = sub(mul(sc[k], sc[kk]), mul(sb[kk], sd[k]));
                    gx[t * dstep] = dvd(sub(mul(sc[kk], sy[k]), mul(sd[k], sy[kk])), deno);
                    gx[(t + df) * dstep] = dvd(sub(mul(sc[k], sy[kk]), mul(sb[kk], sy[k])), deno);
                }
                if (t >= nr - df && t < df) gx[t * dstep] = dvd(sy[k], sc[k]);
            }
        }
    } else {
        // subsystem-major output: row t of subsystem r is row t >> K of
        // subsystem r + (t mod 2^K) G at the next level's stride G 2^K
        const int64_t G2 = p.G << p.K, q2 = nsys / G2, rem2 = nsys % G2;
        const int64_t kmask = (int64_t(1) << p.K) - 1;
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            const int k = tid + q * bd;
            const int64_t t = t0 + k;
            if (k < TR && t >= wlo && t < whi) {
                int64_t gi;
                if (p.dst_sub) {
                    const int64_t r2 = r + (t & kmask) * p.G;
                    gi = dbase + r2 * q2 + min(r2, rem2) + (t >> p.K);
                } else {
                    gi = doff + t * dstep;
                }
                p.dst[A_][gi] = sa[k]; p.dst[B_][gi] = sb[k]; p.dst[C_][gi] = sc[k];
                p.dst[D_][gi] = sd[k]; p.dst[E_][gi] = se[k]; p.dst[Y_][gi] = sy[k];
                p.dst[AL1_][gi] = al1p[q]; p.dst[AL2_][gi] = al2p[q];
            }
        }
    }
}

}  // namespace pcrp
