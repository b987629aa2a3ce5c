/*
 * nf_math.h -- deterministic elementary functions shared by the CUDA kernels and the CPU
 * restatement of the Neofiz timestep.
 *
 * Why these exist. The reference computes its flow stress with Math.pow and Math.log
 * (core/JohnsonCook.java:139,182,196) and its damage band with Math.hypot, Math.atan2,
 * Math.sin and Math.cos (solver/Damage.java:315-322). CUDA's and glibc's versions of those
 * functions differ from each other by an ulp here and there, and a plastic run amplifies a
 * last-bit difference over thousands of steps. Every other operation on the path is a
 * correctly rounded IEEE add, multiply, divide or square root, so if the transcendentals are
 * also the SAME code on both sides -- evaluated as plain IEEE operations with no fused
 * multiply-add contraction (nvcc --fmad=false, gcc -ffp-contract=off) -- the GPU and the CPU
 * produce bit-identical results.
 *
 * Methods (from the mathematics and published methods; every constant is an exact value
 * rounded to double, computed for this file -- the tables by gen_nf_math_tables.py):
 *   log   : Tang's table-driven logarithm (ACM TOMS 16, 1990). x = 2^k z with z in
 *           [0.705, 1.41); z's leading mantissa bits pick one of 128 entries holding
 *           invc ~ 1/c and -log(invc) as hi + lo; r = z invc - 1 is formed exactly as a
 *           product and its fused-multiply-add error (no division), and
 *           log x = k ln2 + (-log invc) + log1p(r), log1p by its Taylor series to r^7
 *           (|r| <= 2^-8). The large terms are summed with their rounding errors, so the
 *           result comes as a double-double (hi + lo) for pow, and rounded once for log.
 *   exp   : Tang's table-driven exponential (ACM TOMS 15, 1989). x = (128 m + j) ln2/128 + r
 *           with ln2/128 split in a 35-bit head (exact products) and a tail, |r| <= ln2/256;
 *           exp x = 2^m 2^(j/128) (1 + r + r^2/2 + ... + r^5/120), 2^(j/128) from a table as
 *           hi + lo. A double-double argument (pow's y log x) enters through r.
 *   pow   : exp(y log x) with log as double-double and y log x formed exactly by a fused
 *           multiply-add, so the result is accurate to about half an ulp rather than
 *           |y log x| ulp.
 * Fused multiply-add is an exactly rounded IEEE operation (fma() in C, the DFMA instruction on
 * the GPU), so it gives the same bits on both sides; only contraction of separate operations
 * is switched off.
 *   atan2 : quadrant folding to atan(t), t in [0,1]; t > tan(pi/8) maps through
 *           atan(t) = pi/4 + atan((t-1)/(t+1)); |u| > 1/8 maps through
 *           atan(u) = atan(1/4) + atan((u-1/4)/(1+u/4)); Taylor series for |v| <= 0.15.
 *   sin/cos: Cody-Waite reduction by pi/2 (valid for |x| < 1e5, which covers every call on
 *           the path: the band angle lies in [-pi/2, pi/2]), Taylor series on [-pi/4, pi/4].
 *   hypot : max * sqrt(1 + (min/max)^2), no overflow for finite inputs.
 * Accuracy against glibc and CUDA's libdevice is asserted by the test suite (a few ulp).
 */
#ifndef NF_MATH_H
#define NF_MATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>

#include "nf_math_tables.h"

#if defined(__CUDACC__)
#define NF_HD static __host__ __device__ inline
#else
#define NF_HD static inline
#endif

NF_HD uint64_t nf_bits(double x) { uint64_t u; memcpy(&u, &x, sizeof u); return u; }
NF_HD double nf_from_bits(uint64_t u) { double x; memcpy(&x, &u, sizeof x); return x; }

#define NF_LN2_HI 0x1.62e42fee00000p-1
#define NF_LN2_LO 0x1.a39ef35793c76p-33
#define NF_INV_LN2 0x1.71547652b82fep+0
#define NF_SQRT2 0x1.6a09e667f3bcdp+0
#define NF_PI 0x1.921fb54442d18p+1
#define NF_PI_LO 0x1.1a62633145c07p-53
#define NF_PIO2 0x1.921fb54442d18p+0
#define NF_PIO2_LO 0x1.1a62633145c07p-54
#define NF_PIO4 0x1.921fb54442d18p-1
#define NF_PIO4_LO 0x1.1a62633145c07p-55
#define NF_PIO2_CW_HI 0x1.921fb54400000p+0
#define NF_PIO2_CW_LO 0x1.0b4611a626331p-34
#define NF_TWO_OVER_PI 0x1.45f306dc9c883p-1
#define NF_TAN_PI_8 0x1.a827999fcef32p-2
#define NF_ATAN_QUARTER_HI 0x1.f5b75f92c80ddp-3
#define NF_ATAN_QUARTER_LO 0x1.8ab6e3cf7afbdp-57

/* 2^k for k in [-1022, 1023]. */
NF_HD double nf_pow2i(int k) { return nf_from_bits((uint64_t)(k + 1023) << 52); }

/* er * 2^k for any k a reduced exponential can produce. */
NF_HD double nf_scale(double er, int k) {
    if (k > 1023) return er * nf_pow2i(1023) * nf_pow2i(k - 1023);
    if (k < -1021) return er * nf_pow2i(k + 600) * nf_pow2i(-600);
    return er * nf_pow2i(k);
}

/* Tables of the logarithm (invc, -log invc hi, lo, 0 per entry) and of 2^(j/128) (hi, lo),
 * one copy for the host and one in device global memory (read through the read-only cache;
 * a warp's lanes index different entries, which constant memory would serialise). */
static const double nf_log_tab_h[4 * 128] = { NF_LOG_TABLE };
static const double nf_exp_tab_h[2 * 128] = { NF_EXP_TABLE };
#if defined(__CUDACC__)
static __device__ const double nf_log_tab_d[4 * 128] = { NF_LOG_TABLE };
static __device__ const double nf_exp_tab_d[2 * 128] = { NF_EXP_TABLE };
#endif

NF_HD double nf_log_tab(int i) {
#if defined(__CUDA_ARCH__)
    return __ldg(nf_log_tab_d + i);
#else
    return nf_log_tab_h[i];
#endif
}
NF_HD double nf_exp_tab(int i) {
#if defined(__CUDA_ARCH__)
    return __ldg(nf_exp_tab_d + i);
#else
    return nf_exp_tab_h[i];
#endif
}

/* exp(p + plo) for p in [-745.2, 709.8] and |plo| <= 2^-40 |p| (or p's own rounding error). */
NF_HD double nf_exp_dd(double p, double plo) {
    const double kd = rint(p * NF_EXP_N_OVER_LN2);
    const int n = (int)kd;
    const double r1 = fma(-kd, NF_EXP_L_HI, p);          /* exact: kd L_HI exact, Sterbenz */
    const double r = fma(-kd, NF_EXP_L_LO, r1) + plo;
    const int j = n & 127;
    const int m = (n - j) / 128;                          /* exact: n - j is a multiple */
    const double thi = nf_exp_tab(2 * j), tlo = nf_exp_tab(2 * j + 1);
    double t = fma(r, 0x1.1111111111111p-7, 0x1.5555555555555p-5);   /* 1/120, 1/24 */
    t = fma(r, t, 0x1.5555555555555p-3);                               /* 1/6 */
    t = fma(r, t, 0.5);
    const double q = fma(r * r, t, r);                    /* exp(r) - 1 */
    return nf_scale(thi + fma(thi, q, tlo), m);
}

NF_HD double nf_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    return nf_exp_dd(x, 0.0);
}

/* log(x) as an unevaluated sum hi + lo, for finite x > 0. */
NF_HD void nf_log_dd(double x, double *hi, double *lo) {
    uint64_t u = nf_bits(x);
    int64_t kadj = 0;
    if (u < 0x0010000000000000ULL) {               /* subnormal: renormalise */
        u = nf_bits(x * 0x1p54);
        kadj = -54;
    }
    const uint64_t tmp = u - NF_LOG_OFF;
    const int64_t k = (int64_t)(tmp & 0xfff0000000000000ULL) / ((int64_t)1 << 52) + kadj;
    const int j = (int)((tmp >> 45) & 127);
    const double z = nf_from_bits(u - (tmp & 0xfff0000000000000ULL));
    const double invc = nf_log_tab(4 * j), chi = nf_log_tab(4 * j + 1);
    const double clo = nf_log_tab(4 * j + 2);
    const double pr = z * invc;
    const double rl = fma(z, invc, -pr);           /* z invc = pr + rl exactly */
    const double rh = pr - 1.0;                    /* exact (Sterbenz) */
    const double dk = (double)k;
    /* k ln2_hi + (-log invc) + rh - rh^2/2, each addition with its error (Fast2Sum: the
     * running sum is never smaller than the term added, or is zero) */
    const double a = dk * NF_LN2_HI;               /* exact */
    const double s1 = a + chi;
    const double e1 = (a - s1) + chi;
    const double s2 = s1 + rh;
    const double e2 = (s1 - s2) + rh;
    const double q = rh * rh;
    const double ql = fma(rh, rh, -q);             /* rh^2 = q + ql exactly */
    const double hq = -0.5 * q;
    const double s3 = s2 + hq;
    const double e3 = (s2 - s3) + hq;
    /* rh^3 (1/3 - rh/4 + rh^2/5 - rh^3/6 + rh^4/7); the remainder is below 2^-67 */
    double t = fma(rh, 0x1.2492492492492p-3, -0x1.5555555555555p-3);   /* 1/7, -1/6 */
    t = fma(rh, t, 0x1.999999999999ap-3);                               /* 1/5 */
    t = fma(rh, t, -0.25);
    t = fma(rh, t, 0x1.5555555555555p-2);                               /* 1/3 */
    const double cubic = (q * rh) * t;
    /* rl (1 - rh) is log1p's first-order response to r's low part */
    const double small = ((dk * NF_LN2_LO + clo) + ((e1 + e2) + e3))
                         + (fma(-rh, rl, rl) - 0.5 * ql);
    const double l = cubic + small;
    const double h = s3 + l;
    *hi = h;
    *lo = l - (h - s3);
}

NF_HD double nf_log(double x) {
    if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;
    if (x == INFINITY) return x;
    double hi, lo;
    nf_log_dd(x, &hi, &lo);
    return hi;
}

/* x^y for x >= 0 (or +inf), y neither 0 nor NaN. Special cases by bit pattern (integer
 * comparisons, which keep the FP64 pipe for the arithmetic). */
NF_HD double nf_pow_nonneg(double x, double y) {
    const uint64_t ux = nf_bits(x), uy = nf_bits(y);
    if (ux == 0x3ff0000000000000ULL) return 1.0;                   /* x == 1 */
    if ((ux << 1) == 0) return (uy >> 63) ? INFINITY : 0.0;        /* x == +-0, y > 0 or < 0 */
    if (ux == 0x7ff0000000000000ULL) return (uy >> 63) ? 0.0 : INFINITY;
    if ((uy << 1) == 0xffe0000000000000ULL) {                      /* y == +-inf */
        const int big = ux > 0x3ff0000000000000ULL;
        return (uy >> 63) ? (big ? 0.0 : INFINITY) : (big ? INFINITY : 0.0);
    }
    double lh, ll;
    nf_log_dd(x, &lh, &ll);
    const double p = y * lh;
    if (p > 709.8) return INFINITY;
    if (p < -745.2) return 0.0;
    const double perr = fma(y, lh, -p);            /* y lh = p + perr exactly */
    return nf_exp_dd(p, fma(y, ll, perr));
}

/* Not recursive: a device call graph without cycles keeps the kernels' stack depth known at
 * compile time, so the driver sizes each launch's per-thread stack itself. */
NF_HD double nf_pow(double x, double y) {
    const uint64_t ux = nf_bits(x), uy = nf_bits(y);
    if ((uy << 1) == 0 || ux == 0x3ff0000000000000ULL) return 1.0;              /* y == 0, x == 1 */
    if ((ux << 1) > 0xffe0000000000000ULL || (uy << 1) > 0xffe0000000000000ULL) return NAN;
    if ((ux >> 63) && (ux << 1) != 0) {                                         /* x < 0 */
        /* Only integer powers of a negative base are real. Never reached on the solver
         * path, whose bases are a plastic strain and a homologous temperature in (0, 1). */
        if (rint(y) != y) return NAN;
        const double m = nf_pow_nonneg(-x, y);
        return fmod(y, 2.0) != 0.0 ? -m : m;
    }
    return nf_pow_nonneg(x, y);
}

/* atan(v) for |v| <= 0.15, Taylor to v^23. */
NF_HD double nf_atan_series(double v) {
    const double z = v * v;
    double p = -0x1.642c8590b2164p-5;              /* -1/23 */
    p = 0x1.8618618618618p-5 + z * p;              /*  1/21 */
    p = -0x1.af286bca1af28p-5 + z * p;             /* -1/19 */
    p = 0x1.e1e1e1e1e1e1ep-5 + z * p;              /*  1/17 */
    p = -0x1.1111111111111p-4 + z * p;             /* -1/15 */
    p = 0x1.3b13b13b13b14p-4 + z * p;              /*  1/13 */
    p = -0x1.745d1745d1746p-4 + z * p;             /* -1/11 */
    p = 0x1.c71c71c71c71cp-4 + z * p;              /*  1/9  */
    p = -0x1.2492492492492p-3 + z * p;             /* -1/7  */
    p = 0x1.999999999999ap-3 + z * p;              /*  1/5  */
    p = -0x1.5555555555555p-2 + z * p;             /* -1/3  */
    return v + v * (z * p);
}

/* atan(u) for |u| <= tan(pi/8). */
NF_HD double nf_atan_mid(double u) {
    const double a = fabs(u);
    double r;
    if (a > 0.125) {
        const double v = (a - 0.25) / (1.0 + 0.25 * a);
        r = NF_ATAN_QUARTER_HI + (nf_atan_series(v) + NF_ATAN_QUARTER_LO);
    } else {
        r = nf_atan_series(a);
    }
    return u < 0.0 ? -r : r;
}

/* atan(t) for t in [0, 1]. */
NF_HD double nf_atan01(double t) {
    if (t > NF_TAN_PI_8) {
        const double u = (t - 1.0) / (t + 1.0);
        return NF_PIO4 + (nf_atan_mid(u) + NF_PIO4_LO);
    }
    return nf_atan_mid(t);
}

NF_HD double nf_atan2(double y, double x) {
    if (x != x || y != y) return NAN;
    const double ax = fabs(x), ay = fabs(y);
    double a;
    if (ay == 0.0 && ax == 0.0) {
        a = signbit(x) ? NF_PI : 0.0;
    } else if (ax == INFINITY && ay == INFINITY) {
        a = x > 0.0 ? NF_PIO4 : 3.0 * NF_PIO4;
    } else {
        if (ay > ax) a = NF_PIO2 - (nf_atan01(ax / ay) - NF_PIO2_LO);
        else a = nf_atan01(ay / ax);
        if (signbit(x)) a = NF_PI - (a - NF_PI_LO);
    }
    return signbit(y) ? -a : a;
}

NF_HD double nf_sin_series(double r) {
    const double z = r * r;
    double p = -0x1.2f49b46814157p-57;             /* -1/19! */
    p = 0x1.952c77030ad4ap-49 + z * p;             /*  1/17! */
    p = -0x1.ae7f3e733b81fp-41 + z * p;            /* -1/15! */
    p = 0x1.6124613a86d09p-33 + z * p;             /*  1/13! */
    p = -0x1.ae64567f544e4p-26 + z * p;            /* -1/11! */
    p = 0x1.71de3a556c734p-19 + z * p;             /*  1/9!  */
    p = -0x1.a01a01a01a01ap-13 + z * p;            /* -1/7!  */
    p = 0x1.1111111111111p-7 + z * p;              /*  1/5!  */
    p = -0x1.5555555555555p-3 + z * p;             /* -1/3!  */
    return r + r * (z * p);
}

NF_HD double nf_cos_series(double r) {
    const double z = r * r;
    double p = -0x1.6827863b97d97p-53;             /* -1/18! */
    p = 0x1.ae7f3e733b81fp-45 + z * p;             /*  1/16! */
    p = -0x1.93974a8c07c9dp-37 + z * p;            /* -1/14! */
    p = 0x1.1eed8eff8d898p-29 + z * p;             /*  1/12! */
    p = -0x1.27e4fb7789f5cp-22 + z * p;            /* -1/10! */
    p = 0x1.a01a01a01a01ap-16 + z * p;             /*  1/8!  */
    p = -0x1.6c16c16c16c17p-10 + z * p;            /* -1/6!  */
    p = 0x1.5555555555555p-5 + z * p;              /*  1/4!  */
    return 1.0 + (-0.5 * z + (z * z) * p);
}

/* x = q pi/2 + r, |r| <= pi/4 (for |x| < 1e5). */
NF_HD double nf_reduce_pio2(double x, int *q) {
    const double kd = rint(x * NF_TWO_OVER_PI);
    *q = (int)kd;
    return (x - kd * NF_PIO2_CW_HI) - kd * NF_PIO2_CW_LO;
}

NF_HD double nf_sin(double x) {
    if (x != x || x == INFINITY || x == -INFINITY) return NAN;
    int q;
    const double r = nf_reduce_pio2(x, &q);
    switch (q & 3) {
        case 0: return nf_sin_series(r);
        case 1: return nf_cos_series(r);
        case 2: return -nf_sin_series(r);
        default: return -nf_cos_series(r);
    }
}

NF_HD double nf_cos(double x) {
    if (x != x || x == INFINITY || x == -INFINITY) return NAN;
    int q;
    const double r = nf_reduce_pio2(x, &q);
    switch (q & 3) {
        case 0: return nf_cos_series(r);
        case 1: return -nf_sin_series(r);
        case 2: return -nf_cos_series(r);
        default: return nf_sin_series(r);
    }
}

NF_HD double nf_hypot(double a, double b) {
    a = fabs(a);
    b = fabs(b);
    if (a == INFINITY || b == INFINITY) return INFINITY;
    if (a != a || b != b) return NAN;
    const double hi = a > b ? a : b;
    const double lo = a > b ? b : a;
    if (hi == 0.0) return 0.0;
    const double q = lo / hi;
    return hi * sqrt(1.0 + q * q);
}

#endif /* NF_MATH_H */
