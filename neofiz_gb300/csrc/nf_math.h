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
 * Methods (all from the mathematics; coefficients are exact Taylor coefficients rounded to
 * double, computed for this file):
 *   log   : x = 2^k m, m in [sqrt(1/2), sqrt(2)]; with f = m - 1 and s = f/(2+f),
 *           log(1+f) = 2 atanh(s) = f - s (f - R),  R = sum_{j>=1} 2 s^(2j) / (2j+1).
 *           k ln2 is added with a Cody-Waite split of ln2 (high part has 32 significant
 *           bits, so k*hi is exact). A double-double form feeds pow.
 *   exp   : Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, Taylor series to r^13.
 *   pow   : exp(y log x) with log in double-double and the product y*log x split exactly by
 *           Veltkamp/Dekker two-product (no fma), so the result is accurate to a few ulp
 *           rather than |y log x| ulp.
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

/* exp(r) for |r| <= ~0.35, Taylor to r^13. */
NF_HD double nf_exp_core(double r) {
    double p = 0x1.6124613a86d09p-33;              /* 1/13! */
    p = 0x1.1eed8eff8d898p-29 + r * p;             /* 1/12! */
    p = 0x1.ae64567f544e4p-26 + r * p;             /* 1/11! */
    p = 0x1.27e4fb7789f5cp-22 + r * p;             /* 1/10! */
    p = 0x1.71de3a556c734p-19 + r * p;             /* 1/9!  */
    p = 0x1.a01a01a01a01ap-16 + r * p;             /* 1/8!  */
    p = 0x1.a01a01a01a01ap-13 + r * p;             /* 1/7!  */
    p = 0x1.6c16c16c16c17p-10 + r * p;             /* 1/6!  */
    p = 0x1.1111111111111p-7 + r * p;              /* 1/5!  */
    p = 0x1.5555555555555p-5 + r * p;              /* 1/4!  */
    p = 0x1.5555555555555p-3 + r * p;              /* 1/3!  */
    p = 0x1.0000000000000p-1 + r * p;              /* 1/2!  */
    return 1.0 + (r + (r * r) * p);
}

NF_HD double nf_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    const double kd = rint(x * NF_INV_LN2);
    const int k = (int)kd;
    const double r = (x - kd * NF_LN2_HI) - kd * NF_LN2_LO;
    return nf_scale(nf_exp_core(r), k);
}

/* log(x) as an unevaluated sum hi + lo, for finite x > 0. */
NF_HD void nf_log_dd(double x, double *hi, double *lo) {
    uint64_t u = nf_bits(x);
    int k = 0;
    if (u < 0x0010000000000000ULL) {               /* subnormal: renormalise */
        x *= 0x1p54;
        u = nf_bits(x);
        k = -54;
    }
    k += (int)(u >> 52) - 1023;
    double m = nf_from_bits((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > NF_SQRT2) { m *= 0.5; k += 1; }
    const double f = m - 1.0;                      /* exact */
    const double s = f / (2.0 + f);
    const double z = s * s;
    double R = 0x1.af286bca1af28p-4;               /* 2/19 */
    R = 0x1.e1e1e1e1e1e1ep-4 + z * R;              /* 2/17 */
    R = 0x1.1111111111111p-3 + z * R;              /* 2/15 */
    R = 0x1.3b13b13b13b14p-3 + z * R;              /* 2/13 */
    R = 0x1.745d1745d1746p-3 + z * R;              /* 2/11 */
    R = 0x1.c71c71c71c71cp-3 + z * R;              /* 2/9  */
    R = 0x1.2492492492492p-2 + z * R;              /* 2/7  */
    R = 0x1.999999999999ap-2 + z * R;              /* 2/5  */
    R = 0x1.5555555555555p-1 + z * R;              /* 2/3  */
    R = z * R;
    const double c = s * (f - R);
    const double lg = f - c;
    const double lglo = (f - lg) - c;              /* |f| >= |c|: Fast2Sum error */
    const double dk = (double)k;
    const double t1 = dk * NF_LN2_HI;              /* exact */
    const double sum = t1 + lg;
    const double bb = sum - t1;
    const double err = (t1 - (sum - bb)) + (lg - bb);
    const double l = err + (lglo + dk * NF_LN2_LO);
    const double h = sum + l;
    *hi = h;
    *lo = l - (h - sum);
}

NF_HD double nf_log(double x) {
    if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;
    if (x == INFINITY) return x;
    double hi, lo;
    nf_log_dd(x, &hi, &lo);
    return hi + lo;
}

/* Veltkamp split of a into hi + lo, each with at most 26 significant bits. */
NF_HD void nf_split(double a, double *hi, double *lo) {
    const double c = 134217729.0 * a;              /* 2^27 + 1 */
    const double h = c - (c - a);
    *hi = h;
    *lo = a - h;
}

/* x^y for x >= 0 (or +inf), y neither 0 nor NaN. */
NF_HD double nf_pow_nonneg(double x, double y) {
    if (x == 1.0) return 1.0;
    if (x == 0.0) return y > 0.0 ? 0.0 : INFINITY;
    if (x == INFINITY) return y > 0.0 ? INFINITY : 0.0;
    if (y == INFINITY) return x > 1.0 ? INFINITY : 0.0;
    if (y == -INFINITY) return x > 1.0 ? 0.0 : INFINITY;
    double lh, ll;
    nf_log_dd(x, &lh, &ll);
    const double p = y * lh;
    if (p > 709.8) return INFINITY;
    if (p < -745.2) return 0.0;
    double yh, yl, hh, hl;
    nf_split(y, &yh, &yl);
    nf_split(lh, &hh, &hl);
    const double perr = ((yh * hh - p) + yh * hl + yl * hh) + yl * hl;  /* exact */
    const double plo = perr + y * ll;
    const double kd = rint(p * NF_INV_LN2);
    const int k = (int)kd;
    const double r = ((p - kd * NF_LN2_HI) + plo) - kd * NF_LN2_LO;
    return nf_scale(nf_exp_core(r), k);
}

/* Not recursive: a device call graph without cycles keeps the kernels' stack depth known at
 * compile time, so the driver sizes each launch's per-thread stack itself. */
NF_HD double nf_pow(double x, double y) {
    if (y == 0.0 || x == 1.0) return 1.0;
    if (x != x || y != y) return NAN;
    if (x < 0.0) {
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
