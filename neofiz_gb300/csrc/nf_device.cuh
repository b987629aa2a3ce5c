// nf_device.cuh -- per-point constitutive arithmetic of the Neofiz timestep, as device
// functions templated on the real type.
//
// The double instantiation is the plain path: each expression keeps the reference's
// evaluation order (Java is strict left-to-right IEEE double), the library is compiled with
// --fmad=false so nothing is fused, and the transcendentals are the deterministic ones of
// nf_math.h, so it is bit-identical to the CPU restatement. The float instantiation is the
// mixed-precision path's element arithmetic: the same algorithm in FP32 with CUDA's float
// math functions and a Johnson-Cook solve tolerance that FP32 can reach.
//
// Reference (src/main/java/org/neofiz/): solver/J2.java:163-296 (update), :332-375 (solve);
// core/JohnsonCook.java:138-209; solver/Damage.java:306-347; solver/Corotational.java:59-98.
#pragma once

#include <cstdint>
#include "nf_math.h"

namespace nf {

constexpr double SQRT_2_3 = 0x1.a20bd700c2c3ep-1;     // Math.sqrt(2.0 / 3.0)
constexpr double TWO_THIRDS = 2.0 / 3.0;
constexpr double SOLVE_TOLERANCE = 1.0e-10;
constexpr int SOLVE_ITERATIONS = 25;
constexpr int COST_NEAR_YIELD = SOLVE_ITERATIONS + 2;   // cost class of an elastic point near yield
constexpr double ISOTROPIC = 1.0e-9;
constexpr double DMAX = 1.7976931348623157e308;        // Double.MAX_VALUE

// Per-material constants, unrolled once at set-up (ExplicitSolver.java:284-300, J2.Flow.of).
template <typename T>
struct MatT {
    T lambda, mu, bulk, density, youngs;
    T sy0, hIso, hKin;
    T a, b, n, c, m, refRate, room, melt, cp, tq, thermalCoefficient;
    int jc;
    int pad;
};
using MatDev = MatT<double>;
using MatF = MatT<float>;

// Elementary functions per real type.
template <typename T> struct Fn;
template <> struct Fn<double> {
    static __device__ __forceinline__ double pow(double a, double b) { return nf_pow(a, b); }
    static __device__ __forceinline__ double log(double a) { return nf_log(a); }
    static __device__ __forceinline__ double sqrt(double a) { return ::sqrt(a); }
    static __device__ __forceinline__ double hypot(double a, double b) { return nf_hypot(a, b); }
    static __device__ __forceinline__ double atan2(double a, double b) { return nf_atan2(a, b); }
    static __device__ __forceinline__ double sin(double a) { return nf_sin(a); }
    static __device__ __forceinline__ double cos(double a) { return nf_cos(a); }
    static __device__ __forceinline__ double abs(double a) { return ::fabs(a); }
    static __device__ __forceinline__ double div3(double a);
    static constexpr double tolerance = SOLVE_TOLERANCE;
};
// The FP32 forms run well inside their error budget with CUDA's fast pow and log (a few ulp
// instead of correctly rounded): the Johnson-Cook solve of a plastic point calls them in
// every Newton iteration.
template <> struct Fn<float> {
    static __device__ __forceinline__ float pow(float a, float b) { return __powf(a, b); }
    static __device__ __forceinline__ float log(float a) { return __logf(a); }
    static __device__ __forceinline__ float sqrt(float a) { return ::sqrtf(a); }
    static __device__ __forceinline__ float hypot(float a, float b) { return ::hypotf(a, b); }
    static __device__ __forceinline__ float atan2(float a, float b) { return ::atan2f(a, b); }
    static __device__ __forceinline__ float sin(float a) { return ::sinf(a); }
    static __device__ __forceinline__ float cos(float a) { return ::cosf(a); }
    static __device__ __forceinline__ float abs(float a) { return ::fabsf(a); }
    static __device__ __forceinline__ float div3(float a) { return a / 3.0f; }
    // 1e-10 A is below FP32 resolution of the residual; 1e-5 A is a few ulp of it.
    static constexpr float tolerance = 1.0e-5f;
};

// x / 3 correctly rounded, without a division. z = RN(1/3) satisfies 3 z = 1 - 2^-54, so
// q0 = RN(x z) lies within one ulp of x / 3; the remainder x - 3 q0 is then exact (one fused
// multiply-add), and one correction q0 + r z rounded once is RN(x / 3) (Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990: a faithful quotient corrected with the correctly rounded reciprocal). The argument
// needs x and the quotient far from underflow and overflow: 2^-1000 <= |x| < 2^1001 takes this
// path, +-0 gives q0 = +-0 (which is x / 3), and anything else is divided.
__device__ __forceinline__ double Fn<double>::div3(double x) {
    const double z = 0x1.5555555555555p-2;
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    const double q0 = x * z;
    if (e - 23u < 2002u) return fma(fma(-q0, 3.0, x), z, q0);
    if ((u << 1) == 0) return q0;
    return x / 3.0;
}

// Damage state of one point (Damage.java:166-200), accessed through pointers so the
// element kernel can leave the rarely-touched geometry in global memory.
template <typename T>
struct DamageRefT {
    T failureStrain;
    T *strength, *softening, *width;
    const T *geometry;           // 5 values: area, uR, uZ, vR, vZ (reference configuration)
    T fractureEnergy, youngs;
};
using DamageRef = DamageRefT<double>;

template <typename T>
__device__ __forceinline__ T jmin(T a, T b) {                      // Math.min
    if (a != a) return a;
    if (b != b) return b;
    if (a == T(0) && b == T(0)) return signbit(a) ? a : b;
    return a <= b ? a : b;
}
template <typename T>
__device__ __forceinline__ T jmax(T a, T b) {                      // Math.max
    if (a != a) return a;
    if (b != b) return b;
    if (a == T(0) && b == T(0)) return signbit(a) ? b : a;
    return a >= b ? a : b;
}
__device__ __forceinline__ int jd2i(double x) {                    // Java (int) cast
    if (x != x) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return (-2147483647 - 1);
    return (int)x;
}

// JohnsonCook.java:138-209
template <typename T>
__device__ __forceinline__ T jc_strainTerm(const MatT<T> &f, T eps) {
    return eps <= T(0) ? f.a : f.a + f.b * Fn<T>::pow(eps, f.n);
}
template <typename T>
__device__ __forceinline__ T jc_rateTerm(const MatT<T> &f, T rate) {
    if (rate <= f.refRate) return T(1);
    // rate / 1 is rate exactly: the common reference rate of 1/s skips the division
    return T(1) + f.c * Fn<T>::log(f.refRate == T(1) ? rate : rate / f.refRate);
}
// isfinite by the exponent field (an integer test, off the FP64 pipe)
__device__ __forceinline__ bool finite_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ULL) !=
           0x7ff0000000000000ULL;
}

// x == +-0 by bit pattern for doubles (an integer test, off the FP64 pipe)
__device__ __forceinline__ bool is_zero(double x) {
    return ((unsigned long long)__double_as_longlong(x) << 1) == 0ULL;
}
__device__ __forceinline__ bool is_zero(float x) { return x == 0.0f; }

template <typename T>
__device__ __forceinline__ T jc_thermalTerm(const MatT<T> &f, T temperature) {
    const T above = temperature - f.room, span = f.melt - f.room;
    // a point that has done no plastic work sits at room temperature: 0 / span is +-0, whose
    // term is 1, for any span but 0 and NaN (which the division below turns into NaN)
    if (is_zero(above) && (span > T(0) || span < T(0))) return T(1);
    const T homologous = above / span;
    if (homologous <= T(0)) return T(1);
    if (homologous >= T(1)) return T(0);
    return T(1) - Fn<T>::pow(homologous, f.m);
}
template <typename T>
__device__ __forceinline__ T jc_quasiStatic(const MatT<T> &f, T eps, T temperature) {
    return jc_strainTerm(f, eps) * jc_thermalTerm(f, temperature);
}

// What J2.solve returns, and what it knew of its answer: the iterations taken and, when it
// converged, the strain term at the returned increment (the new state's, which the caller
// would otherwise evaluate again).
template <typename T>
struct SolveOut {
    T dGamma, strain;
    int iterations, converged;
};

// An ordering hint only (never part of a result): norm / radius above about 0.81, for
// non-negative norm and positive radius, from their bit patterns.
__device__ __forceinline__ bool near_yield(double norm, double radius) {
    return __double_as_longlong(norm) - __double_as_longlong(radius) > -(1351079888211148LL);
}
__device__ __forceinline__ bool near_yield(float norm, float radius) { return norm > 0.81f * radius; }

// J2.solve, J2.java:332-375, given the thermal term jc_thermalTerm(jc, temperature) of the
// point's temperature (the reference evaluates it first thing, from the same argument).
template <typename T>
static __device__ __noinline__ SolveOut<T> j2_solve(T norm, T stiffness, T plasticStrain,
                                                    T thermal, T dt, const MatT<T> &jc) {
    const T tolerance = Fn<T>::tolerance * jc.a;
    T lo = T(0);
    T hi = norm / stiffness;
    T dGamma = hi;
    for (int iteration = 0; iteration < SOLVE_ITERATIONS; iteration++) {
        const T dEps = T(SQRT_2_3) * dGamma;
        const T eps = plasticStrain + dEps;
        const T rate = dt > T(0) ? dEps / dt : T(0);
        const T strain = jc_strainTerm(jc, eps);
        const T rateFactor = jc_rateTerm(jc, rate);
        const T g = norm - stiffness * dGamma - T(SQRT_2_3) * strain * rateFactor * thermal;
        if (g > T(0)) lo = dGamma; else hi = dGamma;
        if (Fn<T>::abs(g) <= tolerance) return SolveOut<T>{dGamma, strain, iteration + 1, 1};
        T slope = -stiffness
                  - T(TWO_THIRDS) * (jc.n * (strain - jc.a) / eps) * rateFactor * thermal;
        if (!(rate <= jc.refRate)) {
            slope -= T(SQRT_2_3) * strain * jc.c * thermal / dGamma;
        }
        T next = dGamma - g / slope;
        if (!(next > lo && next < hi)) next = T(0.5) * (lo + hi);
        dGamma = next;
    }
    return SolveOut<T>{dGamma, T(0), SOLVE_ITERATIONS, 0};
}

// Damage.begin, Damage.java:306-336
template <typename T>
static __device__ __noinline__ void damage_begin(const DamageRefT<T> &d, T flowStress, T nRR,
                                                 T nZZ, T nRZ) {
    const T area = d.geometry[0];
    const T diff = nRR - nZZ;
    const T cross = T(2) * nRZ;
    const T anisotropy = Fn<T>::hypot(diff, cross);
    T h;
    if (anisotropy < T(ISOTROPIC)) {
        h = Fn<T>::sqrt(area);
    } else {
        const T phi = T(0.5) * Fn<T>::atan2(cross, diff);
        const T tR = -Fn<T>::sin(phi), tZ = Fn<T>::cos(phi);
        const T line = Fn<T>::abs(d.geometry[1] * tR + d.geometry[2] * tZ)
                       + Fn<T>::abs(d.geometry[3] * tR + d.geometry[4] * tZ);
        h = area / line;
    }
    *d.width = h;
    *d.strength = flowStress;
    const T slope = -flowStress * flowStress * h / (T(2) * d.fractureEnergy);
    const T floor_ = -d.youngs;
    *d.softening = slope < floor_ ? floor_ : slope;
}

// The Johnson-Cook yield radius sqrt(2/3) A(eps) T(work) of a point's state and its thermal
// term T: the quasi-static flow stress J2.update evaluates (JohnsonCook.java:138-209), in the
// same operations, so a point whose state is unchanged since may use the kept pair instead.
__device__ __forceinline__ double2 jc_yield(const MatDev &f, double epsP, double work) {
    const double thermal = jc_thermalTerm(f, f.room + f.thermalCoefficient * work);
    return make_double2(SQRT_2_3 * (jc_strainTerm(f, epsP) * thermal), thermal);
}

// J2.update, J2.java:163-296. s[4] and bk[4] are the point's stress and back stress
// ({rr, zz, tt, rz}); damage is null for a material that cannot fail, in which case
// dStrength/dSoft are ignored. Returns the plastic multiplier. *cost (when given) receives
// the point's Johnson-Cook cost class: 0 none, 1 the quasi-static flow stress evaluated its
// power laws, 1 + k a return-map solve of k iterations. jcYield (FP64 only, when given) holds
// jc_yield of the point's current plastic strain and work for a Johnson-Cook material; it is
// read in place of the power laws and kept up to date whenever they change.
template <typename T>
__device__ __forceinline__ T j2_update(T *s, T *bk, T &epsP, T &work, T dRR, T dZZ, T dTT,
                                       T dGamRZ, T lambda, T mu, const MatT<T> &flow, T strainDt,
                                       const DamageRefT<T> *damage, T dStrength, T dSoft,
                                       int *cost = nullptr, double2 *jcYield = nullptr) {
    const T lt = lambda * (dRR + dZZ + dTT);
    const T tRR = s[0] + lt + T(2) * mu * dRR;
    const T tZZ = s[1] + lt + T(2) * mu * dZZ;
    const T tTT = s[2] + lt + T(2) * mu * dTT;
    const T tRZ = s[3] + mu * dGamRZ;

    const T p = Fn<T>::div3(tRR + tZZ + tTT);
    const T xRR = tRR - p - bk[0];
    const T xZZ = tZZ - p - bk[1];
    const T xTT = tTT - p - bk[2];
    const T xRZ = tRZ - bk[3];
    const T norm = Fn<T>::sqrt(xRR * xRR + xZZ * xZZ + xTT * xTT + T(2) * xRZ * xRZ);

    const bool jc = flow.jc != 0;
    const bool softening = damage != nullptr && dStrength > T(0);
    T hardening = T(0);
    T flowStress = T(0), radius, thermal = T(1);
    if (softening) {
        flowStress = dStrength + dSoft * (epsP - damage->failureStrain);
        if (flowStress > T(0)) {
            hardening = dSoft;
        } else {
            flowStress = T(0);
        }
        radius = T(SQRT_2_3) * flowStress;
    } else if (!jc) {
        flowStress = flow.sy0 + flow.hIso * epsP;
        hardening = flow.hIso;
        radius = T(SQRT_2_3) * flowStress;
    } else {
        if (jcYield) {
            const double2 y = *jcYield;
            radius = T(y.x);
            thermal = T(y.y);
        } else {                          // jc_quasiStatic, its thermal term kept for the solve
            thermal = jc_thermalTerm(flow, flow.room + flow.thermalCoefficient * work);
            flowStress = jc_strainTerm(flow, epsP) * thermal;
            radius = T(SQRT_2_3) * flowStress;
        }
        if (cost && (epsP > T(0) || work > T(0))) *cost = 1;
    }

    if (!(norm > radius)) {
        s[0] = tRR;
        s[1] = tZZ;
        s[2] = tTT;
        s[3] = tRZ;
        // a Johnson-Cook point within about 20 % of its yield radius is likely to yield soon:
        // the bit patterns of two positive doubles differ by about 2^52 log2 of their ratio,
        // so an integer difference above -0.3 2^52 is a ratio above about 0.81
        if (cost && jc && !softening && near_yield(norm, radius)) *cost = COST_NEAR_YIELD;
        return T(0);
    }

    const T stiffness = T(2) * mu + T(TWO_THIRDS) * flow.hKin;
    T dGamma;
    T strainNew = T(0);                   // the strain term at the new plastic strain, if known
    bool haveStrain = false;
    if (!jc || softening) {
        dGamma = (norm - radius) / (stiffness + T(TWO_THIRDS) * hardening);
        if (softening && flowStress + hardening * T(SQRT_2_3) * dGamma < T(0)) {
            dGamma = norm / stiffness;
        }
    } else {
        const SolveOut<T> r = j2_solve(norm, stiffness, epsP, thermal, strainDt, flow);
        dGamma = r.dGamma;
        // the solve's last strain term was taken at plasticStrain + sqrt(2/3) dGamma, the same
        // sum that forms the new plastic strain below
        strainNew = r.strain;
        haveStrain = r.converged != 0;
        if (cost) *cost = 1 + r.iterations;
    }
    const T inv = T(1) / norm;
    const T nRR = xRR * inv, nZZ = xZZ * inv, nTT = xTT * inv, nRZ = xRZ * inv;

    const T pull = T(2) * mu * dGamma;
    s[0] = tRR - pull * nRR;
    s[1] = tZZ - pull * nZZ;
    s[2] = tTT - pull * nTT;
    s[3] = tRZ - pull * nRZ;

    const T alphaDotN = bk[0] * nRR + bk[1] * nZZ + bk[2] * nTT + T(2) * bk[3] * nRZ;
    work += dGamma * (norm - pull + alphaDotN);

    const T shift = T(TWO_THIRDS) * flow.hKin * dGamma;
    bk[0] += shift * nRR;
    bk[1] += shift * nZZ;
    bk[2] += shift * nTT;
    bk[3] += shift * nRZ;

    epsP += T(SQRT_2_3) * dGamma;

    const bool onset = damage != nullptr && !softening && epsP >= damage->failureStrain;
    if (jc && !haveStrain && (onset || jcYield)) {
        strainNew = jc_strainTerm(flow, epsP);
        haveStrain = true;
    }
    if (onset) {
        // jc_quasiStatic(flow, epsP, temperature): the new strain, the step's own temperature
        damage_begin(*damage, !jc ? flow.sy0 + flow.hIso * epsP : strainNew * thermal,
                     nRR, nZZ, nRZ);
    }
    if (jc && jcYield) {
        const double th = jc_thermalTerm(flow, flow.room + flow.thermalCoefficient * work);
        *jcYield = make_double2(SQRT_2_3 * ((double)strainNew * th), th);
    }
    return dGamma;
}

// Corotational.java:59-98
template <typename T>
__device__ __forceinline__ void corot_rotate(T *t, T c, T sn) {
    const T rr = t[0], zz = t[1], rz = t[3];
    const T cc = c * c, ss = sn * sn, cs = c * sn;
    t[0] = cc * rr - T(2) * cs * rz + ss * zz;
    t[1] = ss * rr + T(2) * cs * rz + cc * zz;
    t[3] = cs * (rr - zz) + (cc - ss) * rz;
}
template <typename T>
__device__ __forceinline__ T corot_cos(T spinDt) {
    const T h = T(0.5) * spinDt;
    return (T(1) - h * h) / (T(1) + h * h);
}
template <typename T>
__device__ __forceinline__ T corot_sin(T spinDt) {
    const T h = T(0.5) * spinDt;
    return T(2) * h / (T(1) + h * h);
}

// corot_rotate of a tensor whose rr, zz and rz are +0 gives +0 in all three when c and sn are
// finite (|c|, |sn| <= 1, so no product overflows) and the rz component's two terms,
// (c sn)(+0) and (c^2 - sn^2)(+0), are not both -0: a product's sign is its factors' sign
// bits xor-ed, and +0 + -0 = +0.
__device__ __forceinline__ bool corot_keeps_zero(double c, double sn) {
    const uint64_t uc = (uint64_t)__double_as_longlong(c), us = (uint64_t)__double_as_longlong(sn);
    const uint64_t ud = (uint64_t)__double_as_longlong(c * c - sn * sn);
    return finite_bits(c) && finite_bits(sn) && !(((uc ^ us) & ud) >> 63);
}

// x is +-0 or 2^-400 <= |x| < 2^400 (the exponent field alone): scaling such values by a
// power of two between 2^-8 and 2^8, and their products and differences, stay normal.
__device__ __forceinline__ bool moderate_or_zero(double x) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    return e - 623u < 800u || (u << 1) == 0;
}

// Bits of four values all zero: every value is +0.
__device__ __forceinline__ bool all_plus_zero(double a, double b, double c, double d) {
    return (__double_as_longlong(a) | __double_as_longlong(b) | __double_as_longlong(c) |
            __double_as_longlong(d)) == 0;
}

template <typename T>
__device__ __forceinline__ T sq2(T a, T b) { return a * a + b * b; }

// Math.min of two squared lengths (+0, positive, +inf or NaN): their bit patterns order as
// their values do, every NaN pattern lies above +inf's, and Math.min's NaN rule is kept, so
// integer comparisons give jmin's answer without using the FP64 pipe.
__device__ __forceinline__ double jmin_nonneg(double a, double b) {
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    if (ua > 0x7ff0000000000000ULL) return a;
    if (ub > 0x7ff0000000000000ULL) return b;
    return ua <= ub ? a : b;
}
__device__ __forceinline__ float jmin_nonneg(float a, float b) { return jmin(a, b); }

// shortestEdge, ExplicitSolver.java:1191-1197 (running is Double.MAX_VALUE or an earlier
// minimum, so every operand is a squared length)
template <typename T>
__device__ __forceinline__ T shortestEdge(T running, T r0, T r1, T r2, T r3, T z0, T z1, T z2,
                                          T z3) {
    return jmin_nonneg(running,
                       jmin_nonneg(jmin_nonneg(sq2(r1 - r0, z1 - z0), sq2(r2 - r1, z2 - z1)),
                                   jmin_nonneg(sq2(r3 - r2, z3 - z2), sq2(r0 - r3, z0 - z3))));
}

// Damage.at, Damage.java:342-347
template <typename T>
__device__ __forceinline__ T damage_at(T strength, T softening, T failureStrain, T plasticStrain) {
    const T sf = strength;
    if (sf <= T(0)) return T(0);
    const T v = -softening * (plasticStrain - failureStrain) / sf;
    return v <= T(0) ? T(0) : (v >= T(1) ? T(1) : v);
}

}  // namespace nf
