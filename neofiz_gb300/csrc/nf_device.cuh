// nf_device.cuh -- per-point constitutive arithmetic of the Neofiz timestep, as device
// functions. Each expression keeps the reference's evaluation order (Java is strict
// left-to-right IEEE double); the library is compiled with --fmad=false so nothing is fused.
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
constexpr double ISOTROPIC = 1.0e-9;
constexpr double DMAX = 1.7976931348623157e308;        // Double.MAX_VALUE

// Per-material constants, unrolled once at set-up (ExplicitSolver.java:284-300, J2.Flow.of).
struct MatDev {
    double lambda, mu, bulk, density, youngs;
    double sy0, hIso, hKin;
    double a, b, n, c, m, refRate, room, melt, cp, tq, thermalCoefficient;
    int jc;
    int pad;
};

// Damage state of one point (Damage.java:166-200), accessed through pointers so the
// element kernel can leave the rarely-touched geometry in global memory.
struct DamageRef {
    double failureStrain;
    double *strength, *softening, *width;
    const double *geometry;      // 5 doubles: area, uR, uZ, vR, vZ (reference configuration)
    double fractureEnergy, youngs;
};

__device__ __forceinline__ double jmin(double a, double b) {      // Math.min
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0 && b == 0.0) return signbit(a) ? a : b;
    return a <= b ? a : b;
}
__device__ __forceinline__ double jmax(double a, double b) {      // Math.max
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0 && b == 0.0) return signbit(a) ? b : a;
    return a >= b ? a : b;
}
__device__ __forceinline__ int jd2i(double x) {                    // Java (int) cast
    if (x != x) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return (-2147483647 - 1);
    return (int)x;
}

// JohnsonCook.java:138-209
__device__ __forceinline__ double jc_strainTerm(const MatDev &f, double eps) {
    return eps <= 0.0 ? f.a : f.a + f.b * nf_pow(eps, f.n);
}
__device__ __forceinline__ double jc_rateTerm(const MatDev &f, double rate) {
    if (rate <= f.refRate) return 1.0;
    return 1.0 + f.c * nf_log(rate / f.refRate);
}
__device__ __forceinline__ double jc_thermalTerm(const MatDev &f, double temperature) {
    const double homologous = (temperature - f.room) / (f.melt - f.room);
    if (homologous <= 0.0) return 1.0;
    if (homologous >= 1.0) return 0.0;
    return 1.0 - nf_pow(homologous, f.m);
}
__device__ __forceinline__ double jc_quasiStatic(const MatDev &f, double eps, double temperature) {
    return jc_strainTerm(f, eps) * jc_thermalTerm(f, temperature);
}

// J2.solve, J2.java:332-375
static __device__ __noinline__ double j2_solve(double norm, double stiffness, double plasticStrain,
                                        double temperature, double dt, const MatDev &jc) {
    const double thermal = jc_thermalTerm(jc, temperature);
    const double tolerance = SOLVE_TOLERANCE * jc.a;
    double lo = 0.0;
    double hi = norm / stiffness;
    double dGamma = hi;
    for (int iteration = 0; iteration < SOLVE_ITERATIONS; iteration++) {
        const double dEps = SQRT_2_3 * dGamma;
        const double eps = plasticStrain + dEps;
        const double rate = dt > 0.0 ? dEps / dt : 0.0;
        const double strain = jc_strainTerm(jc, eps);
        const double rateFactor = jc_rateTerm(jc, rate);
        const double g = norm - stiffness * dGamma - SQRT_2_3 * strain * rateFactor * thermal;
        if (g > 0.0) lo = dGamma; else hi = dGamma;
        if (fabs(g) <= tolerance) return dGamma;
        double slope = -stiffness
                       - TWO_THIRDS * (jc.n * (strain - jc.a) / eps) * rateFactor * thermal;
        if (!(rate <= jc.refRate)) {
            slope -= SQRT_2_3 * strain * jc.c * thermal / dGamma;
        }
        double next = dGamma - g / slope;
        if (!(next > lo && next < hi)) next = 0.5 * (lo + hi);
        dGamma = next;
    }
    return dGamma;
}

// Damage.begin, Damage.java:306-336
static __device__ __noinline__ void damage_begin(const DamageRef &d, double flowStress,
                                          double nRR, double nZZ, double nRZ) {
    const double area = d.geometry[0];
    const double diff = nRR - nZZ;
    const double cross = 2.0 * nRZ;
    const double anisotropy = nf_hypot(diff, cross);
    double h;
    if (anisotropy < ISOTROPIC) {
        h = sqrt(area);
    } else {
        const double phi = 0.5 * nf_atan2(cross, diff);
        const double tR = -nf_sin(phi), tZ = nf_cos(phi);
        const double line = fabs(d.geometry[1] * tR + d.geometry[2] * tZ)
                            + fabs(d.geometry[3] * tR + d.geometry[4] * tZ);
        h = area / line;
    }
    *d.width = h;
    *d.strength = flowStress;
    const double slope = -flowStress * flowStress * h / (2.0 * d.fractureEnergy);
    const double floor_ = -d.youngs;
    *d.softening = slope < floor_ ? floor_ : slope;
}

// J2.update, J2.java:163-296. s[4] and b[4] are the point's stress and back stress
// ({rr, zz, tt, rz}); damage is null for a material that cannot fail, in which case
// dStrength/dSoft are ignored. Returns the plastic multiplier.
__device__ __forceinline__ double j2_update(double *s, double *bk, double &epsP, double &work,
                                            double dRR, double dZZ, double dTT, double dGamRZ,
                                            double lambda, double mu, const MatDev &flow,
                                            double strainDt, const DamageRef *damage,
                                            double dStrength, double dSoft) {
    const double lt = lambda * (dRR + dZZ + dTT);
    const double tRR = s[0] + lt + 2.0 * mu * dRR;
    const double tZZ = s[1] + lt + 2.0 * mu * dZZ;
    const double tTT = s[2] + lt + 2.0 * mu * dTT;
    const double tRZ = s[3] + mu * dGamRZ;

    const double p = (tRR + tZZ + tTT) / 3.0;
    const double xRR = tRR - p - bk[0];
    const double xZZ = tZZ - p - bk[1];
    const double xTT = tTT - p - bk[2];
    const double xRZ = tRZ - bk[3];
    const double norm = sqrt(xRR * xRR + xZZ * xZZ + xTT * xTT + 2.0 * xRZ * xRZ);

    const bool jc = flow.jc != 0;
    const double temperature = !jc ? 0.0 : flow.room + flow.thermalCoefficient * work;

    const bool softening = damage != nullptr && dStrength > 0.0;
    double hardening = 0.0;
    double flowStress;
    if (softening) {
        flowStress = dStrength + dSoft * (epsP - damage->failureStrain);
        if (flowStress > 0.0) {
            hardening = dSoft;
        } else {
            flowStress = 0.0;
        }
    } else if (!jc) {
        flowStress = flow.sy0 + flow.hIso * epsP;
        hardening = flow.hIso;
    } else {
        flowStress = jc_quasiStatic(flow, epsP, temperature);
    }
    const double radius = SQRT_2_3 * flowStress;

    if (!(norm > radius)) {
        s[0] = tRR;
        s[1] = tZZ;
        s[2] = tTT;
        s[3] = tRZ;
        return 0.0;
    }

    const double stiffness = 2.0 * mu + TWO_THIRDS * flow.hKin;
    double dGamma;
    if (!jc || softening) {
        dGamma = (norm - radius) / (stiffness + TWO_THIRDS * hardening);
        if (softening && flowStress + hardening * SQRT_2_3 * dGamma < 0.0) {
            dGamma = norm / stiffness;
        }
    } else {
        dGamma = j2_solve(norm, stiffness, epsP, temperature, strainDt, flow);
    }
    const double inv = 1.0 / norm;
    const double nRR = xRR * inv, nZZ = xZZ * inv, nTT = xTT * inv, nRZ = xRZ * inv;

    const double pull = 2.0 * mu * dGamma;
    s[0] = tRR - pull * nRR;
    s[1] = tZZ - pull * nZZ;
    s[2] = tTT - pull * nTT;
    s[3] = tRZ - pull * nRZ;

    const double alphaDotN = bk[0] * nRR + bk[1] * nZZ + bk[2] * nTT + 2.0 * bk[3] * nRZ;
    work += dGamma * (norm - pull + alphaDotN);

    const double shift = TWO_THIRDS * flow.hKin * dGamma;
    bk[0] += shift * nRR;
    bk[1] += shift * nZZ;
    bk[2] += shift * nTT;
    bk[3] += shift * nRZ;

    epsP += SQRT_2_3 * dGamma;

    if (damage != nullptr && !softening && epsP >= damage->failureStrain) {
        damage_begin(*damage,
                     !jc ? flow.sy0 + flow.hIso * epsP : jc_quasiStatic(flow, epsP, temperature),
                     nRR, nZZ, nRZ);
    }
    return dGamma;
}

// Corotational.java:59-98
__device__ __forceinline__ void corot_rotate(double *t, double c, double sn) {
    const double rr = t[0], zz = t[1], rz = t[3];
    const double cc = c * c, ss = sn * sn, cs = c * sn;
    t[0] = cc * rr - 2.0 * cs * rz + ss * zz;
    t[1] = ss * rr + 2.0 * cs * rz + cc * zz;
    t[3] = cs * (rr - zz) + (cc - ss) * rz;
}
__device__ __forceinline__ double corot_cos(double spinDt) {
    const double h = 0.5 * spinDt;
    return (1.0 - h * h) / (1.0 + h * h);
}
__device__ __forceinline__ double corot_sin(double spinDt) {
    const double h = 0.5 * spinDt;
    return 2.0 * h / (1.0 + h * h);
}

__device__ __forceinline__ double sq2(double a, double b) { return a * a + b * b; }

// shortestEdge, ExplicitSolver.java:1191-1197
__device__ __forceinline__ double shortestEdge(double running, double r0, double r1, double r2,
                                               double r3, double z0, double z1, double z2,
                                               double z3) {
    return jmin(running, jmin(jmin(sq2(r1 - r0, z1 - z0), sq2(r2 - r1, z2 - z1)),
                              jmin(sq2(r3 - r2, z3 - z2), sq2(r0 - r3, z0 - z3))));
}

// Damage.at, Damage.java:342-347
__device__ __forceinline__ double damage_at(double strength, double softening,
                                            double failureStrain, double plasticStrain) {
    const double sf = strength;
    if (sf <= 0.0) return 0.0;
    const double v = -softening * (plasticStrain - failureStrain) / sf;
    return v <= 0.0 ? 0.0 : (v >= 1.0 ? 1.0 : v);
}

}  // namespace nf
