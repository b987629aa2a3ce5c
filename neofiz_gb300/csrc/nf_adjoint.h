/*
 * nf_adjoint.h -- reverse-mode derivatives of one explicit central-difference step, shared by
 * the CUDA adjoint kernel (k_adjoint.cu) and the CPU reference adjoint of the oracle.
 *
 * There is no adjoint in the reference. This file differentiates the reference's step as the
 * forward kernels compute it (ExplicitSolver.step :940-991 with nodalUpdate :998-1062,
 * RigidWall.slide/hold/arrive RigidWall.java:163-259, reducedIntegration :1373-1504,
 * J2.update/solve J2.java:163-375, JohnsonCook.java:138-209, Corotational.java:59-98 and the
 * CFL step :985-990). Each function first recomputes its forward values in exactly the
 * forward kernels' operation order -- so every branch (elastic or plastic point, rate and
 * temperature clamps, wall hold/stick/slip/arrive, the shortest edge) is the one the forward
 * pass took, i.e. frozen -- and then runs the reverse sweep by hand. The Johnson-Cook return
 * map is differentiated through its converged root by the implicit function theorem.
 *
 * Differentiated parameters (NF_ADJ_P_*): Johnson-Cook A, B, n, C, m, the kinematic
 * hardening modulus, the wall friction coefficient, the fracture energy, and the yield stress
 * and isotropic hardening modulus of a linear-hardening material.
 *
 * Plain C (C99) with NF_HD qualifiers, so the oracle (gcc) and the kernels (nvcc) compile the
 * same text; both build with contraction off.
 */
#ifndef NF_ADJOINT_H
#define NF_ADJOINT_H

#include "nf_math.h"

enum { NF_ADJ_P_A = 0, NF_ADJ_P_B, NF_ADJ_P_N, NF_ADJ_P_C, NF_ADJ_P_M, NF_ADJ_P_HKIN,
       NF_ADJ_P_MU, NF_ADJ_P_GF, NF_ADJ_P_SY0, NF_ADJ_P_HISO, NF_ADJ_P_COUNT };

#define NF_ADJ_SQRT_2_3 0x1.a20bd700c2c3ep-1
#define NF_ADJ_TWO_THIRDS (2.0 / 3.0)
/* The reverse differentiates the Johnson-Cook return through its root (implicit function
 * theorem), so the root it evaluates the derivative at is converged further than the forward
 * pass converges it (J2.solve's 1e-10 A, J2.java:332-375, which the forward keeps for parity):
 * at 1e-10 A a solve can stop short of the root -- a bracket closing on the rate term's kink,
 * the iteration cap -- and over a long run the derivatives evaluated there drift from those of
 * the map (0.3 % in d(L/L0)/d(friction) over the 80 us rod). Solved to 1e-14 A the reverse
 * agrees with central differences of the forward map itself. The forward trajectory and the
 * objective values are untouched: the plain step code produces them. */
#define NF_ADJ_TOLERANCE 1.0e-14
#define NF_ADJ_ITERATIONS 80

/* The material constants one point reads (ExplicitSolver.java:289-299, J2.Flow.of). */
typedef struct {
    double lambda, mu, sy0, hIso, hKin;
    double a, b, n, c, m, refRate, room, melt, thermalCoefficient;
    int jc;
} nf_adj_mat;

/* ------------------------------------------------------------------ Johnson-Cook */

NF_HD double nf_adj_strain_term(const nf_adj_mat *f, double eps) {
    return eps <= 0.0 ? f->a : f->a + f->b * nf_pow(eps, f->n);
}
NF_HD double nf_adj_rate_term(const nf_adj_mat *f, double rate) {
    if (rate <= f->refRate) return 1.0;
    return 1.0 + f->c * nf_log(rate / f->refRate);
}
NF_HD double nf_adj_thermal_term(const nf_adj_mat *f, double temperature) {
    const double homologous = (temperature - f->room) / (f->melt - f->room);
    if (homologous <= 0.0) return 1.0;
    if (homologous >= 1.0) return 0.0;
    return 1.0 - nf_pow(homologous, f->m);
}

/* J2.solve, J2.java:332-375, in the forward kernels' order, to the reverse's tolerance. */
NF_HD double nf_adj_solve(double norm, double stiffness, double plasticStrain,
                          double temperature, double dt, const nf_adj_mat *jc) {
    const double thermal = nf_adj_thermal_term(jc, temperature);
    const double tolerance = NF_ADJ_TOLERANCE * jc->a;
    double lo = 0.0, hi = norm / stiffness, dGamma = hi;
    for (int iteration = 0; iteration < NF_ADJ_ITERATIONS; iteration++) {
        const double dEps = NF_ADJ_SQRT_2_3 * dGamma;
        const double eps = plasticStrain + dEps;
        const double rate = dt > 0.0 ? dEps / dt : 0.0;
        const double strain = nf_adj_strain_term(jc, eps);
        const double rateFactor = nf_adj_rate_term(jc, rate);
        const double g = norm - stiffness * dGamma - NF_ADJ_SQRT_2_3 * strain * rateFactor * thermal;
        if (g > 0.0) lo = dGamma; else hi = dGamma;
        if (fabs(g) <= tolerance) return dGamma;
        double slope = -stiffness
                       - NF_ADJ_TWO_THIRDS * (jc->n * (strain - jc->a) / eps) * rateFactor * thermal;
        if (!(rate <= jc->refRate)) slope -= NF_ADJ_SQRT_2_3 * strain * jc->c * thermal / dGamma;
        double next = dGamma - g / slope;
        if (!(next > lo && next < hi)) next = 0.5 * (lo + hi);
        dGamma = next;
    }
    return dGamma;
}

/* ------------------------------------------------------------------ J2 return map */

/* A point's damage state and parameters (Damage.java:166-200): NULL for a material that
 * cannot fail. */
typedef struct {
    double failureStrain, strength, softening, fractureEnergy, youngs;
    const double *geometry;      /* area, uR, uZ, vR, vZ of the reference element */
} nf_adj_damage;

/* The return map's forward values at one point (J2.update, J2.java:163-296, with the damage
 * branches of Damage.java:306-347), kept for its reverse. */
typedef struct {
    double t[4], x[4], norm, temperature, flowStress, radius, hardening, stiffness;
    double dGamma, n[4], pull, alphaDotN, shift, epsP1;
    int plastic, softening, clamped, fallback, onset;
    /* onset: the flow stress at onset and the band width (Damage.begin, :306-336) */
    double fsOnset, width, slope, diff, cross, anisotropy, phi, l1, l2, line;
    int isotropic, floored;
} nf_adj_j2_tape;

/* Forward of the return map in the forward kernels' operation order; fills the tape and the
 * point's new stress, back stress, plastic strain, plastic work and damage state. */
NF_HD void nf_adj_j2_forward(const double *s, const double *bk, double epsP, double work,
                             double dRR, double dZZ, double dTT, double dGamRZ,
                             const nf_adj_mat *f, double strainDt, const nf_adj_damage *dm,
                             nf_adj_j2_tape *tp, double *sOut, double *bOut) {
    const double lambda = f->lambda, mu = f->mu;
    const double lt = lambda * (dRR + dZZ + dTT);
    tp->t[0] = s[0] + lt + 2.0 * mu * dRR;
    tp->t[1] = s[1] + lt + 2.0 * mu * dZZ;
    tp->t[2] = s[2] + lt + 2.0 * mu * dTT;
    tp->t[3] = s[3] + mu * dGamRZ;
    const double p = (tp->t[0] + tp->t[1] + tp->t[2]) / 3.0;
    tp->x[0] = tp->t[0] - p - bk[0];
    tp->x[1] = tp->t[1] - p - bk[1];
    tp->x[2] = tp->t[2] - p - bk[2];
    tp->x[3] = tp->t[3] - bk[3];
    const double *x = tp->x;
    tp->norm = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + 2.0 * x[3] * x[3]);
    const int jc = f->jc != 0;
    tp->temperature = !jc ? 0.0 : f->room + f->thermalCoefficient * work;
    tp->softening = dm != 0 && dm->strength > 0.0;
    tp->clamped = 0;
    tp->hardening = 0.0;
    double fs;
    if (tp->softening) {
        fs = dm->strength + dm->softening * (epsP - dm->failureStrain);
        if (fs > 0.0) {
            tp->hardening = dm->softening;
        } else {
            fs = 0.0;
            tp->clamped = 1;
        }
    } else if (!jc) {
        fs = f->sy0 + f->hIso * epsP;
        tp->hardening = f->hIso;
    } else {
        fs = nf_adj_strain_term(f, epsP) * nf_adj_thermal_term(f, tp->temperature);
    }
    tp->flowStress = fs;
    tp->radius = NF_ADJ_SQRT_2_3 * fs;
    tp->plastic = tp->norm > tp->radius;
    tp->onset = 0;
    tp->fallback = 0;
    if (!tp->plastic) {
        for (int k = 0; k < 4; k++) {
            sOut[k] = tp->t[k];
            bOut[k] = bk[k];
        }
        tp->epsP1 = epsP;
        return;
    }
    tp->stiffness = 2.0 * mu + NF_ADJ_TWO_THIRDS * f->hKin;
    double dGamma;
    if (!jc || tp->softening) {
        dGamma = (tp->norm - tp->radius) / (tp->stiffness + NF_ADJ_TWO_THIRDS * tp->hardening);
        if (tp->softening && fs + tp->hardening * NF_ADJ_SQRT_2_3 * dGamma < 0.0) {
            dGamma = tp->norm / tp->stiffness;
            tp->fallback = 1;
        }
    } else {
        dGamma = nf_adj_solve(tp->norm, tp->stiffness, epsP, tp->temperature, strainDt, f);
    }
    tp->dGamma = dGamma;
    const double inv = 1.0 / tp->norm;
    for (int k = 0; k < 4; k++) tp->n[k] = x[k] * inv;
    const double *n = tp->n;
    tp->pull = 2.0 * mu * dGamma;
    for (int k = 0; k < 4; k++) sOut[k] = tp->t[k] - tp->pull * n[k];
    tp->alphaDotN = bk[0] * n[0] + bk[1] * n[1] + bk[2] * n[2] + 2.0 * bk[3] * n[3];
    tp->shift = NF_ADJ_TWO_THIRDS * f->hKin * dGamma;
    for (int k = 0; k < 4; k++) bOut[k] = bk[k] + tp->shift * n[k];
    tp->epsP1 = epsP + NF_ADJ_SQRT_2_3 * dGamma;
    if (dm != 0 && !tp->softening && tp->epsP1 >= dm->failureStrain) {
        tp->onset = 1;
        tp->fsOnset = !jc ? f->sy0 + f->hIso * tp->epsP1
                          : nf_adj_strain_term(f, tp->epsP1) * nf_adj_thermal_term(f, tp->temperature);
        const double area = dm->geometry[0];
        tp->diff = n[0] - n[1];
        tp->cross = 2.0 * n[3];
        tp->anisotropy = nf_hypot(tp->diff, tp->cross);
        if (tp->anisotropy < 1.0e-9) {
            tp->isotropic = 1;
            tp->width = sqrt(area);
        } else {
            tp->isotropic = 0;
            tp->phi = 0.5 * nf_atan2(tp->cross, tp->diff);
            const double tR = -nf_sin(tp->phi), tZ = nf_cos(tp->phi);
            tp->l1 = dm->geometry[1] * tR + dm->geometry[2] * tZ;
            tp->l2 = dm->geometry[3] * tR + dm->geometry[4] * tZ;
            tp->line = fabs(tp->l1) + fabs(tp->l2);
            tp->width = area / tp->line;
        }
        tp->slope = -tp->fsOnset * tp->fsOnset * tp->width / (2.0 * dm->fractureEnergy);
        tp->floored = tp->slope < -dm->youngs;
    }
}

/* Reverse of the return map at one point from its tape. In: the adjoints of the outputs
 * (sb[4], bb[4], *epsPb, *workb, and the damage state's *strengthb, *softb). Out: the same
 * arrays hold the adjoints of the inputs; dEb[4] the adjoints of dRR, dZZ, dTT, dGamRZ; dt and
 * parameter adjoints are added to *dtb and pb[]. */
NF_HD void nf_adj_j2_reverse(const nf_adj_j2_tape *tp, const double *bk, double epsP,
                             const nf_adj_mat *f, double strainDt, const nf_adj_damage *dm,
                             double *sb, double *bb, double *epsPb, double *workb,
                             double *strengthb, double *softb, double *dEb, double *dtb,
                             double *pb) {
    const double mu = f->mu, lambda = f->lambda;
    const int jc = f->jc != 0;
    double tb[4] = {0.0, 0.0, 0.0, 0.0};
    if (!tp->plastic) {
        for (int k = 0; k < 4; k++) tb[k] = sb[k];
        /* bb, epsPb, workb and the damage state pass through */
    } else {
        const double *n = tp->n, *x = tp->x;
        const double norm = tp->norm, dGamma = tp->dGamma, inv = 1.0 / norm;
        double nb[4] = {0.0, 0.0, 0.0, 0.0};
        double epsP1b = *epsPb;
        double tempb = 0.0;
        /* adjoints of the pre-step damage state: unchanged by the step unless it begins here */
        double strengthIn = strengthb ? *strengthb : 0.0, softIn = softb ? *softb : 0.0;
        if (tp->onset) {
            strengthIn = 0.0;
            softIn = 0.0;
            /* strength' = fsOnset; softening' = max(slope, -E); width from the band direction */
            double fsb = strengthb ? *strengthb : 0.0;
            double widthb = 0.0;
            if (!tp->floored && softb) {
                const double sb_ = *softb;
                fsb -= sb_ * tp->fsOnset * tp->width / dm->fractureEnergy;
                widthb = -sb_ * tp->fsOnset * tp->fsOnset / (2.0 * dm->fractureEnergy);
                pb[NF_ADJ_P_GF] += sb_ * tp->fsOnset * tp->fsOnset * tp->width
                                   / (2.0 * dm->fractureEnergy * dm->fractureEnergy);
            }
            if (!jc) {                              /* fs = sy0 + H_iso epsP' */
                epsP1b += fsb * f->hIso;
                pb[NF_ADJ_P_SY0] += fsb;
                pb[NF_ADJ_P_HISO] += fsb * tp->epsP1;
            } else {
                const double eps = tp->epsP1;
                const double Th = nf_adj_thermal_term(f, tp->temperature);
                const double S = nf_adj_strain_term(f, eps);
                const double en = eps > 0.0 ? nf_pow(eps, f->n) : 0.0;
                if (eps > 0.0) {
                    epsP1b += fsb * f->b * f->n * en / eps * Th;
                    pb[NF_ADJ_P_B] += fsb * Th * en;
                    pb[NF_ADJ_P_N] += fsb * Th * f->b * en * nf_log(eps);
                }
                pb[NF_ADJ_P_A] += fsb * Th;
                const double h = (tp->temperature - f->room) / (f->melt - f->room);
                if (h > 0.0 && h < 1.0) {
                    const double hm = nf_pow(h, f->m);
                    tempb += fsb * S * (-f->m * hm / h / (f->melt - f->room));
                    pb[NF_ADJ_P_M] += fsb * S * (-hm * nf_log(h));
                }
            }
            if (!tp->isotropic) {
                const double area = dm->geometry[0];
                const double lineb = -widthb * area / (tp->line * tp->line);
                const double l1b = tp->l1 >= 0.0 ? lineb : -lineb;
                const double l2b = tp->l2 >= 0.0 ? lineb : -lineb;
                const double tRb = l1b * dm->geometry[1] + l2b * dm->geometry[3];
                const double tZb = l1b * dm->geometry[2] + l2b * dm->geometry[4];
                const double phib = -tRb * cos(tp->phi) - tZb * sin(tp->phi);
                const double rr = tp->diff * tp->diff + tp->cross * tp->cross;
                const double crossb = 0.5 * phib * tp->diff / rr;
                const double diffb = -0.5 * phib * tp->cross / rr;
                nb[0] += diffb;
                nb[1] -= diffb;
                nb[3] += 2.0 * crossb;
            }
        }
        double dGammab = NF_ADJ_SQRT_2_3 * epsP1b;          /* epsP' = epsP + sqrt(2/3) dG */
        double shiftb = 0.0;                                /* bk' = bk + shift n */
        for (int k = 0; k < 4; k++) {
            shiftb += bb[k] * n[k];
            nb[k] += tp->shift * bb[k];
        }
        pb[NF_ADJ_P_HKIN] += NF_ADJ_TWO_THIRDS * dGamma * shiftb;
        dGammab += NF_ADJ_TWO_THIRDS * f->hKin * shiftb;
        const double q = norm - tp->pull + tp->alphaDotN;  /* work' = work + dG q */
        dGammab += q * (*workb);
        const double qb = dGamma * (*workb);
        double normb = qb, pullb = -qb;
        double bkb[4];
        for (int k = 0; k < 3; k++) {
            bkb[k] = bb[k] + qb * n[k];
            nb[k] += qb * bk[k];
        }
        bkb[3] = bb[3] + 2.0 * qb * n[3];
        nb[3] += 2.0 * qb * bk[3];
        for (int k = 0; k < 4; k++) {                       /* s' = trial - pull n */
            tb[k] = sb[k];
            pullb -= sb[k] * n[k];
            nb[k] -= tp->pull * sb[k];
        }
        dGammab += 2.0 * mu * pullb;
        double xb[4], nn = 0.0;                             /* n = x / norm */
        for (int k = 0; k < 4; k++) {
            xb[k] = nb[k] * inv;
            nn += nb[k] * n[k];
        }
        normb -= nn * inv;
        double stiffb = 0.0, epsPbIn = epsP1b;             /* epsP' = epsP + ... */
        if (!jc || tp->softening) {
            if (tp->fallback) {
                normb += dGammab / tp->stiffness;
                stiffb -= dGammab * dGamma / tp->stiffness;
            } else {
                const double den = tp->stiffness + NF_ADJ_TWO_THIRDS * tp->hardening;
                normb += dGammab / den;
                const double radiusb = -dGammab / den;
                stiffb -= dGammab * dGamma / den;
                const double hardb = -dGammab * dGamma / den * NF_ADJ_TWO_THIRDS;
                const double fsb = NF_ADJ_SQRT_2_3 * radiusb;
                if (tp->softening) {
                    if (!tp->clamped) {
                        softIn += hardb;
                        strengthIn += fsb;
                        softIn += fsb * (epsP - dm->failureStrain);
                        epsPbIn += fsb * dm->softening;
                    }
                } else {                            /* fs = sy0 + H_iso epsP */
                    epsPbIn += fsb * f->hIso;
                    pb[NF_ADJ_P_SY0] += fsb;
                    pb[NF_ADJ_P_HISO] += fsb * epsP + hardb;   /* hardening = H_iso */
                }
            }
        } else {
            const double dEps = NF_ADJ_SQRT_2_3 * dGamma;
            const double eps = epsP + dEps;
            const double rate = strainDt > 0.0 ? dEps / strainDt : 0.0;
            const double S = nf_adj_strain_term(f, eps);
            const double R = nf_adj_rate_term(f, rate);
            const double Th = nf_adj_thermal_term(f, tp->temperature);
            const double en = eps > 0.0 ? nf_pow(eps, f->n) : 0.0;
            const double Sp = eps > 0.0 ? f->b * f->n * en / eps : 0.0;
            const int rated = !(rate <= f->refRate);
            const double Rp = rated ? f->c / rate : 0.0;
            const double h = (tp->temperature - f->room) / (f->melt - f->room);
            const int heated = h > 0.0 && h < 1.0;
            const double hm = heated ? nf_pow(h, f->m) : 0.0;
            const double gdg = -tp->stiffness
                               - NF_ADJ_SQRT_2_3 * (Sp * NF_ADJ_SQRT_2_3 * R * Th
                                                    + S * Rp * (strainDt > 0.0 ? NF_ADJ_SQRT_2_3 / strainDt : 0.0) * Th);
            const double w = -dGammab / gdg;
            normb += w;
            stiffb += w * (-dGamma);
            epsPbIn += w * (-NF_ADJ_SQRT_2_3 * Sp * R * Th);
            if (heated) {
                tempb += w * (-NF_ADJ_SQRT_2_3 * S * R * (-f->m * hm / h / (f->melt - f->room)));
                pb[NF_ADJ_P_M] += w * (-NF_ADJ_SQRT_2_3 * S * R * (-hm * nf_log(h)));
            }
            if (rated && strainDt > 0.0) {
                if (dtb) *dtb += w * (NF_ADJ_SQRT_2_3 * S * Th * f->c / strainDt);
                pb[NF_ADJ_P_C] += w * (-NF_ADJ_SQRT_2_3 * S * Th * nf_log(rate / f->refRate));
            }
            pb[NF_ADJ_P_A] += w * (-NF_ADJ_SQRT_2_3 * R * Th);
            if (eps > 0.0) {
                pb[NF_ADJ_P_B] += w * (-NF_ADJ_SQRT_2_3 * R * Th * en);
                pb[NF_ADJ_P_N] += w * (-NF_ADJ_SQRT_2_3 * R * Th * f->b * en * nf_log(eps));
            }
        }
        pb[NF_ADJ_P_HKIN] += NF_ADJ_TWO_THIRDS * stiffb;
        *workb += f->thermalCoefficient * tempb;
        *epsPb = epsPbIn;
        if (strengthb) *strengthb = strengthIn;
        if (softb) *softb = softIn;
        for (int k = 0; k < 3; k++) xb[k] += normb * x[k] * inv;   /* norm */
        xb[3] += normb * 2.0 * x[3] * inv;
        double pbar = 0.0;                                  /* x = dev(trial) - bk */
        for (int k = 0; k < 3; k++) {
            tb[k] += xb[k];
            pbar -= xb[k];
            bkb[k] -= xb[k];
        }
        tb[3] += xb[3];
        bkb[3] -= xb[3];
        for (int k = 0; k < 3; k++) tb[k] += pbar / 3.0;
        for (int k = 0; k < 4; k++) bb[k] = bkb[k];
    }
    /* trial = s + lt I + 2 mu d (normal), s_rz + mu dGamRZ */
    const double ltb = tb[0] + tb[1] + tb[2];
    dEb[0] = 2.0 * mu * tb[0] + lambda * ltb;
    dEb[1] = 2.0 * mu * tb[1] + lambda * ltb;
    dEb[2] = 2.0 * mu * tb[2] + lambda * ltb;
    dEb[3] = mu * tb[3];
    for (int k = 0; k < 4; k++) sb[k] = tb[k];
}

/* ------------------------------------------------------------------ co-rotation */

/* Reverse of Corotational.rotate (Corotational.java:59-71) applied to t with (c, s): t is the
 * tensor before the rotation, tb the adjoint after it (overwritten with the adjoint before);
 * adds to *ccb, *ssb, *csb the adjoints of c^2, s^2 and c s. */
NF_HD void nf_adj_rotate(const double *t, double *tb, double c, double s, double *ccb,
                         double *ssb, double *csb) {
    const double cc = c * c, ss = s * s, cs = c * s;
    const double rr = t[0], zz = t[1], rz = t[3];
    const double rrb = tb[0], zzb = tb[1], rzb = tb[3];
    tb[0] = cc * rrb + ss * zzb + cs * rzb;
    tb[1] = ss * rrb + cc * zzb - cs * rzb;
    tb[3] = -2.0 * cs * rrb + 2.0 * cs * zzb + (cc - ss) * rzb;
    *ccb += rr * rrb + zz * zzb + rz * rzb;
    *ssb += zz * rrb + rr * zzb - rz * rzb;
    *csb += -2.0 * rz * rrb + 2.0 * rz * zzb + (rr - zz) * rzb;
}

NF_HD void nf_adj_rotate_forward(double *t, double c, double sn) {
    const double rr = t[0], zz = t[1], rz = t[3];
    const double cc = c * c, ss = sn * sn, cs = c * sn;
    t[0] = cc * rr - 2.0 * cs * rz + ss * zz;
    t[1] = ss * rr + 2.0 * cs * rz + cc * zz;
    t[3] = cs * (rr - zz) + (cc - ss) * rz;
}

/* ------------------------------------------------------------------ one element */

/* Inputs of one reduced element in one step (the post-nodal state of its four nodes). */
typedef struct {
    double x0r[4], x0z[4];       /* reference coordinates */
    double ur[4], uz[4];         /* displacements after this step's nodal update */
    double vr[4], vz[4];         /* velocities after this step's nodal update */
    double sig[4], back[4];      /* point state before the step */
    double epsP, work;
    double hgR, hgZ;             /* hourglass force before the step */
    int damaged;                 /* the element has damage state (dm below) */
    nf_adj_damage dm;
} nf_adj_elem_in;

/* Adjoints flowing into and out of one element. In: g[8] (adjoints of the contribution
 * slots: radial for corners 0-3, then axial), sig/back/epsP/work/hgR/hgZ (adjoints of the
 * state after the step), edgeOwner (which of the edges 0-1, 1-2, 2-3, 3-0 is this step's
 * shortest, or -1) with edgeb (the adjoint of its squared length). Out: the adjoints of the
 * state before the step (overwritten), ur..vz (adjoints of the nodal inputs), dt and
 * parameters added to *dtb and pb[]. */
typedef struct {
    double g[8];
    double sig[4], back[4], epsP, work, hgR, hgZ;
    double strength, softening;  /* the damage state's */
    int edgeOwner;
    double edgeb;
    double ur[4], uz[4], vr[4], vz[4];
} nf_adj_elem_bar;

/* Reverse of reducedIntegration (ExplicitSolver.java:1373-1504) for one element. */
NF_HD void nf_adj_element_reduced(const nf_adj_elem_in *in, const nf_adj_mat *f, double dt,
                                  int axi, int finite, double thickness, double hourglass,
                                  nf_adj_elem_bar *ab, double *dtb, double *pb) {
    const double mu = f->mu;
    const double mid = -0.5 * dt;
    double r[4], z[4], a[4], c[4];
    for (int k = 0; k < 4; k++) {
        if (finite) {
            r[k] = in->x0r[k] + in->ur[k] + mid * in->vr[k];
            z[k] = in->x0z[k] + in->uz[k] + mid * in->vz[k];
        } else {
            r[k] = in->x0r[k];
            z[k] = in->x0z[k];
        }
        a[k] = in->vr[k] * dt;
        c[k] = in->vz[k] * dt;
    }
    const double J00 = 0.25 * (-r[0] + r[1] + r[2] - r[3]);
    const double J01 = 0.25 * (-z[0] + z[1] + z[2] - z[3]);
    const double J10 = 0.25 * (-r[0] - r[1] + r[2] + r[3]);
    const double J11 = 0.25 * (-z[0] - z[1] + z[2] + z[3]);
    const double det = J00 * J11 - J01 * J10;
    const double inv = 1.0 / det;
    double dr[4], dz[4];
    dr[0] = 0.25 * (J01 - J11) * inv;
    dr[1] = 0.25 * (J01 + J11) * inv;
    dr[2] = -dr[0];
    dr[3] = -dr[1];
    dz[0] = 0.25 * (J10 - J00) * inv;
    dz[1] = -0.25 * (J10 + J00) * inv;
    dz[2] = -dz[0];
    dz[3] = -dz[1];
    const double dEpsR = dr[0] * a[0] + dr[1] * a[1] + dr[2] * a[2] + dr[3] * a[3];
    const double dEpsZ = dz[0] * c[0] + dz[1] * c[1] + dz[2] * c[2] + dz[3] * c[3];
    const double dRdZ = dz[0] * a[0] + dz[1] * a[1] + dz[2] * a[2] + dz[3] * a[3];
    const double dZdR = dr[0] * c[0] + dr[1] * c[1] + dr[2] * c[2] + dr[3] * c[3];
    const double dGamRZ = dRdZ + dZdR;
    double rg = 0.0, dEpsT = 0.0;
    if (axi) {
        rg = 0.25 * (r[0] + r[1] + r[2] + r[3]);
        dEpsT = 0.25 * (a[0] + a[1] + a[2] + a[3]) / rg;
    }
    /* co-rotation (the forward skips it at zero spin; the derivative is taken there too) */
    double s1[4], b1[4];
    for (int k = 0; k < 4; k++) {
        s1[k] = in->sig[k];
        b1[k] = in->back[k];
    }
    const double spinDt = finite ? 0.5 * (dZdR - dRdZ) : 0.0;
    const double hh = 0.5 * spinDt, q1 = 1.0 + hh * hh;
    const double cs = (1.0 - hh * hh) / q1, sn = 2.0 * hh / q1;
    if (finite && spinDt != 0.0) {
        nf_adj_rotate_forward(s1, cs, sn);
        nf_adj_rotate_forward(b1, cs, sn);
    }
    /* the return map, forward (taped), for the stress the forces use */
    double s2[4], b2[4];
    nf_adj_j2_tape tp;
    const nf_adj_damage *dm = in->damaged ? &in->dm : 0;
    nf_adj_j2_forward(s1, b1, in->epsP, in->work, dEpsR, dEpsZ, dEpsT, dGamRZ, f, dt, dm, &tp, s2,
                      b2);
    const double sR = s2[0], sZ = s2[1], sT = s2[2], sRZ = s2[3];
    const double vol = axi ? 2.0 * NF_PI * rg * det : thickness * det;
    const double dV = 4.0 * vol;

    /* ---------------- reverse ---------------- */
    double rb[4] = {0, 0, 0, 0}, zb[4] = {0, 0, 0, 0}, ab_[4] = {0, 0, 0, 0}, cb[4] = {0, 0, 0, 0};
    double drb[4] = {0, 0, 0, 0}, dzb[4] = {0, 0, 0, 0};
    double dVb = 0.0, rgb = 0.0, detb = 0.0;
    double sRb = ab->sig[0], sZb = ab->sig[1], sTb = ab->sig[2], sRZb = ab->sig[3];
    const double *grb = ab->g, *gzb = ab->g + 4;
    /* hourglass: hg' = hg + k (y.a, y.c); g -= y hg' */
    double hgRb = ab->hgR, hgZb = ab->hgZ;
    if (hourglass > 0.0) {
        const double hr = r[0] - r[1] + r[2] - r[3];
        const double hz = z[0] - z[1] + z[2] - z[3];
        double y[4];
        y[0] = 1.0 - hr * dr[0] - hz * dz[0];
        y[1] = -1.0 - hr * dr[1] - hz * dz[1];
        y[2] = 1.0 - hr * dr[2] - hz * dz[2];
        y[3] = -1.0 - hr * dr[3] - hz * dz[3];
        const double sb = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2] + dr[3] * dr[3]
                          + dz[0] * dz[0] + dz[1] * dz[1] + dz[2] * dz[2] + dz[3] * dz[3];
        const double k = hourglass * mu * dV * sb;
        const double sa = y[0] * a[0] + y[1] * a[1] + y[2] * a[2] + y[3] * a[3];
        const double sc = y[0] * c[0] + y[1] * c[1] + y[2] * c[2] + y[3] * c[3];
        const double h2r = in->hgR + k * sa, h2z = in->hgZ + k * sc;
        double yb[4];
        for (int j = 0; j < 4; j++) {
            yb[j] = -grb[j] * h2r - gzb[j] * h2z;
            hgRb -= y[j] * grb[j];
            hgZb -= y[j] * gzb[j];
        }
        /* h2 = hg + k s: */
        const double kb = hgRb * sa + hgZb * sc;
        for (int j = 0; j < 4; j++) {
            yb[j] += k * (hgRb * a[j] + hgZb * c[j]);
            ab_[j] += k * hgRb * y[j];
            cb[j] += k * hgZb * y[j];
        }
        /* k = q mu dV sb */
        dVb += kb * hourglass * mu * sb;
        const double sbb = kb * hourglass * mu * dV;
        for (int j = 0; j < 4; j++) {
            drb[j] += 2.0 * dr[j] * sbb;
            dzb[j] += 2.0 * dz[j] * sbb;
        }
        /* y */
        double hrb = 0.0, hzb = 0.0;
        for (int j = 0; j < 4; j++) {
            hrb -= yb[j] * dr[j];
            hzb -= yb[j] * dz[j];
            drb[j] -= yb[j] * hr;
            dzb[j] -= yb[j] * hz;
        }
        rb[0] += hrb; rb[1] -= hrb; rb[2] += hrb; rb[3] -= hrb;
        zb[0] += hzb; zb[1] -= hzb; zb[2] += hzb; zb[3] -= hzb;
    }
    ab->hgR = hgRb;     /* adjoint of the hourglass force before the step */
    ab->hgZ = hgZb;
    /* forces */
    double hqb = 0.0;
    for (int j = 0; j < 4; j++) {
        const double tr = dr[j] * sR + dz[j] * sRZ;
        const double trb = -grb[j] * dV;
        dVb -= grb[j] * tr;
        if (axi) hqb -= grb[j];
        drb[j] += trb * sR;
        sRb += trb * dr[j];
        dzb[j] += trb * sRZ;
        sRZb += trb * dz[j];
        const double tz = dz[j] * sZ + dr[j] * sRZ;
        const double tzb = -gzb[j] * dV;
        dVb -= gzb[j] * tz;
        dzb[j] += tzb * sZ;
        sZb += tzb * dz[j];
        drb[j] += tzb * sRZ;
        sRZb += tzb * dr[j];
    }
    if (axi) {
        sTb += hqb * dV * 0.25 / rg;
        rgb -= hqb * sT * dV * 0.25 / (rg * rg);
        dVb += hqb * sT / rg * 0.25;
        rgb += dVb * 4.0 * 2.0 * NF_PI * det;
        detb += dVb * 4.0 * 2.0 * NF_PI * rg;
    } else {
        detb += dVb * 4.0 * thickness;
    }
    /* the return map */
    double sb4[4] = {sRb, sZb, sTb, sRZb};
    double bb4[4] = {ab->back[0], ab->back[1], ab->back[2], ab->back[3]};
    double epsPb = ab->epsP, workb = ab->work;
    double dEb[4];
    nf_adj_j2_reverse(&tp, b1, in->epsP, f, dt, dm, sb4, bb4, &epsPb, &workb,
                      dm ? &ab->strength : 0, dm ? &ab->softening : 0, dEb, dtb, pb);
    ab->epsP = epsPb;
    ab->work = workb;
    double dEpsRb = dEb[0], dEpsZb = dEb[1], dEpsTb = dEb[2], dGamRZb = dEb[3];
    /* co-rotation */
    double spinb = 0.0;
    if (finite) {
        double ccb = 0.0, ssb = 0.0, csb = 0.0;
        nf_adj_rotate(in->sig, sb4, cs, sn, &ccb, &ssb, &csb);
        nf_adj_rotate(in->back, bb4, cs, sn, &ccb, &ssb, &csb);
        const double cb_ = 2.0 * cs * ccb + sn * csb;
        const double snb = 2.0 * sn * ssb + cs * csb;
        const double dcdh = -4.0 * hh / (q1 * q1);
        const double dsdh = 2.0 * (1.0 - hh * hh) / (q1 * q1);
        spinb = 0.5 * (cb_ * dcdh + snb * dsdh);
    }
    for (int k = 0; k < 4; k++) {
        ab->sig[k] = sb4[k];
        ab->back[k] = bb4[k];
    }
    const double dZdRb = dGamRZb + 0.5 * spinb;
    const double dRdZb = dGamRZb - 0.5 * spinb;
    /* rg, dEpsT */
    if (axi) {
        for (int k = 0; k < 4; k++) ab_[k] += 0.25 * dEpsTb / rg;
        rgb -= dEpsTb * dEpsT / rg;
        for (int k = 0; k < 4; k++) rb[k] += 0.25 * rgb;
    }
    /* strain increments */
    for (int k = 0; k < 4; k++) {
        drb[k] += dEpsRb * a[k] + dZdRb * c[k];
        dzb[k] += dEpsZb * c[k] + dRdZb * a[k];
        ab_[k] += dEpsRb * dr[k] + dRdZb * dz[k];
        cb[k] += dEpsZb * dz[k] + dZdRb * dr[k];
    }
    /* B from the Jacobian */
    const double d0r = drb[0] - drb[2], d1r = drb[1] - drb[3];
    const double d0z = dzb[0] - dzb[2], d1z = dzb[1] - dzb[3];
    double J00b = 0.0, J01b = 0.0, J10b = 0.0, J11b = 0.0, invb = 0.0;
    J01b += 0.25 * inv * d0r; J11b -= 0.25 * inv * d0r; invb += 0.25 * (J01 - J11) * d0r;
    J01b += 0.25 * inv * d1r; J11b += 0.25 * inv * d1r; invb += 0.25 * (J01 + J11) * d1r;
    J10b += 0.25 * inv * d0z; J00b -= 0.25 * inv * d0z; invb += 0.25 * (J10 - J00) * d0z;
    J10b -= 0.25 * inv * d1z; J00b -= 0.25 * inv * d1z; invb -= 0.25 * (J10 + J00) * d1z;
    detb -= inv * inv * invb;
    J00b += detb * J11; J11b += detb * J00; J01b -= detb * J10; J10b -= detb * J01;
    rb[0] += 0.25 * (-J00b - J10b); rb[1] += 0.25 * (J00b - J10b);
    rb[2] += 0.25 * (J00b + J10b);  rb[3] += 0.25 * (-J00b + J10b);
    zb[0] += 0.25 * (-J01b - J11b); zb[1] += 0.25 * (J01b - J11b);
    zb[2] += 0.25 * (J01b + J11b);  zb[3] += 0.25 * (-J01b + J11b);
    /* the shortest edge (the CFL step of the next step) */
    if (finite && ab->edgeOwner >= 0) {
        const int i = ab->edgeOwner, j = (ab->edgeOwner + 1) & 3;
        const double er = r[j] - r[i], ez = z[j] - z[i];
        rb[j] += 2.0 * er * ab->edgeb; rb[i] -= 2.0 * er * ab->edgeb;
        zb[j] += 2.0 * ez * ab->edgeb; zb[i] -= 2.0 * ez * ab->edgeb;
    }
    /* a = v dt, c = v dt; r = x0 + u + mid v */
    double dtAcc = 0.0, midb = 0.0;
    for (int k = 0; k < 4; k++) {
        ab->vr[k] = ab_[k] * dt;
        ab->vz[k] = cb[k] * dt;
        dtAcc += ab_[k] * in->vr[k] + cb[k] * in->vz[k];
        if (finite) {
            ab->ur[k] = rb[k];
            ab->uz[k] = zb[k];
            ab->vr[k] += mid * rb[k];
            ab->vz[k] += mid * zb[k];
            midb += in->vr[k] * rb[k] + in->vz[k] * zb[k];
        } else {
            ab->ur[k] = 0.0;
            ab->uz[k] = 0.0;
        }
    }
    if (dtb) *dtb += dtAcc - 0.5 * midb;
}

/* The squared edges of an element in the forward order (shortestEdge, :1191-1197): which edge
 * (0..3) attains `value` first in jmin's order, or -1. */
NF_HD int nf_adj_edge_owner(const nf_adj_elem_in *in, double dt, int finite, double value) {
    if (!finite) return -1;
    const double mid = -0.5 * dt;
    double r[4], z[4];
    for (int k = 0; k < 4; k++) {
        r[k] = in->x0r[k] + in->ur[k] + mid * in->vr[k];
        z[k] = in->x0z[k] + in->uz[k] + mid * in->vz[k];
    }
    for (int k = 0; k < 4; k++) {
        const int j = (k + 1) & 3;
        const double dr = r[j] - r[k], dz = z[j] - z[k];
        if (dr * dr + dz * dz == value) return k;
    }
    return -1;
}

/* ------------------------------------------------------------------ pressure edge */

/* Reverse of applyPressure + pressureAt (ExplicitSolver.java:1203-1207, :1511-1556) for one
 * edge (a, b) at time t (after this step's time advance). cb[4]: adjoints of its slots
 * (radial at a, radial at b, axial at a, axial at b). Out: ab[2], bb[2] the adjoints of the
 * edge nodes' displacements (r, z) after the nodal update; the time adjoint added to *tb. */
NF_HD void nf_adj_pressure_edge(double xar, double xaz, double xbr, double xbz, double uar,
                                double uaz, double ubr, double ubz, double t, double target,
                                double rampDuration, int axi, int finite, double thickness,
                                const double *cb, double *ab, double *bb, double *tb) {
    double p = target, dpdt = 0.0;
    if (rampDuration > 0.0) {
        const double s = t / rampDuration < 1.0 ? t / rampDuration : 1.0;
        p = target * s * s * (3.0 - 2.0 * s);
        if (t / rampDuration < 1.0) dpdt = target * (6.0 * s - 6.0 * s * s) / rampDuration;
    }
    double ra = xar, rb = xbr, za = xaz, zb = xbz;
    if (finite) {
        ra = xar + uar; rb = xbr + ubr; za = xaz + uaz; zb = xbz + ubz;
    }
    const double tr = rb - ra, tz = zb - za;
    const double len = sqrt(tr * tr + tz * tz);
    ab[0] = ab[1] = bb[0] = bb[1] = 0.0;
    if (len == 0.0) return;
    const double nr = tz / len, nz = -tr / len;
    double wa, wb;
    if (axi) {
        const double circ = 2.0 * NF_PI * len;
        wa = circ * (ra / 3.0 + rb / 6.0);
        wb = circ * (ra / 6.0 + rb / 3.0);
    } else {
        wa = thickness * len * 0.5;
        wb = wa;
    }
    /* c0 = p nr wa, c1 = p nr wb, c4 = p nz wa, c5 = p nz wb */
    const double pb_ = cb[0] * nr * wa + cb[1] * nr * wb + cb[2] * nz * wa + cb[3] * nz * wb;
    const double nrb = cb[0] * p * wa + cb[1] * p * wb;
    const double nzb = cb[2] * p * wa + cb[3] * p * wb;
    const double wab = cb[0] * p * nr + cb[2] * p * nz;
    const double wbb = cb[1] * p * nr + cb[3] * p * nz;
    double lenb = 0.0, rab = 0.0, rbb = 0.0;
    if (axi) {
        const double circ = 2.0 * NF_PI * len;
        const double circb = wab * (ra / 3.0 + rb / 6.0) + wbb * (ra / 6.0 + rb / 3.0);
        rab += circ * (wab / 3.0 + wbb / 6.0);
        rbb += circ * (wab / 6.0 + wbb / 3.0);
        lenb += 2.0 * NF_PI * circb;
    } else {
        lenb += thickness * 0.5 * (wab + wbb);
    }
    double tzb = nrb / len, trb = -nzb / len;
    lenb += -nrb * tz / (len * len) + nzb * tr / (len * len);
    trb += lenb * tr / len;
    tzb += lenb * tz / len;
    rbb += trb; rab -= trb;
    const double zbb = tzb, zab = -tzb;
    if (finite) {
        ab[0] = rab; ab[1] = zab;
        bb[0] = rbb; bb[1] = zbb;
    }
    if (tb) *tb += pb_ * dpdt;
}

/* ------------------------------------------------------------------ one node */

enum { NF_ADJ_FREE = 0, NF_ADJ_FIXED, NF_ADJ_STUCK, NF_ADJ_SLID, NF_ADJ_HELD, NF_ADJ_ARRIVED };

/* Reverse of one node's nodalUpdate (ExplicitSolver.java:998-1062) with the wall branches.
 * In: the node's state before the step, the step's coefficients, and ub/vb (adjoints of the
 * displacement and velocity after the step). Out: ub, vb, fb = adjoints before the step; the
 * adjoints of decay, gain, dt and the friction coefficient are added to acc[0..3]. */
NF_HD void nf_adj_node(double x0z, double ur, double uz, double vr, double vz, double fr,
                       double fz, double m, double invM, int fixedR, int fixedZ, int onWall,
                       int hasWall, double plane, double friction, double decay, double gain,
                       double dt, double *ub, double *vb, double *fb, double *acc) {
    const int resting = hasWall && onWall && fz <= 0.0;
    double urb = ub[0], uzb = ub[1], vrb = vb[0], vzb = vb[1];
    double frb = 0.0, fzb = 0.0;
    /* radial */
    if (fixedR) {
        vrb = 0.0;
    } else if (resting && friction > 0.0) {
        const double normal = -fz;
        const double trial = -m * decay * vr / gain - fr;
        const double limit = isinf(friction) ? INFINITY : friction * normal;
        if (fabs(trial) <= limit) {
            vrb = 0.0;                           /* stuck: v = 0, u unchanged */
        } else {
            const double sgn = trial < 0.0 ? -1.0 : 1.0;
            const double tangential = copysign(limit, trial);
            const double slid = decay * vr + gain * (fr + tangential) / m;
            const double slidb = vrb + dt * urb;
            acc[2] += slid * urb;
            acc[0] += vr * slidb;
            acc[1] += (fr + tangential) / m * slidb;
            vrb = decay * slidb;
            frb += gain / m * slidb;
            const double tb = gain / m * slidb;
            acc[3] += sgn * normal * tb;
            fzb += -sgn * friction * tb;
        }
    } else {
        const double vn = decay * vr + gain * fr * invM;
        const double vnb = vrb + dt * urb;
        acc[2] += vn * urb;
        acc[0] += vr * vnb;
        acc[1] += fr * invM * vnb;
        vrb = decay * vnb;
        frb += gain * invM * vnb;
    }
    /* axial */
    if (fixedZ) {
        vzb = 0.0;
    } else if (resting) {
        /* held: unchanged */
    } else {
        const double trial = decay * vz + gain * fz * invM;
        const double zc = x0z + uz;
        if (hasWall && zc + trial * dt < plane) {
            uzb = 0.0;                           /* arrived: u = plane - x0, v = 0 */
            vzb = 0.0;
        } else {
            const double tb = vzb + dt * uzb;
            acc[2] += trial * uzb;
            acc[0] += vz * tb;
            acc[1] += fz * invM * tb;
            vzb = decay * tb;
            fzb += gain * invM * tb;
        }
    }
    ub[0] = urb;
    ub[1] = uzb;
    vb[0] = vrb;
    vb[1] = vzb;
    fb[0] = frb;
    fb[1] = fzb;
}

/* dtAvg = (dtPrevious + dt) / 2 feeds decay and gain (:947-956): the adjoint of dtAvg. */
NF_HD double nf_adj_dtavg(double decayb, double gainb, double dtAvg, double damping) {
    const double h = 0.5 * damping * dtAvg;
    const double dh = 0.5 * damping;
    const double ddecay = -2.0 / ((1.0 + h) * (1.0 + h)) * dh;
    const double dgain = 1.0 / (1.0 + h) - dtAvg * dh / ((1.0 + h) * (1.0 + h));
    return decayb * ddecay + gainb * dgain;
}

#endif /* NF_ADJOINT_H */
