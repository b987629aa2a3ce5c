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
 * hardening modulus and the wall friction coefficient.
 *
 * Plain C (C99) with NF_HD qualifiers, so the oracle (gcc) and the kernels (nvcc) compile the
 * same text; both build with contraction off.
 */
#ifndef NF_ADJOINT_H
#define NF_ADJOINT_H

#include "nf_math.h"

enum { NF_ADJ_P_A = 0, NF_ADJ_P_B, NF_ADJ_P_N, NF_ADJ_P_C, NF_ADJ_P_M, NF_ADJ_P_HKIN,
       NF_ADJ_P_MU, NF_ADJ_P_COUNT };

#define NF_ADJ_SQRT_2_3 0x1.a20bd700c2c3ep-1
#define NF_ADJ_TWO_THIRDS (2.0 / 3.0)
#define NF_ADJ_TOLERANCE 1.0e-10
#define NF_ADJ_ITERATIONS 25

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

/* J2.solve, J2.java:332-375, in the forward kernels' order. */
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

/* Reverse of J2.update (J2.java:163-296, no damage) at one point. In: the rotated stress s[4]
 * and back stress bk[4] ({rr, zz, tt, rz}), epsP, work, the strain increments, strainDt, and
 * the adjoints of the outputs (sb, bb, epsPb, workb). Out (overwriting the same arrays):
 * the adjoints of the inputs; *dEb receives the adjoints of dRR, dZZ, dTT, dGamRZ; dt and
 * parameter adjoints are added to *dtb and pb[]. */
NF_HD void nf_adj_j2(const double *s, const double *bk, double epsP, double work, double dRR,
                     double dZZ, double dTT, double dGamRZ, const nf_adj_mat *f, double strainDt,
                     double *sb, double *bb, double *epsPb, double *workb, double *dEb,
                     double *dtb, double *pb) {
    const double lambda = f->lambda, mu = f->mu;
    const double lt = lambda * (dRR + dZZ + dTT);
    const double tRR = s[0] + lt + 2.0 * mu * dRR;
    const double tZZ = s[1] + lt + 2.0 * mu * dZZ;
    const double tTT = s[2] + lt + 2.0 * mu * dTT;
    const double tRZ = s[3] + mu * dGamRZ;
    const double p = (tRR + tZZ + tTT) / 3.0;
    const double x[4] = {tRR - p - bk[0], tZZ - p - bk[1], tTT - p - bk[2], tRZ - bk[3]};
    const double norm = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + 2.0 * x[3] * x[3]);
    const int jc = f->jc != 0;
    const double temperature = !jc ? 0.0 : f->room + f->thermalCoefficient * work;
    double flowStress;
    if (!jc) flowStress = f->sy0 + f->hIso * epsP;
    else flowStress = nf_adj_strain_term(f, epsP) * nf_adj_thermal_term(f, temperature);
    const double radius = NF_ADJ_SQRT_2_3 * flowStress;

    double tb[4] = {0.0, 0.0, 0.0, 0.0};      /* adjoint of the trial stress */
    if (!(norm > radius)) {                    /* elastic: s' = trial, the rest unchanged */
        for (int k = 0; k < 4; k++) tb[k] = sb[k];
    } else {
        const double stiffness = 2.0 * mu + NF_ADJ_TWO_THIRDS * f->hKin;
        double dGamma;
        if (!jc) dGamma = (norm - radius) / (stiffness + NF_ADJ_TWO_THIRDS * f->hIso);
        else dGamma = nf_adj_solve(norm, stiffness, epsP, temperature, strainDt, f);
        const double inv = 1.0 / norm;
        const double n[4] = {x[0] * inv, x[1] * inv, x[2] * inv, x[3] * inv};
        const double pull = 2.0 * mu * dGamma;
        const double alphaDotN = bk[0] * n[0] + bk[1] * n[1] + bk[2] * n[2] + 2.0 * bk[3] * n[3];
        const double shift = NF_ADJ_TWO_THIRDS * f->hKin * dGamma;

        double nb[4] = {0.0, 0.0, 0.0, 0.0};
        double dGammab = NF_ADJ_SQRT_2_3 * (*epsPb);          /* epsP' = epsP + sqrt(2/3) dG */
        /* bk' = bk + shift n */
        double shiftb = 0.0;
        for (int k = 0; k < 4; k++) {
            shiftb += bb[k] * n[k];
            nb[k] += shift * bb[k];
        }
        pb[NF_ADJ_P_HKIN] += NF_ADJ_TWO_THIRDS * dGamma * shiftb;
        dGammab += NF_ADJ_TWO_THIRDS * f->hKin * shiftb;
        /* work' = work + dG (norm - pull + alphaDotN) */
        const double q = norm - pull + alphaDotN;
        dGammab += q * (*workb);
        const double qb = dGamma * (*workb);
        double normb = qb, pullb = -qb;
        const double adnb = qb;
        double bkb[4];
        for (int k = 0; k < 3; k++) {
            bkb[k] = bb[k] + adnb * n[k];
            nb[k] += adnb * bk[k];
        }
        bkb[3] = bb[3] + 2.0 * adnb * n[3];
        nb[3] += 2.0 * adnb * bk[3];
        /* s' = trial - pull n */
        for (int k = 0; k < 4; k++) {
            tb[k] = sb[k];
            pullb -= sb[k] * n[k];
            nb[k] -= pull * sb[k];
        }
        dGammab += 2.0 * mu * pullb;
        /* n = x / norm */
        double xb[4];
        double nn = 0.0;
        for (int k = 0; k < 4; k++) {
            xb[k] = nb[k] * inv;
            nn += nb[k] * n[k];
        }
        normb -= nn * inv;
        /* dGamma(norm, stiffness, epsP, temperature, dt, parameters) */
        double stiffb = 0.0, epsPbIn = *epsPb, tempb = 0.0;
        if (!jc) {
            const double den = stiffness + NF_ADJ_TWO_THIRDS * f->hIso;
            normb += dGammab / den;
            const double radiusb = -dGammab / den;
            stiffb -= dGammab * dGamma / den;
            epsPbIn += NF_ADJ_SQRT_2_3 * f->hIso * radiusb;
        } else {
            const double dEps = NF_ADJ_SQRT_2_3 * dGamma;
            const double eps = epsP + dEps;
            const double rate = strainDt > 0.0 ? dEps / strainDt : 0.0;
            const double S = nf_adj_strain_term(f, eps);
            const double R = nf_adj_rate_term(f, rate);
            const double Th = nf_adj_thermal_term(f, temperature);
            const double en = eps > 0.0 ? nf_pow(eps, f->n) : 0.0;
            const double Sp = eps > 0.0 ? f->b * f->n * en / eps : 0.0;       /* dS/deps */
            const int rated = !(rate <= f->refRate);
            const double Rp = rated ? f->c / rate : 0.0;                      /* dR/drate */
            const double h = (temperature - f->room) / (f->melt - f->room);
            const int heated = h > 0.0 && h < 1.0;
            const double hm = heated ? nf_pow(h, f->m) : 0.0;
            const double gdg = -stiffness
                               - NF_ADJ_SQRT_2_3 * (Sp * NF_ADJ_SQRT_2_3 * R * Th
                                                    + S * Rp * (strainDt > 0.0 ? NF_ADJ_SQRT_2_3 / strainDt : 0.0) * Th);
            const double w = -dGammab / gdg;                                  /* dG = -g_x dx / g_dG */
            normb += w;
            stiffb += w * (-dGamma);
            epsPbIn += w * (-NF_ADJ_SQRT_2_3 * Sp * R * Th);
            if (heated) {
                const double dThdT = -f->m * hm / h / (f->melt - f->room);
                tempb += w * (-NF_ADJ_SQRT_2_3 * S * R * dThdT);
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
        /* norm = sqrt(x . x with 2 rz^2) */
        for (int k = 0; k < 3; k++) xb[k] += normb * x[k] * inv;
        xb[3] += normb * 2.0 * x[3] * inv;
        /* x = dev(trial) - bk */
        double pbar = 0.0;
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
    if (!(norm > radius)) {
        /* elastic: bb, epsPb, workb pass through unchanged */
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
    /* the return map, forward, for the stress the forces use */
    double s2[4];
    {
        const double lambda = f->lambda;
        const double lt = lambda * (dEpsR + dEpsZ + dEpsT);
        const double tRR = s1[0] + lt + 2.0 * mu * dEpsR;
        const double tZZ = s1[1] + lt + 2.0 * mu * dEpsZ;
        const double tTT = s1[2] + lt + 2.0 * mu * dEpsT;
        const double tRZ = s1[3] + mu * dGamRZ;
        const double p = (tRR + tZZ + tTT) / 3.0;
        const double xRR = tRR - p - b1[0], xZZ = tZZ - p - b1[1], xTT = tTT - p - b1[2];
        const double xRZ = tRZ - b1[3];
        const double norm = sqrt(xRR * xRR + xZZ * xZZ + xTT * xTT + 2.0 * xRZ * xRZ);
        const int jc = f->jc != 0;
        const double temperature = !jc ? 0.0 : f->room + f->thermalCoefficient * in->work;
        const double flowStress = !jc ? f->sy0 + f->hIso * in->epsP
                                      : nf_adj_strain_term(f, in->epsP) * nf_adj_thermal_term(f, temperature);
        const double radius = NF_ADJ_SQRT_2_3 * flowStress;
        if (!(norm > radius)) {
            s2[0] = tRR; s2[1] = tZZ; s2[2] = tTT; s2[3] = tRZ;
        } else {
            const double stiffness = 2.0 * mu + NF_ADJ_TWO_THIRDS * f->hKin;
            const double dGamma = !jc ? (norm - radius) / (stiffness + NF_ADJ_TWO_THIRDS * f->hIso)
                                      : nf_adj_solve(norm, stiffness, in->epsP, temperature, dt, f);
            const double iv = 1.0 / norm;
            const double pull = 2.0 * mu * dGamma;
            s2[0] = tRR - pull * (xRR * iv);
            s2[1] = tZZ - pull * (xZZ * iv);
            s2[2] = tTT - pull * (xTT * iv);
            s2[3] = tRZ - pull * (xRZ * iv);
        }
    }
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
    nf_adj_j2(s1, b1, in->epsP, in->work, dEpsR, dEpsZ, dEpsT, dGamRZ, f, dt, sb4, bb4, &epsPb,
              &workb, dEb, dtb, pb);
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
