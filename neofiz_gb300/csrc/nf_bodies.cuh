// nf_bodies.cuh -- the per-node and per-element arithmetic of the timestep, shared by the
// single-scene kernels (k_step.cu, k_mixed.cu) and the batched kernel (k_batch.cu). One copy
// of each body means a batched instance computes exactly what a single scene does.
#pragma once

#include "nf_internal.h"
#include "nf_fpconv.h"

namespace nf {

// One node of nodalUpdate, ExplicitSolver.java:998-1062, with RigidWall.hold/crosses/arrive/
// slide (RigidWall.java:163-259): shared by the single-scene kernel and the batched one. Adds
// the node's wall terms to impulse/loss/fric. When geo.pMid is set (the mixed form) it also
// writes the FP32 geometry of the coming assembly: mid-step and current positions as float
// pairs (hi, lo) and v dt, at index geo.base + i.
struct NodalCoef {
    double decay, gain, dtAvg, dt;
};
struct WallRef {
    int present;
    double plane, friction;
    int *contact, *stuck;
};
struct MixedGeo {
    float4 *pMid, *pCur;
    float2 *vdt;
    int base;
};

static __device__ __forceinline__ void nodal_node(const Dev &d, int i, const NodalCoef &co,
                                                  const WallRef &w, const MixedGeo &geo,
                                                  uint32_t *status, double &impulse,
                                                  double &loss, double &fric) {
    const double decay = co.decay, gain = co.gain, dtAvg = co.dtAvg, dt = co.dt;
    uint8_t fl = d.flags[i];
    const bool fixedR = fl & 1, fixedZ = fl & 2;
    bool onWall = fl & 4;
    double2 u = d.U[i], v = d.V[i];
    const double2 f = d.F[i];
    const double m = d.mass[i];
    const double invM = d.invMass[i];
    const bool resting = w.present && onWall && f.y <= 0.0;
    uint8_t ws = 0;
    if (fixedR) {
        v.x = 0.0;
    } else if (resting && w.friction > 0.0) {
        // RigidWall.slide, RigidWall.java:236-259
        const double normal = -f.y;
        const double trial = -m * decay * v.x / gain - f.x;
        const double limit = isinf(w.friction) ? INFINITY : w.friction * normal;
        if (fabs(trial) <= limit) {
            loss += 0.5 * m * v.x * v.x;
            atomicAdd(w.stuck, 1);
            ws |= NF_WALL_STUCK;
            v.x = 0.0;
        } else {
            const double tangential = copysign(limit, trial);
            const double slid = decay * v.x + gain * (f.x + tangential) / m;
            fric += -tangential * slid * dt;
            ws |= NF_WALL_SLID;
            v.x = slid;
        }
        u.x += v.x * dt;
    } else {
        v.x = decay * v.x + gain * f.x * invM;
        u.x += v.x * dt;
    }
    const double2 x0 = d.X0[i];
    if (fixedZ) {
        v.y = 0.0;
    } else if (resting) {
        impulse += -f.y * dtAvg;                         // RigidWall.hold :178-181
        atomicAdd(w.contact, 1);
        ws |= NF_WALL_HELD;
    } else {
        const double trial = decay * v.y + gain * f.y * invM;
        const double zc = x0.y + u.y;
        if (w.present && zc + trial * dt < w.plane) {
            impulse += -m * trial;                       // RigidWall.arrive :205-209
            loss += 0.5 * m * trial * trial;
            atomicAdd(w.contact, 1);
            u.y += w.plane - zc;
            v.y = 0.0;
            onWall = true;
            ws |= NF_WALL_ARRIVED;
        } else {
            v.y = trial;
            u.y += v.y * dt;
            if (w.present) onWall = false;
        }
    }
    d.U[i] = u;
    d.V[i] = v;
    if (w.present) {
        d.flags[i] = (uint8_t)((fl & 3) | (onWall ? 4 : 0));
        d.wallState[i] = ws;
    }
    if (!(finite_bits(u.x) && finite_bits(u.y) && finite_bits(v.x) && finite_bits(v.y)))
        atomicOr(status, STATUS_NONFINITE);
    if (geo.pMid) {
        // the geometry of the coming assembly: mid-step and current positions as float
        // pairs, and v dt (see k_prepare_mixed)
        const double mid = -0.5 * dt;
        double pr, pz;
        if (d.finite) {
            pr = x0.x + u.x + mid * v.x;
            pz = x0.y + u.y + mid * v.y;
        } else {
            pr = x0.x;
            pz = x0.y;
        }
        const float2 sr = nf_split(pr), sz = nf_split(pz);
        geo.pMid[geo.base + i] = make_float4(sr.x, sr.y, sz.x, sz.y);
        if (geo.pCur) {
            const float2 qr = nf_split(x0.x + u.x), qz = nf_split(x0.y + u.y);
            geo.pCur[geo.base + i] = make_float4(qr.x, qr.y, qz.x, qz.y);
        }
        geo.vdt[geo.base + i] = make_float2(nf_narrow(v.x * dt), nf_narrow(v.y * dt));
    }
}

// The mixed form's geometry of an assembly on its own (the initial one, and steps without the
// fused nodal update): node i's mid-step and current positions as float pairs and v sdt.
static __device__ __forceinline__ void prepare_node(const Dev &d, int i, double sdt,
                                                    const MixedGeo &geo) {
    const double mid = -0.5 * sdt;
    const double2 x = d.X0[i], u = d.U[i], v = d.V[i];
    double pr, pz;
    if (d.finite) {
        pr = x.x + u.x + mid * v.x;
        pz = x.y + u.y + mid * v.y;
    } else {
        pr = x.x;
        pz = x.y;
    }
    const float2 sr = nf_split(pr), sz = nf_split(pz);
    geo.pMid[geo.base + i] = make_float4(sr.x, sr.y, sz.x, sz.y);
    if (geo.pCur) {
        const float2 qr = nf_split(x.x + u.x), qz = nf_split(x.y + u.y);
        geo.pCur[geo.base + i] = make_float4(qr.x, qr.y, qz.x, qz.y);
    }
    geo.vdt[geo.base + i] = make_float2(nf_narrow(v.x * sdt), nf_narrow(v.y * sdt));
}

// reducedIntegration, ExplicitSolver.java:1373-1504, for element e: B at the centroid, strain
// increments, Cayley co-rotation, J2/Johnson-Cook return, FB hourglass, the eight force
// terms into the element's contribution slots; folds its shortest edge into minEdge.
// *cost (when given) receives the point's Johnson-Cook cost class (j2_update).
// The current positions x + u of element e's four nodes (the sums cr/cz and currentArea both
// start from).
static __device__ __forceinline__ void element_current(const Dev &d, int e, double2 *cur) {
    const int4 c = d.conn[e];
    const int n[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double2 x = d.X0[n[k]], u = d.U[n[k]];
        cur[k] = make_double2(x.x + u.x, x.y + u.y);
    }
}

// cur (when given) holds element_current(d, e), already formed for the erosion test.
static __device__ __forceinline__ void element_reduced(const Dev &d, int e, double strainDt,
                                                       double hourglass, double &minEdge,
                                                       int *cost = nullptr,
                                                       const double2 *cur = nullptr) {
    double *ef = d.contribution + 8 * (size_t)e;
    if (d.gone != nullptr && d.gone[e]) {
        for (int k = 0; k < 8; k++) ef[k] = 0.0;
    } else {
        const MatDev &fl = d.mats[d.emat[e]];
        const double lambda = fl.lambda, mu = fl.mu;
        const int4 c = d.conn[e];
        const double mid = -0.5 * strainDt;
        const double2 v0 = d.V[c.x], v1 = d.V[c.y], v2 = d.V[c.z], v3 = d.V[c.w];
        double r0, r1, r2, r3, z0, z1, z2, z3;
        if (d.finite) {                                  // cr/cz, :1176-1182
            double2 p[4];
            if (cur) {
                for (int k = 0; k < 4; k++) p[k] = cur[k];
            } else {
                element_current(d, e, p);
            }
            r0 = p[0].x + mid * v0.x; r1 = p[1].x + mid * v1.x;
            r2 = p[2].x + mid * v2.x; r3 = p[3].x + mid * v3.x;
            z0 = p[0].y + mid * v0.y; z1 = p[1].y + mid * v1.y;
            z2 = p[2].y + mid * v2.y; z3 = p[3].y + mid * v3.y;
        } else {
            const double2 x0 = d.X0[c.x], x1 = d.X0[c.y], x2 = d.X0[c.z], x3 = d.X0[c.w];
            r0 = x0.x; r1 = x1.x; r2 = x2.x; r3 = x3.x;
            z0 = x0.y; z1 = x1.y; z2 = x2.y; z3 = x3.y;
        }
        const double a0 = v0.x * strainDt, a1 = v1.x * strainDt;
        const double a2 = v2.x * strainDt, a3 = v3.x * strainDt;
        const double c0 = v0.y * strainDt, c1 = v1.y * strainDt;
        const double c2 = v2.y * strainDt, c3 = v3.y * strainDt;

        if (d.finite) minEdge = shortestEdge(minEdge, r0, r1, r2, r3, z0, z1, z2, z3);

        // J = S / 4 with S the corner sums, det = D / 16 with D = S00 S11 - S01 S10, and so
        // 0.25 (J01 - J11) / det = (S01 - S11) / D: the powers of two cancel exactly (rounding
        // commutes with them) as long as every scaled value stays normal, which bounding the
        // S and D exponents guarantees; otherwise the reference's own sequence runs
        const double S00 = -r0 + r1 + r2 - r3;
        const double S01 = -z0 + z1 + z2 - z3;
        const double S10 = -r0 - r1 + r2 + r3;
        const double S11 = -z0 - z1 + z2 + z3;
        const double D = S00 * S11 - S01 * S10;
        double det, d0r, d1r, d0z, d1z;
        if (moderate_or_zero(S00) && moderate_or_zero(S01) && moderate_or_zero(S10) &&
            moderate_or_zero(S11) && moderate_or_zero(D)) {
            const double invD = 1.0 / D;
            det = 0.0625 * D;
            d0r = (S01 - S11) * invD;
            d1r = (S01 + S11) * invD;
            d0z = (S10 - S00) * invD;
            d1z = -((S10 + S00) * invD);
        } else {
            const double J00 = 0.25 * S00, J01 = 0.25 * S01, J10 = 0.25 * S10, J11 = 0.25 * S11;
            det = J00 * J11 - J01 * J10;
            const double inv = 1.0 / det;
            d0r = 0.25 * (J01 - J11) * inv;
            d1r = 0.25 * (J01 + J11) * inv;
            d0z = 0.25 * (J10 - J00) * inv;
            d1z = -0.25 * (J10 + J00) * inv;
        }
        const double d2r = -d0r;
        const double d3r = -d1r;
        const double d2z = -d0z;
        const double d3z = -d1z;

        const double dEpsR = d0r * a0 + d1r * a1 + d2r * a2 + d3r * a3;
        const double dEpsZ = d0z * c0 + d1z * c1 + d2z * c2 + d3z * c3;
        const double dRdZ = d0z * a0 + d1z * a1 + d2z * a2 + d3z * a3;
        const double dZdR = d0r * c0 + d1r * c1 + d2r * c2 + d3r * c3;
        const double dGamRZ = dRdZ + dZdR;

        double rg = 0.0, dEpsT = 0.0;
        if (d.axi) {
            rg = 0.25 * (r0 + r1 + r2 + r3);
            dEpsT = 0.25 * (a0 + a1 + a2 + a3) / rg;
        }
        double sg[4], bk[4];
        {
            const double2 *ps = reinterpret_cast<const double2 *>(d.sig + 4 * (size_t)e);
            const double2 *pb = reinterpret_cast<const double2 *>(d.back + 4 * (size_t)e);
            const double2 s01 = ps[0], s23 = ps[1], b01 = pb[0], b23 = pb[1];
            sg[0] = s01.x; sg[1] = s01.y; sg[2] = s23.x; sg[3] = s23.y;
            bk[0] = b01.x; bk[1] = b01.y; bk[2] = b23.x; bk[3] = b23.y;
        }
        if (d.finite) {
            const double spinDt = 0.5 * (dZdR - dRdZ);
            if (!is_zero(spinDt)) {
                const double cs = corot_cos(spinDt), sn = corot_sin(spinDt);
                corot_rotate(sg, cs, sn);
                // a back stress of +0s (no kinematic hardening) rotates to itself
                if (!(all_plus_zero(bk[0], bk[1], bk[2], bk[3]) && corot_keeps_zero(cs, sn)))
                    corot_rotate(bk, cs, sn);
            }
        }
        double epsP = d.epsP[e], work = d.wP[e];
        double2 *const jcYield = d.jcYield && fl.jc ? d.jcYield + e : nullptr;
        if (d.hasDamage) {
            DamageRef dr;
            dr.failureStrain = d.dFail[e];
            dr.strength = d.dStrength + e;
            dr.softening = d.dSoft + e;
            dr.width = d.dWidth + e;
            dr.geometry = d.dGeom + 5 * (size_t)e;
            dr.fractureEnergy = d.dGf[e];
            dr.youngs = fl.youngs;
            j2_update(sg, bk, epsP, work, dEpsR, dEpsZ, dEpsT, dGamRZ, lambda, mu, fl,
                      strainDt, &dr, d.dStrength[e], d.dSoft[e], cost, jcYield);
        } else {
            j2_update(sg, bk, epsP, work, dEpsR, dEpsZ, dEpsT, dGamRZ, lambda, mu, fl,
                      strainDt, (const DamageRef *)nullptr, 0.0, 0.0, cost, jcYield);
        }
        {
            double2 *ps = reinterpret_cast<double2 *>(d.sig + 4 * (size_t)e);
            double2 *pb = reinterpret_cast<double2 *>(d.back + 4 * (size_t)e);
            ps[0] = make_double2(sg[0], sg[1]); ps[1] = make_double2(sg[2], sg[3]);
            pb[0] = make_double2(bk[0], bk[1]); pb[1] = make_double2(bk[2], bk[3]);
            d.epsP[e] = epsP;
            d.wP[e] = work;
        }
        const double sR = sg[0], sZ = sg[1], sT = sg[2], sRZ = sg[3];
        const double dV = 4.0 * (d.axi ? 2.0 * NF_PI * rg * det : d.thickness * det);

        double g0r, g1r, g2r, g3r;
        if (d.axi) {
            const double hh = sT / rg * dV * 0.25;
            g0r = -((d0r * sR + d0z * sRZ) * dV + hh);
            g1r = -((d1r * sR + d1z * sRZ) * dV + hh);
            g2r = -((d2r * sR + d2z * sRZ) * dV + hh);
            g3r = -((d3r * sR + d3z * sRZ) * dV + hh);
        } else {
            g0r = -(d0r * sR + d0z * sRZ) * dV;
            g1r = -(d1r * sR + d1z * sRZ) * dV;
            g2r = -(d2r * sR + d2z * sRZ) * dV;
            g3r = -(d3r * sR + d3z * sRZ) * dV;
        }
        double g0z = -(d0z * sZ + d0r * sRZ) * dV;
        double g1z = -(d1z * sZ + d1r * sRZ) * dV;
        double g2z = -(d2z * sZ + d2r * sRZ) * dV;
        double g3z = -(d3z * sZ + d3r * sRZ) * dV;

        const double qhg = hourglass;
        if (qhg > 0.0) {
            const double hr = r0 - r1 + r2 - r3;
            const double hz = z0 - z1 + z2 - z3;
            const double y0 = 1.0 - hr * d0r - hz * d0z;
            const double y1 = -1.0 - hr * d1r - hz * d1z;
            const double y2 = 1.0 - hr * d2r - hz * d2z;
            const double y3 = -1.0 - hr * d3r - hz * d3z;
            const double k = qhg * mu * dV
                             * (d0r * d0r + d1r * d1r + d2r * d2r + d3r * d3r
                                + d0z * d0z + d1z * d1z + d2z * d2z + d3z * d3z);
            double2 hg = d.hg[e];
            hg.x += k * (y0 * a0 + y1 * a1 + y2 * a2 + y3 * a3);
            hg.y += k * (y0 * c0 + y1 * c1 + y2 * c2 + y3 * c3);
            d.hg[e] = hg;
            const double qr = hg.x, qz = hg.y;
            g0r -= y0 * qr; g1r -= y1 * qr; g2r -= y2 * qr; g3r -= y3 * qr;
            g0z -= y0 * qz; g1z -= y1 * qz; g2z -= y2 * qz; g3z -= y3 * qz;
            d.hgK[e] = k;
        }
        double2 *ef2 = reinterpret_cast<double2 *>(ef);
        ef2[0] = make_double2(g0r, g1r);
        ef2[1] = make_double2(g2r, g3r);
        ef2[2] = make_double2(g0z, g1z);
        ef2[3] = make_double2(g2z, g3z);
    }
}

static __device__ __forceinline__ float diff_hl(float4 a, float4 b, int comp) {
    // (a - b) for component comp (0: r, 1: z) of two hi/lo pairs
    return comp == 0 ? (a.x - b.x) + (a.y - b.y) : (a.z - b.z) + (a.w - b.w);
}

// One point's update in FP32; shared by the reduced and full kernels.
static __device__ __forceinline__ void point_update_mixed(const Dev &d, int e, int p, const MatF &fl,
                                                   float dEpsR, float dEpsZ, float dEpsT,
                                                   float dGamRZ, float spinDt, float strainDt,
                                                   float *sg) {
    float bk[4];
    {
        const float4 s = reinterpret_cast<const float4 *>(d.sigF)[p];
        const float4 b = reinterpret_cast<const float4 *>(d.backF)[p];
        sg[0] = s.x; sg[1] = s.y; sg[2] = s.z; sg[3] = s.w;
        bk[0] = b.x; bk[1] = b.y; bk[2] = b.z; bk[3] = b.w;
    }
    if (d.finite && spinDt != 0.0f) {
        const float cs = corot_cos(spinDt), sn = corot_sin(spinDt);
        corot_rotate(sg, cs, sn);
        corot_rotate(bk, cs, sn);
    }
    float epsP = d.epsPF[p], work = d.wPF[p];
    if (d.hasDamage) {
        DamageRefT<float> dr;
        dr.failureStrain = d.dFailF[e];
        dr.strength = d.dStrF + p;
        dr.softening = d.dSoftF + p;
        dr.width = d.dWidthF + p;
        dr.geometry = d.dGeomF + 5 * (size_t)e;
        dr.fractureEnergy = d.dGfF[e];
        dr.youngs = fl.youngs;
        j2_update(sg, bk, epsP, work, dEpsR, dEpsZ, dEpsT, dGamRZ, fl.lambda, fl.mu, fl,
                  strainDt, &dr, d.dStrF[p], d.dSoftF[p]);
    } else {
        j2_update(sg, bk, epsP, work, dEpsR, dEpsZ, dEpsT, dGamRZ, fl.lambda, fl.mu, fl,
                  strainDt, (const DamageRefT<float> *)nullptr, 0.0f, 0.0f);
    }
    reinterpret_cast<float4 *>(d.sigF)[p] = make_float4(sg[0], sg[1], sg[2], sg[3]);
    reinterpret_cast<float4 *>(d.backF)[p] = make_float4(bk[0], bk[1], bk[2], bk[3]);
    d.epsPF[p] = epsP;
    d.wPF[p] = work;
}

// reducedIntegration (ExplicitSolver.java:1373-1504) in FP32 for element e, on the float
// geometry pMid/vdt of its nodes (node n at index n - base). Shared by the single-scene and
// batched kernels.
static __device__ __forceinline__ void element_reduced_f32(const Dev &d, int e, float strainDt,
                                                           float hourglass, const float4 *pMid,
                                                           const float2 *vdt, int base,
                                                           float &minEdge) {
    float4 *ef = reinterpret_cast<float4 *>(d.contribF + 8 * (size_t)e);
    if (d.gone != nullptr && d.gone[e]) {
        ef[0] = make_float4(0.f, 0.f, 0.f, 0.f);
        ef[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        const MatF &fl = d.matsF[d.emat[e]];
        const float mu = fl.mu;
        const int4 c = d.conn[e];
        const float4 p0 = pMid[c.x - base], p1 = pMid[c.y - base], p2 = pMid[c.z - base],
                     p3 = pMid[c.w - base];
        const float2 w0 = vdt[c.x - base], w1 = vdt[c.y - base], w2 = vdt[c.z - base],
                     w3 = vdt[c.w - base];
        const float r0 = 0.0f, z0 = 0.0f;
        const float r1 = diff_hl(p1, p0, 0), r2 = diff_hl(p2, p0, 0), r3 = diff_hl(p3, p0, 0);
        const float z1 = diff_hl(p1, p0, 1), z2 = diff_hl(p2, p0, 1), z3 = diff_hl(p3, p0, 1);
        const float a0 = w0.x, a1 = w1.x, a2 = w2.x, a3 = w3.x;
        const float c0 = w0.y, c1 = w1.y, c2 = w2.y, c3 = w3.y;
        if (d.finite) minEdge = shortestEdge(minEdge, r0, r1, r2, r3, z0, z1, z2, z3);

        const float J00 = 0.25f * (-r0 + r1 + r2 - r3);
        const float J01 = 0.25f * (-z0 + z1 + z2 - z3);
        const float J10 = 0.25f * (-r0 - r1 + r2 + r3);
        const float J11 = 0.25f * (-z0 - z1 + z2 + z3);
        const float det = J00 * J11 - J01 * J10;
        const float inv = 1.0f / det;
        const float d0r = 0.25f * (J01 - J11) * inv;
        const float d1r = 0.25f * (J01 + J11) * inv;
        const float d2r = -d0r, d3r = -d1r;
        const float d0z = 0.25f * (J10 - J00) * inv;
        const float d1z = -0.25f * (J10 + J00) * inv;
        const float d2z = -d0z, d3z = -d1z;

        const float dEpsR = d0r * a0 + d1r * a1 + d2r * a2 + d3r * a3;
        const float dEpsZ = d0z * c0 + d1z * c1 + d2z * c2 + d3z * c3;
        const float dRdZ = d0z * a0 + d1z * a1 + d2z * a2 + d3z * a3;
        const float dZdR = d0r * c0 + d1r * c1 + d2r * c2 + d3r * c3;
        const float dGamRZ = dRdZ + dZdR;
        float rg = 0.0f, dEpsT = 0.0f;
        if (d.axi) {
            rg = 0.25f * (p0.x + p1.x + p2.x + p3.x);
            dEpsT = 0.25f * (a0 + a1 + a2 + a3) / rg;
        }
        float sg[4];
        point_update_mixed(d, e, e, fl, dEpsR, dEpsZ, dEpsT, dGamRZ,
                           0.5f * (dZdR - dRdZ), strainDt, sg);
        const float sR = sg[0], sZ = sg[1], sT = sg[2], sRZ = sg[3];
        const float dV = 4.0f * (d.axi ? 2.0f * 3.14159265358979f * rg * det
                                       : (float)d.thickness * det);
        float g0r, g1r, g2r, g3r;
        if (d.axi) {
            const float hh = sT / rg * dV * 0.25f;
            g0r = -((d0r * sR + d0z * sRZ) * dV + hh);
            g1r = -((d1r * sR + d1z * sRZ) * dV + hh);
            g2r = -((d2r * sR + d2z * sRZ) * dV + hh);
            g3r = -((d3r * sR + d3z * sRZ) * dV + hh);
        } else {
            g0r = -(d0r * sR + d0z * sRZ) * dV;
            g1r = -(d1r * sR + d1z * sRZ) * dV;
            g2r = -(d2r * sR + d2z * sRZ) * dV;
            g3r = -(d3r * sR + d3z * sRZ) * dV;
        }
        float g0z = -(d0z * sZ + d0r * sRZ) * dV;
        float g1z = -(d1z * sZ + d1r * sRZ) * dV;
        float g2z = -(d2z * sZ + d2r * sRZ) * dV;
        float g3z = -(d3z * sZ + d3r * sRZ) * dV;
        const float qhg = hourglass;
        if (qhg > 0.0f) {
            const float hr = r0 - r1 + r2 - r3;
            const float hz = z0 - z1 + z2 - z3;
            const float y0 = 1.0f - hr * d0r - hz * d0z;
            const float y1 = -1.0f - hr * d1r - hz * d1z;
            const float y2 = 1.0f - hr * d2r - hz * d2z;
            const float y3 = -1.0f - hr * d3r - hz * d3z;
            const float k = qhg * mu * dV
                            * (d0r * d0r + d1r * d1r + d2r * d2r + d3r * d3r
                               + d0z * d0z + d1z * d1z + d2z * d2z + d3z * d3z);
            float2 hg = d.hgF[e];
            hg.x += k * (y0 * a0 + y1 * a1 + y2 * a2 + y3 * a3);
            hg.y += k * (y0 * c0 + y1 * c1 + y2 * c2 + y3 * c3);
            d.hgF[e] = hg;
            g0r -= y0 * hg.x; g1r -= y1 * hg.x; g2r -= y2 * hg.x; g3r -= y3 * hg.x;
            g0z -= y0 * hg.y; g1z -= y1 * hg.y; g2z -= y2 * hg.y; g3z -= y3 * hg.y;
            d.hgKF[e] = k;
        }
        ef[0] = make_float4(g0r, g1r, g2r, g3r);
        ef[1] = make_float4(g0z, g1z, g2z, g3z);
    }
}

// applyPressure + pressureAt, ExplicitSolver.java:1203-1207, :1511-1556, for pressure edge e at
// time t (the ramp's target and duration given): writes the edge's contribution slots.
static __device__ __forceinline__ void pressure_edge(const Dev &d, int e, double t, double target,
                                                     double rampDuration) {
    double p = target;
    if (rampDuration > 0.0) {
        const double s = jmin(1.0, t / rampDuration);
        p = target * s * s * (3.0 - 2.0 * s);
    }
    double *c = d.contribution + 8 * (size_t)(d.E + e);
    const int2 ed = d.pedges[e];
    const double2 xa = d.X0[ed.x], xb = d.X0[ed.y];
    double ra, rb, za, zb;
    if (d.finite) {
        const double2 ua = d.U[ed.x], ub = d.U[ed.y], va = d.V[ed.x], vb = d.V[ed.y];
        ra = xa.x + ua.x + 0.0 * va.x; rb = xb.x + ub.x + 0.0 * vb.x;
        za = xa.y + ua.y + 0.0 * va.y; zb = xb.y + ub.y + 0.0 * vb.y;
    } else {
        ra = xa.x; rb = xb.x; za = xa.y; zb = xb.y;
    }
    const double tr = rb - ra;
    const double tz = zb - za;
    const double len = sqrt(tr * tr + tz * tz);
    if (len == 0.0) {
        c[0] = 0.0; c[1] = 0.0; c[4] = 0.0; c[5] = 0.0;
        return;
    }
    const double nr = tz / len;
    const double nz = -tr / len;
    double wa, wb;
    if (d.axi) {
        const double circumference = 2.0 * NF_PI * len;
        wa = circumference * (ra / 3.0 + rb / 6.0);
        wb = circumference * (ra / 6.0 + rb / 3.0);
    } else {
        wa = d.thickness * len * 0.5;
        wb = wa;
    }
    c[0] = p * nr * wa;
    c[1] = p * nr * wb;
    c[4] = p * nz * wa;
    c[5] = p * nz * wb;
}

// The same edge in the mixed form: FP64 geometry and load, float contribution slots.
static __device__ __forceinline__ void pressure_edge_f32(const Dev &d, int e, double t,
                                                         double target, double rampDuration) {
    double p = target;
    if (rampDuration > 0.0) {
        const double s = jmin(1.0, t / rampDuration);
        p = target * s * s * (3.0 - 2.0 * s);
    }
    float *c = d.contribF + 8 * (size_t)(d.E + e);
    const int2 ed = d.pedges[e];
    const double2 xa = d.X0[ed.x], xb = d.X0[ed.y];
    double ra = xa.x, rb = xb.x, za = xa.y, zb = xb.y;
    if (d.finite) {
        const double2 ua = d.U[ed.x], ub = d.U[ed.y];
        ra += ua.x; rb += ub.x; za += ua.y; zb += ub.y;
    }
    const double tr = rb - ra, tz = zb - za;
    const double len = sqrt(tr * tr + tz * tz);
    if (len == 0.0) {
        c[0] = 0.f; c[1] = 0.f; c[4] = 0.f; c[5] = 0.f;
        return;
    }
    const double nr = tz / len, nz = -tr / len;
    double wa, wb;
    if (d.axi) {
        const double circumference = 2.0 * NF_PI * len;
        wa = circumference * (ra / 3.0 + rb / 6.0);
        wb = circumference * (ra / 6.0 + rb / 3.0);
    } else {
        wa = d.thickness * len * 0.5;
        wb = wa;
    }
    c[0] = (float)(p * nr * wa);
    c[1] = (float)(p * nr * wb);
    c[4] = (float)(p * nz * wa);
    c[5] = (float)(p * nz * wb);
}

// ---------------------------------------------------------------- the compensated form
// FP32 nodal arithmetic with each displacement carried as an unevaluated float pair hi + lo
// (Kahan-style compensated accumulation, about 48 significant bits), FP32 velocities and an
// FP32 gather. The error-free transformations are additions only; the increment v dt that
// feeds one is rounded on its own (__fmul_rn), so a contracted multiply-add cannot change
// what the compensation sees.

// TwoSum (Knuth): s + e == a + b exactly.
static __device__ __forceinline__ float2 two_sum_f(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return make_float2(s, (a - (s - bb)) + (b - bb));
}

// (hi, lo) += x, renormalised (|lo| <= ulp(hi) / 2).
static __device__ __forceinline__ void ff_add(float &hi, float &lo, float x) {
    const float2 s = two_sum_f(hi, x);
    const float l = s.y + lo;
    hi = s.x + l;
    lo = l - (hi - s.x);
}

// The pair nearest xh + xl + uh + ul + c for a small c (a node's position, mid-step or current).
static __device__ __forceinline__ float2 ff_point(float xh, float xl, float uh, float ul, float c) {
    const float2 s = two_sum_f(xh, uh);
    const float l = s.y + ((xl + ul) + c);
    const float hi = s.x + l;
    return make_float2(hi, l - (hi - s.x));
}

static __device__ __forceinline__ float2 ff_from(double x) {
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// nodalUpdate (:998-1062) with the rigid wall (RigidWall.java:163-259) for node i in the
// compensated form, the same branch structure as nodal_node; also writes the node's float
// geometry for the coming assembly. The audit terms are summed in FP64.
static __device__ __forceinline__ void nodal_node_comp(const Dev &d, int i, float decay,
                                                       float gain, float dtAvg, float dt,
                                                       float plane, float friction,
                                                       const WallRef &w, const MixedGeo &geo,
                                                       uint32_t *status, double &impulse,
                                                       double &loss, double &fric) {
    const uint8_t fl = d.flags[i];
    const bool fixedR = fl & 1, fixedZ = fl & 2;
    bool onWall = fl & 4;
    float4 u = d.uC[i];
    float2 v = d.vC[i];
    const float2 f = d.fC[i];
    const float2 mm = d.mC[i];
    const float m = mm.x, invM = mm.y;
    const float4 x0 = d.x0C[i];
    const bool resting = w.present && onWall && f.y <= 0.0f;
    uint8_t ws = 0;
    if (fixedR) {
        v.x = 0.0f;
    } else if (resting && friction > 0.0f) {
        const float normal = -f.y;
        const float trial = -m * decay * v.x / gain - f.x;
        const float limit = isinf(friction) ? INFINITY : friction * normal;
        if (fabsf(trial) <= limit) {
            loss += 0.5 * (double)m * (double)v.x * (double)v.x;
            atomicAdd(w.stuck, 1);
            ws |= NF_WALL_STUCK;
            v.x = 0.0f;
        } else {
            const float tangential = copysignf(limit, trial);
            const float slid = decay * v.x + gain * (f.x + tangential) / m;
            fric += -(double)tangential * (double)slid * (double)dt;
            ws |= NF_WALL_SLID;
            v.x = slid;
        }
        ff_add(u.x, u.y, __fmul_rn(v.x, dt));
    } else {
        v.x = decay * v.x + gain * f.x * invM;
        ff_add(u.x, u.y, __fmul_rn(v.x, dt));
    }
    if (fixedZ) {
        v.y = 0.0f;
    } else if (resting) {
        impulse += -(double)f.y * (double)dtAvg;
        atomicAdd(w.contact, 1);
        ws |= NF_WALL_HELD;
    } else {
        const float trial = decay * v.y + gain * f.y * invM;
        // z + trial dt < plane, with z = x0 + u as a pair
        const float2 s = two_sum_f(x0.z, u.z);
        const float below = (s.x - plane) + ((s.y + (x0.w + u.w)) + trial * dt);
        if (w.present && below < 0.0f) {
            impulse += -(double)m * (double)trial;
            loss += 0.5 * (double)m * (double)trial * (double)trial;
            atomicAdd(w.contact, 1);
            // u = plane - x0
            const float2 t = two_sum_f(plane, -x0.z);
            const float l = t.y - x0.w;
            u.z = t.x + l;
            u.w = l - (u.z - t.x);
            v.y = 0.0f;
            onWall = true;
            ws |= NF_WALL_ARRIVED;
        } else {
            v.y = trial;
            ff_add(u.z, u.w, __fmul_rn(v.y, dt));
            if (w.present) onWall = false;
        }
    }
    d.uC[i] = u;
    d.vC[i] = v;
    if (w.present) {
        d.flags[i] = (uint8_t)((fl & 3) | (onWall ? 4 : 0));
        d.wallState[i] = ws;
    }
    if (!(isfinite(u.x) && isfinite(u.z) && isfinite(v.x) && isfinite(v.y)))
        atomicOr(status, STATUS_NONFINITE);
    if (geo.pMid) {
        const float mid = -0.5f * dt;
        float2 pr, pz;
        if (d.finite) {
            pr = ff_point(x0.x, x0.y, u.x, u.y, mid * v.x);
            pz = ff_point(x0.z, x0.w, u.z, u.w, mid * v.y);
        } else {
            pr = make_float2(x0.x, x0.y);
            pz = make_float2(x0.z, x0.w);
        }
        geo.pMid[geo.base + i] = make_float4(pr.x, pr.y, pz.x, pz.y);
        geo.vdt[geo.base + i] = make_float2(v.x * dt, v.y * dt);
    }
}

// The pressure edge of the mixed form with the edge's current geometry read from the
// compensated pairs.
static __device__ __forceinline__ void pressure_edge_comp(const Dev &d, int e, double t,
                                                          double target, double rampDuration) {
    double p = target;
    if (rampDuration > 0.0) {
        const double s = jmin(1.0, t / rampDuration);
        p = target * s * s * (3.0 - 2.0 * s);
    }
    float *c = d.contribF + 8 * (size_t)(d.E + e);
    const int2 ed = d.pedges[e];
    const float4 xa = d.x0C[ed.x], xb = d.x0C[ed.y];
    double ra = (double)xa.x + (double)xa.y, rb = (double)xb.x + (double)xb.y;
    double za = (double)xa.z + (double)xa.w, zb = (double)xb.z + (double)xb.w;
    if (d.finite) {
        const float4 ua = d.uC[ed.x], ub = d.uC[ed.y];
        ra += (double)ua.x + (double)ua.y; rb += (double)ub.x + (double)ub.y;
        za += (double)ua.z + (double)ua.w; zb += (double)ub.z + (double)ub.w;
    }
    const double tr = rb - ra, tz = zb - za;
    const double len = sqrt(tr * tr + tz * tz);
    if (len == 0.0) {
        c[0] = 0.f; c[1] = 0.f; c[4] = 0.f; c[5] = 0.f;
        return;
    }
    const double nr = tz / len, nz = -tr / len;
    double wa, wb;
    if (d.axi) {
        const double circumference = 2.0 * NF_PI * len;
        wa = circumference * (ra / 3.0 + rb / 6.0);
        wb = circumference * (ra / 6.0 + rb / 3.0);
    } else {
        wa = d.thickness * len * 0.5;
        wb = wa;
    }
    c[0] = (float)(p * nr * wa);
    c[1] = (float)(p * nr * wb);
    c[4] = (float)(p * nz * wa);
    c[5] = (float)(p * nz * wb);
}

// The gather of float contributions into float sums, in CSR order, then m g.
static __device__ __forceinline__ float2 gather_node_comp(const Dev &d, int n, float gR,
                                                          float gZ) {
    float sr = 0.0f, sz = 0.0f;
    const int end = d.nodeSlotStart[n + 1];
    for (int k = d.nodeSlotStart[n]; k < end; k++) {
        const int slot = d.nodeSlot[k];
        sr += d.contribF[slot];
        sz += d.contribF[slot + 4];
    }
    const float m = d.mC[n].x;
    return make_float2(sr + m * gR, sz + m * gZ);
}

// gather, ExplicitSolver.java:1147-1165: node n's sources in ascending order, then m g.
// Four slots at a time: their indices, then their values, are loaded before any is added, so
// the loads overlap; the sums still take the slots in order.
static __device__ __forceinline__ double2 gather_node(const Dev &d, int n) {
    double sr = 0.0, sz = 0.0;
    const int end = d.nodeSlotStart[n + 1];
    const double m = d.mass[n];
    for (int k = d.nodeSlotStart[n]; k < end; k += 4) {
        const int cnt = end - k < 4 ? end - k : 4;
        int slot[4];
        double vr[4], vz[4];
#pragma unroll
        for (int j = 0; j < 4; j++) slot[j] = j < cnt ? d.nodeSlot[k + j] : 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            vr[j] = j < cnt ? d.contribution[slot[j]] : 0.0;
            vz[j] = j < cnt ? d.contribution[slot[j] + 4] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (j < cnt) {
                sr += vr[j];
                sz += vz[j];
            }
        }
    }
    return make_double2(sr + m * d.gravR, sz + m * d.gravZ);
}

// The same gather of float contributions into FP64 sums (the mixed form), four slots at a
// time like gather_node. Each float is widened to double by integer arithmetic (exact, the
// value the conversion gives): only the sums use the FP64 pipe.
static __device__ __forceinline__ double2 gather_node_f32(const Dev &d, int n) {
    double sr = 0.0, sz = 0.0;
    const int end = d.nodeSlotStart[n + 1];
    const double m = d.mass[n];
    for (int k = d.nodeSlotStart[n]; k < end; k += 4) {
        const int cnt = end - k < 4 ? end - k : 4;
        int slot[4];
        float vr[4], vz[4];
#pragma unroll
        for (int j = 0; j < 4; j++) slot[j] = j < cnt ? d.nodeSlot[k + j] : 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            vr[j] = j < cnt ? d.contribF[slot[j]] : 0.0f;
            vz[j] = j < cnt ? d.contribF[slot[j] + 4] : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (j < cnt) {
                sr += nf_widen(vr[j]);
                sz += nf_widen(vz[j]);
            }
        }
    }
    return make_double2(sr + m * d.gravR, sz + m * d.gravZ);
}

}  // namespace nf
