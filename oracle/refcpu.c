/*
 * refcpu.c -- ORACLE. Test infrastructure only: a CPU restatement, in plain C, of the
 * reference's explicit central-difference timestep. It is the checker that the GPU path in
 * neofiz_gb300 is compared against; nothing in the product links, loads or calls it.
 *
 * It follows the Java source statement by statement and keeps its floating-point
 * evaluation order (Java evaluates strictly left to right in IEEE double; this file is built
 * with -O2 -ffp-contract=off, so no multiply-add is fused and every expression below rounds
 * exactly where the Java one does). Citations are to src/main/java/org/neofiz/ in the
 * reference:
 *   solver/ExplicitSolver.java  constructor :264-339, node slots :347-366, setters :386-808,
 *                               step :940-991, nodal update :998-1062, advance :1069-1075,
 *                               assembly :1081-1165, kernels :1191-1504, pressure :1511-1556,
 *                               lumped mass :1559-1597, audits :1610-1965
 *   solver/J2.java              update :163-296, solve :332-375
 *   core/JohnsonCook.java       :138-226
 *   solver/Damage.java          :196-412
 *   solver/Corotational.java    :59-98
 *   solver/RigidWall.java       :110-279
 *   solver/Contact.java         :209-762
 *   mesh/QuadMesh.java          :59-226
 *
 * The transcendental functions (Math.pow, Math.log, Math.hypot, Math.atan2, Math.sin,
 * Math.cos) are the deterministic implementations in nf_math.h, shared with the kernels so
 * that the two sides are bit-comparable; nf_math itself is pinned against glibc and CUDA.
 *
 * Parity pin: the reference ships no stored vectors and no JDK exists here, so this file is
 * pinned by re-expressing the reference's own known-answer tests (GravityTest, J2Test,
 * RateDependentReturnMapTest, DamageTest, HourglassTest, FiniteStrainTest, MassScalingTest,
 * ContactTest, ErosionTest, EnergyAuditTest, ThreadingTest) and its published Taylor-impact
 * results (README.md:306-312) against it; see tests/test_oracle_pins.py.
 *
 * Threading: nfo_set_threads(n > 1) splits the element assembly, the gather and the contact
 * search across n POSIX threads exactly where the reference's Parallel pool does
 * (ExplicitSolver.java:1087-1093, :1105). Each element writes only its own contribution slot
 * and each node sums its own slots in a fixed order, so results are bit-identical at any
 * thread count (ThreadingTest.java:117-157).
 */
#include "../include/neofiz.h"
#include "../neofiz_gb300/csrc/nf_math.h"
#include "../neofiz_gb300/csrc/nf_adjoint.h"

#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <time.h>

#define COMPONENTS 4
#define GEOMETRY_STRIDE 5
static const double SQRT_2_3 = 0x1.a20bd700c2c3ep-1;     /* Math.sqrt(2.0 / 3.0) */
static const double TWO_THIRDS = 2.0 / 3.0;
static const double SOLVE_TOLERANCE = 1.0e-10;
static const int SOLVE_ITERATIONS = 25;
static const double G_PT = 0.5773502691896258;
static const double GP_XI[4] = {-0.5773502691896258, 0.5773502691896258, 0.5773502691896258, -0.5773502691896258};
static const double GP_ETA[4] = {-0.5773502691896258, -0.5773502691896258, 0.5773502691896258, 0.5773502691896258};
static const double W_REDUCED = 4.0;
static const double HG[4] = {1.0, -1.0, 1.0, -1.0};
static const double DEFAULT_HOURGLASS_COEFFICIENT = 0.05;
static const double ISOTROPIC = 1.0e-9;
static const double CONTACT_DEFAULT_SCALE = 0.1;
static const double MAX_DEPTH = 0.5;
static const double STICK_RELAXATION = 0.5;
static const double FACING = 0.25;

/* ------------------------------------------------------------------ Java semantics */

static double jmin(double a, double b) {          /* Math.min */
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0 && b == 0.0) return signbit(a) ? a : b;
    return a <= b ? a : b;
}
static double jmax(double a, double b) {          /* Math.max */
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0 && b == 0.0) return signbit(a) ? b : a;
    return a >= b ? a : b;
}
static int jd2i(double x) {                       /* (int) cast of a double */
    if (x != x) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return (-2147483647 - 1);
    return (int)x;
}

/* ------------------------------------------------------------------ material */

typedef struct {
    double sy0, hIso, hKin;
    int jc;
    double a, b, n, c, m, refRate, room, melt, cp, tq;
    double thermalCoefficient;
} flow_t;

static double mat_lambda(const nf_material *m) {  /* Material.java:93-95 */
    return m->youngs_modulus * m->poisson_ratio
           / ((1.0 + m->poisson_ratio) * (1.0 - 2.0 * m->poisson_ratio));
}
static double mat_mu(const nf_material *m) {      /* Material.java:98-100 */
    return m->youngs_modulus / (2.0 * (1.0 + m->poisson_ratio));
}
static double mat_wave(const nf_material *m) {    /* Material.java:106-108 */
    return sqrt((mat_lambda(m) + 2.0 * mat_mu(m)) / m->density);
}
static flow_t flow_of(const nf_material *m) {     /* J2.Flow.of, J2.java:105-110 */
    flow_t f;
    memset(&f, 0, sizeof f);
    f.sy0 = m->yield_stress;
    f.hIso = m->isotropic_hardening;
    f.hKin = m->kinematic_hardening;
    f.jc = m->has_johnson_cook != 0;
    if (f.jc) {
        f.a = m->jc_a; f.b = m->jc_b; f.n = m->jc_n; f.c = m->jc_c; f.m = m->jc_m;
        f.refRate = m->jc_reference_strain_rate;
        f.room = m->jc_room_temperature;
        f.melt = m->jc_melt_temperature;
        f.cp = m->jc_specific_heat;
        f.tq = m->jc_taylor_quinney;
        f.thermalCoefficient = f.tq / (m->density * f.cp);   /* JohnsonCook.java:224-226 */
    }
    return f;
}

static const char *material_invalid(const nf_material *m) {
    /* Material.java:23-39, JohnsonCook.java:71-89 */
    if (m->youngs_modulus <= 0) return "E must be positive";
    if (m->poisson_ratio <= -1.0 || m->poisson_ratio >= 0.5) return "nu must lie in (-1, 0.5)";
    if (m->density <= 0) return "density must be positive";
    if (m->yield_stress <= 0) return "yield stress must be positive";
    if (m->isotropic_hardening < 0 || m->kinematic_hardening < 0)
        return "hardening moduli must be non-negative";
    if (m->has_johnson_cook) {
        if (m->jc_a <= 0) return "A must be positive";
        if (m->jc_b < 0) return "B must be non-negative";
        if (m->jc_n <= 0 || m->jc_n > 1) return "n must lie in (0, 1]";
        if (m->jc_c < 0) return "C must be non-negative";
        if (m->jc_m <= 0) return "m must be positive";
        if (m->jc_reference_strain_rate <= 0) return "reference strain rate must be positive";
        if (m->jc_melt_temperature <= m->jc_room_temperature)
            return "melt temperature must exceed room temperature";
        if (m->jc_specific_heat <= 0) return "specific heat must be positive";
        if (m->jc_taylor_quinney < 0 || m->jc_taylor_quinney > 1)
            return "Taylor-Quinney fraction must lie in [0, 1]";
        if (m->yield_stress != m->jc_a)
            return "yield stress disagrees with the Johnson-Cook A";
    }
    return NULL;
}

/* JohnsonCook.java:138-209 */
static double jc_strainTerm(const flow_t *f, double eps) {
    return eps <= 0.0 ? f->a : f->a + f->b * nf_pow(eps, f->n);
}
static double jc_strainSlopeFrom(const flow_t *f, double strainTerm, double eps) {
    return f->n * (strainTerm - f->a) / eps;
}
static double jc_rateTerm(const flow_t *f, double rate) {
    if (rate <= f->refRate) return 1.0;
    return 1.0 + f->c * nf_log(rate / f->refRate);
}
static int jc_rateIsClamped(const flow_t *f, double rate) { return rate <= f->refRate; }
static double jc_thermalTerm(const flow_t *f, double temperature) {
    const double homologous = (temperature - f->room) / (f->melt - f->room);
    if (homologous <= 0.0) return 1.0;
    if (homologous >= 1.0) return 0.0;
    return 1.0 - nf_pow(homologous, f->m);
}
static double jc_quasiStatic(const flow_t *f, double eps, double temperature) {
    return jc_strainTerm(f, eps) * jc_thermalTerm(f, temperature);
}

/* ------------------------------------------------------------------ damage */

typedef struct {
    const double *failureStrain, *fractureEnergy, *youngsModulus, *geometry;
    double *strength, *softening, *width;
} damage_t;

/* Damage.begin, Damage.java:306-336 */
static void damage_begin(const damage_t *d, int point, double flowStress,
                         double nRR, double nZZ, double nRZ) {
    const int g = GEOMETRY_STRIDE * point;
    const double area = d->geometry[g];
    const double diff = nRR - nZZ;
    const double cross = 2.0 * nRZ;
    const double anisotropy = nf_hypot(diff, cross);
    double h;
    if (anisotropy < ISOTROPIC) {
        h = sqrt(area);
    } else {
        const double phi = 0.5 * nf_atan2(cross, diff);
        const double tR = -nf_sin(phi), tZ = nf_cos(phi);
        const double line = fabs(d->geometry[g + 1] * tR + d->geometry[g + 2] * tZ)
                            + fabs(d->geometry[g + 3] * tR + d->geometry[g + 4] * tZ);
        h = area / line;
    }
    d->width[point] = h;
    d->strength[point] = flowStress;
    const double slope = -flowStress * flowStress * h / (2.0 * d->fractureEnergy[point]);
    const double floor_ = -d->youngsModulus[point];
    d->softening[point] = slope < floor_ ? floor_ : slope;
}

/* Damage.at, Damage.java:342-347 */
static double damage_at(const damage_t *d, int point, double plasticStrain) {
    const double sf = d->strength[point];
    if (sf <= 0.0) return 0.0;
    const double v = -d->softening[point] * (plasticStrain - d->failureStrain[point]) / sf;
    return v <= 0.0 ? 0.0 : (v >= 1.0 ? 1.0 : v);
}

/* Damage.dissipation, Damage.java:362-372 */
static double damage_dissipation(const damage_t *d, int point, double plasticStrain) {
    const double sf = d->strength[point];
    if (sf <= 0.0) return 0.0;
    const double slope = d->softening[point];
    const double full = -sf / slope;
    double excess = plasticStrain - d->failureStrain[point];
    if (excess <= 0.0) return 0.0;
    if (excess > full) excess = full;
    return excess * (sf + 0.5 * slope * excess);
}

/* ------------------------------------------------------------------ J2 */

/* J2.solve, J2.java:332-375 */
static double j2_solve(double norm, double stiffness, double plasticStrain,
                       double temperature, double dt, const flow_t *jc) {
    const double thermal = jc_thermalTerm(jc, temperature);
    const double tolerance = SOLVE_TOLERANCE * jc->a;
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
                       - TWO_THIRDS * jc_strainSlopeFrom(jc, strain, eps) * rateFactor * thermal;
        if (!jc_rateIsClamped(jc, rate)) {
            slope -= SQRT_2_3 * strain * jc->c * thermal / dGamma;
        }
        double next = dGamma - g / slope;
        if (!(next > lo && next < hi)) next = 0.5 * (lo + hi);
        dGamma = next;
    }
    return dGamma;
}

/* J2.update, J2.java:163-296 */
static double j2_update(double *sig, double *back, double *epsP, double *work, int e,
                        double dRR, double dZZ, double dTT, double dGamRZ,
                        double lambda, double mu, const flow_t *flow, double strainDt,
                        const damage_t *damage) {
    const int s = COMPONENTS * e;
    const double lt = lambda * (dRR + dZZ + dTT);
    const double tRR = sig[s] + lt + 2.0 * mu * dRR;
    const double tZZ = sig[s + 1] + lt + 2.0 * mu * dZZ;
    const double tTT = sig[s + 2] + lt + 2.0 * mu * dTT;
    const double tRZ = sig[s + 3] + mu * dGamRZ;

    const double p = (tRR + tZZ + tTT) / 3.0;
    const double xRR = tRR - p - back[s];
    const double xZZ = tZZ - p - back[s + 1];
    const double xTT = tTT - p - back[s + 2];
    const double xRZ = tRZ - back[s + 3];
    const double norm = sqrt(xRR * xRR + xZZ * xZZ + xTT * xTT + 2.0 * xRZ * xRZ);

    const int jc = flow->jc;
    const double temperature = !jc ? 0.0 : flow->room + flow->thermalCoefficient * work[e];

    const int softening = damage != NULL && damage->strength[e] > 0.0;
    double hardening = 0.0;
    double flowStress;
    if (softening) {
        flowStress = damage->strength[e]
                     + damage->softening[e] * (epsP[e] - damage->failureStrain[e]);
        if (flowStress > 0.0) {
            hardening = damage->softening[e];
        } else {
            flowStress = 0.0;
        }
    } else if (!jc) {
        flowStress = flow->sy0 + flow->hIso * epsP[e];
        hardening = flow->hIso;
    } else {
        flowStress = jc_quasiStatic(flow, epsP[e], temperature);
    }
    const double radius = SQRT_2_3 * flowStress;

    if (!(norm > radius)) {
        sig[s] = tRR;
        sig[s + 1] = tZZ;
        sig[s + 2] = tTT;
        sig[s + 3] = tRZ;
        return 0.0;
    }

    const double stiffness = 2.0 * mu + TWO_THIRDS * flow->hKin;
    double dGamma;
    if (!jc || softening) {
        dGamma = (norm - radius) / (stiffness + TWO_THIRDS * hardening);
        if (softening && flowStress + hardening * SQRT_2_3 * dGamma < 0.0) {
            dGamma = norm / stiffness;
        }
    } else {
        dGamma = j2_solve(norm, stiffness, epsP[e], temperature, strainDt, flow);
    }
    const double inv = 1.0 / norm;
    const double nRR = xRR * inv, nZZ = xZZ * inv, nTT = xTT * inv, nRZ = xRZ * inv;

    const double pull = 2.0 * mu * dGamma;
    sig[s] = tRR - pull * nRR;
    sig[s + 1] = tZZ - pull * nZZ;
    sig[s + 2] = tTT - pull * nTT;
    sig[s + 3] = tRZ - pull * nRZ;

    const double alphaDotN = back[s] * nRR + back[s + 1] * nZZ + back[s + 2] * nTT
                             + 2.0 * back[s + 3] * nRZ;
    work[e] += dGamma * (norm - pull + alphaDotN);

    const double shift = TWO_THIRDS * flow->hKin * dGamma;
    back[s] += shift * nRR;
    back[s + 1] += shift * nZZ;
    back[s + 2] += shift * nTT;
    back[s + 3] += shift * nRZ;

    epsP[e] += SQRT_2_3 * dGamma;

    if (damage != NULL && !softening && epsP[e] >= damage->failureStrain[e]) {
        damage_begin(damage, e,
                     !jc ? flow->sy0 + flow->hIso * epsP[e]
                         : jc_quasiStatic(flow, epsP[e], temperature),
                     nRR, nZZ, nRZ);
    }
    return dGamma;
}

/* ------------------------------------------------------------------ corotational */

static void corot_rotate(double *t, int index, double c, double sn) {  /* :59-71 */
    const int s = COMPONENTS * index;
    const double rr = t[s], zz = t[s + 1], rz = t[s + 3];
    const double cc = c * c, ss = sn * sn, cs = c * sn;
    t[s] = cc * rr - 2.0 * cs * rz + ss * zz;
    t[s + 1] = ss * rr + 2.0 * cs * rz + cc * zz;
    t[s + 3] = cs * (rr - zz) + (cc - ss) * rz;
}
static double corot_cos(double spinDt) {                                /* :88-91 */
    const double h = 0.5 * spinDt;
    return (1.0 - h * h) / (1.0 + h * h);
}
static double corot_sin(double spinDt) {                                /* :94-97 */
    const double h = 0.5 * spinDt;
    return 2.0 * h / (1.0 + h * h);
}

/* ------------------------------------------------------------------ free surface */

typedef struct { int32_t *edges; int32_t *owner; int32_t *nodes; int edgeCount, nodeCount; } surface_t;

typedef struct { int64_t key; int idx; } keyidx_t;
static int cmp_keyidx(const void *a, const void *b) {
    const keyidx_t *x = (const keyidx_t *)a, *y = (const keyidx_t *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->idx - y->idx;
}

/* QuadMesh.surface(skip), QuadMesh.java:188-226. The HashMap count is a sort here; the
 * emission order is element order as in the reference. */
static surface_t mesh_surface(int E, int N, const int32_t *conn, const uint8_t *skip) {
    surface_t out;
    keyidx_t *keys = (keyidx_t *)malloc(sizeof(keyidx_t) * (size_t)(4 * (E > 0 ? E : 1)));
    int *count = (int *)calloc((size_t)(4 * (E > 0 ? E : 1)), sizeof(int));
    int nk = 0;
    for (int e = 0; e < E; e++) {
        if (skip && skip[e]) continue;
        for (int k = 0; k < 4; k++) {
            const int a = conn[e * 4 + k], b = conn[e * 4 + (k + 1) % 4];
            const int lo = a < b ? a : b, hi = a < b ? b : a;
            keys[nk].key = ((int64_t)lo << 32) | (uint32_t)hi;
            keys[nk].idx = e * 4 + k;
            nk++;
        }
    }
    qsort(keys, (size_t)nk, sizeof(keyidx_t), cmp_keyidx);
    for (int i = 0; i < nk;) {
        int j = i;
        while (j < nk && keys[j].key == keys[i].key) j++;
        for (int q = i; q < j; q++) count[keys[q].idx] = j - i;
        i = j;
    }
    int freeEdges = 0;
    for (int e = 0; e < E; e++) {
        if (skip && skip[e]) continue;
        for (int k = 0; k < 4; k++) if (count[e * 4 + k] == 1) freeEdges++;
    }
    out.edgeCount = freeEdges;
    out.edges = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * freeEdges + 2));
    out.owner = (int32_t *)malloc(sizeof(int32_t) * (size_t)(freeEdges + 1));
    uint8_t *onSurface = (uint8_t *)calloc((size_t)(N + 1), 1);
    int at = 0;
    for (int e = 0; e < E; e++) {
        if (skip && skip[e]) continue;
        for (int k = 0; k < 4; k++) {
            if (count[e * 4 + k] != 1) continue;
            const int a = conn[e * 4 + k], b = conn[e * 4 + (k + 1) % 4];
            out.edges[2 * at] = a;
            out.edges[2 * at + 1] = b;
            out.owner[at] = e;
            at++;
            onSurface[a] = 1;
            onSurface[b] = 1;
        }
    }
    int n = 0;
    for (int i = 0; i < N; i++) if (onSurface[i]) n++;
    out.nodeCount = n;
    out.nodes = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int m = 0;
    for (int i = 0; i < N; i++) if (onSurface[i]) out.nodes[m++] = i;
    free(onSurface);
    free(count);
    free(keys);
    return out;
}

static void surface_free(surface_t *s) {
    free(s->edges); free(s->owner); free(s->nodes);
    memset(s, 0, sizeof *s);
}

/* ------------------------------------------------------------------ contact */

typedef struct {
    uint8_t *dead;
    int stale;
    surface_t surface;
    int32_t *slot, *segStart, *segOf;
    double friction, scale, damping;
    double step, reference;
    double *cr, *cz, *nr, *nz, *length, *pnr, *pnz;
    int32_t *lastMaster, *master;
    uint8_t *dropped;
    double cellSize, gridR0, gridZ0;
    int gridCols, gridRows, buckets;
    int32_t *bucketStart, *bucketOf;
    int bucketStartCap, bucketOfCap;
    int pairs, escaped;
    double energy, dissipation, maxPenetration;
} contact_t;

typedef struct nfo_solver nfo_solver;

typedef struct {
    nfo_solver *h;
    int from, to, worker;
    int kind;
} job_t;

struct nfo_solver {
    int N, E, K;
    double *r, *z;
    int32_t *conn, *pedges;
    int formulation, integration, kinematics;
    double thickness, cflSafety;
    int nmat;
    flow_t *flows;
    nf_material *mats;
    int32_t *emat;
    double *lambdaOf, *muOf, *bulkOf, *densityOf;
    double fastestWave, dt0, dt, dtPrevious, minEdgeSquared, time;
    int64_t stepCount;
    double *ur, *uz, *vr, *vz, *fr, *fz, *mass;
    uint8_t *fixedR, *fixedZ, *onWall, *wallState;
    int ppe;
    double *sig, *back, *epsP, *wPlastic, *hgR, *hgZ, *hgK;
    double *contribution;
    int edgeSlotBase;
    int32_t *nodeSlotStart, *nodeSlot;
    double damping, targetPressure, rampDuration, hourglassCoefficient;
    double kernelStrainDt, kernelPressure, nodalDecay, nodalGain, nodalDtAvg;
    int hasWall;
    double wallPlane, wallFriction, wImpulse, wEnergyLoss, wFriction;
    int wContact, wStuck;
    contact_t *contact;
    uint8_t *contactState;
    double gravR, gravZ;
    uint8_t *gone;
    double massScale, erosionDamage, erodedEnergy;
    int erodedCount, invertedCount;
    int hasDamage;
    double *dFailure, *dGf, *dE, *dGeom, *dStrength, *dSoft, *dWidth;
    damage_t dmg;
    int threads;
    double *minEdgeLocal;
    char err[512];
};

static __thread char g_err[512];

static nf_status fail(nfo_solver *h, nf_status st, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(h ? h->err : g_err, 512, fmt, ap);
    va_end(ap);
    return st;
}

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }
static int32_t *ialloc(size_t n) { return (int32_t *)calloc(n ? n : 1, sizeof(int32_t)); }
static uint8_t *balloc(size_t n) { return (uint8_t *)calloc(n ? n : 1, 1); }

/* Contact.adopt, Contact.java:290-322 */
static void contact_adopt(nfo_solver *h, contact_t *c) {
    surface_free(&c->surface);
    free(c->segStart); free(c->segOf); free(c->nr); free(c->nz); free(c->length);
    free(c->pnr); free(c->pnz); free(c->lastMaster); free(c->master); free(c->dropped);
    c->surface = mesh_surface(h->E, h->N, h->conn, c->dead);
    const int32_t *seg = c->surface.edges;
    const int nn = c->surface.nodeCount;
    for (int i = 0; i < h->N; i++) c->slot[i] = -1;
    for (int i = 0; i < nn; i++) c->slot[c->surface.nodes[i]] = i;
    const int segments = c->surface.edgeCount;
    c->segStart = ialloc((size_t)nn + 1);
    for (int s = 0; s < segments; s++) {
        c->segStart[c->slot[seg[2 * s]] + 1]++;
        c->segStart[c->slot[seg[2 * s + 1]] + 1]++;
    }
    for (int i = 0; i < nn; i++) c->segStart[i + 1] += c->segStart[i];
    c->segOf = ialloc((size_t)c->segStart[nn]);
    int32_t *fill = ialloc((size_t)nn + 1);
    memcpy(fill, c->segStart, sizeof(int32_t) * (size_t)(nn + 1));
    for (int s = 0; s < segments; s++) {
        c->segOf[fill[c->slot[seg[2 * s]]]++] = s;
        c->segOf[fill[c->slot[seg[2 * s + 1]]]++] = s;
    }
    free(fill);
    c->nr = dalloc((size_t)segments);
    c->nz = dalloc((size_t)segments);
    c->length = dalloc((size_t)segments);
    c->pnr = dalloc((size_t)nn);
    c->pnz = dalloc((size_t)nn);
    c->lastMaster = ialloc((size_t)nn);
    for (int i = 0; i < nn; i++) c->lastMaster[i] = -1;
    c->master = ialloc((size_t)nn);
    c->dropped = balloc((size_t)nn);
    c->stale = 0;
}

static contact_t *contact_new(nfo_solver *h) {
    contact_t *c = (contact_t *)calloc(1, sizeof(contact_t));
    c->dead = balloc((size_t)h->E);
    c->cr = dalloc((size_t)h->N);
    c->cz = dalloc((size_t)h->N);
    c->slot = ialloc((size_t)h->N);
    c->scale = CONTACT_DEFAULT_SCALE;
    c->damping = 0.0;
    contact_adopt(h, c);
    return c;
}

static void contact_free(contact_t *c) {
    if (!c) return;
    surface_free(&c->surface);
    free(c->dead); free(c->cr); free(c->cz); free(c->slot); free(c->segStart); free(c->segOf);
    free(c->nr); free(c->nz); free(c->length); free(c->pnr); free(c->pnz);
    free(c->lastMaster); free(c->master); free(c->dropped); free(c->bucketStart);
    free(c->bucketOf);
    free(c);
}

/* Contact.geometry, Contact.java:467-500 */
static void contact_geometry(nfo_solver *h, contact_t *c) {
    const int32_t *seg = c->surface.edges;
    for (int i = 0; i < c->surface.nodeCount; i++) {
        const int n = c->surface.nodes[i];
        c->cr[n] = h->r[n] + h->ur[n];
        c->cz[n] = h->z[n] + h->uz[n];
    }
    for (int s = 0; s < c->surface.edgeCount; s++) {
        const int a = seg[2 * s], b = seg[2 * s + 1];
        const double dr = c->cr[b] - c->cr[a], dz = c->cz[b] - c->cz[a];
        const double len = sqrt(dr * dr + dz * dz);
        c->length[s] = len;
        if (len > 0.0) {
            c->nr[s] = dz / len;
            c->nz[s] = -dr / len;
        } else {
            c->nr[s] = 0.0;
            c->nz[s] = 0.0;
        }
    }
    for (int i = 0; i < c->surface.nodeCount; i++) {
        double sr = 0.0, sz = 0.0;
        for (int k = c->segStart[i]; k < c->segStart[i + 1]; k++) {
            sr += c->nr[c->segOf[k]];
            sz += c->nz[c->segOf[k]];
        }
        const double len = sqrt(sr * sr + sz * sz);
        c->pnr[i] = len > 0.0 ? sr / len : 0.0;
        c->pnz[i] = len > 0.0 ? sz / len : 0.0;
    }
}

static int iclamp(int v, int n) { return v < 0 ? 0 : v >= n ? n - 1 : v; }

static int contact_cellOf(const contact_t *c, double r, double z) {   /* :547-551 */
    const int i = iclamp(jd2i((r - c->gridR0) / c->cellSize), c->gridCols);
    const int j = iclamp(jd2i((z - c->gridZ0) / c->cellSize), c->gridRows);
    return j * c->gridCols + i;
}

/* Contact.grid, Contact.java:515-545 */
static void contact_grid(contact_t *c) {
    const int segments = c->surface.edgeCount;
    const int32_t *seg = c->surface.edges;
    double rlo = DBL_MAX, zlo = DBL_MAX, rhi = -DBL_MAX, zhi = -DBL_MAX;
    double longest = 0.0;
    for (int i = 0; i < c->surface.nodeCount; i++) {
        const int n = c->surface.nodes[i];
        if (c->cr[n] < rlo) rlo = c->cr[n];
        if (c->cr[n] > rhi) rhi = c->cr[n];
        if (c->cz[n] < zlo) zlo = c->cz[n];
        if (c->cz[n] > zhi) zhi = c->cz[n];
    }
    for (int s = 0; s < segments; s++) if (c->length[s] > longest) longest = c->length[s];
    c->cellSize = longest > 0.0 ? 1.5 * longest : 1.0;
    c->gridR0 = rlo;
    c->gridZ0 = zlo;
    {
        const int a = jd2i((rhi - rlo) / c->cellSize) + 1;
        const int b = jd2i((zhi - zlo) / c->cellSize) + 1;
        c->gridCols = a > 1 ? a : 1;
        c->gridRows = b > 1 ? b : 1;
    }
    c->buckets = c->gridCols * c->gridRows;
    if (c->bucketStartCap < c->buckets + 1) {
        free(c->bucketStart);
        c->bucketStartCap = c->buckets + 1;
        c->bucketStart = ialloc((size_t)c->bucketStartCap);
    } else {
        memset(c->bucketStart, 0, sizeof(int32_t) * (size_t)(c->buckets + 1));
    }
    if (c->bucketOfCap < 2 * segments) {
        free(c->bucketOf);
        c->bucketOfCap = 2 * segments;
        c->bucketOf = ialloc((size_t)c->bucketOfCap);
    }
    for (int s = 0; s < segments; s++) {
        c->bucketStart[contact_cellOf(c, c->cr[seg[2 * s]], c->cz[seg[2 * s]]) + 1]++;
        c->bucketStart[contact_cellOf(c, c->cr[seg[2 * s + 1]], c->cz[seg[2 * s + 1]]) + 1]++;
    }
    for (int q = 0; q < c->buckets; q++) c->bucketStart[q + 1] += c->bucketStart[q];
    int32_t *fill = ialloc((size_t)c->buckets + 1);
    memcpy(fill, c->bucketStart, sizeof(int32_t) * (size_t)(c->buckets + 1));
    for (int s = 0; s < segments; s++) {
        c->bucketOf[fill[contact_cellOf(c, c->cr[seg[2 * s]], c->cz[seg[2 * s]])]++] = s;
        c->bucketOf[fill[contact_cellOf(c, c->cr[seg[2 * s + 1]], c->cz[seg[2 * s + 1]])]++] = s;
    }
    free(fill);
}

/* Contact.excluded, Contact.java:620-639 */
static int contact_excluded(const contact_t *c, int i, int n, int s) {
    const int32_t *seg = c->surface.edges;
    const int a = seg[2 * s], b = seg[2 * s + 1];
    if (c->pnr[i] * c->nr[s] + c->pnz[i] * c->nz[s] > -FACING) return 1;
    if (a == n || b == n) return 1;
    for (int k = c->segStart[i]; k < c->segStart[i + 1]; k++) {
        const int own = c->segOf[k];
        const int p = seg[2 * own], q = seg[2 * own + 1];
        if (p == a || p == b || q == a || q == b) return 1;
    }
    return 0;
}

/* Contact.depth, Contact.java:642-652 */
static double contact_depth(const contact_t *c, int n, int s) {
    const int32_t *seg = c->surface.edges;
    const int a = seg[2 * s], b = seg[2 * s + 1];
    const double len = c->length[s];
    if (len <= 0.0) return 0.0;
    const double tr = (c->cr[b] - c->cr[a]) / len, tz = (c->cz[b] - c->cz[a]) / len;
    const double dr = c->cr[n] - c->cr[a], dz = c->cz[n] - c->cz[a];
    const double along = dr * tr + dz * tz;
    if (along < 0.0 || along > len) return 0.0;
    const double gap = dr * c->nr[s] + dz * c->nz[s];
    return gap < 0.0 ? -gap : 0.0;
}

/* Contact.parameter, Contact.java:655-661 */
static double contact_parameter(const contact_t *c, int n, int s) {
    const int32_t *seg = c->surface.edges;
    const int a = seg[2 * s];
    const double len = c->length[s];
    const double tr = (c->cr[seg[2 * s + 1]] - c->cr[a]) / len;
    const double tz = (c->cz[seg[2 * s + 1]] - c->cz[a]) / len;
    return ((c->cr[n] - c->cr[a]) * tr + (c->cz[n] - c->cz[a]) * tz) / len;
}

/* Contact.nearestPenetrated, Contact.java:570-606 */
static int contact_nearest(contact_t *c, int i, int n) {
    const int ci = iclamp(jd2i((c->cr[n] - c->gridR0) / c->cellSize), c->gridCols);
    const int cj = iclamp(jd2i((c->cz[n] - c->gridZ0) / c->cellSize), c->gridRows);
    int best = -1;
    double deepest = 0.0;
    int fell = 0;
    for (int dj = -1; dj <= 1; dj++) {
        const int j = cj + dj;
        if (j < 0 || j >= c->gridRows) continue;
        for (int di = -1; di <= 1; di++) {
            const int ii = ci + di;
            if (ii < 0 || ii >= c->gridCols) continue;
            const int cell = j * c->gridCols + ii;
            for (int k = c->bucketStart[cell]; k < c->bucketStart[cell + 1]; k++) {
                const int s = c->bucketOf[k];
                if (contact_excluded(c, i, n, s)) continue;
                const double depth = contact_depth(c, n, s);
                if (depth <= 0.0) continue;
                if (depth > MAX_DEPTH * c->length[s]) {
                    if (s == c->lastMaster[i]) fell = 1;
                    continue;
                }
                if (depth > deepest) {
                    deepest = depth;
                    best = s;
                }
            }
        }
    }
    c->dropped[i] = (uint8_t)fell;
    return best;
}

/* Contact.resolve, Contact.java:663-762 */
static void contact_resolve(nfo_solver *h, contact_t *c, int i, int n, int s) {
    (void)i;
    double *vr = h->vr, *vz = h->vz, *mass = h->mass, *fr = h->fr, *fz = h->fz;
    const int32_t *seg = c->surface.edges;
    const double dt = c->step;
    const int a = seg[2 * s], b = seg[2 * s + 1];
    const double depth = contact_depth(c, n, s);
    const double t = contact_parameter(c, n, s);
    const double wa = 1.0 - t, wb = t;
    const double invMaster = 0.25 / mass[a] + 0.25 / mass[b];
    if (!(invMaster > 0.0)) return;
    const double mMaster = 1.0 / invMaster;
    const double mSlave = mass[n];
    const double mStar = mSlave * mMaster / (mSlave + mMaster);
    const double k = c->scale * mStar / (c->reference * c->reference);
    const double nR = c->nr[s], nZ = c->nz[s];
    const double mTrue = 1.0 / (wa * wa / mass[a] + wb * wb / mass[b]);
    const double mTangent = mSlave * mTrue / (mSlave + mTrue);
    const double closing = (vr[n] - wa * vr[a] - wb * vr[b]) * nR
                           + (vz[n] - wa * vz[a] - wb * vz[b]) * nZ;
    const double damper = 2.0 * c->damping * mStar * sqrt(c->scale) / c->reference;
    const double normal = jmax(0.0, k * depth - damper * closing);

    fr[n] += normal * nR;
    fz[n] += normal * nZ;
    fr[a] -= wa * normal * nR;
    fz[a] -= wa * normal * nZ;
    fr[b] -= wb * normal * nR;
    fz[b] -= wb * normal * nZ;

    c->pairs++;
    c->energy += 0.5 * k * depth * depth;
    if (depth > c->maxPenetration) c->maxPenetration = depth;
    const double damperForce = normal - k * depth;
    if (damperForce != 0.0) {
        const double closingAfter = closing + damperForce * dt / mTangent;
        c->dissipation -= damperForce * 0.5 * (closing + closingAfter) * dt;
    }
    h->contactState[n] = NF_CONTACT_PAIR;
    if (c->friction <= 0.0) return;

    const double tR = -nZ, tZ = nR;
    const double slide = (vr[n] - wa * vr[a] - wb * vr[b]) * tR
                         + (vz[n] - wa * vz[a] - wb * vz[b]) * tZ;
    double tangent = -STICK_RELAXATION * mTangent * slide / dt;
    const double cone = c->friction * normal;
    int slipped = 0;
    if (tangent > cone) { tangent = cone; slipped = 1; }
    else if (tangent < -cone) { tangent = -cone; slipped = 1; }
    h->contactState[n] = (uint8_t)(NF_CONTACT_PAIR | (slipped ? NF_CONTACT_SLIP : NF_CONTACT_STICK));

    fr[n] += tangent * tR;
    fz[n] += tangent * tZ;
    fr[a] -= wa * tangent * tR;
    fz[a] -= wa * tangent * tZ;
    fr[b] -= wb * tangent * tR;
    fz[b] -= wb * tangent * tZ;

    const double after = slide + tangent * dt / mTangent;
    c->dissipation += -tangent * 0.5 * (slide + after) * dt;
}

/* Contact.begin, Contact.java:424-436 */
static int contact_begin(nfo_solver *h, contact_t *c, double dt, double referenceStep) {
    c->step = dt;
    c->reference = referenceStep;
    if (c->stale) contact_adopt(h, c);
    c->pairs = 0;
    c->energy = 0.0;
    c->maxPenetration = 0.0;
    if (c->surface.edgeCount == 0) return 0;
    contact_geometry(h, c);
    contact_grid(c);
    return c->surface.nodeCount;
}

static void contact_search(contact_t *c, int from, int to) {          /* :439-443 */
    for (int i = from; i < to; i++) c->master[i] = contact_nearest(c, i, c->surface.nodes[i]);
}

static void contact_accumulate(nfo_solver *h, contact_t *c) {         /* :446-462 */
    for (int i = 0; i < c->surface.nodeCount; i++) {
        const int n = c->surface.nodes[i];
        const int best = c->master[i];
        if (best < 0) {
            if (c->lastMaster[i] >= 0 && c->dropped[i]) c->escaped++;
            c->lastMaster[i] = -1;
            continue;
        }
        c->lastMaster[i] = best;
        contact_resolve(h, c, i, n, best);
    }
}

/* ------------------------------------------------------------------ solver kernels */

static double cr_(const nfo_solver *h, int node, double shift) {      /* :1176-1178 */
    return h->kinematics == NF_FINITE_STRAIN ? h->r[node] + h->ur[node] + shift * h->vr[node]
                                             : h->r[node];
}
static double cz_(const nfo_solver *h, int node, double shift) {      /* :1180-1182 */
    return h->kinematics == NF_FINITE_STRAIN ? h->z[node] + h->uz[node] + shift * h->vz[node]
                                             : h->z[node];
}
static double sq(double a, double b) { return a * a + b * b; }
static double shortestEdge(double running, double r0, double r1, double r2, double r3,
                           double z0, double z1, double z2, double z3) {   /* :1191-1197 */
    return jmin(running, jmin(jmin(sq(r1 - r0, z1 - z0), sq(r2 - r1, z2 - z1)),
                              jmin(sq(r3 - r2, z3 - z2), sq(r0 - r3, z0 - z3))));
}

static double pressureAt(const nfo_solver *h, double t) {             /* :1203-1207 */
    if (h->rampDuration <= 0.0) return h->targetPressure;
    double s = jmin(1.0, t / h->rampDuration);
    return h->targetPressure * s * s * (3.0 - 2.0 * s);
}

static const damage_t *dmg_of(const nfo_solver *h) { return h->hasDamage ? &h->dmg : NULL; }

/* fullIntegration, ExplicitSolver.java:1219-1339 */
static double fullIntegration(nfo_solver *h, double strainDt, int from, int to) {
    const int32_t *conn = h->conn;
    double *ef = h->contribution;
    const int axi = h->formulation == NF_AXISYMMETRIC;
    const int finite = h->kinematics == NF_FINITE_STRAIN;
    const double mid = -0.5 * strainDt;
    const damage_t *dmg = dmg_of(h);
    double minEdge = DBL_MAX;
    (void)G_PT;

    for (int e = from; e < to; e++) {
        const int b = e * 4;
        if (h->gone != NULL && h->gone[e]) {
            for (int k = 0; k < 8; k++) ef[b * 2 + k] = 0.0;
            continue;
        }
        const flow_t *fl = &h->flows[h->emat[e]];
        const double lambda = h->lambdaOf[e], mu = h->muOf[e];
        const int n0 = conn[b], n1 = conn[b + 1], n2 = conn[b + 2], n3 = conn[b + 3];
        const double r0 = cr_(h, n0, mid), r1 = cr_(h, n1, mid), r2 = cr_(h, n2, mid), r3 = cr_(h, n3, mid);
        const double z0 = cz_(h, n0, mid), z1 = cz_(h, n1, mid), z2 = cz_(h, n2, mid), z3 = cz_(h, n3, mid);
        const double a0 = h->vr[n0] * strainDt, a1 = h->vr[n1] * strainDt;
        const double a2 = h->vr[n2] * strainDt, a3 = h->vr[n3] * strainDt;
        const double c0 = h->vz[n0] * strainDt, c1 = h->vz[n1] * strainDt;
        const double c2 = h->vz[n2] * strainDt, c3 = h->vz[n3] * strainDt;

        if (finite) minEdge = shortestEdge(minEdge, r0, r1, r2, r3, z0, z1, z2, z3);

        double g0r = 0, g1r = 0, g2r = 0, g3r = 0;
        double g0z = 0, g1z = 0, g2z = 0, g3z = 0;

        for (int g = 0; g < 4; g++) {
            const double xi = GP_XI[g], eta = GP_ETA[g];
            const double xm = 1.0 - xi, xp = 1.0 + xi;
            const double em = 1.0 - eta, ep = 1.0 + eta;
            const double N0 = 0.25 * xm * em, N1 = 0.25 * xp * em;
            const double N2 = 0.25 * xp * ep, N3 = 0.25 * xm * ep;
            const double dN0x = -0.25 * em, dN1x = 0.25 * em, dN2x = 0.25 * ep, dN3x = -0.25 * ep;
            const double dN0e = -0.25 * xm, dN1e = -0.25 * xp, dN2e = 0.25 * xp, dN3e = 0.25 * xm;

            const double J00 = dN0x * r0 + dN1x * r1 + dN2x * r2 + dN3x * r3;
            const double J01 = dN0x * z0 + dN1x * z1 + dN2x * z2 + dN3x * z3;
            const double J10 = dN0e * r0 + dN1e * r1 + dN2e * r2 + dN3e * r3;
            const double J11 = dN0e * z0 + dN1e * z1 + dN2e * z2 + dN3e * z3;
            const double det = J00 * J11 - J01 * J10;
            const double inv = 1.0 / det;

            const double d0r = (J11 * dN0x - J01 * dN0e) * inv;
            const double d1r = (J11 * dN1x - J01 * dN1e) * inv;
            const double d2r = (J11 * dN2x - J01 * dN2e) * inv;
            const double d3r = (J11 * dN3x - J01 * dN3e) * inv;
            const double d0z = (-J10 * dN0x + J00 * dN0e) * inv;
            const double d1z = (-J10 * dN1x + J00 * dN1e) * inv;
            const double d2z = (-J10 * dN2x + J00 * dN2e) * inv;
            const double d3z = (-J10 * dN3x + J00 * dN3e) * inv;

            const double dEpsR = d0r * a0 + d1r * a1 + d2r * a2 + d3r * a3;
            const double dEpsZ = d0z * c0 + d1z * c1 + d2z * c2 + d3z * c3;
            const double dRdZ = d0z * a0 + d1z * a1 + d2z * a2 + d3z * a3;
            const double dZdR = d0r * c0 + d1r * c1 + d2r * c2 + d3r * c3;
            const double dGamRZ = dRdZ + dZdR;

            double rg = 0.0, dEpsT = 0.0;
            if (axi) {
                rg = N0 * r0 + N1 * r1 + N2 * r2 + N3 * r3;
                dEpsT = (N0 * a0 + N1 * a1 + N2 * a2 + N3 * a3) / rg;
            }
            const int p = e * 4 + g;
            if (finite) {
                const double spinDt = 0.5 * (dZdR - dRdZ);
                if (spinDt != 0.0) {
                    const double cs = corot_cos(spinDt), sn = corot_sin(spinDt);
                    corot_rotate(h->sig, p, cs, sn);
                    corot_rotate(h->back, p, cs, sn);
                }
            }
            j2_update(h->sig, h->back, h->epsP, h->wPlastic, p, dEpsR, dEpsZ, dEpsT, dGamRZ,
                      lambda, mu, fl, strainDt, dmg);

            const int s = COMPONENTS * p;
            const double sR = h->sig[s], sZ = h->sig[s + 1], sT = h->sig[s + 2], sRZ = h->sig[s + 3];
            const double dV = axi ? 2.0 * NF_PI * rg * det : h->thickness * det;
            if (axi) {
                const double hh = sT / rg * dV;
                g0r -= (d0r * sR + d0z * sRZ) * dV + N0 * hh;
                g1r -= (d1r * sR + d1z * sRZ) * dV + N1 * hh;
                g2r -= (d2r * sR + d2z * sRZ) * dV + N2 * hh;
                g3r -= (d3r * sR + d3z * sRZ) * dV + N3 * hh;
            } else {
                g0r -= (d0r * sR + d0z * sRZ) * dV;
                g1r -= (d1r * sR + d1z * sRZ) * dV;
                g2r -= (d2r * sR + d2z * sRZ) * dV;
                g3r -= (d3r * sR + d3z * sRZ) * dV;
            }
            g0z -= (d0z * sZ + d0r * sRZ) * dV;
            g1z -= (d1z * sZ + d1r * sRZ) * dV;
            g2z -= (d2z * sZ + d2r * sRZ) * dV;
            g3z -= (d3z * sZ + d3r * sRZ) * dV;
        }
        ef[b * 2] = g0r; ef[b * 2 + 1] = g1r; ef[b * 2 + 2] = g2r; ef[b * 2 + 3] = g3r;
        ef[b * 2 + 4] = g0z; ef[b * 2 + 5] = g1z; ef[b * 2 + 6] = g2z; ef[b * 2 + 7] = g3z;
    }
    return minEdge;
}

/* reducedIntegration, ExplicitSolver.java:1373-1504 */
static double reducedIntegration(nfo_solver *h, double strainDt, int from, int to) {
    const int32_t *conn = h->conn;
    double *ef = h->contribution;
    const int axi = h->formulation == NF_AXISYMMETRIC;
    const int finite = h->kinematics == NF_FINITE_STRAIN;
    const double mid = -0.5 * strainDt;
    const double qhg = h->hourglassCoefficient;
    const damage_t *dmg = dmg_of(h);
    double minEdge = DBL_MAX;

    for (int e = from; e < to; e++) {
        const int b = e * 4;
        if (h->gone != NULL && h->gone[e]) {
            for (int k = 0; k < 8; k++) ef[b * 2 + k] = 0.0;
            continue;
        }
        const flow_t *fl = &h->flows[h->emat[e]];
        const double lambda = h->lambdaOf[e], mu = h->muOf[e];
        const int n0 = conn[b], n1 = conn[b + 1], n2 = conn[b + 2], n3 = conn[b + 3];
        const double r0 = cr_(h, n0, mid), r1 = cr_(h, n1, mid), r2 = cr_(h, n2, mid), r3 = cr_(h, n3, mid);
        const double z0 = cz_(h, n0, mid), z1 = cz_(h, n1, mid), z2 = cz_(h, n2, mid), z3 = cz_(h, n3, mid);
        const double a0 = h->vr[n0] * strainDt, a1 = h->vr[n1] * strainDt;
        const double a2 = h->vr[n2] * strainDt, a3 = h->vr[n3] * strainDt;
        const double c0 = h->vz[n0] * strainDt, c1 = h->vz[n1] * strainDt;
        const double c2 = h->vz[n2] * strainDt, c3 = h->vz[n3] * strainDt;

        if (finite) minEdge = shortestEdge(minEdge, r0, r1, r2, r3, z0, z1, z2, z3);

        const double J00 = 0.25 * (-r0 + r1 + r2 - r3);
        const double J01 = 0.25 * (-z0 + z1 + z2 - z3);
        const double J10 = 0.25 * (-r0 - r1 + r2 + r3);
        const double J11 = 0.25 * (-z0 - z1 + z2 + z3);
        const double det = J00 * J11 - J01 * J10;
        const double inv = 1.0 / det;

        const double d0r = 0.25 * (J01 - J11) * inv;
        const double d1r = 0.25 * (J01 + J11) * inv;
        const double d2r = -d0r;
        const double d3r = -d1r;
        const double d0z = 0.25 * (J10 - J00) * inv;
        const double d1z = -0.25 * (J10 + J00) * inv;
        const double d2z = -d0z;
        const double d3z = -d1z;

        const double dEpsR = d0r * a0 + d1r * a1 + d2r * a2 + d3r * a3;
        const double dEpsZ = d0z * c0 + d1z * c1 + d2z * c2 + d3z * c3;
        const double dRdZ = d0z * a0 + d1z * a1 + d2z * a2 + d3z * a3;
        const double dZdR = d0r * c0 + d1r * c1 + d2r * c2 + d3r * c3;
        const double dGamRZ = dRdZ + dZdR;

        double rg = 0.0, dEpsT = 0.0;
        if (axi) {
            rg = 0.25 * (r0 + r1 + r2 + r3);
            dEpsT = 0.25 * (a0 + a1 + a2 + a3) / rg;
        }
        if (finite) {
            const double spinDt = 0.5 * (dZdR - dRdZ);
            if (spinDt != 0.0) {
                const double cs = corot_cos(spinDt), sn = corot_sin(spinDt);
                corot_rotate(h->sig, e, cs, sn);
                corot_rotate(h->back, e, cs, sn);
            }
        }
        j2_update(h->sig, h->back, h->epsP, h->wPlastic, e, dEpsR, dEpsZ, dEpsT, dGamRZ,
                  lambda, mu, fl, strainDt, dmg);

        const int s = COMPONENTS * e;
        const double sR = h->sig[s], sZ = h->sig[s + 1], sT = h->sig[s + 2], sRZ = h->sig[s + 3];
        const double dV = W_REDUCED * (axi ? 2.0 * NF_PI * rg * det : h->thickness * det);

        double g0r, g1r, g2r, g3r;
        if (axi) {
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

        if (qhg > 0.0) {
            const double hr = r0 - r1 + r2 - r3;
            const double hz = z0 - z1 + z2 - z3;
            const double y0 = HG[0] - hr * d0r - hz * d0z;
            const double y1 = HG[1] - hr * d1r - hz * d1z;
            const double y2 = HG[2] - hr * d2r - hz * d2z;
            const double y3 = HG[3] - hr * d3r - hz * d3z;
            const double k = qhg * mu * dV
                             * (d0r * d0r + d1r * d1r + d2r * d2r + d3r * d3r
                                + d0z * d0z + d1z * d1z + d2z * d2z + d3z * d3z);
            h->hgR[e] += k * (y0 * a0 + y1 * a1 + y2 * a2 + y3 * a3);
            h->hgZ[e] += k * (y0 * c0 + y1 * c1 + y2 * c2 + y3 * c3);
            const double qr = h->hgR[e], qz = h->hgZ[e];
            g0r -= y0 * qr; g1r -= y1 * qr; g2r -= y2 * qr; g3r -= y3 * qr;
            g0z -= y0 * qz; g1z -= y1 * qz; g2z -= y2 * qz; g3z -= y3 * qz;
            h->hgK[e] = k;
        }
        ef[b * 2] = g0r; ef[b * 2 + 1] = g1r; ef[b * 2 + 2] = g2r; ef[b * 2 + 3] = g3r;
        ef[b * 2 + 4] = g0z; ef[b * 2 + 5] = g1z; ef[b * 2 + 6] = g2z; ef[b * 2 + 7] = g3z;
    }
    return minEdge;
}

/* applyPressure, ExplicitSolver.java:1511-1556 */
static void applyPressure(nfo_solver *h, double p, int from, int to) {
    const int32_t *edges = h->pedges;
    double *c = h->contribution;
    for (int e = from; e < to; e++) {
        const int k = 2 * e;
        const int slot = (h->edgeSlotBase + e) * 8;
        const int a = edges[k], bnode = edges[k + 1];
        const double ra = cr_(h, a, 0.0), rb = cr_(h, bnode, 0.0);
        const double tr = rb - ra;
        const double tz = cz_(h, bnode, 0.0) - cz_(h, a, 0.0);
        const double len = sqrt(tr * tr + tz * tz);
        if (len == 0.0) {
            c[slot] = 0.0; c[slot + 1] = 0.0; c[slot + 4] = 0.0; c[slot + 5] = 0.0;
            continue;
        }
        const double nr = tz / len;
        const double nz = -tr / len;
        double wa, wb;
        if (h->formulation == NF_AXISYMMETRIC) {
            const double circumference = 2.0 * NF_PI * len;
            wa = circumference * (ra / 3.0 + rb / 6.0);
            wb = circumference * (ra / 6.0 + rb / 3.0);
        } else {
            wa = h->thickness * len * 0.5;
            wb = wa;
        }
        c[slot] = p * nr * wa;
        c[slot + 1] = p * nr * wb;
        c[slot + 4] = p * nz * wa;
        c[slot + 5] = p * nz * wb;
    }
}

/* assemble, ExplicitSolver.java:1126-1137 */
static void assemble(nfo_solver *h, int from, int to, int worker) {
    const int ne = h->edgeSlotBase;
    if (from < ne) {
        const int end = to < ne ? to : ne;
        const double edge = h->integration == NF_FULL
                            ? fullIntegration(h, h->kernelStrainDt, from, end)
                            : reducedIntegration(h, h->kernelStrainDt, from, end);
        if (edge < h->minEdgeLocal[worker]) h->minEdgeLocal[worker] = edge;
    }
    if (to > ne) applyPressure(h, h->kernelPressure, (from > ne ? from : ne) - ne, to - ne);
}

/* gather, ExplicitSolver.java:1147-1165 */
static void gather(nfo_solver *h, int from, int to) {
    const double *c = h->contribution;
    const int32_t *slots = h->nodeSlot;
    for (int n = from; n < to; n++) {
        double sr = 0.0, sz = 0.0;
        const int end = h->nodeSlotStart[n + 1];
        for (int k = h->nodeSlotStart[n]; k < end; k++) {
            const int slot = slots[k];
            sr += c[slot];
            sz += c[slot + 4];
        }
        h->fr[n] = sr + h->mass[n] * h->gravR;
        h->fz[n] = sz + h->mass[n] * h->gravZ;
    }
}

/* ---- the thread pool: fixed contiguous chunks, joined per region */

enum { JOB_ASSEMBLE = 0, JOB_GATHER = 1, JOB_SEARCH = 2 };

static void *job_run(void *arg) {
    job_t *j = (job_t *)arg;
    if (j->kind == JOB_ASSEMBLE) assemble(j->h, j->from, j->to, j->worker);
    else if (j->kind == JOB_GATHER) gather(j->h, j->from, j->to);
    else contact_search(j->h->contact, j->from, j->to);
    return NULL;
}

static void parallel_run(nfo_solver *h, int count, int kind) {
    const int t = h->threads;
    if (t <= 1 || count < 2 * t) {
        job_t j = {h, 0, count, 0, kind};
        job_run(&j);
        return;
    }
    pthread_t tid[64];
    job_t jobs[64];
    for (int w = 0; w < t; w++) {
        jobs[w].h = h;
        jobs[w].from = (int)((int64_t)count * w / t);
        jobs[w].to = (int)((int64_t)count * (w + 1) / t);
        jobs[w].worker = w;
        jobs[w].kind = kind;
    }
    for (int w = 1; w < t; w++) pthread_create(&tid[w], NULL, job_run, &jobs[w]);
    job_run(&jobs[0]);
    for (int w = 1; w < t; w++) pthread_join(tid[w], NULL);
}

/* advanceMaterialAndAssemble, ExplicitSolver.java:1081-1115 */
static void advanceMaterialAndAssemble(nfo_solver *h, double strainDt) {
    h->kernelStrainDt = strainDt;
    h->kernelPressure = pressureAt(h, h->time);
    const int workers = h->threads > 0 ? h->threads : 1;
    for (int w = 0; w < workers; w++) h->minEdgeLocal[w] = DBL_MAX;
    const int sources = h->edgeSlotBase + h->K;
    parallel_run(h, sources, JOB_ASSEMBLE);
    parallel_run(h, h->N, JOB_GATHER);
    if (h->contact != NULL) {
        memset(h->contactState, 0, (size_t)h->N);
        const int slaves = contact_begin(h, h->contact, h->dt, h->dt0);
        if (slaves > 0) {
            parallel_run(h, slaves, JOB_SEARCH);
            contact_accumulate(h, h->contact);
        }
    }
    h->minEdgeSquared = DBL_MAX;
    for (int w = 0; w < workers; w++) h->minEdgeSquared = jmin(h->minEdgeSquared, h->minEdgeLocal[w]);
}

/* RigidWall.slide, RigidWall.java:236-259 */
static double wall_slide(nfo_solver *h, int i, double forceR, double forceZ, double velocityR,
                         double decay, double gain, double nodeMass, double dt) {
    const double normal = -forceZ;
    const double trial = -nodeMass * decay * velocityR / gain - forceR;
    const double limit = isinf(h->wallFriction) ? INFINITY : h->wallFriction * normal;
    if (fabs(trial) <= limit) {
        h->wEnergyLoss += 0.5 * nodeMass * velocityR * velocityR;
        h->wStuck++;
        h->wallState[i] |= NF_WALL_STUCK;
        return 0.0;
    }
    const double tangential = copysign(limit, trial);
    const double slid = decay * velocityR + gain * (forceR + tangential) / nodeMass;
    h->wFriction += -tangential * slid * dt;
    h->wallState[i] |= NF_WALL_SLID;
    return slid;
}

/* nodalUpdate, ExplicitSolver.java:998-1062 */
static void nodalUpdate(nfo_solver *h, int from, int to) {
    const double decay = h->nodalDecay;
    const double gain = h->nodalGain;
    const double dtAvg = h->nodalDtAvg;
    const double dt = h->dt;
    for (int i = from; i < to; i++) {
        const double invM = 1.0 / h->mass[i];
        const int resting = h->hasWall && h->onWall[i] && h->fz[i] <= 0.0;
        h->wallState[i] = 0;
        if (h->fixedR[i]) {
            h->vr[i] = 0.0;
        } else if (resting && h->wallFriction > 0.0) {
            h->vr[i] = wall_slide(h, i, h->fr[i], h->fz[i], h->vr[i], decay, gain, h->mass[i], dt);
            h->ur[i] += h->vr[i] * dt;
        } else {
            h->vr[i] = decay * h->vr[i] + gain * h->fr[i] * invM;
            h->ur[i] += h->vr[i] * dt;
        }
        if (h->fixedZ[i]) {
            h->vz[i] = 0.0;
        } else if (resting) {
            h->wImpulse += -h->fz[i] * dtAvg;        /* RigidWall.hold, :178-181 */
            h->wContact++;
            h->wallState[i] |= NF_WALL_HELD;
        } else {
            const double trial = decay * h->vz[i] + gain * h->fz[i] * invM;
            const double zc = h->z[i] + h->uz[i];
            if (h->hasWall && zc + trial * dt < h->wallPlane) {   /* RigidWall.crosses :187-189 */
                h->wImpulse += -h->mass[i] * trial;                /* RigidWall.arrive :205-209 */
                h->wEnergyLoss += 0.5 * h->mass[i] * trial * trial;
                h->wContact++;
                h->uz[i] += h->wallPlane - zc;
                h->vz[i] = 0.0;
                h->onWall[i] = 1;
                h->wallState[i] |= NF_WALL_ARRIVED;
            } else {
                h->vz[i] = trial;
                h->uz[i] += h->vz[i] * dt;
                if (h->hasWall) h->onWall[i] = 0;
            }
        }
    }
}

/* gaussVolume, ExplicitSolver.java:1939-1965 */
static double gaussVolume(const nfo_solver *h, int element, int g) {
    const int b = element * 4;
    const int n0 = h->conn[b], n1 = h->conn[b + 1], n2 = h->conn[b + 2], n3 = h->conn[b + 3];
    const double r0 = h->r[n0], r1 = h->r[n1], r2 = h->r[n2], r3 = h->r[n3];
    const double z0 = h->z[n0], z1 = h->z[n1], z2 = h->z[n2], z3 = h->z[n3];
    const double xi = h->ppe == 1 ? 0.0 : GP_XI[g];
    const double eta = h->ppe == 1 ? 0.0 : GP_ETA[g];
    const double weight = h->ppe == 1 ? W_REDUCED : 1.0;
    const double xm = 1.0 - xi, xp = 1.0 + xi, em = 1.0 - eta, ep = 1.0 + eta;
    const double N0 = 0.25 * xm * em, N1 = 0.25 * xp * em;
    const double N2 = 0.25 * xp * ep, N3 = 0.25 * xm * ep;
    const double dN0x = -0.25 * em, dN1x = 0.25 * em, dN2x = 0.25 * ep, dN3x = -0.25 * ep;
    const double dN0e = -0.25 * xm, dN1e = -0.25 * xp, dN2e = 0.25 * xp, dN3e = 0.25 * xm;
    const double J00 = dN0x * r0 + dN1x * r1 + dN2x * r2 + dN3x * r3;
    const double J01 = dN0x * z0 + dN1x * z1 + dN2x * z2 + dN3x * z3;
    const double J10 = dN0e * r0 + dN1e * r1 + dN2e * r2 + dN3e * r3;
    const double J11 = dN0e * z0 + dN1e * z1 + dN2e * z2 + dN3e * z3;
    const double det = J00 * J11 - J01 * J10;
    const double rg = N0 * r0 + N1 * r1 + N2 * r2 + N3 * r3;
    return weight * (h->formulation == NF_AXISYMMETRIC ? 2.0 * NF_PI * rg * det : h->thickness * det);
}

/* pointStrainEnergy, ExplicitSolver.java:1666-1675 */
static double pointStrainEnergy(const nfo_solver *h, int e, int g) {
    const int p = e * h->ppe + g;
    const int s = COMPONENTS * p;
    const double *sig = h->sig;
    const double press = (sig[s] + sig[s + 1] + sig[s + 2]) / 3.0;
    const double a = sig[s] - press, bb = sig[s + 1] - press, c = sig[s + 2] - press;
    const double d = sig[s + 3];
    const double density = (a * a + bb * bb + c * c + 2.0 * d * d) / (4.0 * h->muOf[e])
                           + press * press / (2.0 * h->bulkOf[e]);
    return density * gaussVolume(h, e, g);
}

static double elementDamage(const nfo_solver *h, int element) {     /* :1764-1772 */
    if (!h->hasDamage) return 0.0;
    double sum = 0.0;
    for (int g = 0; g < h->ppe; g++) {
        const int p = element * h->ppe + g;
        sum += damage_at(&h->dmg, p, h->epsP[p]);
    }
    return sum / h->ppe;
}

static double currentArea(const nfo_solver *h, int element) {       /* :681-691 */
    const int b = element * 4;
    double a = 0.0;
    for (int k = 0; k < 4; k++) {
        const int i = h->conn[b + k];
        const int j = h->conn[b + (k + 1) % 4];
        a += (h->r[i] + h->ur[i]) * (h->z[j] + h->uz[j])
             - (h->r[j] + h->ur[j]) * (h->z[i] + h->uz[i]);
    }
    return 0.5 * a;
}

/* erode, ExplicitSolver.java:663-678 */
static void erode(nfo_solver *h) {
    for (int e = 0; e < h->E; e++) {
        if (h->gone[e]) continue;
        const int failed = h->hasDamage && elementDamage(h, e) >= h->erosionDamage;
        const int inverted = currentArea(h, e) <= 0.0;
        if (!failed && !inverted) continue;
        h->gone[e] = 1;
        h->erodedCount++;
        if (inverted && !failed) h->invertedCount++;
        for (int g = 0; g < h->ppe; g++) h->erodedEnergy += pointStrainEnergy(h, e, g);
        if (h->contact != NULL) {
            h->contact->dead[e] = 1;               /* Contact.forget, :329-332 */
            h->contact->stale = 1;
        }
    }
}

/* step, ExplicitSolver.java:940-991 */
static void step_body(nfo_solver *h);
static void step(nfo_solver *h) {
    if (h->stepCount == 0) advanceMaterialAndAssemble(h, 0.0);
    step_body(h);
}
static void step_body(nfo_solver *h) {
    const double dtAvg = 0.5 * (h->dtPrevious + h->dt);
    const double half = 0.5 * h->damping * dtAvg;
    h->nodalDecay = (1.0 - half) / (1.0 + half);
    h->nodalGain = dtAvg / (1.0 + half);
    h->nodalDtAvg = dtAvg;
    if (h->hasWall) { h->wContact = 0; h->wStuck = 0; }     /* RigidWall.beginStep :153-156 */
    nodalUpdate(h, 0, h->N);
    h->time += h->dt;
    h->stepCount++;
    if (h->gone != NULL) erode(h);
    advanceMaterialAndAssemble(h, h->dt);
    if (h->kinematics == NF_FINITE_STRAIN) {
        h->dtPrevious = h->dt;
        h->dt = h->cflSafety * sqrt(h->minEdgeSquared * h->massScale) / h->fastestWave;
    }
}

/* lumpMass, ExplicitSolver.java:1559-1597 */
static void lumpMass(nfo_solver *h) {
    const int axi = h->formulation == NF_AXISYMMETRIC;
    for (int e = 0; e < h->E; e++) {
        const double rho = h->densityOf[e];
        const int b = e * 4;
        const int n0 = h->conn[b], n1 = h->conn[b + 1], n2 = h->conn[b + 2], n3 = h->conn[b + 3];
        const double r0 = h->r[n0], r1 = h->r[n1], r2 = h->r[n2], r3 = h->r[n3];
        const double z0 = h->z[n0], z1 = h->z[n1], z2 = h->z[n2], z3 = h->z[n3];
        for (int g = 0; g < 4; g++) {
            const double xi = GP_XI[g], eta = GP_ETA[g];
            const double xm = 1.0 - xi, xp = 1.0 + xi;
            const double em = 1.0 - eta, ep = 1.0 + eta;
            const double N0 = 0.25 * xm * em, N1 = 0.25 * xp * em;
            const double N2 = 0.25 * xp * ep, N3 = 0.25 * xm * ep;
            const double dN0x = -0.25 * em, dN1x = 0.25 * em, dN2x = 0.25 * ep, dN3x = -0.25 * ep;
            const double dN0e = -0.25 * xm, dN1e = -0.25 * xp, dN2e = 0.25 * xp, dN3e = 0.25 * xm;
            const double J00 = dN0x * r0 + dN1x * r1 + dN2x * r2 + dN3x * r3;
            const double J01 = dN0x * z0 + dN1x * z1 + dN2x * z2 + dN3x * z3;
            const double J10 = dN0e * r0 + dN1e * r1 + dN2e * r2 + dN3e * r3;
            const double J11 = dN0e * z0 + dN1e * z1 + dN2e * z2 + dN3e * z3;
            const double det = J00 * J11 - J01 * J10;
            const double rg = N0 * r0 + N1 * r1 + N2 * r2 + N3 * r3;
            const double dV = axi ? 2.0 * NF_PI * rg * det : h->thickness * det;
            h->mass[n0] += rho * N0 * dV;
            h->mass[n1] += rho * N1 * dV;
            h->mass[n2] += rho * N2 * dV;
            h->mass[n3] += rho * N3 * dV;
        }
    }
}

static double signedArea(const nfo_solver *h, int element) {        /* QuadMesh.java:78-87 */
    const int b = element * 4;
    double a = 0.0;
    for (int k = 0; k < 4; k++) {
        const int i = h->conn[b + k];
        const int j = h->conn[b + (k + 1) % 4];
        a += h->r[i] * h->z[j] - h->r[j] * h->z[i];
    }
    return 0.5 * a;
}

/* ------------------------------------------------------------------ API */

#define API __attribute__((visibility("default")))

API const char *nfo_last_error(const nfo_solver *h) { return h ? h->err : g_err; }

API void nfo_destroy(nfo_solver *h) {
    if (!h) return;
    free(h->r); free(h->z); free(h->conn); free(h->pedges); free(h->flows); free(h->mats);
    free(h->emat); free(h->lambdaOf); free(h->muOf); free(h->bulkOf); free(h->densityOf);
    free(h->ur); free(h->uz); free(h->vr); free(h->vz); free(h->fr); free(h->fz); free(h->mass);
    free(h->fixedR); free(h->fixedZ); free(h->onWall); free(h->wallState);
    free(h->sig); free(h->back); free(h->epsP); free(h->wPlastic); free(h->hgR); free(h->hgZ);
    free(h->hgK); free(h->contribution); free(h->nodeSlotStart); free(h->nodeSlot);
    free(h->contactState); free(h->gone); free(h->dFailure); free(h->dGf); free(h->dE);
    free(h->dGeom); free(h->dStrength); free(h->dSoft); free(h->dWidth); free(h->minEdgeLocal);
    contact_free(h->contact);
    free(h);
}

/* ExplicitSolver constructor, :264-339 */
API nf_status nfo_create(const nf_mesh *mesh, const nf_material *materials, int32_t material_count,
                         const int32_t *element_material, int32_t formulation, int32_t integration,
                         int32_t kinematics, double thickness, double cfl_safety, nfo_solver **out) {
    *out = NULL;
    if (!mesh || !materials || material_count < 1)
        return fail(NULL, NF_EINVAL, "mesh and at least one material are required");
    if (mesh->node_count < 0 || mesh->element_count < 0 || mesh->pressure_edge_count < 0)
        return fail(NULL, NF_EINVAL, "negative mesh size");
    if (formulation < 0 || formulation > 2 || integration < 0 || integration > 1
        || kinematics < 0 || kinematics > 1)
        return fail(NULL, NF_EINVAL, "unknown formulation, integration or kinematics");
    for (int m = 0; m < material_count; m++) {
        const char *why = material_invalid(&materials[m]);
        if (why) return fail(NULL, NF_EINVAL, "%s", why);
        if (formulation == NF_PLANE_STRESS && !isinf(materials[m].yield_stress))
            return fail(NULL, NF_EINVAL,
                        "plane stress plasticity needs its own return map; not implemented");
    }
    const int N = mesh->node_count, E = mesh->element_count, K = mesh->pressure_edge_count;
    for (int k = 0; k < 4 * E; k++)
        if (mesh->conn[k] < 0 || mesh->conn[k] >= N)
            return fail(NULL, NF_EINVAL, "connectivity refers to node %d of %d", mesh->conn[k], N);
    for (int k = 0; k < 2 * K; k++)
        if (mesh->pressure_edges[k] < 0 || mesh->pressure_edges[k] >= N)
            return fail(NULL, NF_EINVAL, "pressure edge refers to node %d of %d",
                        mesh->pressure_edges[k], N);
    if (element_material)
        for (int e = 0; e < E; e++)
            if (element_material[e] < 0 || element_material[e] >= material_count)
                return fail(NULL, NF_EINVAL, "element %d has no material", e);

    nfo_solver *h = (nfo_solver *)calloc(1, sizeof(nfo_solver));
    h->N = N; h->E = E; h->K = K;
    h->r = dalloc((size_t)N); memcpy(h->r, mesh->r, sizeof(double) * (size_t)N);
    h->z = dalloc((size_t)N); memcpy(h->z, mesh->z, sizeof(double) * (size_t)N);
    h->conn = ialloc((size_t)4 * E); memcpy(h->conn, mesh->conn, sizeof(int32_t) * (size_t)(4 * E));
    h->pedges = ialloc((size_t)2 * K);
    if (K) memcpy(h->pedges, mesh->pressure_edges, sizeof(int32_t) * (size_t)(2 * K));
    for (int e = 0; e < E; e++) {
        if (signedArea(h, e) <= 0.0) {
            nfo_destroy(h);
            return fail(NULL, NF_ESTATE,
                        "element %d has non-positive area; node ordering must be "
                        "counter-clockwise in (r, z)", e);
        }
    }
    h->formulation = formulation; h->integration = integration; h->kinematics = kinematics;
    h->thickness = thickness; h->cflSafety = cfl_safety;
    h->nmat = material_count;
    h->mats = (nf_material *)malloc(sizeof(nf_material) * (size_t)material_count);
    memcpy(h->mats, materials, sizeof(nf_material) * (size_t)material_count);
    h->flows = (flow_t *)malloc(sizeof(flow_t) * (size_t)material_count);
    for (int m = 0; m < material_count; m++) h->flows[m] = flow_of(&materials[m]);
    h->emat = ialloc((size_t)E);
    if (element_material) memcpy(h->emat, element_material, sizeof(int32_t) * (size_t)E);
    h->lambdaOf = dalloc((size_t)E); h->muOf = dalloc((size_t)E);
    h->bulkOf = dalloc((size_t)E); h->densityOf = dalloc((size_t)E);
    for (int e = 0; e < E; e++) {
        const nf_material *m = &materials[h->emat[e]];
        const double lam = formulation == NF_PLANE_STRESS
                           ? 2.0 * mat_lambda(m) * mat_mu(m) / (mat_lambda(m) + 2.0 * mat_mu(m))
                           : mat_lambda(m);
        h->lambdaOf[e] = lam;
        h->muOf[e] = mat_mu(m);
        h->bulkOf[e] = lam + 2.0 * mat_mu(m) / 3.0;
        h->densityOf[e] = m->density;
    }
    /* Materials.fastestWave, Materials.java:118-127 */
    if (!element_material || material_count == 1) {
        h->fastestWave = mat_wave(&materials[0]);
    } else {
        double fastest = 0.0;
        for (int e = 0; e < E; e++) {
            const double c = mat_wave(&materials[h->emat[e]]);
            if (c > fastest) fastest = c;
        }
        h->fastestWave = fastest;
    }
    h->ur = dalloc((size_t)N); h->uz = dalloc((size_t)N); h->vr = dalloc((size_t)N);
    h->vz = dalloc((size_t)N); h->fr = dalloc((size_t)N); h->fz = dalloc((size_t)N);
    h->mass = dalloc((size_t)N);
    h->fixedR = balloc((size_t)N); h->fixedZ = balloc((size_t)N); h->onWall = balloc((size_t)N);
    h->wallState = balloc((size_t)N); h->contactState = balloc((size_t)N);
    h->ppe = integration == NF_FULL ? 4 : 1;
    const size_t points = (size_t)E * (size_t)h->ppe;
    h->sig = dalloc(COMPONENTS * points); h->back = dalloc(COMPONENTS * points);
    h->epsP = dalloc(points); h->wPlastic = dalloc(points);
    h->hgR = dalloc((size_t)E); h->hgZ = dalloc((size_t)E); h->hgK = dalloc((size_t)E);
    h->edgeSlotBase = E;
    h->contribution = dalloc((size_t)8 * (size_t)(E + K));
    h->nodeSlotStart = ialloc((size_t)N + 1);
    h->nodeSlot = ialloc((size_t)4 * E + 2 * K);
    /* buildNodeSlots, :347-366 */
    for (int k = 0; k < 4 * E; k++) h->nodeSlotStart[h->conn[k] + 1]++;
    for (int k = 0; k < 2 * K; k++) h->nodeSlotStart[h->pedges[k] + 1]++;
    for (int i = 0; i < N; i++) h->nodeSlotStart[i + 1] += h->nodeSlotStart[i];
    {
        int32_t *cursor = ialloc((size_t)N + 1);
        memcpy(cursor, h->nodeSlotStart, sizeof(int32_t) * (size_t)(N + 1));
        for (int e = 0; e < E; e++)
            for (int c = 0; c < 4; c++) h->nodeSlot[cursor[h->conn[e * 4 + c]]++] = e * 8 + c;
        for (int k = 0; k < 2 * K; k += 2) {
            const int slot = (h->edgeSlotBase + k / 2) * 8;
            h->nodeSlot[cursor[h->pedges[k]]++] = slot;
            h->nodeSlot[cursor[h->pedges[k + 1]]++] = slot + 1;
        }
        free(cursor);
    }
    h->threads = 1;
    h->minEdgeLocal = dalloc(64);
    h->hourglassCoefficient = DEFAULT_HOURGLASS_COEFFICIENT;
    h->massScale = 1.0;
    h->erosionDamage = INFINITY;
    lumpMass(h);
    /* QuadMesh.minimumEdgeLength, QuadMesh.java:59-75 */
    double edge = DBL_MAX;
    for (int e = 0; e < E; e++) {
        for (int k = 0; k < 4; k++) {
            const int i = h->conn[e * 4 + k], j = h->conn[e * 4 + (k + 1) % 4];
            const double dr = h->r[j] - h->r[i], dz = h->z[j] - h->z[i];
            const double len = sqrt(dr * dr + dz * dz);
            if (len < edge) edge = len;
        }
    }
    h->minEdgeSquared = edge * edge;
    h->dt = cfl_safety * edge / h->fastestWave;
    h->dt0 = h->dt;
    h->dtPrevious = h->dt;
    *out = h;
    return NF_OK;
}

API nf_status nfo_set_threads(nfo_solver *h, int32_t n) {
    if (n < 1) return fail(h, NF_EINVAL, "need at least one thread");
    h->threads = n > 64 ? 64 : n;
    return NF_OK;
}
API nf_status nfo_fix_radial(nfo_solver *h, int32_t node) {
    if (node < 0 || node >= h->N) return fail(h, NF_EINVAL, "node %d out of range", node);
    h->fixedR[node] = 1;
    return NF_OK;
}
API nf_status nfo_fix_axial(nfo_solver *h, int32_t node) {
    if (node < 0 || node >= h->N) return fail(h, NF_EINVAL, "node %d out of range", node);
    h->fixedZ[node] = 1;
    return NF_OK;
}
API nf_status nfo_fix_all_axial(nfo_solver *h) {
    memset(h->fixedZ, 1, (size_t)h->N);
    return NF_OK;
}
API nf_status nfo_set_pressure_ramp(nfo_solver *h, double pascals, double ramp) {
    h->targetPressure = pascals;
    h->rampDuration = ramp;
    return NF_OK;
}
API nf_status nfo_set_relaxation_damping(nfo_solver *h, double fraction, double omega) {
    if (omega <= 0.0) return fail(h, NF_EINVAL, "angular frequency must be positive");
    h->damping = 2.0 * fraction * omega;
    return NF_OK;
}
API nf_status nfo_set_hourglass_coefficient(nfo_solver *h, double q) {
    if (q < 0.0) return fail(h, NF_EINVAL, "hourglass coefficient must be >= 0");
    h->hourglassCoefficient = q;
    return NF_OK;
}
API nf_status nfo_set_rigid_wall(nfo_solver *h, double plane, double friction) {
    if (friction < 0.0 || friction != friction)
        return fail(h, NF_EINVAL, "friction coefficient must be >= 0");
    h->hasWall = 1;
    h->wallPlane = plane;
    h->wallFriction = friction;
    h->wImpulse = h->wEnergyLoss = h->wFriction = 0.0;
    h->wContact = h->wStuck = 0;
    return NF_OK;
}
API nf_status nfo_clear_rigid_wall(nfo_solver *h) { h->hasWall = 0; return NF_OK; }
API nf_status nfo_set_contact(nfo_solver *h, double friction, double damping, double scale) {
    if (friction < 0.0) return fail(h, NF_EINVAL, "friction must not be negative");
    if (damping < 0.0 || damping > 1.0)
        return fail(h, NF_EINVAL,
                    "contact damping is a fraction of critical, so it lies in [0, 1]; was %.17g",
                    damping);
    if (!(scale > 0.0) || scale >= 2.0)
        return fail(h, NF_EINVAL,
                    "the stiffness scale must lie in (0, 2); a pair is found from both sides, "
                    "so the effective stiffness is twice this and above 2 the contact "
                    "frequency exceeds what central difference can integrate, was %.17g", scale);
    contact_free(h->contact);
    h->contact = contact_new(h);
    h->contact->friction = friction;
    h->contact->damping = damping;
    h->contact->scale = scale;
    return NF_OK;
}
API nf_status nfo_clear_contact(nfo_solver *h) {
    contact_free(h->contact);
    h->contact = NULL;
    return NF_OK;
}
API nf_status nfo_set_gravity(nfo_solver *h, double ar, double az) {
    h->gravR = ar;
    h->gravZ = az;
    return NF_OK;
}
API nf_status nfo_set_erosion(nfo_solver *h, double threshold) {
    if (!h->hasDamage)
        return fail(h, NF_ESTATE, "erosion needs a failure model; call setDamage first");
    if (!(threshold > 0.0) || threshold > 1.0)
        return fail(h, NF_EINVAL,
                    "the erosion threshold is a damage, so it lies in (0, 1]; was %.17g", threshold);
    h->erosionDamage = threshold;
    if (h->gone == NULL) h->gone = balloc((size_t)h->E);
    return NF_OK;
}
API nf_status nfo_set_mass_scaling(nfo_solver *h, double target) {
    if (!(target > 0.0)) return fail(h, NF_EINVAL, "the target step must be positive");
    if (target < h->dt)
        return fail(h, NF_EINVAL,
                    "the step is already %.17g s, longer than the target %.17g; mass scaling adds "
                    "mass and cannot shorten a step", h->dt, target);
    const double factor = (target / h->dt) * (target / h->dt);
    for (int i = 0; i < h->N; i++) h->mass[i] *= factor;
    h->massScale *= factor;
    h->dt = target;
    h->dtPrevious = h->dt;
    h->dt0 = h->dt;
    return NF_OK;
}

/* setDamage(double[], double[]), ExplicitSolver.java:729-791 and the Damage constructor
 * Damage.java:224-262 */
API nf_status nfo_set_damage(nfo_solver *h, const double *gf, const double *eps) {
    for (int m = 0; m < h->nmat; m++) {
        const nf_material *mm = &h->mats[m];
        const double worst = 2.0 * mat_mu(mm) + (2.0 / 3.0) * (mm->kinematic_hardening - mm->youngs_modulus);
        if (!(worst > 0.0))
            return fail(h, NF_EINVAL,
                        "a fully clamped softening modulus would make the return map singular: "
                        "2mu + (2/3)(H_kin - E) = %.17g <= 0", worst);
    }
    const int P = h->E * h->ppe;
    double *perPoint = dalloc((size_t)P), *gfOf = dalloc((size_t)P), *eOf = dalloc((size_t)P);
    double *geometry = dalloc((size_t)GEOMETRY_STRIDE * P);
    for (int e = 0; e < h->E; e++) {
        const int b = e * 4;
        const int n0 = h->conn[b], n1 = h->conn[b + 1], n2 = h->conn[b + 2], n3 = h->conn[b + 3];
        const double uR = 0.5 * (h->r[n1] - h->r[n0] + h->r[n2] - h->r[n3]);
        const double uZ = 0.5 * (h->z[n1] - h->z[n0] + h->z[n2] - h->z[n3]);
        const double vR = 0.5 * (h->r[n3] - h->r[n0] + h->r[n2] - h->r[n1]);
        const double vZ = 0.5 * (h->z[n3] - h->z[n0] + h->z[n2] - h->z[n1]);
        const double area = fabs(signedArea(h, e));
        for (int g = 0; g < h->ppe; g++) {
            const int p = e * h->ppe + g;
            perPoint[p] = eps[e];
            gfOf[p] = gf[e];
            eOf[p] = h->mats[h->emat[e]].youngs_modulus;
            const int q = GEOMETRY_STRIDE * p;
            geometry[q] = area;
            geometry[q + 1] = uR;
            geometry[q + 2] = uZ;
            geometry[q + 3] = vR;
            geometry[q + 4] = vZ;
        }
    }
    nf_status st = NF_OK;
    for (int p = 0; p < P && st == NF_OK; p++) {
        if (!(gfOf[p] > 0.0)) st = fail(h, NF_EINVAL, "fracture energy must be positive, was %.17g", gfOf[p]);
        else if (!(eOf[p] > 0.0)) st = fail(h, NF_EINVAL, "Young's modulus must be positive, was %.17g", eOf[p]);
    }
    for (int p = 0; p < P && st == NF_OK; p++) {
        if (!(perPoint[p] > 0.0))
            st = fail(h, NF_EINVAL, "failure strain must be positive; point %d has %.17g", p, perPoint[p]);
        else if (!(geometry[GEOMETRY_STRIDE * p] > 0.0))
            st = fail(h, NF_EINVAL, "area must be positive; point %d has %.17g", p, geometry[GEOMETRY_STRIDE * p]);
    }
    if (st != NF_OK) {
        free(perPoint); free(gfOf); free(eOf); free(geometry);
        return st;
    }
    free(h->dFailure); free(h->dGf); free(h->dE); free(h->dGeom);
    free(h->dStrength); free(h->dSoft); free(h->dWidth);
    h->dFailure = perPoint; h->dGf = gfOf; h->dE = eOf; h->dGeom = geometry;
    h->dStrength = dalloc((size_t)P); h->dSoft = dalloc((size_t)P); h->dWidth = dalloc((size_t)P);
    h->dmg.failureStrain = h->dFailure;
    h->dmg.fractureEnergy = h->dGf;
    h->dmg.youngsModulus = h->dE;
    h->dmg.geometry = h->dGeom;
    h->dmg.strength = h->dStrength;
    h->dmg.softening = h->dSoft;
    h->dmg.width = h->dWidth;
    h->hasDamage = 1;
    return NF_OK;
}
API nf_status nfo_set_velocity(nfo_solver *h, int32_t node, double vr, double vz) {
    if (node < 0 || node >= h->N) return fail(h, NF_EINVAL, "node %d out of range", node);
    h->vr[node] = vr;
    h->vz[node] = vz;
    return NF_OK;
}
API nf_status nfo_set_uniform_velocity(nfo_solver *h, double vr, double vz) {
    for (int i = 0; i < h->N; i++) { h->vr[i] = vr; h->vz[i] = vz; }
    return NF_OK;
}
API nf_status nfo_set_velocities(nfo_solver *h, const double *vr, const double *vz) {
    memcpy(h->vr, vr, sizeof(double) * (size_t)h->N);
    memcpy(h->vz, vz, sizeof(double) * (size_t)h->N);
    return NF_OK;
}
API nf_status nfo_step(nfo_solver *h, int64_t steps) {
    for (int64_t i = 0; i < steps; i++) step(h);
    return NF_OK;
}
API nf_status nfo_advance(nfo_solver *h) {                    /* :1069-1075 */
    for (int i = 0; i < h->N; i++) {
        if (!h->fixedR[i]) h->ur[i] += h->vr[i] * h->dt;
        if (!h->fixedZ[i]) h->uz[i] += h->vz[i] * h->dt;
    }
    advanceMaterialAndAssemble(h, h->dt);
    return NF_OK;
}
API nf_status nfo_run_until(nfo_solver *h, double t_end, int64_t max_steps, int64_t *taken) {
    int64_t n = 0;
    while (h->time < t_end && n < max_steps) { step(h); n++; }
    if (taken) *taken = n;
    return NF_OK;
}
API nf_status nfo_synchronize(nfo_solver *h) { (void)h; return NF_OK; }
API nf_status nfo_status_word(nfo_solver *h, uint32_t *w) { (void)h; *w = 0; return NF_OK; }
/* The CPU twin of nf_check: nothing here waits, so only the finiteness of the nodal
 * velocities and displacements is checked (the device's NF_STATUS_NONFINITE test). */
API nf_status nfo_check(nfo_solver *h) {
    for (int i = 0; i < h->N; i++)
        if (!isfinite(h->ur[i]) || !isfinite(h->uz[i]) || !isfinite(h->vr[i]) ||
            !isfinite(h->vz[i]))
            return fail(h, NF_EDEVICE, "a nodal velocity or displacement is not finite "
                                       "(status word 0x%x)", 1u);
    return NF_OK;
}
API nf_status nfo_set_wait_limit(nfo_solver *h, int64_t polls, int64_t ns) {
    if (polls < 0 || ns < 0)
        return fail(h, NF_EINVAL, "wait limits must be >= 0 (0 restores the default)");
    return NF_OK;
}

API nf_status nfo_set_grid_slots(nfo_solver *h, int32_t slots) {
    /* the oracle files its buckets by a counting sort only; the setting is validated */
    if (slots < 0 || slots > 64) return fail(h, NF_EINVAL, "grid slots must be in [0, 64]");
    return NF_OK;
}

static nf_status field_desc(nfo_solver *h, int field, void **ptr, size_t *count, size_t *bytes) {
    const size_t N = (size_t)h->N, E = (size_t)h->E, P = (size_t)h->E * (size_t)h->ppe;
    *ptr = NULL; *count = 0; *bytes = 8;
    switch (field) {
        case NF_FIELD_UR: *ptr = h->ur; *count = N; break;
        case NF_FIELD_UZ: *ptr = h->uz; *count = N; break;
        case NF_FIELD_VR: *ptr = h->vr; *count = N; break;
        case NF_FIELD_VZ: *ptr = h->vz; *count = N; break;
        case NF_FIELD_FR: *ptr = h->fr; *count = N; break;
        case NF_FIELD_FZ: *ptr = h->fz; *count = N; break;
        case NF_FIELD_MASS: *ptr = h->mass; *count = N; break;
        case NF_FIELD_STRESS: *ptr = h->sig; *count = 4 * P; break;
        case NF_FIELD_BACK_STRESS: *ptr = h->back; *count = 4 * P; break;
        case NF_FIELD_PLASTIC_STRAIN: *ptr = h->epsP; *count = P; break;
        case NF_FIELD_PLASTIC_WORK: *ptr = h->wPlastic; *count = P; break;
        case NF_FIELD_HOURGLASS_R: *ptr = h->hgR; *count = E; break;
        case NF_FIELD_HOURGLASS_Z: *ptr = h->hgZ; *count = E; break;
        case NF_FIELD_HOURGLASS_STIFFNESS: *ptr = h->hgK; *count = E; break;
        case NF_FIELD_DAMAGE_STRENGTH: *ptr = h->dStrength; *count = h->hasDamage ? P : 0; break;
        case NF_FIELD_DAMAGE_SOFTENING: *ptr = h->dSoft; *count = h->hasDamage ? P : 0; break;
        case NF_FIELD_DAMAGE_WIDTH: *ptr = h->dWidth; *count = h->hasDamage ? P : 0; break;
        case NF_FIELD_ERODED: *ptr = h->gone; *count = h->gone ? E : 0; *bytes = 1; break;
        case NF_FIELD_ON_WALL: *ptr = h->onWall; *count = N; *bytes = 1; break;
        case NF_FIELD_WALL_STATE: *ptr = h->wallState; *count = N; *bytes = 1; break;
        case NF_FIELD_CONTACT_STATE: *ptr = h->contactState; *count = N; *bytes = 1; break;
        case NF_FIELD_FIXED: *ptr = NULL; *count = N; *bytes = 1; break;
        case NF_FIELD_CONTACT_MASTER: *ptr = NULL; *count = N; *bytes = 4; break;
        case NF_FIELD_SURFACE_EDGES:
            *ptr = h->contact ? h->contact->surface.edges : NULL;
            *count = h->contact ? 2 * (size_t)h->contact->surface.edgeCount : 0; *bytes = 4; break;
        case NF_FIELD_SURFACE_NODES:
            *ptr = h->contact ? h->contact->surface.nodes : NULL;
            *count = h->contact ? (size_t)h->contact->surface.nodeCount : 0; *bytes = 4; break;
        default: return fail(h, NF_EINVAL, "unknown field %d", field);
    }
    return NF_OK;
}

API nf_status nfo_field_size(nfo_solver *h, int32_t field, size_t *count, size_t *bytes) {
    void *p;
    return field_desc(h, field, &p, count, bytes);
}

API nf_status nfo_read_field(nfo_solver *h, int32_t field, void *dst, size_t nbytes) {
    void *p; size_t count, eb;
    nf_status st = field_desc(h, field, &p, &count, &eb);
    if (st) return st;
    if (nbytes != count * eb)
        return fail(h, NF_EINVAL, "field %d holds %zu bytes, caller passed %zu", field, count * eb, nbytes);
    if (field == NF_FIELD_FIXED) {
        uint8_t *d = (uint8_t *)dst;
        for (int i = 0; i < h->N; i++) d[i] = (uint8_t)(h->fixedR[i] | (h->fixedZ[i] << 1));
        return NF_OK;
    }
    if (field == NF_FIELD_CONTACT_MASTER) {
        int32_t *d = (int32_t *)dst;
        for (int i = 0; i < h->N; i++) d[i] = -1;
        if (h->contact)
            for (int i = 0; i < h->contact->surface.nodeCount; i++)
                d[h->contact->surface.nodes[i]] = h->contact->master[i];
        return NF_OK;
    }
    if (count) memcpy(dst, p, nbytes);
    return NF_OK;
}

API nf_status nfo_write_field(nfo_solver *h, int32_t field, const void *src, size_t nbytes) {
    switch (field) {
        case NF_FIELD_UR: case NF_FIELD_UZ: case NF_FIELD_VR: case NF_FIELD_VZ:
        case NF_FIELD_STRESS: case NF_FIELD_BACK_STRESS: case NF_FIELD_PLASTIC_STRAIN:
        case NF_FIELD_PLASTIC_WORK: break;
        default: return fail(h, NF_EINVAL, "field %d is not writable", field);
    }
    void *p; size_t count, eb;
    nf_status st = field_desc(h, field, &p, &count, &eb);
    if (st) return st;
    if (nbytes != count * eb)
        return fail(h, NF_EINVAL, "field %d holds %zu bytes, caller passed %zu", field, count * eb, nbytes);
    memcpy(p, src, nbytes);
    return NF_OK;
}

API nf_status nfo_get_state(nfo_solver *h, nf_state *o) {
    memset(o, 0, sizeof *o);
    o->time = h->time; o->timestep = h->dt; o->timestep_previous = h->dtPrevious;
    o->reference_timestep = h->dt0; o->mass_scale = h->massScale;
    o->min_edge_squared = h->minEdgeSquared; o->fastest_wave = h->fastestWave;
    o->eroded_energy = h->erodedEnergy; o->bore_pressure = pressureAt(h, h->time);
    o->steps = h->stepCount; o->eroded_elements = h->erodedCount;
    o->inverted_elements = h->invertedCount; o->node_count = h->N; o->element_count = h->E;
    o->points_per_element = h->ppe; o->pressure_edge_count = h->K;
    return NF_OK;
}

/* Audits, ExplicitSolver.java:875-886, :1610-1860 */
API nf_status nfo_audits(nfo_solver *h, nf_audit *o) {
    memset(o, 0, sizeof *o);
    const int N = h->N, E = h->E, ppe = h->ppe, P = E * ppe;
    double ke = 0.0, cke = 0.0, pz = 0.0, pr = 0.0;
    const double hh = 0.5 * h->dt;
    for (int i = 0; i < N; i++) {
        const double invM = 1.0 / h->mass[i];
        const int held = h->hasWall && h->onWall[i] && h->fz[i] <= 0.0;
        const double cvr = h->fixedR[i] ? h->vr[i] : h->vr[i] + hh * h->fr[i] * invM;
        const double cvz = h->fixedZ[i] || held ? h->vz[i] : h->vz[i] + hh * h->fz[i] * invM;
        cke += 0.5 * h->mass[i] * (cvr * cvr + cvz * cvz);
        ke += h->mass[i] * (h->vr[i] * h->vr[i] + h->vz[i] * h->vz[i]);
        pz += h->mass[i] * h->vz[i];
        pr += h->mass[i] * h->vr[i];
    }
    o->kinetic_energy = 0.5 * ke;
    o->centred_kinetic_energy = cke;
    o->axial_momentum = pz;
    o->radial_momentum = pr;
    double se = 0.0, wp = 0.0, fd = 0.0;
    for (int e = 0; e < E; e++) {
        for (int g = 0; g < ppe; g++) {
            const int p = e * ppe + g;
            const double vol = gaussVolume(h, e, g);
            if (!(h->gone != NULL && h->gone[e])) se += pointStrainEnergy(h, e, g);
            wp += h->wPlastic[p] * vol;
            if (h->hasDamage) fd += damage_dissipation(&h->dmg, p, h->epsP[p]) * vol;
        }
    }
    o->strain_energy = se;
    o->plastic_dissipation = wp;
    o->fracture_dissipation = fd;
    double hg = 0.0;
    if (!(h->integration == NF_FULL || h->hourglassCoefficient == 0.0)) {
        for (int e = 0; e < E; e++) {
            const double k = h->hgK[e];
            if (k > 0.0) hg += 0.5 * (h->hgR[e] * h->hgR[e] + h->hgZ[e] * h->hgZ[e]) / k;
        }
    }
    o->hourglass_energy = hg;
    double mx = 0.0; int yielded = 0;
    for (int p = 0; p < P; p++) { if (h->epsP[p] > mx) mx = h->epsP[p]; if (h->epsP[p] > 0.0) yielded++; }
    o->max_plastic_strain = mx;
    o->yielded_fraction = (double)yielded / P;
    o->most_damaged_element = -1;
    if (h->hasDamage) {
        double md = 0.0, worstv = 0.0; int begun = 0, failed = 0, clamped = 0, worst = -1;
        for (int p = 0; p < P; p++) {
            const double d = damage_at(&h->dmg, p, h->epsP[p]);
            if (d > md) md = d;
            if (h->dStrength[p] > 0.0) begun++;
            if (d >= 1.0) failed++;
            if (h->dSoft[p] == -h->dE[p]) clamped++;
        }
        for (int e = 0; e < E; e++)
            for (int g = 0; g < ppe; g++) {
                const int p = e * ppe + g;
                const double d = damage_at(&h->dmg, p, h->epsP[p]);
                if (d > worstv) { worstv = d; worst = e; }
            }
        o->max_damage = md;
        o->damaged_fraction = (double)begun / P;
        o->failed_fraction = (double)failed / P;
        o->clamped_points = clamped;
        o->most_damaged_element = worst;
    }
    /* maxTemperature, :1842-1846; NaN when some point has no thermal model */
    double tmax = -INFINITY;
    for (int p = 0; p < P; p++) {
        const int e = p / ppe;
        const flow_t *f = &h->flows[h->emat[e]];
        if (!f->jc) { tmax = NAN; break; }
        const double t = f->room + f->tq * h->wPlastic[p] / (h->densityOf[e] * f->cp);
        tmax = jmax(tmax, t);
    }
    o->max_temperature = tmax;
    return NF_OK;
}

API nf_status nfo_wall_stats(nfo_solver *h, nf_wall_info *o) {
    memset(o, 0, sizeof *o);
    o->present = h->hasWall;
    o->plane = h->wallPlane; o->friction = h->wallFriction;
    o->impulse = h->wImpulse; o->energy_loss = h->wEnergyLoss;
    o->friction_dissipation = h->wFriction;
    o->contact_count = h->wContact; o->stuck_count = h->wStuck;
    return NF_OK;
}

API nf_status nfo_contact_stats(nfo_solver *h, nf_contact_info *o) {
    memset(o, 0, sizeof *o);
    if (!h->contact) return NF_OK;
    contact_t *c = h->contact;
    o->present = 1; o->friction = c->friction; o->energy = c->energy;
    o->dissipation = c->dissipation; o->max_penetration = c->maxPenetration;
    o->pair_count = c->pairs; o->escaped_nodes = c->escaped; o->segment_count = c->surface.edgeCount;
    return NF_OK;
}

/* TaylorImpactCase.java:272-288 */
API nf_status nfo_measure_body(nfo_solver *h, nf_measure *o) {
    double zMax = -INFINITY, zMin = INFINITY, rMax = 0.0;
    for (int n = 0; n < h->N; n++) {
        const double zc = h->z[n] + h->uz[n];
        zMax = jmax(zMax, zc);
        zMin = jmin(zMin, zc);
        rMax = jmax(rMax, h->r[n] + h->ur[n]);
    }
    o->z_max = zMax; o->z_min = zMin; o->length = zMax - zMin; o->mushroom_diameter = 2.0 * rMax;
    return NF_OK;
}

/* J2.update per point, for the material-point tests (J2Test, RateDependentReturnMapTest,
 * DamageTest). */
API nf_status nfo_material_point_update(const nf_material *material, int32_t formulation,
                                        int32_t count, double *sig, double *back, double *eps_p,
                                        double *work, const double *strain, double strain_dt,
                                        const nf_damage_points *damage, double *dgamma) {
    const char *why = material_invalid(material);
    if (why) return fail(NULL, NF_EINVAL, "%s", why);
    const flow_t flow = flow_of(material);
    const double lam = formulation == NF_PLANE_STRESS
                       ? 2.0 * mat_lambda(material) * mat_mu(material)
                             / (mat_lambda(material) + 2.0 * mat_mu(material))
                       : mat_lambda(material);
    const double mu = mat_mu(material);
    damage_t d;
    const damage_t *dp = NULL;
    if (damage && damage->failure_strain) {
        d.failureStrain = damage->failure_strain;
        d.fractureEnergy = damage->fracture_energy;
        d.youngsModulus = damage->youngs_modulus;
        d.geometry = damage->geometry;
        d.strength = damage->strength;
        d.softening = damage->softening;
        d.width = damage->width;
        dp = &d;
    }
    for (int p = 0; p < count; p++) {
        const double g = j2_update(sig, back, eps_p, work, p, strain[4 * p], strain[4 * p + 1],
                                   strain[4 * p + 2], strain[4 * p + 3], lam, mu, &flow,
                                   strain_dt, dp);
        if (dgamma) dgamma[p] = g;
    }
    return NF_OK;
}

/* Scalar hooks into the Johnson-Cook law and the math layer, for the known-value tests. */
API double nfo_jc_flow_stress(const nf_material *m, double eps, double rate, double temperature) {
    const flow_t f = flow_of(m);
    return jc_strainTerm(&f, eps) * jc_rateTerm(&f, rate) * jc_thermalTerm(&f, temperature);
}
API double nfo_math(int which, double x, double y) {
    switch (which) {
        case 0: return nf_log(x);
        case 1: return nf_exp(x);
        case 2: return nf_pow(x, y);
        case 3: return nf_atan2(x, y);
        case 4: return nf_sin(x);
        case 5: return nf_cos(x);
        case 6: return nf_hypot(x, y);
        default: return NAN;
    }
}

/* Device-only entry points of the ABI: no-ops on the CPU. */
API nf_status nfo_set_stream(nfo_solver *h, void *stream) { (void)h; (void)stream; return NF_OK; }
/* The oracle is the FP64 algorithm; a precision request leaves it unchanged. */
API nf_status nfo_set_precision(nfo_solver *h, int32_t precision) { (void)h; (void)precision; return NF_OK; }
API nf_status nfo_profile(nfo_solver *h, int32_t enable) { (void)h; (void)enable; return NF_OK; }
API nf_status nfo_profile_read(nfo_solver *h, double *ms, int64_t *steps) {
    (void)h;
    for (int g = 0; g < NF_GROUP_COUNT; g++) ms[g] = 0.0;
    if (steps) *steps = 0;
    return NF_OK;
}
API nf_status nfo_launch_count(nfo_solver *h, int64_t *launches) { (void)h; *launches = 0; return NF_OK; }

/* ------------------------------------------------------------------ batched scenes */

/* The batched surface of include/neofiz.h as the reference runs a sweep: one solver per
 * instance, a pool of host threads over the instances (Sweep.over, app/Sweep.java:82-105),
 * each instance stepped while time < t_end. Every instance is FP64 whatever precision is
 * asked for (the oracle has one precision); launch shapes do not exist here, so the config
 * calls only store and echo what they are given. */
struct nfo_batch {
    int count;
    nfo_solver **s;
    double *tEnd;
    int32_t *nodeOff, *elemOff;
    int threads;
    double lastMs;
    nf_batch_config config;
    char err[512];
    /* the pool's shared cursor */
    pthread_mutex_t lock;
    int next;
    int64_t maxSteps;
    /* the adjoint's checkpoints, per instance */
    struct adj_ctx_s *adj;
    double adjForwardMs, adjBackwardMs;
    /* burst measurement (nfo_batch_set_burst) */
    nf_batch_burst burst;
    double *meanRadius;
    nf_burst_result *burstRes;
    double *burstTrace;
};
typedef struct nfo_batch nfo_batch;

static char g_batch_err[512];

static nf_status bfail(nfo_batch *b, nf_status st, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b ? b->err : g_batch_err, 512, fmt, ap);
    va_end(ap);
    return st;
}

API const char *nfo_batch_last_error(const nfo_batch *b) { return b ? b->err : g_batch_err; }

static void adj_free_all(nfo_batch *b);

API nf_status nfo_batch_destroy(nfo_batch *b) {
    if (!b) return NF_OK;
    adj_free_all(b);
    for (int k = 0; k < b->count; k++) nfo_destroy(b->s[k]);
    free(b->s); free(b->tEnd); free(b->nodeOff); free(b->elemOff);
    free(b->meanRadius); free(b->burstRes); free(b->burstTrace);
    pthread_mutex_destroy(&b->lock);
    free(b);
    return NF_OK;
}

API nf_status nfo_batch_create(const nf_batch_mesh *mesh, const nf_batch_instance *inst,
                               int32_t formulation, int32_t kinematics, double thickness,
                               double cfl_safety, int32_t precision, nfo_batch **out) {
    *out = NULL;
    if (!mesh || !inst || mesh->instance_count < 1)
        return bfail(NULL, NF_EINVAL, "a batch needs at least one instance and its mesh arrays");
    if (precision != NF_PRECISION_FP64 && precision != NF_PRECISION_MIXED &&
        precision != NF_PRECISION_COMPENSATED)
        return bfail(NULL, NF_EINVAL, "unknown precision %d", precision);
    const int count = mesh->instance_count;
    nfo_batch *b = (nfo_batch *)calloc(1, sizeof *b);
    b->count = count;
    b->s = (nfo_solver **)calloc((size_t)count, sizeof *b->s);
    b->tEnd = (double *)calloc((size_t)count, sizeof(double));
    b->nodeOff = ialloc((size_t)count + 1);
    b->elemOff = ialloc((size_t)count + 1);
    pthread_mutex_init(&b->lock, NULL);
    b->config.threads = 1;
    b->config.blocks_per_sm = 1;
    b->config.chunk_steps = 1;
    const char *env = getenv("NFO_THREADS");
    b->threads = env ? atoi(env) : 1;
    if (b->threads < 1) b->threads = 1;
    memcpy(b->nodeOff, mesh->node_offset, sizeof(int32_t) * ((size_t)count + 1));
    memcpy(b->elemOff, mesh->element_offset, sizeof(int32_t) * ((size_t)count + 1));
    for (int k = 0; k < count; k++) {
        const int n0 = mesh->node_offset[k], e0 = mesh->element_offset[k];
        nf_mesh m;
        m.node_count = mesh->node_offset[k + 1] - n0;
        m.element_count = mesh->element_offset[k + 1] - e0;
        const int k0 = mesh->pressure_offset ? mesh->pressure_offset[k] : 0;
        m.pressure_edge_count = mesh->pressure_offset ? mesh->pressure_offset[k + 1] - k0 : 0;
        m.r = mesh->r + n0;
        m.z = mesh->z + n0;
        m.conn = mesh->conn + 4 * (size_t)e0;
        m.pressure_edges = m.pressure_edge_count ? mesh->pressure_edges + 2 * (size_t)k0 : NULL;
        nf_status st = nfo_create(&m, &inst[k].material, 1, NULL, formulation, NF_REDUCED,
                                  kinematics, thickness, cfl_safety, &b->s[k]);
        if (!st) st = nfo_set_hourglass_coefficient(b->s[k], inst[k].hourglass);
        if (!st) st = nfo_set_pressure_ramp(b->s[k], inst[k].pressure, inst[k].pressure_ramp);
        if (!st && inst[k].damping_omega > 0.0)
            st = nfo_set_relaxation_damping(b->s[k], inst[k].damping_fraction, inst[k].damping_omega);
        if (!st && mesh->failure_strain)
            st = nfo_set_damage(b->s[k], mesh->fracture_energy + e0, mesh->failure_strain + e0);
        for (int i = 0; !st && mesh->fixed && i < m.node_count; i++) {
            if (mesh->fixed[n0 + i] & 1) st = nfo_fix_radial(b->s[k], i);
            if (!st && (mesh->fixed[n0 + i] & 2)) st = nfo_fix_axial(b->s[k], i);
        }
        if (!st && inst[k].wall_plane == inst[k].wall_plane)
            st = nfo_set_rigid_wall(b->s[k], inst[k].wall_plane, inst[k].wall_friction);
        if (!st) st = nfo_set_uniform_velocity(b->s[k], inst[k].velocity_r, inst[k].velocity_z);
        if (st) {
            bfail(NULL, st, "instance %d: %s", k, b->s[k] ? nfo_last_error(b->s[k]) : nfo_last_error(NULL));
            nfo_batch_destroy(b);
            return st;
        }
        b->tEnd[k] = inst[k].t_end;
    }
    *out = b;
    return NF_OK;
}

API nf_status nfo_batch_tune(nfo_batch *b, int32_t trial_steps, nf_batch_config *chosen) {
    (void)trial_steps;
    if (chosen) *chosen = b->config;
    return NF_OK;
}
API nf_status nfo_batch_set_config(nfo_batch *b, const nf_batch_config *c) {
    b->config = *c;
    return NF_OK;
}
API nf_status nfo_batch_get_config(nfo_batch *b, nf_batch_config *c) {
    *c = b->config;
    return NF_OK;
}

static void burst_run_instance(nfo_batch *b, int k);

static void *batch_worker(void *arg) {
    nfo_batch *b = (nfo_batch *)arg;
    for (;;) {
        pthread_mutex_lock(&b->lock);
        const int k = b->next++;
        pthread_mutex_unlock(&b->lock);
        if (k >= b->count) return NULL;
        if (b->burst.sample_every > 0) burst_run_instance(b, k);
        else nfo_run_until(b->s[k], b->tEnd[k], b->maxSteps, NULL);
    }
}

API nf_status nfo_batch_run(nfo_batch *b, int64_t max_steps) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    b->next = 0;
    b->maxSteps = max_steps;
    const int n = b->threads < b->count ? b->threads : b->count;
    pthread_t *tid = (pthread_t *)calloc((size_t)n, sizeof(pthread_t));
    for (int t = 1; t < n; t++) pthread_create(&tid[t], NULL, batch_worker, b);
    batch_worker(b);
    for (int t = 1; t < n; t++) pthread_join(tid[t], NULL);
    free(tid);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    b->lastMs = (double)(t1.tv_sec - t0.tv_sec) * 1e3 + (double)(t1.tv_nsec - t0.tv_nsec) * 1e-6;
    return NF_OK;
}

API nf_status nfo_batch_elapsed(nfo_batch *b, double *ms) { *ms = b->lastMs; return NF_OK; }
API nf_status nfo_batch_launch_count(nfo_batch *b, int64_t *n) { (void)b; *n = 0; return NF_OK; }

API nf_status nfo_batch_field_size(nfo_batch *b, int32_t field, size_t *count, size_t *bytes) {
    size_t total = 0, eb = 8;
    for (int k = 0; k < b->count; k++) {
        size_t c;
        nf_status st = nfo_field_size(b->s[k], field, &c, &eb);
        if (st) return bfail(b, st, "%s", nfo_last_error(b->s[k]));
        total += c;
    }
    *count = total;
    *bytes = eb;
    return NF_OK;
}

API nf_status nfo_batch_read(nfo_batch *b, int32_t field, void *dst, size_t nbytes) {
    size_t total, eb;
    nf_status st = nfo_batch_field_size(b, field, &total, &eb);
    if (st) return st;
    if (nbytes < total * eb) return bfail(b, NF_EINVAL, "buffer smaller than the field");
    char *o = (char *)dst;
    for (int k = 0; k < b->count; k++) {
        size_t c;
        nfo_field_size(b->s[k], field, &c, &eb);
        st = nfo_read_field(b->s[k], field, o, c * eb);
        if (st) return bfail(b, st, "%s", nfo_last_error(b->s[k]));
        o += c * eb;
    }
    return NF_OK;
}

API nf_status nfo_batch_state(nfo_batch *b, nf_batch_progress *out) {
    for (int k = 0; k < b->count; k++) {
        nf_state s;
        nfo_get_state(b->s[k], &s);
        out[k].time = s.time;
        out[k].timestep = s.timestep;
        out[k].steps = s.steps;
        out[k].status = 0;
        const int every = b->burst.sample_every;
        out[k].done = every > 0 ? (b->burstRes[k].traversed ||
                                   (s.steps % every == 0 && !(s.time < b->tEnd[k])))
                                : !(s.time < b->tEnd[k]);
    }
    return NF_OK;
}

API nf_status nfo_batch_measure(nfo_batch *b, nf_measure *out) {
    for (int k = 0; k < b->count; k++) nfo_measure_body(b->s[k], &out[k]);
    return NF_OK;
}

API nf_status nfo_batch_wall_stats(nfo_batch *b, nf_wall_info *out) {
    for (int k = 0; k < b->count; k++) nfo_wall_stats(b->s[k], &out[k]);
    return NF_OK;
}


/* ------------------------------------------------------------------ reference adjoint */

/* The FP64 reference adjoint (no counterpart in the reference): gradients of the length
 * ratio L/L0 or the mushroom diameter after the forward run's N steps with respect to the
 * Johnson-Cook A, B, n, C, m, the kinematic hardening modulus and the wall friction, by the
 * reverse sweep of nf_adjoint.h over checkpointed segments. Reduced integration, no damage,
 * erosion, contact or pressure (the Taylor scene); the first (zero-strain) assembly of a
 * stress-free start depends on no parameter. */
typedef struct {
    double *ur, *uz, *vr, *vz, *fr, *fz;
    uint8_t *onWall;
    double *sig, *back, *epsP, *work, *hgR, *hgZ, *hgK;
    double *dStrength, *dSoft, *dWidth;          /* when the solver has damage */
    double dt, dtPrevious, minEdgeSquared, time;
    int64_t stepCount;
} adj_state;

static void adj_alloc(const nfo_solver *h, adj_state *s) {
    const size_t N = (size_t)h->N, E = (size_t)h->E;
    s->ur = dalloc(N); s->uz = dalloc(N); s->vr = dalloc(N); s->vz = dalloc(N);
    s->fr = dalloc(N); s->fz = dalloc(N); s->onWall = balloc(N);
    s->sig = dalloc(4 * E); s->back = dalloc(4 * E); s->epsP = dalloc(E); s->work = dalloc(E);
    s->hgR = dalloc(E); s->hgZ = dalloc(E); s->hgK = dalloc(E);
    s->dStrength = h->hasDamage ? dalloc(E) : NULL;
    s->dSoft = h->hasDamage ? dalloc(E) : NULL;
    s->dWidth = h->hasDamage ? dalloc(E) : NULL;
}
static void adj_free(adj_state *s) {
    free(s->ur); free(s->uz); free(s->vr); free(s->vz); free(s->fr); free(s->fz); free(s->onWall);
    free(s->sig); free(s->back); free(s->epsP); free(s->work); free(s->hgR); free(s->hgZ);
    free(s->hgK); free(s->dStrength); free(s->dSoft); free(s->dWidth);
}
static void adj_copy(nfo_solver *h, adj_state *s, int save) {
    const size_t N = (size_t)h->N, E = (size_t)h->E;
#define C_(a, b, n) do { if (save) memcpy(a, b, n); else memcpy(b, a, n); } while (0)
    C_(s->ur, h->ur, 8 * N); C_(s->uz, h->uz, 8 * N); C_(s->vr, h->vr, 8 * N);
    C_(s->vz, h->vz, 8 * N); C_(s->fr, h->fr, 8 * N); C_(s->fz, h->fz, 8 * N);
    C_(s->onWall, h->onWall, N);
    C_(s->sig, h->sig, 32 * E); C_(s->back, h->back, 32 * E); C_(s->epsP, h->epsP, 8 * E);
    C_(s->work, h->wPlastic, 8 * E); C_(s->hgR, h->hgR, 8 * E); C_(s->hgZ, h->hgZ, 8 * E);
    C_(s->hgK, h->hgK, 8 * E);
    if (h->hasDamage) {
        C_(s->dStrength, h->dStrength, 8 * E); C_(s->dSoft, h->dSoft, 8 * E);
        C_(s->dWidth, h->dWidth, 8 * E);
    }
#undef C_
    if (save) {
        s->dt = h->dt; s->dtPrevious = h->dtPrevious; s->minEdgeSquared = h->minEdgeSquared;
        s->time = h->time; s->stepCount = h->stepCount;
    } else {
        h->dt = s->dt; h->dtPrevious = s->dtPrevious; h->minEdgeSquared = s->minEdgeSquared;
        h->time = s->time; h->stepCount = s->stepCount;
    }
}

typedef struct adj_ctx_s {
    int every, sampleEvery;
    int64_t steps;
    int checkpoints;
    adj_state *ckpt;
    /* the largest sampled capacity (BurstCase.loadCapacity) and the state it was read from */
    double peak;
    int64_t peakStep;
    adj_state peakState;
    int hasPeak;
} adj_ctx;

static void adj_ctx_free(adj_ctx *c) {
    for (int j = 0; j < c->checkpoints; j++) adj_free(&c->ckpt[j]);
    free(c->ckpt);
    c->ckpt = NULL;
    c->checkpoints = 0;
    if (c->hasPeak) adj_free(&c->peakState);
    c->hasPeak = 0;
}

static void adj_free_all(nfo_batch *b) {
    if (!b->adj) return;
    for (int k = 0; k < b->count; k++) adj_ctx_free(&b->adj[k]);
    free(b->adj);
    b->adj = NULL;
}

static nf_adj_mat adj_mat(const nfo_solver *h, int e) {
    const flow_t *f = &h->flows[h->emat[e]];
    nf_adj_mat m;
    m.lambda = h->lambdaOf[e]; m.mu = h->muOf[e];
    m.sy0 = f->sy0; m.hIso = f->hIso; m.hKin = f->hKin;
    m.a = f->a; m.b = f->b; m.n = f->n; m.c = f->c; m.m = f->m; m.refRate = f->refRate;
    m.room = f->room; m.melt = f->melt; m.thermalCoefficient = f->thermalCoefficient;
    m.jc = f->jc;
    return m;
}

static void adj_elem_in(const nfo_solver *h, int e, nf_adj_elem_in *in) {
    for (int k = 0; k < 4; k++) {
        const int n = h->conn[4 * e + k];
        in->x0r[k] = h->r[n]; in->x0z[k] = h->z[n];
        in->ur[k] = h->ur[n]; in->uz[k] = h->uz[n];
        in->vr[k] = h->vr[n]; in->vz[k] = h->vz[n];
        in->sig[k] = h->sig[4 * e + k]; in->back[k] = h->back[4 * e + k];
    }
    in->epsP = h->epsP[e]; in->work = h->wPlastic[e];
    in->hgR = h->hgR[e]; in->hgZ = h->hgZ[e];
    in->damaged = h->hasDamage;
    if (h->hasDamage) {
        in->dm.failureStrain = h->dFailure[e];
        in->dm.strength = h->dStrength[e];
        in->dm.softening = h->dSoft[e];
        in->dm.fractureEnergy = h->dGf[e];
        in->dm.youngs = h->dE[e];
        in->dm.geometry = h->dGeom + GEOMETRY_STRIDE * (size_t)e;
    }
}

typedef struct {
    double *ur, *uz, *vr, *vz, *fr, *fz;           /* node adjoints */
    double *sig, *back, *epsP, *work, *hgR, *hgZ;  /* element adjoints */
    double *strength, *soft;                       /* damage state adjoints */
    double *corner;                                /* [E][4][4] per-corner node adjoints */
    double *edge;                                  /* [K][4] pressure edges: a (r, z), b (r, z) */
    double dt, dtPrevious, time;                   /* of the next step's dt, dtPrevious, time */
    double p[NF_ADJ_P_COUNT];
} adj_bar;

/* The reverse of one step whose pre-step state is `pre` and whose shortest squared edge
 * (the next step's CFL input) was minEdge. */
static void adj_reverse_step(nfo_solver *h, adj_state *pre, double minEdge, adj_bar *a) {
    adj_copy(h, pre, 0);
    const double dt = h->dt;
    const double dtAvg = 0.5 * (h->dtPrevious + h->dt);
    const double half = 0.5 * h->damping * dtAvg;
    const double decay = (1.0 - half) / (1.0 + half), gain = dtAvg / (1.0 + half);
    h->nodalDecay = decay; h->nodalGain = gain; h->nodalDtAvg = dtAvg;
    nodalUpdate(h, 0, h->N);                       /* u', v' of this step */
    const int axi = h->formulation == NF_AXISYMMETRIC;
    const int finite = h->kinematics == NF_FINITE_STRAIN;
    double edgeb = 0.0;
    int owner = -1, ownerEdge = -1;
    if (finite && minEdge > 0.0 && minEdge < DBL_MAX) {
        edgeb = a->dt * h->cflSafety * sqrt(h->massScale) / h->fastestWave * 0.5 / sqrt(minEdge);
        for (int e = 0; e < h->E && owner < 0; e++) {
            nf_adj_elem_in in;
            adj_elem_in(h, e, &in);
            const int k = nf_adj_edge_owner(&in, dt, finite, minEdge);
            if (k >= 0) { owner = e; ownerEdge = k; }
        }
    }
    double dtb = a->dtPrevious;
    for (int e = 0; e < h->E; e++) {
        nf_adj_elem_in in;
        adj_elem_in(h, e, &in);
        nf_adj_elem_bar bar;
        for (int k = 0; k < 4; k++) {
            const int n = h->conn[4 * e + k];
            bar.g[k] = a->fr[n];
            bar.g[4 + k] = a->fz[n];
            bar.sig[k] = a->sig[4 * e + k];
            bar.back[k] = a->back[4 * e + k];
        }
        bar.epsP = a->epsP[e]; bar.work = a->work[e]; bar.hgR = a->hgR[e]; bar.hgZ = a->hgZ[e];
        bar.strength = h->hasDamage ? a->strength[e] : 0.0;
        bar.softening = h->hasDamage ? a->soft[e] : 0.0;
        bar.edgeOwner = e == owner ? ownerEdge : -1;
        bar.edgeb = edgeb;
        const nf_adj_mat m = adj_mat(h, e);
        nf_adj_element_reduced(&in, &m, dt, axi, finite, h->thickness, h->hourglassCoefficient,
                               &bar, &dtb, a->p);
        for (int k = 0; k < 4; k++) {
            a->sig[4 * e + k] = bar.sig[k];
            a->back[4 * e + k] = bar.back[k];
            double *c = a->corner + 16 * (size_t)e + 4 * k;
            c[0] = bar.ur[k]; c[1] = bar.uz[k]; c[2] = bar.vr[k]; c[3] = bar.vz[k];
        }
        a->epsP[e] = bar.epsP; a->work[e] = bar.work; a->hgR[e] = bar.hgR; a->hgZ[e] = bar.hgZ;
        if (h->hasDamage) {
            a->strength[e] = bar.strength;
            a->soft[e] = bar.softening;
        }
    }
    /* pressure edges (their load at this step's end time) */
    double tpress = 0.0;
    const double tnow = pre->time + dt;
    for (int j = 0; j < h->K; j++) {
        const int na = h->pedges[2 * j], nb = h->pedges[2 * j + 1];
        const double cb[4] = {a->fr[na], a->fr[nb], a->fz[na], a->fz[nb]};
        nf_adj_pressure_edge(h->r[na], h->z[na], h->r[nb], h->z[nb], h->ur[na], h->uz[na],
                             h->ur[nb], h->uz[nb], tnow, h->targetPressure, h->rampDuration, axi,
                             finite, h->thickness, cb, a->edge + 4 * (size_t)j,
                             a->edge + 4 * (size_t)j + 2, &tpress);
    }
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < h->N; i++) {
        double ub[2] = {a->ur[i], a->uz[i]}, vb[2] = {a->vr[i], a->vz[i]}, fb[2];
        for (int s = h->nodeSlotStart[i]; s < h->nodeSlotStart[i + 1]; s++) {
            const int slot = h->nodeSlot[s];
            if (slot >= 8 * h->E) {
                const double *c = a->edge + 4 * (size_t)((slot >> 3) - h->E) + 2 * (slot & 7);
                ub[0] += c[0]; ub[1] += c[1];
                continue;
            }
            const double *c = a->corner + 16 * (size_t)(slot >> 3) + 4 * (slot & 7);
            ub[0] += c[0]; ub[1] += c[1]; vb[0] += c[2]; vb[1] += c[3];
        }
        nf_adj_node(h->z[i], pre->ur[i], pre->uz[i], pre->vr[i], pre->vz[i], pre->fr[i],
                    pre->fz[i], h->mass[i], 1.0 / h->mass[i], h->fixedR[i], h->fixedZ[i],
                    pre->onWall[i], h->hasWall, h->wallPlane, h->wallFriction, decay, gain, dt,
                    ub, vb, fb, acc);
        a->ur[i] = ub[0]; a->uz[i] = ub[1]; a->vr[i] = vb[0]; a->vz[i] = vb[1];
        a->fr[i] = fb[0]; a->fz[i] = fb[1];
    }
    dtb += acc[2];
    a->p[NF_ADJ_P_MU] += acc[3];
    a->time += tpress;                             /* time' = time + dt */
    dtb += a->time;
    const double dtAvgb = nf_adj_dtavg(acc[0], acc[1], dtAvg, h->damping);
    dtb += 0.5 * dtAvgb;
    a->dt = dtb;
    a->dtPrevious = 0.5 * dtAvgb;
}

static nf_status adj_check(nfo_solver *h) {
    if (h->integration != NF_REDUCED || h->gone != NULL || h->contact != NULL)
        return fail(h, NF_EINVAL, "the adjoint covers reduced integration without erosion or "
                                  "contact");
    return NF_OK;
}

/* BurstCase.loadCapacity (BurstCase.java:533-553) of the solver's current state; with the
 * extremal nodes, for the seed. */
static double adj_capacity(const nfo_solver *h, const double *ur, const double *uz,
                           const double *sig, int *iBore, int *iLow, int *iHigh) {
    const int finite = h->kinematics == NF_FINITE_STRAIN;
    double hoop = 0.0;
    for (int e = 0; e < h->E; e++) {
        double sum = 0.0;
        for (int k = 0; k < 4; k++) {
            const int i = h->conn[4 * e + k], j = h->conn[4 * e + (k + 1) % 4];
            const double ri = finite ? h->r[i] + ur[i] : h->r[i];
            const double rj = finite ? h->r[j] + ur[j] : h->r[j];
            const double zi = finite ? h->z[i] + uz[i] : h->z[i];
            const double zj = finite ? h->z[j] + uz[j] : h->z[j];
            sum += ri * zj - rj * zi;
        }
        hoop += sig[4 * e + 2] * (0.5 * sum);
    }
    double bore = DBL_MAX, low = DBL_MAX, high = -DBL_MAX;
    for (int i = 0; i < h->N; i++) {
        const double r = finite ? h->r[i] + ur[i] : h->r[i];
        const double z = finite ? h->z[i] + uz[i] : h->z[i];
        if (r < bore) { bore = r; *iBore = i; }
        if (z < low) { low = z; *iLow = i; }
        if (z > high) { high = z; *iHigh = i; }
    }
    return hoop / (bore * (high - low));
}

static void adj_forward(nfo_solver *h, adj_ctx *c, double tEnd, int every, int sampleEvery) {
    c->every = every;
    c->sampleEvery = sampleEvery;
    c->hasPeak = 0;
    c->peak = -DBL_MAX;
    c->peakStep = 0;
    int cap = 16;
    c->ckpt = (adj_state *)calloc((size_t)cap, sizeof(adj_state));
    c->checkpoints = 0;
    while (h->time < tEnd) {
        if (h->stepCount % every == 0) {
            if (c->checkpoints == cap) {
                cap *= 2;
                c->ckpt = (adj_state *)realloc(c->ckpt, (size_t)cap * sizeof(adj_state));
            }
            adj_alloc(h, &c->ckpt[c->checkpoints]);
            adj_copy(h, &c->ckpt[c->checkpoints], 1);
            c->checkpoints++;
        }
        step(h);
        if (sampleEvery > 0 && h->stepCount % sampleEvery == 0) {
            int ib, il, ih;
            const double cap = adj_capacity(h, h->ur, h->uz, h->sig, &ib, &il, &ih);
            if (cap > c->peak) {
                c->peak = cap;
                c->peakStep = h->stepCount;
                if (!c->hasPeak) adj_alloc(h, &c->peakState);
                c->hasPeak = 1;
                adj_copy(h, &c->peakState, 1);
            }
        }
    }
    c->steps = h->stepCount;
}

/* The capacity's seed: adjoints of the displacements and of the hoop stress in `s`. */
static double adj_capacity_seed(const nfo_solver *h, const adj_state *s, double *urb,
                                double *uzb, double *sigb) {
    const int finite = h->kinematics == NF_FINITE_STRAIN;
    int ib = 0, il = 0, ih = 0;
    const double cap = adj_capacity(h, s->ur, s->uz, s->sig, &ib, &il, &ih);
    const double bore = finite ? h->r[ib] + s->ur[ib] : h->r[ib];
    const double zl = finite ? h->z[il] + s->uz[il] : h->z[il];
    const double zh = finite ? h->z[ih] + s->uz[ih] : h->z[ih];
    const double den = bore * (zh - zl);
    for (int e = 0; e < h->E; e++) {
        double r[4], z[4];
        int nn[4];
        for (int k = 0; k < 4; k++) {
            nn[k] = h->conn[4 * e + k];
            r[k] = finite ? h->r[nn[k]] + s->ur[nn[k]] : h->r[nn[k]];
            z[k] = finite ? h->z[nn[k]] + s->uz[nn[k]] : h->z[nn[k]];
        }
        double sum = 0.0;
        for (int k = 0; k < 4; k++) sum += r[k] * z[(k + 1) & 3] - r[(k + 1) & 3] * z[k];
        sigb[4 * e + 2] += 0.5 * sum / den;
        if (finite) {
            const double w = s->sig[4 * e + 2] / den;
            for (int k = 0; k < 4; k++) {
                urb[nn[k]] += w * 0.5 * (z[(k + 1) & 3] - z[(k + 3) & 3]);
                uzb[nn[k]] += w * 0.5 * (r[(k + 3) & 3] - r[(k + 1) & 3]);
            }
        }
    }
    if (finite) {
        urb[ib] -= cap / bore;
        uzb[ih] -= cap / (zh - zl);
        uzb[il] += cap / (zh - zl);
    }
    return cap;
}

static double adj_objective(const nfo_solver *h, int objective, double *ur, double *uz) {
    double zmax = -DBL_MAX, zmin = DBL_MAX, z0max = -DBL_MAX, z0min = DBL_MAX, rmax = -DBL_MAX;
    int imax = 0, imin = 0, irmax = 0;
    for (int i = 0; i < h->N; i++) {
        const double z = h->z[i] + h->uz[i], r = h->r[i] + h->ur[i];
        if (z > zmax) { zmax = z; imax = i; }
        if (z < zmin) { zmin = z; imin = i; }
        if (r > rmax) { rmax = r; irmax = i; }
        if (h->z[i] > z0max) z0max = h->z[i];
        if (h->z[i] < z0min) z0min = h->z[i];
    }
    memset(ur, 0, 8 * (size_t)h->N);
    memset(uz, 0, 8 * (size_t)h->N);
    if (objective == 0) {
        const double L0 = z0max - z0min;
        uz[imax] += 1.0 / L0;
        uz[imin] -= 1.0 / L0;
        return (zmax - zmin) / L0;
    }
    ur[irmax] += 2.0;
    return 2.0 * rmax;
}

static nf_status adj_backward(nfo_solver *h, adj_ctx *c, int objective, double *value,
                              double *grad) {
    const size_t N = (size_t)h->N, E = (size_t)h->E;
    adj_bar a;
    memset(&a, 0, sizeof a);
    a.ur = dalloc(N); a.uz = dalloc(N); a.vr = dalloc(N); a.vz = dalloc(N);
    a.fr = dalloc(N); a.fz = dalloc(N);
    a.sig = dalloc(4 * E); a.back = dalloc(4 * E); a.epsP = dalloc(E); a.work = dalloc(E);
    a.hgR = dalloc(E); a.hgZ = dalloc(E); a.corner = dalloc(16 * E);
    a.strength = dalloc(E); a.soft = dalloc(E); a.edge = dalloc(4 * (size_t)h->K);
    /* the objective's seed enters the sweep after step m (the final step, or the capacity's
       sampled peak) */
    int64_t m = c->steps;
    double *seedR = dalloc(N), *seedZ = dalloc(N), *seedSig = dalloc(4 * E);
    if (objective == NF_OBJECTIVE_PEAK_CAPACITY) {
        if (!c->hasPeak) {
            free(seedR); free(seedZ); free(seedSig);
            return fail(h, NF_ESTATE, "no capacity was sampled in the forward pass");
        }
        m = c->peakStep;
        *value = adj_capacity_seed(h, &c->peakState, seedR, seedZ, seedSig);
    } else {
        *value = adj_objective(h, objective, seedR, seedZ);
    }
    adj_state final_;
    adj_alloc(h, &final_);
    adj_copy(h, &final_, 1);
    const int every = c->every;
    adj_state *tape = (adj_state *)calloc((size_t)every, sizeof(adj_state));
    double *minEdge = (double *)calloc((size_t)every, sizeof(double));
    for (int j = 0; j < every; j++) adj_alloc(h, &tape[j]);
    for (int s = c->checkpoints - 1; s >= 0; s--) {
        adj_copy(h, &c->ckpt[s], 0);
        const int64_t start = (int64_t)s * every;
        const int64_t end = start + every < c->steps ? start + every : c->steps;
        for (int64_t j = start; j < end; j++) {
            if (h->stepCount == 0) advanceMaterialAndAssemble(h, 0.0);
            adj_copy(h, &tape[j - start], 1);
            step_body(h);
            minEdge[j - start] = h->minEdgeSquared;
        }
        for (int64_t j = end - 1; j >= start; j--) {
            if (j == m - 1) {
                for (size_t i = 0; i < N; i++) { a.ur[i] += seedR[i]; a.uz[i] += seedZ[i]; }
                for (size_t i = 0; i < 4 * E; i++) a.sig[i] += seedSig[i];
            }
            adj_reverse_step(h, &tape[j - start], minEdge[j - start], &a);
        }
    }
    for (int k = 0; k < NF_ADJ_P_COUNT; k++) grad[k] = a.p[k];
    adj_copy(h, &final_, 0);
    adj_free(&final_);
    for (int j = 0; j < every; j++) adj_free(&tape[j]);
    free(tape); free(minEdge);
    free(a.ur); free(a.uz); free(a.vr); free(a.vz); free(a.fr); free(a.fz);
    free(a.sig); free(a.back); free(a.epsP); free(a.work); free(a.hgR); free(a.hgZ);
    free(a.corner); free(a.strength); free(a.soft); free(a.edge);
    free(seedR); free(seedZ); free(seedSig);
    return NF_OK;
}

/* The batch surface: every instance of the oracle's batch, one after another. */
static double now_ms(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec * 1e3 + (double)t.tv_nsec * 1e-6;
}

API nf_status nfo_batch_adjoint_forward(nfo_batch *b, int32_t checkpoint_every,
                                        int32_t sample_every) {
    if (checkpoint_every < 1) return bfail(b, NF_EINVAL, "checkpoint interval must be positive");
    if (sample_every < 0) return bfail(b, NF_EINVAL, "sampling interval must not be negative");
    for (int k = 0; k < b->count; k++) {
        nf_status st = adj_check(b->s[k]);
        if (st) return bfail(b, st, "%s", nfo_last_error(b->s[k]));
        if (b->s[k]->stepCount != 0)
            return bfail(b, NF_ESTATE, "the adjoint's forward pass starts from a fresh batch");
    }
    const double t0 = now_ms();
    if (b->adj)
        for (int k = 0; k < b->count; k++) adj_ctx_free(&b->adj[k]);
    else
        b->adj = (adj_ctx *)calloc((size_t)b->count, sizeof(adj_ctx));
    for (int k = 0; k < b->count; k++)
        adj_forward(b->s[k], &b->adj[k], b->tEnd[k], checkpoint_every, sample_every);
    b->adjForwardMs = now_ms() - t0;
    return NF_OK;
}

API nf_status nfo_batch_adjoint_backward(nfo_batch *b, int32_t objective, double *values,
                                         double *gradients) {
    if (!b->adj) return bfail(b, NF_ESTATE, "run the adjoint's forward pass first");
    if (objective != NF_OBJECTIVE_LENGTH_RATIO && objective != NF_OBJECTIVE_MUSHROOM &&
        objective != NF_OBJECTIVE_PEAK_CAPACITY)
        return bfail(b, NF_EINVAL, "unknown objective %d", objective);
    const double t0 = now_ms();
    for (int k = 0; k < b->count; k++) {
        nf_status st = adj_backward(b->s[k], &b->adj[k], objective, &values[k],
                                    gradients + (size_t)k * NF_ADJ_P_COUNT);
        if (st) return bfail(b, st, "instance %d: %s", k, nfo_last_error(b->s[k]));
    }
    b->adjBackwardMs = now_ms() - t0;
    return NF_OK;
}

/* Several objectives: one reference backward pass per objective (the reference adjoint has
 * no shared recompute; its gradients are those of the single passes). */
API nf_status nfo_batch_adjoint_backward_many(nfo_batch *b, const int32_t *objectives,
                                              int32_t count, double *values, double *gradients) {
    if (count < 1 || count > 3)
        return bfail(b, NF_EINVAL, "1 to 3 objectives per backward pass, not %d", count);
    double total = 0.0;
    for (int w = 0; w < count; w++) {
        nf_status st = nfo_batch_adjoint_backward(b, objectives[w], values + (size_t)w * b->count,
                                                  gradients + (size_t)w * b->count * NF_ADJ_P_COUNT);
        if (st) return st;
        total += b->adjBackwardMs;
    }
    b->adjBackwardMs = total;
    return NF_OK;
}

API nf_status nfo_batch_adjoint_elapsed(nfo_batch *b, double *forward_ms, double *backward_ms) {
    *forward_ms = b->adjForwardMs;
    *backward_ms = b->adjBackwardMs;
    return NF_OK;
}

/* ---------------------------------------------------------------- burst measurement */

/* BurstCase.run's sampling (validate/BurstCase.java:446-490) for instance k after its step
 * count reached a multiple of sample_every: loadCapacity (:533-553), hoopStrain (:560-569),
 * borePressure, the running peak and the turnover test. */
static void burst_sample(nfo_batch *b, int k) {
    nfo_solver *h = b->s[k];
    int ib, il, ih;
    const double capacity = adj_capacity(h, h->ur, h->uz, h->sig, &ib, &il, &ih);
    double bore = DBL_MAX, rim = -DBL_MAX;
    for (int i = 0; i < h->N; i++) {
        const double r = h->r[i] + h->ur[i];
        if (r < bore) bore = r;
        if (r > rim) rim = r;
    }
    const double strain = nf_log(0.5 * (bore + rim) / b->meanRadius[k]);
    const double applied = pressureAt(h, h->time);
    nf_burst_result *st = &b->burstRes[k];
    if (b->burst.trace_capacity > 0 && st->samples < b->burst.trace_capacity) {
        double *t = b->burstTrace + 4 * ((size_t)k * b->burst.trace_capacity + st->samples);
        t[0] = h->time; t[1] = strain; t[2] = capacity; t[3] = applied;
    }
    st->samples += 1;
    st->capacity = capacity;
    st->strain = strain;
    st->applied = applied;
    if (capacity > st->peak_capacity) {
        st->peak_capacity = capacity;
        st->peak_strain = strain;
        st->peak_applied = applied;
    } else if (applied >= h->targetPressure && capacity < st->peak_capacity * (1.0 - b->burst.margin)) {
        st->traversed = 1;
    }
}

/* Whole samples of steps until the peak is traversed, the deadline is passed at a sample
 * point, or the run's step bound is reached. */
static void burst_run_instance(nfo_batch *b, int k) {
    nfo_solver *h = b->s[k];
    const int every = b->burst.sample_every;
    int64_t taken = 0;
    for (;;) {
        if (b->burstRes[k].traversed || taken >= b->maxSteps) break;
        if (h->stepCount % every == 0 && !(h->time < b->tEnd[k])) break;
        step(h);
        taken++;
        if (h->stepCount % every == 0) burst_sample(b, k);
    }
}

API nf_status nfo_batch_set_burst(nfo_batch *b, const nf_batch_burst *config,
                                  const double *mean_radius) {
    if (!config || config->sample_every < 0 || config->trace_capacity < 0 ||
        !(config->margin >= 0.0 && config->margin < 1.0))
        return bfail(b, NF_EINVAL, "burst sampling needs sample_every >= 0, trace_capacity >= 0 "
                                   "and a margin in [0, 1)");
    if (config->sample_every > 0 && !mean_radius)
        return bfail(b, NF_EINVAL, "burst sampling needs each instance's mean radius");
    free(b->meanRadius); free(b->burstRes); free(b->burstTrace);
    b->meanRadius = NULL; b->burstRes = NULL; b->burstTrace = NULL;
    b->burst = *config;
    if (config->sample_every == 0) return NF_OK;
    b->meanRadius = (double *)malloc(sizeof(double) * (size_t)b->count);
    memcpy(b->meanRadius, mean_radius, sizeof(double) * (size_t)b->count);
    b->burstRes = (nf_burst_result *)calloc((size_t)b->count, sizeof(nf_burst_result));
    b->burstTrace = (double *)calloc(4 * (size_t)b->count * (size_t)config->trace_capacity + 1,
                                     sizeof(double));
    return NF_OK;
}

API nf_status nfo_batch_burst_results(nfo_batch *b, nf_burst_result *out) {
    if (b->burst.sample_every == 0) return bfail(b, NF_ESTATE, "burst sampling is not set");
    memcpy(out, b->burstRes, sizeof(nf_burst_result) * (size_t)b->count);
    return NF_OK;
}

API nf_status nfo_batch_burst_trace(nfo_batch *b, double *trace) {
    if (b->burst.sample_every == 0) return bfail(b, NF_ESTATE, "burst sampling is not set");
    memcpy(trace, b->burstTrace,
           sizeof(double) * 4 * (size_t)b->count * (size_t)b->burst.trace_capacity);
    return NF_OK;
}
