/*
 * defect_field.c -- the Weibull defect field's arithmetic on the host: the failure strains
 * handed to ExplicitSolver.setDamage by a defect-driven scene.
 *
 * Restates core/DefectField.java (the hash-seeded white noise :325-347, the separable Gaussian
 * window :289-319 and the copula transform :262-274), core/Normal.java (Cody's rational
 * erfc, :50-129) and core/Weibull.java (the quantiles and the size effect, :114-164) in the
 * reference's operation order, over the deterministic elementary functions of nf_math.h
 * (log, exp, pow, cos) instead of a platform's libm. The same seed then gives the same field,
 * bit for bit, on every host (x86-64 and aarch64 alike), and the window's sums are the
 * reference's sequential ones. Built with contraction off (-ffp-contract=off).
 *
 * The lattice noise is evaluated once per site over the points' bounding box and gathered, as
 * DefectField.sampleOnto memoises it (:350-378); a point whose window leaves the box hashes
 * the site directly, which gives the same value. Points are split over host threads; each
 * point's value does not depend on the split.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "nf_math.h"

#define API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ the lattice noise */

static uint64_t field_mix(uint64_t z) {                       /* DefectField.mix, :335-339 */
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double unit_open(uint64_t bits) {                      /* :346-348 */
    return ((double)(bits >> 11) + 0.5) * 0x1.0p-53;
}

/* DefectField.white, :325-332: Box-Muller over two SplitMix64-style hashes of the site. */
static double field_white(uint64_t seed, int64_t i, int64_t j) {
    uint64_t h = field_mix(seed + 0x9E3779B97F4A7C15ULL);
    h = field_mix(h ^ ((uint64_t)i * 0xBF58476D1CE4E5B9ULL));
    h = field_mix(h ^ ((uint64_t)j * 0x94D049BB133111EBULL));
    const double u1 = unit_open(h);
    const double u2 = unit_open(field_mix(h ^ 0xD6E8FEB86659FD93ULL));
    return sqrt(-2.0 * nf_log(u1)) * nf_cos(2.0 * NF_PI * u2);
}

/* ------------------------------------------------------------------ Normal (Cody's erfc) */

/* W. J. Cody, "Rational Chebyshev approximations for the error function", Math. Comp. 23
 * (1969) 631-637: the published coefficients of the three intervals, as core/Normal.java
 * holds them. */
static const double ERF_A[5] = {3.16112374387056560e0, 1.13864154151050156e2,
                                3.77485237685302021e2, 3.20937758913846947e3,
                                1.85777706184603153e-1};
static const double ERF_B[4] = {2.36012909523441209e1, 2.44024637934444173e2,
                                1.28261652607737228e3, 2.84423683343917062e3};
static const double ERF_C[9] = {5.64188496988670089e-1, 8.88314979438837594e0,
                                6.61191906371416295e1, 2.98635138197400131e2,
                                8.81952221241769090e2, 1.71204761263407058e3,
                                2.05107837782607147e3, 1.23033935479799725e3,
                                2.15311535474403846e-8};
static const double ERF_D[8] = {1.57449261107098347e1, 1.17693950891312499e2,
                                5.37181101862009858e2, 1.62138957456669019e3,
                                3.29079923573345963e3, 4.36261909014324716e3,
                                3.43936767414372164e3, 1.23033935480374942e3};
static const double ERF_P[6] = {3.05326634961232344e-1, 3.60344899949804439e-1,
                                1.25781726111229246e-1, 1.60837851487422766e-2,
                                6.58749161529837803e-4, 1.63153871373020978e-2};
static const double ERF_Q[5] = {2.56852019228982242e0, 1.87295284992346047e0,
                                5.27905102951428412e-1, 6.05183413124413191e-2,
                                2.33520497626869185e-3};
static const double ERF_THRESHOLD = 0.46875;
static const double SQRT_HALF = 0.70710678118654752440;
static const double INV_SQRT_PI = 5.6418958354775628695e-1;

static double small_erf(double sq) {                         /* Normal.smallErf, :105-113 */
    double num = ERF_A[4] * sq, den = sq;
    for (int i = 0; i < 3; i++) {
        num = (num + ERF_A[i]) * sq;
        den = (den + ERF_B[i]) * sq;
    }
    return (num + ERF_A[3]) / (den + ERF_B[3]);
}

static double cody_erfc(double x) {                          /* Normal.erfc, :62-101 */
    const double y = fabs(x);
    double result;
    if (y <= ERF_THRESHOLD) return 1.0 - x * small_erf(y * y);
    if (y <= 4.0) {
        double num = ERF_C[8] * y, den = y;
        for (int i = 0; i < 7; i++) {
            num = (num + ERF_C[i]) * y;
            den = (den + ERF_D[i]) * y;
        }
        result = (num + ERF_C[7]) / (den + ERF_D[7]);
    } else {
        const double inv = 1.0 / (y * y);
        double num = ERF_P[5] * inv, den = inv;
        for (int i = 0; i < 4; i++) {
            num = (num + ERF_P[i]) * inv;
            den = (den + ERF_Q[i]) * inv;
        }
        result = inv * (num + ERF_P[4]) / (den + ERF_Q[4]);
        result = (INV_SQRT_PI - result) / y;
    }
    const double trunc = (double)(int)(y * 16.0) / 16.0;
    const double del = (y - trunc) * (y + trunc);
    result *= nf_exp(-trunc * trunc) * nf_exp(-del);
    return x < 0.0 ? 2.0 - result : result;
}

/* ------------------------------------------------------------------ Weibull */

/* log(1 + x) for x > -1: log of u = 1 + x (rounded) corrected by (x - (u - 1)) / u, the
 * classical compensation (Goldberg, "What every computer scientist should know about
 * floating-point arithmetic", 1991, theorem 4), with log as nf_math's double-double. */
static double field_log1p(double x) {
    const double u = 1.0 + x;
    if (u == 1.0) return x;
    double hi, lo;
    nf_log_dd(u, &hi, &lo);
    return hi + (lo + (x - (u - 1.0)) / u);
}

/* Weibull.quantile (:114-119) and quantileFromSurvival (:126-131). */
static double weibull_quantile(double scale, double modulus, double p) {
    return scale * nf_pow(-field_log1p(-p), 1.0 / modulus);
}
static double weibull_quantile_survival(double scale, double modulus, double s) {
    return scale * nf_pow(-nf_log(s), 1.0 / modulus);
}

/* ------------------------------------------------------------------ the field */

typedef struct {
    uint64_t seed;
    double cell, sigmaCells;
    int radius;
    /* memoised noise over [i0, i0 + ni) x [j0, j0 + nj), or NULL */
    const double *grid;
    int64_t i0, j0, ni, nj;
} field_t;

static void field_init(field_t *f, double correlationLength, uint64_t seed) {
    memset(f, 0, sizeof *f);
    f->seed = seed;
    f->cell = correlationLength / 3.0;                                /* :133 */
    f->sigmaCells = (correlationLength / sqrt(2.0)) / f->cell;        /* :136 */
    f->radius = (int)ceil(4.0 * f->sigmaCells);                       /* :137 */
}

static double field_noise(const field_t *f, int64_t i, int64_t j) {
    const int64_t a = i - f->i0, b = j - f->j0;
    if (f->grid && a >= 0 && a < f->ni && b >= 0 && b < f->nj) return f->grid[b * f->ni + a];
    return field_white(f->seed, i, j);
}

/* DefectField.smooth, :289-319: the separable window, each row summed over a, the rows over
 * b, normalised by the root of the product of the squared weights' sums. */
static double field_gaussian(const field_t *f, double r, double z) {
    double wr[64], wz[64];
    const double gr = r / f->cell, gz = z / f->cell;
    const int64_t i0 = (int64_t)floor(gr) - f->radius;
    const int64_t j0 = (int64_t)floor(gz) - f->radius;
    const int taps = 2 * f->radius + 2;
    const double twoSigmaSq = 2.0 * f->sigmaCells * f->sigmaCells;
    double sumRSq = 0.0, sumZSq = 0.0;
    for (int k = 0; k < taps; k++) {
        const double dr = gr - (double)(i0 + k);
        const double dz = gz - (double)(j0 + k);
        wr[k] = nf_exp(-dr * dr / twoSigmaSq);
        wz[k] = nf_exp(-dz * dz / twoSigmaSq);
        sumRSq += wr[k] * wr[k];
        sumZSq += wz[k] * wz[k];
    }
    double sum = 0.0;
    for (int b = 0; b < taps; b++) {
        double row = 0.0;
        for (int a = 0; a < taps; a++) row += wr[a] * field_noise(f, i0 + a, j0 + b);
        sum += wz[b] * row;
    }
    return sum / sqrt(sumRSq * sumZSq);
}

/* DefectField.transform, :262-274, with Weibull.forVolume's scale (:139-158). */
static double field_transform(double scale, double modulus, double referenceVolume, double g,
                              double volume) {
    const double local = scale * nf_pow(volume / referenceVolume, -1.0 / modulus);
    const double c = fmax(-9.0, fmin(9.0, g));
    return c <= 0.0
           ? weibull_quantile(local, modulus, 0.5 * cody_erfc(-c * SQRT_HALF))
           : weibull_quantile_survival(local, modulus, 0.5 * cody_erfc(c * SQRT_HALF));
}

/* ------------------------------------------------------------------ threads */

typedef struct {
    const field_t *f;
    double scale, modulus, referenceVolume;
    const double *r, *z, *volume;
    double *out;
    int64_t lo, hi;
    int transform;
} work_t;

static void *work_run(void *arg) {
    const work_t *w = (const work_t *)arg;
    for (int64_t k = w->lo; k < w->hi; k++) {
        const double g = field_gaussian(w->f, w->r[k], w->z[k]);
        w->out[k] = w->transform
                    ? field_transform(w->scale, w->modulus, w->referenceVolume, g, w->volume[k])
                    : g;
    }
    return NULL;
}

static void *grid_run(void *arg) {
    const work_t *w = (const work_t *)arg;                  /* rows [lo, hi) of the grid */
    const field_t *f = w->f;
    double *grid = w->out;
    for (int64_t b = w->lo; b < w->hi; b++)
        for (int64_t a = 0; a < f->ni; a++)
            grid[b * f->ni + a] = field_white(f->seed, f->i0 + a, f->j0 + b);
    return NULL;
}

static int thread_count(int64_t items) {
    long cpus = sysconf(_SC_NPROCESSORS_ONLN);
    if (cpus < 1) cpus = 1;
    if (cpus > 32) cpus = 32;
    const int64_t want = items / 4096 + 1;
    return (int)(want < cpus ? want : cpus);
}

static void run_split(void *(*fn)(void *), work_t *base, int64_t items) {
    const int t = thread_count(items);
    pthread_t th[32];
    work_t w[32];
    int started[32] = {0};
    for (int k = 0; k < t; k++) {
        w[k] = *base;
        w[k].lo = items * k / t;
        w[k].hi = items * (k + 1) / t;
        started[k] = k > 0 && pthread_create(&th[k], NULL, fn, &w[k]) == 0;
    }
    fn(&w[0]);
    for (int k = 1; k < t; k++) {
        if (started[k]) pthread_join(th[k], NULL);
        else fn(&w[k]);                         /* a thread that could not start: run here */
    }
}

/* Field values (transform = 0: the Gaussian field, gaussianAt :253-255; 1: failure strains,
 * failureStrainForVolume :233-236) at n points. Returns 0, or -1 when out of memory. */
static int field_eval(double scale, double modulus, double referenceVolume,
                      double correlationLength, uint64_t seed, int64_t n, const double *r,
                      const double *z, const double *volume, double *out, int transform) {
    field_t f;
    field_init(&f, correlationLength, seed);
    if (f.radius > 31) return -2;                 /* taps beyond the window arrays */
    double *grid = NULL;
    if (n > 0) {
        double gr0 = r[0] / f.cell, gr1 = gr0, gz0 = z[0] / f.cell, gz1 = gz0;
        for (int64_t k = 1; k < n; k++) {
            const double gr = r[k] / f.cell, gz = z[k] / f.cell;
            gr0 = fmin(gr0, gr); gr1 = fmax(gr1, gr);
            gz0 = fmin(gz0, gz); gz1 = fmax(gz1, gz);
        }
        const int64_t i0 = (int64_t)floor(gr0) - f.radius, j0 = (int64_t)floor(gz0) - f.radius;
        const int64_t ni = (int64_t)floor(gr1) + f.radius + 2 - i0;
        const int64_t nj = (int64_t)floor(gz1) + f.radius + 2 - j0;
        if (ni > 0 && nj > 0 && ni * nj <= ((int64_t)1 << 24) && ni * nj <= 64 * n + 4096) {
            grid = (double *)malloc(sizeof(double) * (size_t)(ni * nj));
            if (!grid) return -1;
            f.i0 = i0; f.j0 = j0; f.ni = ni; f.nj = nj;
            work_t g = {&f, 0, 0, 0, NULL, NULL, NULL, grid, 0, 0, 0};
            run_split(grid_run, &g, nj);
            f.grid = grid;
        }
    }
    work_t w = {&f, scale, modulus, referenceVolume, r, z, volume, out, 0, 0, transform};
    run_split(work_run, &w, n);
    free(grid);
    return 0;
}

/* ------------------------------------------------------------------ exports */

API int nf_field_gaussian(double correlationLength, uint64_t seed, int64_t n, const double *r,
                          const double *z, double *out) {
    return field_eval(0.0, 1.0, 1.0, correlationLength, seed, n, r, z, NULL, out, 0);
}

API int nf_field_failure_strain(double scale, double modulus, double referenceVolume,
                                double correlationLength, uint64_t seed, int64_t n,
                                const double *r, const double *z, const double *volume,
                                double *out) {
    return field_eval(scale, modulus, referenceVolume, correlationLength, seed, n, r, z, volume,
                      out, 1);
}

API void nf_field_white(uint64_t seed, int64_t n, const int64_t *i, const int64_t *j,
                        double *out) {
    for (int64_t k = 0; k < n; k++) out[k] = field_white(seed, i[k], j[k]);
}

/* Normal.cdf (:33-35) and survival (:43-45) of each x. */
API void nf_normal(int64_t n, const double *x, double *cdf, double *survival) {
    for (int64_t k = 0; k < n; k++) {
        if (cdf) cdf[k] = 0.5 * cody_erfc(-x[k] * SQRT_HALF);
        if (survival) survival[k] = 0.5 * cody_erfc(x[k] * SQRT_HALF);
    }
}

/* Weibull.quantile (from_survival = 0) or quantileFromSurvival (1) of each probability. */
API void nf_weibull_quantile(double scale, double modulus, int from_survival, int64_t n,
                             const double *p, double *out) {
    for (int64_t k = 0; k < n; k++)
        out[k] = from_survival ? weibull_quantile_survival(scale, modulus, p[k])
                               : weibull_quantile(scale, modulus, p[k]);
}

/* Weibull.minimumOf's scale factor n^(-1/m) (:139-144). */
API double nf_weibull_size_factor(double count, double modulus) {
    return nf_pow(count, -1.0 / modulus);
}
