/*
 * CPU oracle for the StatER statistics hot path (see oracle.h for the scope).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library, never part of it.
 * Compiled with -ffp-contract=off so that every operation is separately rounded.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Parallel-for over [0, total) in contiguous chunks.                         */
/* ------------------------------------------------------------------------- */
typedef void (*range_fn)(void *ctx, int64_t begin, int64_t end);
typedef struct {
    range_fn fn;
    void *ctx;
    int64_t begin, end;
} range_job;

static void *range_thread(void *arg) {
    range_job *j = (range_job *)arg;
    j->fn(j->ctx, j->begin, j->end);
    return NULL;
}

static void parallel_for(int64_t total, int nthreads, range_fn fn, void *ctx) {
    if (nthreads <= 1 || total < 2) {
        fn(ctx, 0, total);
        return;
    }
    if (nthreads > 256) nthreads = 256;
    if (nthreads > total) nthreads = (int)total;
    pthread_t th[256];
    range_job jobs[256];
    for (int t = 0; t < nthreads; t++) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].begin = total * t / nthreads;
        jobs[t].end = total * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, range_thread, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------- */
/* Transforms. Box-Cox follows boxCox() (estimator.h:43-76): identity when    */
/* lambda == 1, else (x^lambda - 1) / lambda. The other monotone transforms   */
/* (log1p, sqrt, cbrt, asinh) are the multi-transform set of the target.      */
/* ------------------------------------------------------------------------- */
double orc_transform_f64(int kind, double lambda, double x) {
    switch (kind) {
        case ORC_TK_LOG1P: return log1p(x);
        case ORC_TK_SQRT: return sqrt(x);
        case ORC_TK_CBRT: return cbrt(x);
        case ORC_TK_ASINH: return asinh(x);
        case ORC_TK_BOXCOX:
            if (lambda == 1.0) return x;
            return (pow(x, lambda) - 1.0) / lambda;
        default: return x;
    }
}

float orc_transform_f32(int kind, float lambda, float x) {
    switch (kind) {
        case ORC_TK_LOG1P: return log1pf(x);
        case ORC_TK_SQRT: return sqrtf(x);
        case ORC_TK_CBRT: return cbrtf(x);
        case ORC_TK_ASINH: return asinhf(x);
        case ORC_TK_BOXCOX:
            if (lambda == 1.f) return x;
            return (powf(x, lambda) - 1.f) / lambda;
        default: return x;
    }
}

/* ------------------------------------------------------------------------- */
/* Stage 1: accumulation (two precisions from one body).                      */
/* ------------------------------------------------------------------------- */
#define REAL double
#define SFX(name) name##_f64
#define TRANSFORM(k, l, x) orc_transform_f64((k), (l), (x))
#define SQRT_REAL sqrt
#include "oracle_acc.inc"
#undef REAL
#undef SFX
#undef TRANSFORM
#undef SQRT_REAL

#define REAL float
#define SFX(name) name##_f32
#define TRANSFORM(k, l, x) orc_transform_f32((k), (l), (x))
#define SQRT_REAL sqrtf
#include "oracle_acc.inc"
#undef REAL
#undef SFX
#undef TRANSFORM
#undef SQRT_REAL

typedef struct {
    int W, H, G, S, K, max_moment;
    const float *samples;
    const int32_t *count;
    const int32_t *tkind;
    const void *tlambda;
    int32_t *n;
    void *stats, *gmean;
} acc_ctx;

/* Work is split over 16x16 tiles, as ParallelFor2D splits the render
 * (statpath.cpp:85-90, 178-406). */
#define TILE 16
static void acc_range_f64(void *vctx, int64_t b, int64_t e) {
    acc_ctx *c = (acc_ctx *)vctx;
    const int ntx = (c->W + TILE - 1) / TILE;
    const size_t HW = (size_t)c->W * c->H;
    for (int64_t t = b; t < e; t++) {
        const int tx = (int)(t % ntx), ty = (int)(t / ntx);
        for (int y = ty * TILE; y < ty * TILE + TILE && y < c->H; y++)
            for (int x = tx * TILE; x < tx * TILE + TILE && x < c->W; x++)
                acc_pixel_f64((size_t)y * c->W + x, HW, c->G, c->S, c->samples, c->count, c->K,
                              c->tkind, (const double *)c->tlambda, c->max_moment, c->n,
                              (double *)c->stats, (double *)c->gmean);
    }
}
static void acc_range_f32(void *vctx, int64_t b, int64_t e) {
    acc_ctx *c = (acc_ctx *)vctx;
    const int ntx = (c->W + TILE - 1) / TILE;
    const size_t HW = (size_t)c->W * c->H;
    for (int64_t t = b; t < e; t++) {
        const int tx = (int)(t % ntx), ty = (int)(t / ntx);
        for (int y = ty * TILE; y < ty * TILE + TILE && y < c->H; y++)
            for (int x = tx * TILE; x < tx * TILE + TILE && x < c->W; x++)
                acc_pixel_f32((size_t)y * c->W + x, HW, c->G, c->S, c->samples, c->count, c->K,
                              c->tkind, (const float *)c->tlambda, c->max_moment, c->n,
                              (float *)c->stats, (float *)c->gmean);
    }
}

void orc_accumulate_f64(int W, int H, int G, int S, const float *samples, const int32_t *count,
                        int K, const int32_t *tkind, const double *tlambda, int max_moment,
                        int32_t *n, double *stats, double *gmean, int nthreads) {
    acc_ctx c = {W, H, G, S, K, max_moment, samples, count, tkind, tlambda, n, stats, gmean};
    const int64_t ntiles = (int64_t)((W + TILE - 1) / TILE) * ((H + TILE - 1) / TILE);
    parallel_for(ntiles, nthreads, acc_range_f64, &c);
}

void orc_accumulate_f32(int W, int H, int G, int S, const float *samples, const int32_t *count,
                        int K, const int32_t *tkind, const float *tlambda, int max_moment,
                        int32_t *n, float *stats, float *gmean, int nthreads) {
    acc_ctx c = {W, H, G, S, K, max_moment, samples, count, tkind, tlambda, n, stats, gmean};
    const int64_t ntiles = (int64_t)((W + TILE - 1) / TILE) * ((H + TILE - 1) / TILE);
    parallel_for(ntiles, nthreads, acc_range_f32, &c);
}

/* ------------------------------------------------------------------------- */
/* Tile merge: Estimator::MergeTransformTile (estimator.cpp:301-324) copies   */
/* each StatTilePixel<Vec3> of a tile into the full-image planes. Record      */
/* layout of the float build: uint64 n at 0, t0 at 64, t1 at 192, each set    */
/* seven float3 (mean, m2, m3, m4, c2X, c2Y, m1); 320 bytes per pixel.        */
/* ------------------------------------------------------------------------- */
void orc_merge_transform_tiles_f32(int W, int H, int ntiles, const int32_t *bounds,
                                   const uint8_t *records, int32_t *n, float *stats) {
    const size_t HW = (size_t)W * H;
    size_t rec = 0;
    for (int t = 0; t < ntiles; t++) {
        const int x0 = bounds[4 * t], y0 = bounds[4 * t + 1], x1 = bounds[4 * t + 2],
                  y1 = bounds[4 * t + 3];
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++, rec++) {
                const uint8_t *r = records + rec * 320;
                const size_t p = (size_t)y * W + x;
                uint64_t nn;
                memcpy(&nn, r, 8);
                n[p] = (int32_t)nn;
                for (int set = 0; set < 2; set++) {
                    const float *v = (const float *)(r + (set == 0 ? 64 : 192));
                    for (int q = 0; q < ORC_NQ; q++)
                        for (int c = 0; c < 3; c++)
                            stats[(((size_t)set * ORC_NQ + q) * 3 + c) * HW + p] = v[q * 3 + c];
                }
            }
    }
}

/* ------------------------------------------------------------------------- */
/* Pairwise combine of moment sets (Chan et al. 1979; Pebay 2008, eqs. 2.1-   */
/* 2.3 for M2..M4). The co-moments c2X/c2Y and the absolute-deviation sum m1   */
/* add, which matches how the reference's online update ignores the shift of  */
/* the mean for those three accumulators (estimator.h:301-304).               */
/* ------------------------------------------------------------------------- */
void orc_merge_moments_f64(int HW, int K, int max_moment, int32_t *nA, double *statsA,
                           const int32_t *nB, const double *statsB) {
    for (int p = 0; p < HW; p++) {
        const int32_t na = nA[p], nb = nB[p];
        if (nb == 0) continue;
        for (int k = 0; k < K; k++)
            for (int c = 0; c < 3; c++) {
                double *a[ORC_NQ];
                const double *b[ORC_NQ];
                for (int q = 0; q < ORC_NQ; q++) {
                    a[q] = statsA + (((size_t)k * ORC_NQ + q) * 3 + c) * HW + p;
                    b[q] = statsB + (((size_t)k * ORC_NQ + q) * 3 + c) * HW + p;
                }
                if (na == 0) {
                    for (int q = 0; q < ORC_NQ; q++) *a[q] = *b[q];
                    continue;
                }
                const double fa = na, fb = nb, f = fa + fb;
                const double delta = *b[ORC_Q_MEAN] - *a[ORC_Q_MEAN];
                const double m2a = *a[ORC_Q_M2], m2b = *b[ORC_Q_M2];
                const double m3a = *a[ORC_Q_M3], m3b = *b[ORC_Q_M3];
                const double m4a = *a[ORC_Q_M4], m4b = *b[ORC_Q_M4];
                *a[ORC_Q_MEAN] = *a[ORC_Q_MEAN] + delta * fb / f;
                if (max_moment >= 2) *a[ORC_Q_M2] = m2a + m2b + delta * delta * fa * fb / f;
                if (max_moment >= 3)
                    *a[ORC_Q_M3] = m3a + m3b + delta * delta * delta * fa * fb * (fa - fb) / (f * f) +
                                   3.0 * delta * (fa * m2b - fb * m2a) / f;
                if (max_moment >= 4)
                    *a[ORC_Q_M4] = m4a + m4b +
                                   delta * delta * delta * delta * fa * fb * (fa * fa - fa * fb + fb * fb) /
                                       (f * f * f) +
                                   6.0 * delta * delta * (fa * fa * m2b + fb * fb * m2a) / (f * f) +
                                   4.0 * delta * (fa * m3b - fb * m3a) / f;
                if (max_moment >= 5) {
                    *a[ORC_Q_C2X] = *a[ORC_Q_C2X] + *b[ORC_Q_C2X];
                    *a[ORC_Q_C2Y] = *a[ORC_Q_C2Y] + *b[ORC_Q_C2Y];
                    *a[ORC_Q_M1] = *a[ORC_Q_M1] + *b[ORC_Q_M1];
                }
            }
        nA[p] = na + nb;
    }
}

/* ------------------------------------------------------------------------- */
/* Student-t quantiles. The upper tail of Student's t with nu degrees of      */
/* freedom is P(T > t) = I_x(nu/2, 1/2) / 2 with x = nu / (nu + t^2). The     */
/* regularised incomplete beta I_x(a, b) is evaluated from its continued      */
/* fraction (DLMF 8.17.22) with the modified Lentz method, switching to        */
/* 1 - I_{1-x}(b, a) beyond x = (a+1)/(a+b+2) where the fraction converges     */
/* slowly. The quantile is found by bisection in t.                           */
/* ------------------------------------------------------------------------- */
static double lentz_guard(double v) { return fabs(v) < 1e-300 ? 1e-300 : v; }

static double inc_beta_cf(double a, double b, double x) {
    /* g = 1 + d1/(1 + d2/(1 + ...)) by the modified Lentz method (b_0 = b_j = 1,
     * a_j = d_j) with d_{2m} = m(b-m)x/((a+2m-1)(a+2m)) and
     * d_{2m+1} = -(a+m)(a+b+m)x/((a+2m)(a+2m+1)); the fraction of DLMF 8.17.22
     * is 1/g. */
    double g = 1.0, C = 1.0, D = 0.0;
    for (int j = 1; j < 100000; j++) {
        double dj;
        if (j % 2 == 0) {
            const double m = (double)(j / 2);
            dj = m * (b - m) * x / ((a + 2.0 * m - 1.0) * (a + 2.0 * m));
        } else {
            const double m = (double)((j - 1) / 2);
            dj = -(a + m) * (a + b + m) * x / ((a + 2.0 * m) * (a + 2.0 * m + 1.0));
        }
        D = 1.0 / lentz_guard(1.0 + dj * D);
        C = lentz_guard(1.0 + dj / C);
        const double delta = C * D;
        g *= delta;
        if (fabs(delta - 1.0) < 1e-16) break;
    }
    return 1.0 / g;
}

static double inc_beta(double a, double b, double x) {
    if (x <= 0.0) return 0.0;
    if (x >= 1.0) return 1.0;
    const double front = exp(lgamma(a + b) - lgamma(a) - lgamma(b) + a * log(x) + b * log1p(-x));
    if (x < (a + 1.0) / (a + b + 2.0)) return front * inc_beta_cf(a, b, x) / a;
    return 1.0 - front * inc_beta_cf(b, a, 1.0 - x) / b;
}

static double t_upper(double t, double nu) {
    if (nu <= 0.0) return 0.5 * erfc(t / sqrt(2.0));
    return 0.5 * inc_beta(0.5 * nu, 0.5, nu / (nu + t * t));
}

double orc_t_quantile(double p, double nu) {
    /* p > 0.5: the t with P(T <= t) = p. */
    const double target = 1.0 - p;
    double lo = 0.0, hi = 1.0;
    while (t_upper(hi, nu) > target && hi < 1e12) hi *= 2.0;
    for (int it = 0; it < 400; it++) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (t_upper(mid, nu) > target) lo = mid;
        else hi = mid;
    }
    return 0.5 * (lo + hi);
}

void orc_tcrit2_table(double alpha, int N, double *table) {
    const double p = 1.0 - 0.5 * alpha;
    for (int m = 0; m <= N; m++) {
        const double t = m == 0 ? orc_t_quantile(p, 0.0) : orc_t_quantile(p, (double)N / m);
        table[m] = t * t;
    }
}

static double tcrit2_lookup(double u, int N, const double *table) {
    if (u > 1.0) u = 1.0;
    const double f = u * (double)N;
    int m = (int)f;
    if (m > N - 1) m = N - 1;
    const double frac = f - (double)m;
    return table[m] + frac * (table[m + 1] - table[m]);
}

/* ------------------------------------------------------------------------- */
/* Stage 2: per-pixel variance statistics and the variance filter.            */
/* ------------------------------------------------------------------------- */
#define S2_FLOOR 1e-30

static double range_arg(int nG, const orc_gbuf *gb, const double *gmean, size_t HW, size_t i,
                        size_t j) {
    double a = 0.0;
    for (int g = 0; g < nG; g++) {
        double d2 = 0.0;
        for (int ch = 0; ch < gb[g].channels; ch++) {
            const double *pl = gmean + (size_t)(gb[g].first_channel + ch) * HW;
            const double d = pl[i] - pl[j];
            d2 = d2 + d * d;
        }
        a = a + gb[g].dr_factor * d2;
    }
    return a;
}

typedef struct {
    int W, H, K, max_moment, R, nG;
    const int32_t *n;
    const double *stats, *gmean, *m2c_ext;
    double ds_factor, var_z;
    const orc_gbuf *gbufs;
    double *jb, *lnS2, *se2, *m2C, *varD, *varCD;
    double *s2, *s2c; /* scratch [K][3][HW] */
} vars_ctx;

static void vars_stats_range(void *vctx, int64_t b, int64_t e) {
    vars_ctx *c = (vars_ctx *)vctx;
    const size_t HW = (size_t)c->W * c->H;
    const double z = c->var_z;
    for (int64_t p = b; p < e; p++) {
        const int nn = c->n[p];
        const double n = (double)nn;
        for (int k = 0; k < c->K; k++) {
            double jbsum = 0.0;
            for (int ch = 0; ch < 3; ch++) {
                const size_t o = ((size_t)k * 3 + ch) * HW + p;
                const double *st = c->stats + ((size_t)(k * ORC_NQ) * 3 + ch) * HW + p;
                if (nn < 2) {
                    c->s2[o] = c->s2c[o] = 0.0;
                    c->lnS2[o] = c->se2[o] = c->m2C[o] = 0.0;
                    continue;
                }
                const double M2 = st[(size_t)ORC_Q_M2 * 3 * HW];
                const double M3 = st[(size_t)ORC_Q_M3 * 3 * HW];
                const double M4 = st[(size_t)ORC_Q_M4 * 3 * HW];
                const double s2 = M2 / (n - 1.0);
                const double cB = n > z + 1.0 ? n / (n - z) : 1.0;
                const double kurt = (c->max_moment >= 4 && M2 > 0.0) ? n * M4 / (M2 * M2) : 3.0;
                double m2c = M2;
                if (k == 0 && c->m2c_ext) {
                    m2c = c->m2c_ext[(size_t)ch * HW + p];
                } else if (c->max_moment >= 5) {
                    const double cx = st[(size_t)ORC_Q_C2X * 3 * HW];
                    const double cy = st[(size_t)ORC_Q_C2Y * 3 * HW];
                    m2c = M2 - 12.0 * (cx * cx + cy * cy) / n;
                    if (m2c < 0.0) m2c = 0.0;
                }
                c->s2[o] = s2;
                c->s2c[o] = m2c / (n - 1.0);
                c->m2C[o] = m2c;
                c->lnS2[o] = log(cB * (s2 > S2_FLOOR ? s2 : S2_FLOOR));
                c->se2[o] = cB * cB * (kurt - (n - 3.0) / n) / (n - 1.0);
                if (M2 > 0.0) {
                    const double skew2 = n * M3 * M3 / (M2 * M2 * M2);
                    double jbc = skew2;
                    if (c->max_moment >= 4) jbc = jbc + (kurt - 3.0) * (kurt - 3.0) / 4.0;
                    jbsum = jbsum + n / 6.0 * jbc;
                }
            }
            c->jb[(size_t)k * HW + p] = nn < 2 ? 0.0 : jbsum;
        }
    }
}

static void vars_filter_range(void *vctx, int64_t b, int64_t e) {
    vars_ctx *c = (vars_ctx *)vctx;
    const int W = c->W, H = c->H, R = c->R, K = c->K;
    const size_t HW = (size_t)W * H;
    const double z2 = c->var_z * c->var_z;
    double *sw = (double *)malloc(sizeof(double) * K * 3 * 3);
    for (int64_t row = b; row < e; row++) {
        const int y = (int)row;
        for (int x = 0; x < W; x++) {
            const size_t i = (size_t)y * W + x;
            if (c->n[i] < 2) {
                for (int k = 0; k < K; k++)
                    for (int ch = 0; ch < 3; ch++) {
                        c->varD[((size_t)k * 3 + ch) * HW + i] = 0.0;
                        c->varCD[((size_t)k * 3 + ch) * HW + i] = 0.0;
                    }
                continue;
            }
            memset(sw, 0, sizeof(double) * K * 9);
            for (int dy = -R; dy <= R; dy++) {
                const int yy = y + dy;
                if (yy < 0 || yy >= H) continue;
                for (int dx = -R; dx <= R; dx++) {
                    const int xx = x + dx;
                    if (xx < 0 || xx >= W) continue;
                    const size_t j = (size_t)yy * W + xx;
                    if (c->n[j] < 2) continue;
                    const double w = exp(c->ds_factor * (double)(dx * dx + dy * dy) +
                                         range_arg(c->nG, c->gbufs, c->gmean, HW, i, j));
                    for (int k = 0; k < K; k++)
                        for (int ch = 0; ch < 3; ch++) {
                            const size_t oi = ((size_t)k * 3 + ch) * HW + i;
                            const size_t oj = ((size_t)k * 3 + ch) * HW + j;
                            if (j != i) {
                                const double dl = c->lnS2[oi] - c->lnS2[oj];
                                if (dl * dl > z2 * (c->se2[oi] + c->se2[oj])) continue;
                            }
                            double *a = sw + (k * 3 + ch) * 3;
                            a[0] = a[0] + w;
                            a[1] = a[1] + w * c->s2[oj];
                            a[2] = a[2] + w * c->s2c[oj];
                        }
                }
            }
            for (int k = 0; k < K; k++)
                for (int ch = 0; ch < 3; ch++) {
                    const double *a = sw + (k * 3 + ch) * 3;
                    c->varD[((size_t)k * 3 + ch) * HW + i] = a[1] / a[0];
                    c->varCD[((size_t)k * 3 + ch) * HW + i] = a[2] / a[0];
                }
        }
    }
    free(sw);
}

void orc_denoise_vars_f64(int W, int H, int K, int max_moment, const int32_t *n,
                          const double *stats, int R, double ds_factor, double var_z, int nG,
                          const orc_gbuf *gbufs, const double *gmean, const double *m2c_ext,
                          double *jb, double *lnS2, double *se2, double *m2C, double *varD,
                          double *varCD, int nthreads) {
    const size_t HW = (size_t)W * H;
    vars_ctx c;
    c.W = W; c.H = H; c.K = K; c.max_moment = max_moment; c.R = R; c.nG = nG;
    c.n = n; c.stats = stats; c.gmean = gmean; c.m2c_ext = m2c_ext;
    c.ds_factor = ds_factor; c.var_z = var_z; c.gbufs = gbufs;
    c.jb = jb; c.lnS2 = lnS2; c.se2 = se2; c.m2C = m2C; c.varD = varD; c.varCD = varCD;
    c.s2 = (double *)malloc(sizeof(double) * K * 3 * HW);
    c.s2c = (double *)malloc(sizeof(double) * K * 3 * HW);
    parallel_for((int64_t)HW, nthreads, vars_stats_range, &c);
    parallel_for(H, nthreads, vars_filter_range, &c);
    free(c.s2);
    free(c.s2c);
}

/* ------------------------------------------------------------------------- */
/* Stage 2c: Welch-discriminated mean filter (denoiseFilm).                   */
/* ------------------------------------------------------------------------- */
typedef struct {
    int W, H, K, R, nG, use_levc, discr_source, mt_mode, lut_n;
    const int32_t *n;
    const double *stats, *varD, *varCD, *m2C, *jb, *tcrit2, *gmean, *film;
    double ds_factor;
    const orc_gbuf *gbufs;
    double *discr, *filmD;
    double *ediv; /* scratch [K][3][HW]: discr^2 / (n-1) */
    uint32_t *accept_bits;
} film_ctx;

static void film_discr_range(void *vctx, int64_t b, int64_t e) {
    film_ctx *c = (film_ctx *)vctx;
    const size_t HW = (size_t)c->W * c->H;
    for (int64_t p = b; p < e; p++) {
        const double n = (double)c->n[p];
        for (int k = 0; k < c->K; k++)
            for (int ch = 0; ch < 3; ch++) {
                const size_t o = ((size_t)k * 3 + ch) * HW + p;
                if (c->n[p] < 2) {
                    c->discr[o] = 0.0;
                    c->ediv[o] = 0.0;
                    continue;
                }
                /* the reference's CASCADE_MODE: denoised variance (1, default) or the
                 * pixel's own sample variance (0, the "M" build) */
                double v;
                if (c->discr_source == 1) {
                    const double m2 = c->use_levc ? c->m2C[o]
                                                  : c->stats[((size_t)(k * ORC_NQ + ORC_Q_M2) * 3 + ch) * HW + p];
                    v = m2 / (n - 1.0);
                } else {
                    v = c->use_levc ? c->varCD[o] : c->varD[o];
                }
                const double d = v / n;
                c->discr[o] = d;
                c->ediv[o] = d * d / (n - 1.0);
            }
    }
}

static int welch_accept(const film_ctx *c, size_t HW, int k, size_t i, size_t j) {
    for (int ch = 0; ch < 3; ch++) {
        const size_t oi = ((size_t)k * 3 + ch) * HW + i;
        const size_t oj = ((size_t)k * 3 + ch) * HW + j;
        /* transform 0 compares the film, as denoiseFilm receives filmBuffer for the
         * untransformed set (estimator.cpp:432) */
        double diff;
        if (k == 0) {
            diff = c->film[(size_t)ch * HW + i] - c->film[(size_t)ch * HW + j];
        } else {
            const size_t mi = ((size_t)(k * ORC_NQ + ORC_Q_MEAN) * 3 + ch) * HW + i;
            const size_t mj = ((size_t)(k * ORC_NQ + ORC_Q_MEAN) * 3 + ch) * HW + j;
            diff = c->stats[mi] - c->stats[mj];
        }
        const double s = c->discr[oi] + c->discr[oj];
        if (!(s > 0.0)) {
            if (diff != 0.0) return 0;
            continue;
        }
        const double u = (c->ediv[oi] + c->ediv[oj]) / (s * s);
        const double t2 = tcrit2_lookup(u, c->lut_n, c->tcrit2);
        if (diff * diff > t2 * s) return 0;
    }
    return 1;
}

static void film_filter_range(void *vctx, int64_t b, int64_t e) {
    film_ctx *c = (film_ctx *)vctx;
    const int W = c->W, H = c->H, R = c->R, K = c->K;
    const size_t HW = (size_t)W * H;
    const int D = 2 * R + 1;
    const int words = (D * D + 31) / 32;
    for (int64_t row = b; row < e; row++) {
        const int y = (int)row;
        for (int x = 0; x < W; x++) {
            const size_t i = (size_t)y * W + x;
            uint32_t *bits = c->accept_bits ? c->accept_bits + i * (size_t)K * words : NULL;
            if (bits) memset(bits, 0, sizeof(uint32_t) * K * words);
            if (c->n[i] < 2) {
                for (int ch = 0; ch < 3; ch++) c->filmD[(size_t)ch * HW + i] = c->film[(size_t)ch * HW + i];
                continue;
            }
            int ksel = -1;
            if (c->mt_mode == ORC_MT_JB) {
                ksel = 0;
                for (int k = 1; k < K; k++)
                    if (c->jb[(size_t)k * HW + i] < c->jb[(size_t)ksel * HW + i]) ksel = k;
            }
            double sw = 0.0, sf[3] = {0.0, 0.0, 0.0};
            for (int dy = -R; dy <= R; dy++) {
                const int yy = y + dy;
                if (yy < 0 || yy >= H) continue;
                for (int dx = -R; dx <= R; dx++) {
                    const int xx = x + dx;
                    if (xx < 0 || xx >= W) continue;
                    const size_t j = (size_t)yy * W + xx;
                    if (c->n[j] < 2) continue;
                    const int bit = (dy + R) * D + (dx + R);
                    int acc = 1;
                    for (int k = 0; k < K; k++) {
                        const int a = (j == i) ? 1 : welch_accept(c, HW, k, i, j);
                        if (bits && a) bits[k * words + bit / 32] |= 1u << (bit % 32);
                        if (ksel < 0 || ksel == k) acc = acc && a;
                    }
                    if (!acc) continue;
                    const double w = exp(c->ds_factor * (double)(dx * dx + dy * dy) +
                                         range_arg(c->nG, c->gbufs, c->gmean, HW, i, j));
                    sw = sw + w;
                    for (int ch = 0; ch < 3; ch++) sf[ch] = sf[ch] + w * c->film[(size_t)ch * HW + j];
                }
            }
            for (int ch = 0; ch < 3; ch++) c->filmD[(size_t)ch * HW + i] = sf[ch] / sw;
        }
    }
}

void orc_denoise_film_f64(int W, int H, int K, const int32_t *n, const double *stats,
                          const double *varD, const double *varCD, const double *jb, int use_levc,
                          int discr_source, const double *m2C,
                          int mt_mode, int R, double ds_factor, int lut_n, const double *tcrit2,
                          int nG, const orc_gbuf *gbufs, const double *gmean, const double *film,
                          double *discr, double *filmD, uint32_t *accept_bits, int nthreads) {
    const size_t HW = (size_t)W * H;
    film_ctx c;
    c.W = W; c.H = H; c.K = K; c.R = R; c.nG = nG; c.use_levc = use_levc; c.mt_mode = mt_mode;
    c.discr_source = discr_source; c.m2C = m2C;
    c.lut_n = lut_n; c.n = n; c.stats = stats; c.varD = varD; c.varCD = varCD; c.jb = jb;
    c.tcrit2 = tcrit2; c.gmean = gmean; c.film = film; c.ds_factor = ds_factor; c.gbufs = gbufs;
    c.discr = discr; c.filmD = filmD; c.accept_bits = accept_bits;
    c.ediv = (double *)malloc(sizeof(double) * K * 3 * HW);
    parallel_for((int64_t)HW, nthreads, film_discr_range, &c);
    parallel_for(H, nthreads, film_filter_range, &c);
    free(c.ediv);
}

/* ------------------------------------------------------------------------- */
/* Target SPP.                                                                */
/* ------------------------------------------------------------------------- */
#define TREE_BLOCK 1024
#define TREE_THREADS 256

static double tree_block(const double *x, int64_t m) {
    double part[TREE_THREADS];
    for (int t = 0; t < TREE_THREADS; t++) {
        double v[4];
        for (int r = 0; r < 4; r++) {
            const int64_t idx = t + (int64_t)TREE_THREADS * r;
            v[r] = idx < m ? x[idx] : 0.0;
        }
        part[t] = ((v[0] + v[1]) + v[2]) + v[3];
    }
    for (int s = TREE_THREADS / 2; s >= 1; s >>= 1)
        for (int t = 0; t < s; t++) part[t] = part[t] + part[t + s];
    return part[0];
}

double orc_tree_sum(const double *v, int64_t len) {
    if (len <= 0) return 0.0;
    double *cur = (double *)malloc(sizeof(double) * len);
    memcpy(cur, v, sizeof(double) * len);
    while (len > 1) {
        const int64_t nb = (len + TREE_BLOCK - 1) / TREE_BLOCK;
        double *next = (double *)malloc(sizeof(double) * nb);
        for (int64_t bb = 0; bb < nb; bb++) {
            const int64_t m = len - bb * TREE_BLOCK < TREE_BLOCK ? len - bb * TREE_BLOCK : TREE_BLOCK;
            next[bb] = tree_block(cur + bb * TREE_BLOCK, m);
        }
        free(cur);
        cur = next;
        len = nb;
    }
    const double r = cur[0];
    free(cur);
    return r;
}

void orc_calc_target_spp(int W, int H, int spp, const int32_t *n, const double *varD,
                         const double *mean, double eps, int tmin, int tmax, int32_t *target) {
    orc_calc_target_spp_src(W, H, spp, n, varD, NULL, 0, mean, eps, tmin, tmax, target);
}

void orc_calc_target_spp_src(int W, int H, int spp, const int32_t *n, const double *varD,
                             const double *m2, int as_source, const double *mean, double eps, int tmin,
                             int tmax, int32_t *target) {
    const size_t HW = (size_t)W * H;
    double *e = (double *)calloc(HW ? HW : 1, sizeof(double));
    for (size_t p = 0; p < HW; p++) {
        if (n[p] < 2) {
            e[p] = 0.0;
            continue;
        }
        const double nn = (double)n[p];
        double acc = 0.0;
        for (int ch = 0; ch < 3; ch++) {
            /* the reference's AS_MODE: denoised variance ("ASM") or the sample variance ("ASN") */
            const double var = as_source == 1 ? m2[(size_t)ch * HW + p] / (nn - 1.0) : varD[(size_t)ch * HW + p];
            double v = var / nn;
            if (mean) {
                const double m = mean[(size_t)ch * HW + p];
                v = v / (m * m + eps);
            }
            acc = acc + v;
        }
        e[p] = acc;
    }
    const double total = orc_tree_sum(e, (int64_t)HW);
    const double budget = (double)spp * (double)HW;
    for (size_t p = 0; p < HW; p++) {
        double t;
        if (n[p] < 2) t = (double)tmax;
        else if (!(total > 0.0)) t = (double)spp;
        else t = rint(budget * e[p] / total);
        if (t < tmin) t = tmin;
        if (t > tmax) t = tmax;
        target[p] = (int32_t)t;
    }
    free(e);
}

void orc_calc_mean_var_f32(int HW, const int32_t *n, const float *m2, float *var) {
    for (int ch = 0; ch < 3; ch++)
        for (int p = 0; p < HW; p++) {
            const float nPF = (float)n[p];
            var[(size_t)ch * HW + p] = m2[(size_t)ch * HW + p] / ((nPF - 1.f) * nPF);
        }
}

/* ------------------------------------------------------------------------- */
/* LEV: per-pixel ridge regression of radiance on the feature channels.       */
/* ------------------------------------------------------------------------- */
int orc_lev_nstate(int G) {
    const int P0 = G + 3;
    return 1 + 2 * P0 + G * (G + 1) / 2 + 3 * G + 3;
}

typedef struct {
    int W, H, G, S;
    const float *samples;
    const int32_t *count;
    double *state;
    double lambda;
    const double *cstate;
    double *beta, *m2C, *r2;
} lev_ctx;

static void lev_acc_range(void *vctx, int64_t b, int64_t e) {
    lev_ctx *c = (lev_ctx *)vctx;
    const int G = c->G, P0 = G + 3, NCH = 5 + G;
    const size_t HW = (size_t)c->W * c->H;
    const int oP = 1, oS = 1 + P0, oFF = 1 + 2 * P0, oFY = oFF + G * (G + 1) / 2, oYY = oFY + 3 * G;
    double z[64];
    for (int64_t p = b; p < e; p++) {
        double *st = c->state + p;
#define ST(i) st[(size_t)(i) * HW]
        const int cnt = c->count ? c->count[p] : c->S;
        for (int s = 0; s < cnt; s++) {
            const float *sp = c->samples + (size_t)s * NCH * HW + p;
            double v[64];
            for (int g = 0; g < G; g++) v[g] = (double)sp[(size_t)(5 + g) * HW];
            for (int ch = 0; ch < 3; ch++) v[G + ch] = (double)sp[(size_t)ch * HW];
            if (ST(0) == 0.0)
                for (int a = 0; a < P0; a++) ST(oP + a) = v[a];
            ST(0) = ST(0) + 1.0;
            for (int a = 0; a < P0; a++) {
                z[a] = v[a] - ST(oP + a);
                ST(oS + a) = ST(oS + a) + z[a];
            }
            int q = 0;
            for (int a = 0; a < G; a++)
                for (int bb = a; bb < G; bb++, q++) ST(oFF + q) = ST(oFF + q) + z[a] * z[bb];
            for (int a = 0; a < G; a++)
                for (int ch = 0; ch < 3; ch++)
                    ST(oFY + a * 3 + ch) = ST(oFY + a * 3 + ch) + z[a] * z[G + ch];
            for (int ch = 0; ch < 3; ch++) ST(oYY + ch) = ST(oYY + ch) + z[G + ch] * z[G + ch];
        }
#undef ST
    }
}

void orc_lev_accumulate_f64(int W, int H, int G, int S, const float *samples, const int32_t *count,
                            double *state, int nthreads) {
    lev_ctx c;
    memset(&c, 0, sizeof(c));
    c.W = W; c.H = H; c.G = G; c.S = S; c.samples = samples; c.count = count; c.state = state;
    parallel_for((int64_t)W * H, nthreads, lev_acc_range, &c);
}

static void lev_solve_range(void *vctx, int64_t b, int64_t e) {
    lev_ctx *c = (lev_ctx *)vctx;
    const int G = c->G, P0 = G + 3;
    const size_t HW = (size_t)c->W * c->H;
    const int oP = 1, oS = 1 + P0, oFF = 1 + 2 * P0, oFY = oFF + G * (G + 1) / 2, oYY = oFY + 3 * G;
    double Cff[16][16], L[16][16], cfy[16][3], cyy[3], mean[32], beta[16], tmp[16];
    for (int64_t p = b; p < e; p++) {
        const double *st = c->cstate + p;
#define ST(i) st[(size_t)(i) * HW]
        const double n = ST(0);
        if (n < 2.0) {
            for (int ch = 0; ch < 3; ch++) {
                c->m2C[(size_t)ch * HW + p] = 0.0;
                c->r2[(size_t)ch * HW + p] = 0.0;
                for (int a = 0; a <= G; a++) c->beta[((size_t)ch * (G + 1) + a) * HW + p] = 0.0;
            }
            continue;
        }
        for (int a = 0; a < P0; a++) mean[a] = ST(oP + a) + ST(oS + a) / n;
        int q = 0;
        for (int a = 0; a < G; a++)
            for (int bb = a; bb < G; bb++, q++) {
                const double v = ST(oFF + q) - ST(oS + a) * ST(oS + bb) / n;
                Cff[a][bb] = v;
                Cff[bb][a] = v;
            }
        for (int a = 0; a < G; a++)
            for (int ch = 0; ch < 3; ch++)
                cfy[a][ch] = ST(oFY + a * 3 + ch) - ST(oS + a) * ST(oS + G + ch) / n;
        for (int ch = 0; ch < 3; ch++) cyy[ch] = ST(oYY + ch) - ST(oS + G + ch) * ST(oS + G + ch) / n;
#undef ST
        /* Cholesky of A = Cff/n + lambda*I. */
        for (int a = 0; a < G; a++)
            for (int bb = 0; bb <= a; bb++) {
                double sum = Cff[a][bb] / n + (a == bb ? c->lambda : 0.0);
                for (int m = 0; m < bb; m++) sum = sum - L[a][m] * L[bb][m];
                if (a == bb) L[a][a] = sqrt(sum > 0.0 ? sum : 1e-300);
                else L[a][bb] = sum / L[bb][bb];
            }
        for (int ch = 0; ch < 3; ch++) {
            for (int a = 0; a < G; a++) {
                double sum = cfy[a][ch] / n;
                for (int m = 0; m < a; m++) sum = sum - L[a][m] * tmp[m];
                tmp[a] = sum / L[a][a];
            }
            for (int a = G - 1; a >= 0; a--) {
                double sum = tmp[a];
                for (int m = a + 1; m < G; m++) sum = sum - L[m][a] * beta[m];
                beta[a] = sum / L[a][a];
            }
            double bc = 0.0, bab = 0.0, icpt = mean[G + ch];
            for (int a = 0; a < G; a++) {
                bc = bc + beta[a] * cfy[a][ch];
                double row = 0.0;
                for (int bb = 0; bb < G; bb++) row = row + Cff[a][bb] * beta[bb];
                bab = bab + beta[a] * row;
                icpt = icpt - beta[a] * mean[a];
            }
            double rss = cyy[ch] - 2.0 * bc + bab;
            if (rss < 0.0) rss = 0.0;
            c->m2C[(size_t)ch * HW + p] = rss;
            c->r2[(size_t)ch * HW + p] = cyy[ch] > 0.0 ? 1.0 - rss / cyy[ch] : 0.0;
            c->beta[((size_t)ch * (G + 1)) * HW + p] = icpt;
            for (int a = 0; a < G; a++) c->beta[((size_t)ch * (G + 1) + 1 + a) * HW + p] = beta[a];
        }
    }
}

void orc_lev_solve_f64(int W, int H, int G, const double *state, double lambda, double *beta,
                       double *m2C, double *r2, int nthreads) {
    lev_ctx c;
    memset(&c, 0, sizeof(c));
    c.W = W; c.H = H; c.G = G; c.cstate = state; c.lambda = lambda;
    c.beta = beta; c.m2C = m2C; c.r2 = r2;
    parallel_for((int64_t)W * H, nthreads, lev_solve_range, &c);
}

/* ---------------------------------------------------------------------------
 * Film path: FilmTile::AddSample with the box filter of radius 0.5
 * (core/film.h:152-190; filter width forced in core/api.cpp:1713-1739) and
 * Film::UpdateImage (core/film.cpp:187-222), colour matrices of
 * core/spectrum.h:66-76, luminance weights of core/spectrum.h:483-486.
 * ------------------------------------------------------------------------- */
static const float kRgbToXyz[3][3] = {{0.412453f, 0.357580f, 0.180423f},
                                      {0.212671f, 0.715160f, 0.072169f},
                                      {0.019334f, 0.119193f, 0.950227f}};
static const float kXyzToRgb[3][3] = {{3.240479f, -1.537150f, -0.498535f},
                                      {-0.969256f, 1.875991f, 0.041556f},
                                      {0.055648f, -0.204043f, 1.057311f}};
static const float kYWeight[3] = {0.212671f, 0.715160f, 0.072169f};

void orc_film_constants(float *rgb_to_xyz, float *xyz_to_rgb, float *y_weight) {
    memcpy(rgb_to_xyz, kRgbToXyz, sizeof(kRgbToXyz));
    memcpy(xyz_to_rgb, kXyzToRgb, sizeof(kXyzToRgb));
    memcpy(y_weight, kYWeight, sizeof(kYWeight));
}

/* The box filter's support of a sample at pFilm = pixel + (u, v) covers pixels
 * ceil(x + u - 1) .. floor(x + u) (film.h:158-161 with radius 0.5): the own
 * pixel, plus the left one when u == 0 and the right one when u == 1 (same in
 * y). Every covered pixel inside the image gets weight 1 (BoxFilter::Evaluate).
 * Samples of pixel p go to contrib_sum/weight_sum of p in sample order; those
 * that also cover a neighbour q are summed into spill of q, visiting pixels in
 * row-major order and their samples in order. */
void orc_film_add_samples(int W, int H, int G, int S, const float *samples, const int32_t *count,
                          float max_lum, float *contrib_sum, float *weight_sum, float *spill) {
    const size_t HW = (size_t)W * H;
    const size_t NCH = 5 + (size_t)G;
    for (size_t p = 0; p < HW; p++) {
        const int x = (int)(p % W), y = (int)(p / W);
        int cnt = count ? count[p] : S;
        if (cnt < 0) cnt = 0;
        if (cnt > S) cnt = S;
        for (int s = 0; s < cnt; s++) {
            const float *sp = samples + (size_t)s * NCH * HW + p;
            float L[3] = {sp[0], sp[HW], sp[2 * HW]};
            const float u = sp[3 * HW], v = sp[4 * HW];
            const float lum = kYWeight[0] * L[0] + kYWeight[1] * L[1] + kYWeight[2] * L[2];
            if (lum > max_lum) {
                const float f = max_lum / lum;
                for (int c = 0; c < 3; c++) L[c] = L[c] * f;
            }
            for (int c = 0; c < 3; c++) contrib_sum[c * HW + p] = contrib_sum[c * HW + p] + L[c];
            weight_sum[p] = weight_sum[p] + 1.0f;
            const int dx0 = u == 0.0f ? -1 : 0, dx1 = u == 1.0f ? 1 : 0;
            const int dy0 = v == 0.0f ? -1 : 0, dy1 = v == 1.0f ? 1 : 0;
            for (int dy = dy0; dy <= dy1; dy++)
                for (int dx = dx0; dx <= dx1; dx++) {
                    if (dx == 0 && dy == 0) continue;
                    const int qx = x + dx, qy = y + dy;
                    if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
                    const size_t q = (size_t)qy * W + qx;
                    for (int c = 0; c < 3; c++) spill[c * HW + q] = spill[c * HW + q] + L[c];
                    spill[3 * HW + q] = spill[3 * HW + q] + 1.0f;
                }
        }
    }
}

static void rgb_to_xyz(const float *rgb, float *xyz) {
    for (int i = 0; i < 3; i++)
        xyz[i] = kRgbToXyz[i][0] * rgb[0] + kRgbToXyz[i][1] * rgb[1] + kRgbToXyz[i][2] * rgb[2];
}

/* Film::UpdateImage without splats (the statistics integrator splats nothing):
 * xyz = RGBToXYZ(own sum) + RGBToXYZ(spill), as MergeFilmTile adds each tile's
 * converted sum (film.cpp:140-149); rgb = max(0, XYZToRGB(xyz) / w) when w != 0;
 * times scale. */
void orc_film_update_image(int W, int H, const float *contrib_sum, const float *weight_sum,
                           const float *spill, float scale, float *rgb) {
    const size_t HW = (size_t)W * H;
    for (size_t p = 0; p < HW; p++) {
        float own[3], sp[3], a[3], b[3], xyz[3], out[3];
        for (int c = 0; c < 3; c++) {
            own[c] = contrib_sum[c * HW + p];
            sp[c] = spill ? spill[c * HW + p] : 0.0f;
        }
        rgb_to_xyz(own, a);
        rgb_to_xyz(sp, b);
        for (int i = 0; i < 3; i++) xyz[i] = (0.0f + a[i]) + b[i];
        for (int i = 0; i < 3; i++)
            out[i] = kXyzToRgb[i][0] * xyz[0] + kXyzToRgb[i][1] * xyz[1] + kXyzToRgb[i][2] * xyz[2];
        const float w = weight_sum[p] + (spill ? spill[3 * HW + p] : 0.0f);
        if (w != 0.0f) {
            const float inv = 1.0f / w;
            for (int i = 0; i < 3; i++) {
                const float t = out[i] * inv;
                out[i] = 0.0f < t ? t : 0.0f;
            }
        }
        for (int i = 0; i < 3; i++) rgb[i * HW + p] = out[i] * scale;
    }
}
