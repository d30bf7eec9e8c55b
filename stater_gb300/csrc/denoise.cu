// Stage 2, plain FP64 form: one image per launch, one thread per
// (pixel, transform), neighbours read through L1/L2. Compiled with
// -fmad=false so that every operation rounds like the FP64 oracle.
//
// Formulas (per pixel i, transform b, channel c; n = n_i):
//   s2    = m2 / (n - 1)
//   cB    = n / (n - z) if n > z + 1 else 1           (Bonett 2006 small-sample factor)
//   kurt  = n m4 / m2^2 (3 when m4 is not tracked or m2 == 0)
//   lnS2  = ln(cB * max(s2, 1e-30)),  se2 = cB^2 (kurt - (n-3)/n) / (n - 1)
//   jb    = sum_c n/6 (n m3^2 / m2^3 + (kurt - 3)^2 / 4)  (kurtosis term only with m4)
//   m2C   = max(m2 - 12 (c2X^2 + c2Y^2) / n, 0)        (regression on the uniform
//           in-pixel offset, variance 1/12), or the external LEV result
//   varD  = sum_j w_ij a_ij s2_j / sum_j w_ij a_ij, varCD likewise with m2C_j/(n_j-1)
//   a_ij  = [ (lnS2_i - lnS2_j)^2 <= z^2 (se2_i + se2_j) ]
//   w_ij  = exp(ds |p_i - p_j|^2 + sum_g dr_g |G_g(i) - G_g(j)|^2)
//   discr = v / n (v = varCD with LEV, else varD), e = discr^2 / (n - 1)
//   Welch: reject if (mu_i - mu_j)^2 > t2(u) (d_i + d_j), u = (e_i + e_j)/(d_i + d_j)^2 = 1/df
//   filmD = sum_j w_ij A_ij film_j / sum_j w_ij A_ij
#include <cmath>

#include "denoise_params.cuh"

namespace stater {

namespace {

__device__ inline double range_arg(const GBuf<double> &gb, size_t i, size_t j, size_t HW) {
    double a = 0.0;
    for (int g = 0; g < gb.count; g++) {
        double d2 = 0.0;
        for (int ch = 0; ch < gb.channels[g]; ch++) {
            const double *pl = gb.planes[g] + (size_t)ch * HW;
            const double d = pl[i] - pl[j];
            d2 = d2 + d * d;
        }
        a = a + gb.dr[g] * d2;
    }
    return a;
}

__global__ void vars_stats_f64(VarsParams<double> P) {
    const size_t HW = (size_t)P.W * P.H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (p >= HW) return;
    const int nn = P.n[p];
    const double n = (double)nn;
    const double z = P.z;
    double jbsum = 0.0;
    for (int c = 0; c < 3; c++) {
        const size_t o = (size_t)c * HW + p;
        const size_t so = ((size_t)k * 3 + c) * HW + p;
        if (nn < 2) {
            P.s2[so] = 0.0;
            P.s2c[so] = 0.0;
            P.lnS2[k][o] = 0.0;
            P.se2[k][o] = 0.0;
            P.m2C[k][o] = 0.0;
            continue;
        }
        const double M2 = P.m2[k][o];
        const double M3 = P.m3[k][o];
        const double M4 = P.max_moment >= 4 ? P.m4[k][o] : 0.0;
        const double s2 = M2 / (n - 1.0);
        const double cB = n > z + 1.0 ? n / (n - z) : 1.0;
        const double kurt = (P.max_moment >= 4 && M2 > 0.0) ? n * M4 / (M2 * M2) : 3.0;
        double m2c = M2;
        if (k == 0 && P.m2c_in) {
            m2c = P.m2c_in[o];
        } else if (P.max_moment >= 5) {
            const double cx = P.cx[k][o], cy = P.cy[k][o];
            m2c = M2 - 12.0 * (cx * cx + cy * cy) / n;
            if (m2c < 0.0) m2c = 0.0;
        }
        P.s2[so] = s2;
        P.s2c[so] = m2c / (n - 1.0);
        P.m2C[k][o] = m2c;
        P.lnS2[k][o] = log(cB * (s2 > (double)kS2Floor ? s2 : (double)kS2Floor));
        P.se2[k][o] = cB * cB * (kurt - (n - 3.0) / n) / (n - 1.0);
        if (M2 > 0.0) {
            double jbc = n * M3 * M3 / (M2 * M2 * M2);
            if (P.max_moment >= 4) jbc = jbc + (kurt - 3.0) * (kurt - 3.0) / 4.0;
            jbsum = jbsum + n / 6.0 * jbc;
        }
    }
    P.jb[k][p] = nn < 2 ? 0.0 : jbsum;
}

__global__ void vars_filter_f64(VarsParams<double> P) {
    const size_t HW = (size_t)P.W * P.H;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (i >= HW) return;
    if (P.n[i] < 2) {
        for (int c = 0; c < 3; c++) {
            P.varD[k][(size_t)c * HW + i] = 0.0;
            P.varCD[k][(size_t)c * HW + i] = 0.0;
        }
        return;
    }
    const int x = (int)(i % P.W), y = (int)(i / P.W);
    const int R = P.R;
    const double z2 = P.z * P.z;
    const double *lnS2 = P.lnS2[k];
    const double *se2 = P.se2[k];
    const double *s2 = P.s2 + (size_t)k * 3 * HW;
    const double *s2c = P.s2c + (size_t)k * 3 * HW;
    double sw[3] = {0.0, 0.0, 0.0}, sv[3] = {0.0, 0.0, 0.0}, svc[3] = {0.0, 0.0, 0.0};
    for (int dy = -R; dy <= R; dy++) {
        const int yy = y + dy;
        if (yy < 0 || yy >= P.H) continue;
        for (int dx = -R; dx <= R; dx++) {
            const int xx = x + dx;
            if (xx < 0 || xx >= P.W) continue;
            const size_t j = (size_t)yy * P.W + xx;
            if (P.n[j] < 2) continue;
            const double w = exp(P.ds * (double)(dx * dx + dy * dy) + range_arg(P.gb, i, j, HW));
            for (int c = 0; c < 3; c++) {
                const size_t oi = (size_t)c * HW + i, oj = (size_t)c * HW + j;
                if (j != i) {
                    const double dl = lnS2[oi] - lnS2[oj];
                    if (dl * dl > z2 * (se2[oi] + se2[oj])) continue;
                }
                sw[c] = sw[c] + w;
                sv[c] = sv[c] + w * s2[oj];
                svc[c] = svc[c] + w * s2c[oj];
            }
        }
    }
    for (int c = 0; c < 3; c++) {
        P.varD[k][(size_t)c * HW + i] = sv[c] / sw[c];
        P.varCD[k][(size_t)c * HW + i] = svc[c] / sw[c];
    }
}

__global__ void film_discr_f64(FilmParams<double> P) {
    const size_t HW = (size_t)P.W * P.H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (p >= HW) return;
    const double n = (double)P.n[p];
    for (int c = 0; c < 3; c++) {
        const size_t o = (size_t)c * HW + p;
        double *e = P.ediv + (size_t)k * 3 * HW;
        if (P.n[p] < 2) {
            P.discr[k][o] = 0.0;
            e[o] = 0.0;
            continue;
        }
        // CASCADE_MODE: the denoised variance, or the pixel's own sample variance
        const double v = P.discr_source == STATER_DISCR_SAMPLE ? P.m2s[k][o] / (n - 1.0)
                                                               : (P.use_levc ? P.varCD[k][o] : P.varD[k][o]);
        const double d = v / n;
        P.discr[k][o] = d;
        e[o] = d * d / (n - 1.0);
    }
}

__device__ inline double lut_lookup(const double *lut, int N, double u) {
    if (u > 1.0) u = 1.0;
    const double f = u * (double)N;
    int m = (int)f;
    if (m > N - 1) m = N - 1;
    const double frac = f - (double)m;
    return lut[m] + frac * (lut[m + 1] - lut[m]);
}

__device__ inline int welch_accept_f64(const FilmParams<double> &P, size_t HW, int k, size_t i, size_t j) {
    const double *mu = k == 0 ? P.film : P.mean[k];
    const double *d = P.discr[k];
    const double *e = P.ediv + (size_t)k * 3 * HW;
    for (int c = 0; c < 3; c++) {
        const size_t oi = (size_t)c * HW + i, oj = (size_t)c * HW + j;
        const double diff = mu[oi] - mu[oj];
        const double s = d[oi] + d[oj];
        if (!(s > 0.0)) {
            if (diff != 0.0) return 0;
            continue;
        }
        const double u = (e[oi] + e[oj]) / (s * s);
        const double t2 = lut_lookup(P.lut, P.lut_n, u);
        if (diff * diff > t2 * s) return 0;
    }
    return 1;
}

__global__ void film_filter_f64(FilmParams<double> P) {
    const size_t HW = (size_t)P.W * P.H;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= HW) return;
    const int R = P.R, D = 2 * R + 1, words = (D * D + 31) / 32;
    uint32_t *bits = P.bits ? P.bits + i * (size_t)P.K * words : nullptr;
    if (bits)
        for (int w = 0; w < P.K * words; w++) bits[w] = 0u;
    if (P.n[i] < 2) {
        for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + i] = P.film[(size_t)c * HW + i];
        return;
    }
    int ksel = -1;
    if (P.mt_mode == STATER_MT_JB) {
        ksel = 0;
        for (int k = 1; k < P.K; k++)
            if (P.jb[k][i] < P.jb[ksel][i]) ksel = k;
    }
    const int x = (int)(i % P.W), y = (int)(i / P.W);
    double sw = 0.0, sf[3] = {0.0, 0.0, 0.0};
    for (int dy = -R; dy <= R; dy++) {
        const int yy = y + dy;
        if (yy < 0 || yy >= P.H) continue;
        for (int dx = -R; dx <= R; dx++) {
            const int xx = x + dx;
            if (xx < 0 || xx >= P.W) continue;
            const size_t j = (size_t)yy * P.W + xx;
            if (P.n[j] < 2) continue;
            const int bit = (dy + R) * D + (dx + R);
            int acc = 1;
            for (int k = 0; k < P.K; k++) {
                const int a = (j == i) ? 1 : welch_accept_f64(P, HW, k, i, j);
                if (bits && a) bits[k * words + bit / 32] |= 1u << (bit % 32);
                if (ksel < 0 || ksel == k) acc = acc && a;
            }
            if (!acc) continue;
            const double w = exp(P.ds * (double)(dx * dx + dy * dy) + range_arg(P.gb, i, j, HW));
            sw = sw + w;
            for (int c = 0; c < 3; c++) sf[c] = sf[c] + w * P.film[(size_t)c * HW + j];
        }
    }
    for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + i] = sf[c] / sw;
}

}  // namespace

}  // namespace stater

using namespace stater;

namespace {
stater_status check_vars_args(const stater_denoise_vars_args *a) {
    if (!a) return set_error(STATER_ERR_INVALID, "stater_denoise_vars: null args");
    if (a->n_buffers < 1 || a->n_buffers > STATER_MAX_TRANSFORMS || a->width <= 0 || a->height <= 0)
        return set_error(STATER_ERR_INVALID, "stater_denoise_vars: bad geometry");
    if (a->filter_radius < 0 || a->filter_radius > STATER_MAX_RADIUS)
        return set_error(STATER_ERR_INVALID, "stater_denoise_vars: filter_radius must be 0..20");
    if (a->max_moment < 3 || a->max_moment > 5)
        return set_error(STATER_ERR_INVALID, "stater_denoise_vars: needs max_moment >= 3 (m2, m3)");
    if (!a->n) return set_error(STATER_ERR_INVALID, "stater_denoise_vars: null n");
    for (int k = 0; k < a->n_buffers; k++) {
        if (!a->m2[k] || !a->m3[k] || !a->jb[k] || !a->lnS2[k] || !a->se2[k] || !a->m2C[k] || !a->varD[k] ||
            !a->varCD[k])
            return set_error(STATER_ERR_INVALID, "stater_denoise_vars: null buffer pointer");
        if (a->max_moment >= 4 && !a->m4[k])
            return set_error(STATER_ERR_INVALID, "stater_denoise_vars: null m4 with max_moment >= 4");
        if (a->max_moment >= 5 && (!a->c2X[k] || !a->c2Y[k]))
            return set_error(STATER_ERR_INVALID, "stater_denoise_vars: null c2X/c2Y with max_moment 5");
    }
    return STATER_OK;
}

stater_status check_film_args(const stater_denoise_film_args *a) {
    if (!a) return set_error(STATER_ERR_INVALID, "stater_denoise_film: null args");
    if (a->n_buffers < 1 || a->n_buffers > STATER_MAX_TRANSFORMS || a->width <= 0 || a->height <= 0)
        return set_error(STATER_ERR_INVALID, "stater_denoise_film: bad geometry");
    if (a->filter_radius < 0 || a->filter_radius > STATER_MAX_RADIUS)
        return set_error(STATER_ERR_INVALID, "stater_denoise_film: filter_radius must be 0..20");
    if (!(a->alpha > 0.f && a->alpha < 1.f))
        return set_error(STATER_ERR_INVALID, "stater_denoise_film: alpha must be in (0, 1)");
    if (a->mt_mode != STATER_MT_ALL && a->mt_mode != STATER_MT_JB)
        return set_error(STATER_ERR_INVALID, "stater_denoise_film: mt_mode must be 2 or 3");
    if (!a->n || !a->film || !a->filmD) return set_error(STATER_ERR_INVALID, "stater_denoise_film: null buffer");
    if (a->discr_source != STATER_DISCR_DENOISED && a->discr_source != STATER_DISCR_SAMPLE)
        return set_error(STATER_ERR_INVALID, "stater_denoise_film: discr_source must be 0 or 1");
    const bool sample = a->discr_source == STATER_DISCR_SAMPLE;
    for (int k = 0; k < a->n_buffers; k++) {
        const void *var = sample ? (a->use_levc ? a->m2C[k] : a->m2[k]) : (a->use_levc ? a->varCD[k] : a->varD[k]);
        if ((k > 0 && !a->mean[k]) || !a->discr[k] || !var)
            return set_error(STATER_ERR_INVALID, "stater_denoise_film: null buffer pointer");
        if (a->mt_mode == STATER_MT_JB && !a->jb[k])
            return set_error(STATER_ERR_INVALID, "stater_denoise_film: mt_mode 3 needs jb");
    }
    return STATER_OK;
}
}  // namespace

extern "C" {

stater_status stater_denoise_vars(const stater_denoise_vars_args *a, stater_stream stream) {
    clear_error();
    stater_status st = check_vars_args(a);
    if (st != STATER_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (a->precision == STATER_F32) return denoise_vars_f32(a, s);
    if (a->precision != STATER_F64) return set_error(STATER_ERR_INVALID, "stater_denoise_vars: bad precision");

    VarsParams<double> P;
    P.W = a->width;
    P.H = a->height;
    P.K = a->n_buffers;
    P.max_moment = a->max_moment;
    P.R = a->filter_radius;
    P.ds = (double)a->ds_factor;
    P.z = (double)a->var_z;
    P.n = a->n;
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        P.m2[k] = (const double *)a->m2[k];
        P.m3[k] = (const double *)a->m3[k];
        P.m4[k] = (const double *)a->m4[k];
        P.cx[k] = (const double *)a->c2X[k];
        P.cy[k] = (const double *)a->c2Y[k];
        P.jb[k] = (double *)a->jb[k];
        P.lnS2[k] = (double *)a->lnS2[k];
        P.se2[k] = (double *)a->se2[k];
        P.m2C[k] = (double *)a->m2C[k];
        P.varD[k] = (double *)a->varD[k];
        P.varCD[k] = (double *)a->varCD[k];
    }
    P.m2c_in = (const double *)a->m2C_in;
    if (!fill_gbuf(P.gb, a->gbuffers)) return set_error(STATER_ERR_INVALID, "stater_denoise_vars: bad gbuffers");
    const size_t HW = (size_t)P.W * P.H;
    double *scr = (double *)scratch(0, sizeof(double) * 2 * 3 * P.K * HW, s);
    if (!scr) return set_error(STATER_ERR_NOMEM, "stater_denoise_vars: scratch allocation failed");
    P.s2 = scr;
    P.s2c = scr + (size_t)3 * P.K * HW;
    dim3 grid((unsigned)((HW + 127) / 128), P.K);
    vars_stats_f64<<<grid, 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("vars_stats_f64");
    vars_filter_f64<<<grid, 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("vars_filter_f64");
    return STATER_OK;
}

stater_status stater_denoise_film(const stater_denoise_film_args *a, stater_stream stream) {
    clear_error();
    stater_status st = check_film_args(a);
    if (st != STATER_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (a->precision == STATER_F32) return denoise_film_f32(a, s);
    if (a->precision != STATER_F64) return set_error(STATER_ERR_INVALID, "stater_denoise_film: bad precision");

    FilmParams<double> P;
    P.W = a->width;
    P.H = a->height;
    P.K = a->n_buffers;
    P.R = a->filter_radius;
    P.mt_mode = a->mt_mode;
    P.use_levc = a->use_levc;
    P.discr_source = a->discr_source;
    P.lut_n = tcrit_intervals();
    P.ds = (double)a->ds_factor;
    P.n = a->n;
    P.film = (const double *)a->film;
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        P.mean[k] = (const double *)a->mean[k];
        P.varD[k] = (const double *)a->varD[k];
        P.varCD[k] = (const double *)a->varCD[k];
        P.jb[k] = (const double *)a->jb[k];
        P.discr[k] = (double *)a->discr[k];
        P.m2s[k] = (const double *)(a->use_levc ? a->m2C[k] : a->m2[k]);
    }
    P.filmD = (double *)a->filmD;
    P.bits = a->accept_bits;
    P.lut = (const double *)tcrit_table_device((double)a->alpha, true, s);
    if (!P.lut) return set_error(STATER_ERR_NOMEM, "stater_denoise_film: t table allocation failed");
    if (!fill_gbuf(P.gb, a->gbuffers)) return set_error(STATER_ERR_INVALID, "stater_denoise_film: bad gbuffers");
    const size_t HW = (size_t)P.W * P.H;
    P.ediv = (double *)scratch(1, sizeof(double) * 3 * P.K * HW, s);
    if (!P.ediv) return set_error(STATER_ERR_NOMEM, "stater_denoise_film: scratch allocation failed");
    dim3 grid((unsigned)((HW + 127) / 128), P.K);
    film_discr_f64<<<grid, 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("film_discr_f64");
    film_filter_f64<<<(unsigned)((HW + 127) / 128), 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("film_filter_f64");
    return STATER_OK;
}

}  // extern "C"
