// Stage 1 entry points: accumulate, synthetic sample source, tile merge,
// pairwise moment merge, meanVar. Compiled with -fmad=false: every kernel here
// rounds each operation separately, like the reference's CPU code and the oracle.
#include <cmath>
#include <mutex>

#include "acc_kernels.cuh"
#include "common.cuh"

namespace stater {

cudaError_t launch_acc_fast_f32(const AccParams &P, int max_moment, cudaStream_t s);
cudaError_t launch_acc_tma_f32(const AccParams &P, int max_moment, cudaStream_t s);

// ---------------------------------------------------------------------------
// Synthetic sample source.
// ---------------------------------------------------------------------------
struct GenParams {
    int W, H, S, G, region;
    const int32_t *pix;  // nullable: column i generates pixel pix[i]
    size_t ncols;        // sample columns (W*H, or entries of pix)
    uint32_t k0, k1;
    float mean_mu, mean_sigma, noise_sigma, ff_prob, ff_scale, lev_r2, lev_b;
    const int32_t *first_index;
    const int32_t *count;
    float *samples;
};

__device__ inline void box_muller(uint32_t a, uint32_t b, float &z0, float &z1) {
    const float r = sqrtf(-2.0f * logf(u01_open(a)));
    float s, c;
    sincospif(2.0f * u01(b), &s, &c);
    z0 = r * c;
    z1 = r * s;
}

__global__ void generate_kernel(GenParams g) {
    const size_t HW = g.ncols;  // column stride of the sample planes
    const size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= HW) return;
    size_t p = col;
    if (g.pix) {
        const int32_t q = g.pix[col];
        if (q < 0 || (size_t)q >= (size_t)g.W * g.H) return;
        p = (size_t)q;
    }
    const int x = (int)(p % g.W), y = (int)(p / g.W);
    const int rw = (g.W + g.region - 1) / g.region;
    const uint32_t rid = (uint32_t)((y / g.region) * rw + x / g.region);
    const uint32_t first = g.first_index ? (uint32_t)g.first_index[col] : 0u;
    const int NCH = 5 + g.G;

    // Per-region radiance mean and feature base values.
    float mu[3];
    {
        U4 r = philox4x32_10({rid, 0xFFFFFFFFu, 3u, 0u}, g.k0, g.k1);
        float z0, z1, z2, z3;
        box_muller(r.x, r.y, z0, z1);
        box_muller(r.z, r.w, z2, z3);
        mu[0] = expf(g.mean_mu + g.mean_sigma * z0);
        mu[1] = expf(g.mean_mu + g.mean_sigma * z1);
        mu[2] = expf(g.mean_mu + g.mean_sigma * z2);
    }
    float base[STATER_MAX_FEATURES];
    for (int f = 0; f < g.G; f += 4) {
        U4 r = philox4x32_10({rid, 0xFFFFFFFFu, 4u + (uint32_t)(f / 4), 0u}, g.k0, g.k1);
        const uint32_t v[4] = {r.x, r.y, r.z, r.w};
        for (int j = 0; j < 4 && f + j < g.G; j++) base[f + j] = u01(v[j]);
    }

    const int ns = g.count ? min(max(g.count[col], 0), g.S) : g.S;
    for (int s = 0; s < ns; s++) {
        const uint32_t sidx = first + (uint32_t)s;
        float *out = g.samples + (size_t)s * NCH * HW + col;
        const U4 a = philox4x32_10({(uint32_t)p, sidx, 0u, 0u}, g.k0, g.k1);
        const U4 b = philox4x32_10({(uint32_t)p, sidx, 1u, 0u}, g.k0, g.k1);
        float z[4];
        box_muller(b.x, b.y, z[0], z[1]);
        box_muller(b.z, b.w, z[2], z[3]);
        float feat[STATER_MAX_FEATURES];
        for (int f = 0; f < g.G; f += 4) {
            U4 r = philox4x32_10({(uint32_t)p, sidx, 2u + (uint32_t)(f / 4), 0u}, g.k0, g.k1);
            const uint32_t v[4] = {r.x, r.y, r.z, r.w};
            for (int j = 0; j < 4 && f + j < g.G; j++) {
                if (g.lev_r2 > 0.f) {
                    feat[f + j] = u01(v[j]);
                } else {
                    const float jit = base[f + j] + 0.02f * (u01(v[j]) - 0.5f);
                    feat[f + j] = fminf(fmaxf(jit, 0.f), 1.f);
                }
            }
        }
        float rad[3];
        if (g.lev_r2 > 0.f) {
            const float mlog = expf(0.5f * g.noise_sigma * g.noise_sigma);
            for (int c = 0; c < 3; c++) {
                float wn = 0.f, lin = 0.f;
                for (int f = 0; f < g.G; f++) {
                    const float w = cosf(1.3f * f + 2.1f * c);
                    wn += w * w;
                    lin += w * (feat[f] - 0.5f);
                }
                lin = g.G > 0 ? lin * rsqrtf(wn) : 0.f;
                rad[c] = mu[c] * (1.f + 0.5f * lin) + mu[c] * g.lev_b * (expf(g.noise_sigma * z[c]) - mlog);
            }
        } else {
            const float ff = u01(a.z) < g.ff_prob ? g.ff_scale : 1.f;
            for (int c = 0; c < 3; c++) rad[c] = mu[c] * expf(g.noise_sigma * z[c]) * ff;
        }
        out[0] = rad[0];
        out[HW] = rad[1];
        out[2 * HW] = rad[2];
        out[3 * HW] = u01(a.x);
        out[4 * HW] = u01(a.y);
        for (int f = 0; f < g.G; f++) out[(size_t)(5 + f) * HW] = feat[f];
    }
}

// ---------------------------------------------------------------------------
// Tile merge (Estimator::MergeTransformTile / MergeTile, estimator.cpp:267-324).
// ---------------------------------------------------------------------------
__global__ void merge_tiles_kernel(int W, int H, const int32_t *__restrict__ bounds,
                                   const unsigned char *__restrict__ records, int n_sets,
                                   int32_t *n, float *stats) {
    __shared__ unsigned long long partial[256];
    const int t = blockIdx.x;
    // Record offset of this tile = sum of the areas of the tiles before it.
    unsigned long long acc = 0;
    for (int i = threadIdx.x; i < t; i += blockDim.x) {
        const int4 b = reinterpret_cast<const int4 *>(bounds)[i];
        acc += (unsigned long long)(max(b.z - b.x, 0) * max(b.w - b.y, 0));
    }
    partial[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) partial[threadIdx.x] += partial[threadIdx.x + s];
        __syncthreads();
    }
    const unsigned long long first = partial[0];
    const int4 b = reinterpret_cast<const int4 *>(bounds)[t];
    const int tw = max(b.z - b.x, 0), th = max(b.w - b.y, 0);
    const size_t HW = (size_t)W * H;
    for (int j = threadIdx.x; j < tw * th; j += blockDim.x) {
        const int x = b.x + j % tw, y = b.y + j / tw;
        if (x < 0 || y < 0 || x >= W || y >= H) continue;
        const unsigned char *r = records + (first + (unsigned long long)j) * 320ull;
        const size_t p = (size_t)y * W + x;
        n[p] = (int32_t) * reinterpret_cast<const unsigned long long *>(r);
        // a plain tile (MergeTile) sets mean, M2, M3 and M4 only; a transform
        // tile (MergeTransformTile) all seven quantities of both sets
        const int nq = n_sets == 1 ? STATER_Q_M4 + 1 : kNQ;
        for (int set = 0; set < n_sets; set++) {
            const float *v = reinterpret_cast<const float *>(r + (set == 0 ? 64 : 192));
#pragma unroll
            for (int q = 0; q < kNQ; q++) {
                if (q >= nq) break;
#pragma unroll
                for (int c = 0; c < 3; c++) stats[stat_index(set, q, c, HW) + p] = v[q * 3 + c];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Pairwise moment merge (Chan et al. 1979; Pebay 2008).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void merge_moments_kernel(size_t HW, int K, int max_moment, int32_t *nA, T *A,
                                     const int32_t *nB, const T *B) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    const int32_t na = nA[p], nb = nB[p];
    if (nb == 0) return;
    for (int k = 0; k < K; k++)
        for (int c = 0; c < 3; c++) {
            const size_t o = stat_index(k, 0, c, HW) + p;
            const size_t qs = 3 * HW;
            if (na == 0) {
                for (int q = 0; q < kNQ; q++) A[o + q * qs] = B[o + q * qs];
                continue;
            }
            const T fa = (T)na, fb = (T)nb, f = fa + fb;
            const T delta = B[o] - A[o];
            const T m2a = A[o + qs], m2b = B[o + qs];
            const T m3a = A[o + 2 * qs], m3b = B[o + 2 * qs];
            const T m4a = A[o + 3 * qs], m4b = B[o + 3 * qs];
            A[o] = A[o] + delta * fb / f;
            if (max_moment >= 2) A[o + qs] = m2a + m2b + delta * delta * fa * fb / f;
            if (max_moment >= 3)
                A[o + 2 * qs] = m3a + m3b + delta * delta * delta * fa * fb * (fa - fb) / (f * f) +
                                (T)3.0 * delta * (fa * m2b - fb * m2a) / f;
            if (max_moment >= 4)
                A[o + 3 * qs] = m4a + m4b +
                                delta * delta * delta * delta * fa * fb * (fa * fa - fa * fb + fb * fb) / (f * f * f) +
                                (T)6.0 * delta * delta * (fa * fa * m2b + fb * fb * m2a) / (f * f) +
                                (T)4.0 * delta * (fa * m3b - fb * m3a) / f;
            if (max_moment >= 5)
                for (int q = STATER_Q_C2X; q <= STATER_Q_M1; q++) A[o + q * qs] = A[o + q * qs] + B[o + q * qs];
        }
    nA[p] = na + nb;
}

// calcMatMeanVar (estimator.cpp:462-474): var = m2 / ((n - 1) * n) in float.
__global__ void mean_var_kernel(size_t HW, const int32_t *n, const float *m2, float *var) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * HW) return;
    const size_t p = i % HW;
    const float nPF = (float)n[p];
    var[i] = m2[i] / ((nPF - 1.f) * nPF);
}

// Warp order set by stater_debug_set_warp_order (n = 0: none).
std::mutex g_order_mu;
int g_order_n = 0;
int8_t g_order[STATER_MAX_TRANSFORMS];

void apply_warp_order(AccParams &P) {
    std::lock_guard<std::mutex> lock(g_order_mu);
    if (g_order_n == 0 || g_order_n != P.K) return;
    // the features stay with their transforms; only the warps change
    std::copy(g_order, g_order + P.K, P.wt);
}

}  // namespace stater

using namespace stater;

stater_status stater_debug_set_warp_order(const int32_t *order, int32_t n_transforms) {
    clear_error();
    if (n_transforms < 0 || n_transforms > STATER_MAX_TRANSFORMS || (n_transforms > 0 && !order))
        return set_error(STATER_ERR_INVALID, "stater_debug_set_warp_order: bad arguments");
    bool seen[STATER_MAX_TRANSFORMS] = {false};
    for (int w = 0; w < n_transforms; w++) {
        if (order[w] < 0 || order[w] >= n_transforms || seen[order[w]])
            return set_error(STATER_ERR_INVALID, "stater_debug_set_warp_order: not a permutation");
        seen[order[w]] = true;
    }
    std::lock_guard<std::mutex> lock(g_order_mu);
    for (int w = 0; w < n_transforms; w++) g_order[w] = (int8_t)order[w];
    g_order_n = n_transforms;
    return STATER_OK;
}

extern "C" {

stater_status stater_accumulate(const stater_accumulate_args *a, stater_stream stream) {
    clear_error();
    if (!a) return set_error(STATER_ERR_INVALID, "stater_accumulate: null args");
    if (a->width <= 0 || a->height <= 0 || a->n_samples < 0 || a->n_features < 0 ||
        a->n_features > STATER_MAX_FEATURES)
        return set_error(STATER_ERR_INVALID, "stater_accumulate: bad geometry");
    if (a->n_transforms < 1 || a->n_transforms > STATER_MAX_TRANSFORMS)
        return set_error(STATER_ERR_INVALID, "stater_accumulate: n_transforms must be 1..8");
    if (a->transforms[0].kind != STATER_TK_IDENTITY)
        return set_error(STATER_ERR_INVALID, "stater_accumulate: transform 0 must be the identity");
    if (a->max_moment < 1 || a->max_moment > 5)
        return set_error(STATER_ERR_INVALID, "stater_accumulate: max_moment must be 1..5");
    if (!a->n || !a->stats || (a->n_samples > 0 && !a->samples) || (a->n_features > 0 && !a->gmean))
        return set_error(STATER_ERR_INVALID, "stater_accumulate: null buffer");
    if (a->precision != STATER_F32 && a->precision != STATER_F64)
        return set_error(STATER_ERR_INVALID, "stater_accumulate: bad precision");
    if (a->mode == STATER_ACC_FAST && a->precision != STATER_F32)
        return set_error(STATER_ERR_INVALID, "stater_accumulate: the fast mode is FP32 only");
    for (int k = 0; k < a->n_transforms; k++)
        if (a->transforms[k].kind < 0 || a->transforms[k].kind > STATER_TK_BOXCOX)
            return set_error(STATER_ERR_INVALID, "stater_accumulate: unknown transform kind");
    if (a->film_contrib_sum && (!a->film_weight_sum || !a->film_spill || !(a->film_max_sample_luminance > 0.0f)))
        return set_error(STATER_ERR_INVALID, "stater_accumulate: incomplete film buffers");
    if (a->pixel_index && a->n_active <= 0)
        return set_error(STATER_ERR_INVALID, "stater_accumulate: pixel_index needs n_active > 0");
    if (a->n_samples == 0) return STATER_OK;

    AccParams P;
    P.HWs = (size_t)a->width * a->height;
    P.pix = a->pixel_index;
    P.HW = a->pixel_index ? (size_t)a->n_active : P.HWs;
    P.S = a->n_samples;
    P.G = a->n_features;
    P.K = a->n_transforms;
    P.NCH = 5 + a->n_features;
    P.samples = a->samples;
    P.count = a->count;
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        P.ts.kind[k] = k < a->n_transforms ? a->transforms[k].kind : 0;
        P.ts.lambda[k] = k < a->n_transforms ? a->transforms[k].lambda : 1.f;
    }
    P.n = a->n;
    P.stats = a->stats;
    P.gmean = a->gmean;
    P.film.W = a->width;
    P.film.H = a->height;
    P.film.max_lum = a->film_max_sample_luminance;
    P.film.sum = a->film_contrib_sum;
    P.film.weight = a->film_weight_sum;
    P.film.spill = a->film_spill;
    P.maxf = acc_assign_features(P);
    apply_warp_order(P);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if (a->mode == STATER_ACC_FAST) {
        e = launch_acc_tma_f32(P, a->max_moment, s);
        if (e == cudaErrorNotSupported) {
            cudaGetLastError();
            e = launch_acc_fast_f32(P, a->max_moment, s);
        }
    }
    else if (a->precision == STATER_F64)
        e = launch_acc<double, false>(P, a->max_moment, s);
    else
        e = launch_acc<float, false>(P, a->max_moment, s);
    return cuda_status(e, "stater_accumulate launch");
}

stater_status stater_generate_samples(const stater_generate_args *a, stater_stream stream) {
    clear_error();
    if (!a || !a->samples || a->width <= 0 || a->height <= 0 || a->n_samples < 0 ||
        a->n_features < 0 || a->n_features > STATER_MAX_FEATURES || a->region < 1)
        return set_error(STATER_ERR_INVALID, "stater_generate_samples: bad arguments");
    if (a->n_samples == 0) return STATER_OK;
    GenParams g;
    g.W = a->width;
    g.H = a->height;
    g.S = a->n_samples;
    g.G = a->n_features;
    g.region = a->region;
    g.k0 = (uint32_t)a->seed;
    g.k1 = (uint32_t)(a->seed >> 32);
    g.mean_mu = a->mean_mu;
    g.mean_sigma = a->mean_sigma;
    g.noise_sigma = a->noise_sigma;
    g.ff_prob = a->firefly_prob;
    g.ff_scale = a->firefly_scale;
    g.lev_r2 = a->lev_r2;
    g.lev_b = 0.f;
    if (a->lev_r2 > 0.f) {
        const double s2 = (double)a->noise_sigma * a->noise_sigma;
        const double var_ln = (std::exp(s2) - 1.0) * std::exp(s2);
        const double r2 = a->lev_r2 >= 1.f ? 0.999999 : a->lev_r2;
        g.lev_b = (float)std::sqrt((1.0 - r2) / r2 * (1.0 / 48.0) / var_ln);
    }
    g.first_index = a->first_index;
    g.count = a->count;
    g.samples = a->samples;
    g.pix = a->pixel_index;
    g.ncols = a->pixel_index ? (size_t)a->n_active : (size_t)g.W * g.H;
    if (a->pixel_index && a->n_active <= 0)
        return set_error(STATER_ERR_INVALID, "stater_generate_samples: pixel_index needs n_active > 0");
    generate_kernel<<<(unsigned)((g.ncols + 255) / 256), 256, 0, (cudaStream_t)stream>>>(g);
    return cuda_status(cudaGetLastError(), "stater_generate_samples launch");
}

stater_status stater_merge_tiles(int32_t width, int32_t height, int32_t n_tiles, const int32_t *bounds,
                                 const void *records, int32_t n_sets, int32_t *n, float *stats,
                                 stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || n_tiles < 0 || (n_tiles > 0 && (!bounds || !records)) || !n ||
        !stats || (n_sets != 1 && n_sets != 2))
        return set_error(STATER_ERR_INVALID, "stater_merge_tiles: bad arguments");
    if (((uintptr_t)bounds & 15) != 0 || ((uintptr_t)records & 15) != 0)
        return set_error(STATER_ERR_INVALID, "stater_merge_tiles: bounds and records must be 16-byte aligned");
    if (n_tiles == 0) return STATER_OK;
    merge_tiles_kernel<<<n_tiles, 256, 0, (cudaStream_t)stream>>>(
        width, height, bounds, (const unsigned char *)records, n_sets, n, stats);
    return cuda_status(cudaGetLastError(), "stater_merge_tiles launch");
}

stater_status stater_merge_moments(int32_t width, int32_t height, int32_t n_transforms, int32_t max_moment,
                                   stater_precision precision, int32_t *nA, void *statsA, const int32_t *nB,
                                   const void *statsB, stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || n_transforms < 1 || n_transforms > STATER_MAX_TRANSFORMS ||
        max_moment < 1 || max_moment > 5 || !nA || !statsA || !nB || !statsB)
        return set_error(STATER_ERR_INVALID, "stater_merge_moments: bad arguments");
    const size_t HW = (size_t)width * height;
    const unsigned grid = (unsigned)((HW + 255) / 256);
    if (precision == STATER_F64)
        merge_moments_kernel<double><<<grid, 256, 0, (cudaStream_t)stream>>>(
            HW, n_transforms, max_moment, nA, (double *)statsA, nB, (const double *)statsB);
    else if (precision == STATER_F32)
        merge_moments_kernel<float><<<grid, 256, 0, (cudaStream_t)stream>>>(
            HW, n_transforms, max_moment, nA, (float *)statsA, nB, (const float *)statsB);
    else
        return set_error(STATER_ERR_INVALID, "stater_merge_moments: bad precision");
    return cuda_status(cudaGetLastError(), "stater_merge_moments launch");
}

stater_status stater_calc_mean_var(int32_t width, int32_t height, const int32_t *n, const float *m2,
                                   float *mean_var, stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || !n || !m2 || !mean_var)
        return set_error(STATER_ERR_INVALID, "stater_calc_mean_var: bad arguments");
    const size_t HW = (size_t)width * height;
    mean_var_kernel<<<(unsigned)((3 * HW + 255) / 256), 256, 0, (cudaStream_t)stream>>>(HW, n, m2, mean_var);
    return cuda_status(cudaGetLastError(), "stater_calc_mean_var launch");
}

}  // extern "C"
