// Linear explained variance: per-pixel ridge regression of the three radiance
// channels on the G feature channels plus an intercept. Compiled with
// -fmad=false (the FP64 form matches the CPU restatement operation by operation).
//
// Accumulation state per pixel (planes of W*H, index order):
//   n, pivot[G+3], S[G+3] (pivot-shifted sums), Sff[G(G+1)/2] (upper triangle,
//   row-major), Sfy[G][3], Syy[3]
// Shifting by the pixel's first sample keeps the raw cross-products close to the
// centred ones, so the conversion to co-moments (C_ab = S_ab - S_a S_b / n)
// does not cancel catastrophically. The solve is FP64 Cholesky of
// Cff/n + lambda I (ridge on the slopes, intercept free).
#include <cmath>

#include "common.cuh"

namespace stater {

cudaError_t lev_accumulate_f32_launch(int G, size_t HW, int S, const float *samples, const int32_t *count,
                                      float *state, cudaStream_t s);

namespace {

constexpr int kLevMaxG = 8;

__host__ __device__ constexpr int lev_nstate(int G) { return 1 + 2 * (G + 3) + G * (G + 1) / 2 + 3 * G + 3; }

template <int G>
__global__ void __launch_bounds__(128) lev_acc_f64(size_t HW, int S, const float *__restrict__ samples,
                                                   const int32_t *__restrict__ count, double *state) {
    constexpr int P0 = G + 3;
    constexpr int oP = 1, oS = 1 + P0, oFF = 1 + 2 * P0, oFY = oFF + G * (G + 1) / 2, oYY = oFY + 3 * G;
    constexpr int NS = lev_nstate(G);
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    double st[NS];
#pragma unroll
    for (int q = 0; q < NS; q++) st[q] = state[(size_t)q * HW + p];
    const int cnt = count ? min(max(count[p], 0), S) : S;
    const size_t NCH = 5 + G;
    const float *sp = samples + p;
    for (int s = 0; s < cnt; s++, sp += NCH * HW) {
        double v[P0];
#pragma unroll
        for (int g = 0; g < G; g++) v[g] = (double)__ldg(sp + (size_t)(5 + g) * HW);
#pragma unroll
        for (int c = 0; c < 3; c++) v[G + c] = (double)__ldg(sp + (size_t)c * HW);
        if (st[0] == 0.0) {
#pragma unroll
            for (int a = 0; a < P0; a++) st[oP + a] = v[a];
        }
        st[0] = st[0] + 1.0;
        double z[P0];
#pragma unroll
        for (int a = 0; a < P0; a++) {
            z[a] = v[a] - st[oP + a];
            st[oS + a] = st[oS + a] + z[a];
        }
        int q = 0;
#pragma unroll
        for (int a = 0; a < G; a++)
#pragma unroll
            for (int b = a; b < G; b++, q++) st[oFF + q] = st[oFF + q] + z[a] * z[b];
#pragma unroll
        for (int a = 0; a < G; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) st[oFY + a * 3 + c] = st[oFY + a * 3 + c] + z[a] * z[G + c];
#pragma unroll
        for (int c = 0; c < 3; c++) st[oYY + c] = st[oYY + c] + z[G + c] * z[G + c];
    }
#pragma unroll
    for (int q = 0; q < NS; q++) state[(size_t)q * HW + p] = st[q];
}

// Reads the state (FP64: one plane set; FP32: hi and lo plane sets, summed in FP64).
template <int G, typename T>
__global__ void __launch_bounds__(128) lev_solve_kernel(size_t HW, const T *__restrict__ state, double lambda,
                                                        T *beta, T *m2C, T *r2) {
    constexpr int P0 = G + 3;
    constexpr int oP = 1, oS = 1 + P0, oFF = 1 + 2 * P0, oFY = oFF + G * (G + 1) / 2, oYY = oFY + 3 * G;
    constexpr int NS = lev_nstate(G);
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    double st[NS];
#pragma unroll
    for (int q = 0; q < NS; q++) {
        double v = (double)state[(size_t)q * HW + p];
        if (sizeof(T) == 4) v = v + (double)state[(size_t)(NS + q) * HW + p];
        st[q] = v;
    }
    const double n = st[0];
    if (n < 2.0) {
        for (int c = 0; c < 3; c++) {
            m2C[(size_t)c * HW + p] = T(0);
            r2[(size_t)c * HW + p] = T(0);
            for (int a = 0; a <= G; a++) beta[((size_t)c * (G + 1) + a) * HW + p] = T(0);
        }
        return;
    }
    // One reciprocal of n and of each Cholesky pivot instead of a division per
    // term (FP64 division is a long instruction sequence on this part), and
    // fused multiply-adds in the dot products.
    const double inv_n = 1.0 / n;
    double mean[P0], Cff[G > 0 ? G : 1][G > 0 ? G : 1], L[G > 0 ? G : 1][G > 0 ? G : 1], inv_d[G > 0 ? G : 1];
    double cfy[G > 0 ? G : 1][3], cyy[3];
#pragma unroll
    for (int a = 0; a < P0; a++) mean[a] = fma(st[oS + a], inv_n, st[oP + a]);
    {
        int q = 0;
#pragma unroll
        for (int a = 0; a < G; a++)
#pragma unroll
            for (int b = a; b < G; b++, q++) {
                const double v = fma(-st[oS + a], st[oS + b] * inv_n, st[oFF + q]);
                Cff[a][b] = v;
                Cff[b][a] = v;
            }
    }
#pragma unroll
    for (int a = 0; a < G; a++)
#pragma unroll
        for (int c = 0; c < 3; c++) cfy[a][c] = fma(-st[oS + a], st[oS + G + c] * inv_n, st[oFY + a * 3 + c]);
#pragma unroll
    for (int c = 0; c < 3; c++) cyy[c] = fma(-st[oS + G + c], st[oS + G + c] * inv_n, st[oYY + c]);
#pragma unroll
    for (int a = 0; a < G; a++)
#pragma unroll
        for (int b = 0; b <= a; b++) {
            double sum = fma(Cff[a][b], inv_n, a == b ? lambda : 0.0);
#pragma unroll
            for (int m = 0; m < b; m++) sum = fma(-L[a][m], L[b][m], sum);
            if (a == b) {
                L[a][a] = sqrt(sum > 0.0 ? sum : 1e-300);
                inv_d[a] = 1.0 / L[a][a];
            } else {
                L[a][b] = sum * inv_d[b];
            }
        }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double tmp[G > 0 ? G : 1], bt[G > 0 ? G : 1];
#pragma unroll
        for (int a = 0; a < G; a++) {
            double sum = cfy[a][c] * inv_n;
#pragma unroll
            for (int m = 0; m < a; m++) sum = fma(-L[a][m], tmp[m], sum);
            tmp[a] = sum * inv_d[a];
        }
#pragma unroll
        for (int a = G - 1; a >= 0; a--) {
            double sum = tmp[a];
#pragma unroll
            for (int m = a + 1; m < G; m++) sum = fma(-L[m][a], bt[m], sum);
            bt[a] = sum * inv_d[a];
        }
        double bc = 0.0, bab = 0.0, icpt = mean[G + c];
#pragma unroll
        for (int a = 0; a < G; a++) {
            bc = fma(bt[a], cfy[a][c], bc);
            double row = 0.0;
#pragma unroll
            for (int b = 0; b < G; b++) row = fma(Cff[a][b], bt[b], row);
            bab = fma(bt[a], row, bab);
            icpt = fma(-bt[a], mean[a], icpt);
        }
        double rss = cyy[c] - 2.0 * bc + bab;
        if (rss < 0.0) rss = 0.0;
        m2C[(size_t)c * HW + p] = (T)rss;
        r2[(size_t)c * HW + p] = (T)(cyy[c] > 0.0 ? 1.0 - rss / cyy[c] : 0.0);
        beta[((size_t)c * (G + 1)) * HW + p] = (T)icpt;
#pragma unroll
        for (int a = 0; a < G; a++) beta[((size_t)c * (G + 1) + 1 + a) * HW + p] = (T)bt[a];
    }
}

template <template <int> class F, typename... Args>
cudaError_t dispatch_g(int G, Args... args) {
    switch (G) {
        case 0: return F<0>::run(args...);
        case 1: return F<1>::run(args...);
        case 2: return F<2>::run(args...);
        case 3: return F<3>::run(args...);
        case 4: return F<4>::run(args...);
        case 5: return F<5>::run(args...);
        case 6: return F<6>::run(args...);
        case 7: return F<7>::run(args...);
        case 8: return F<8>::run(args...);
        default: return cudaErrorInvalidValue;
    }
}

template <int G>
struct AccF64 {
    static cudaError_t run(size_t HW, int S, const float *samples, const int32_t *count, double *state,
                           cudaStream_t s) {
        lev_acc_f64<G><<<(unsigned)((HW + 127) / 128), 128, 0, s>>>(HW, S, samples, count, state);
        return cudaGetLastError();
    }
};

template <int G>
struct SolveF64 {
    static cudaError_t run(size_t HW, const void *state, double lambda, void *beta, void *m2C, void *r2,
                           cudaStream_t s) {
        lev_solve_kernel<G, double><<<(unsigned)((HW + 127) / 128), 128, 0, s>>>(
            HW, (const double *)state, lambda, (double *)beta, (double *)m2C, (double *)r2);
        return cudaGetLastError();
    }
};

template <int G>
struct SolveF32 {
    static cudaError_t run(size_t HW, const void *state, double lambda, void *beta, void *m2C, void *r2,
                           cudaStream_t s) {
        lev_solve_kernel<G, float><<<(unsigned)((HW + 127) / 128), 128, 0, s>>>(
            HW, (const float *)state, lambda, (float *)beta, (float *)m2C, (float *)r2);
        return cudaGetLastError();
    }
};

}  // namespace
}  // namespace stater

using namespace stater;

extern "C" {

int32_t stater_lev_state_size(int32_t n_features, stater_precision precision) {
    if (n_features < 0 || n_features > kLevMaxG) return -1;
    const int ns = lev_nstate(n_features);
    return precision == STATER_F32 ? 2 * ns : ns;
}

stater_status stater_lev_accumulate(int32_t width, int32_t height, int32_t n_features, int32_t n_samples,
                                    const float *samples, const int32_t *count, stater_precision precision,
                                    void *state, stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || n_features < 0 || n_samples < 0 || !state || (n_samples > 0 && !samples))
        return set_error(STATER_ERR_INVALID, "stater_lev_accumulate: bad arguments");
    if (n_features > kLevMaxG)
        return set_error(STATER_ERR_UNSUPPORTED, "stater_lev_accumulate: at most 8 feature channels");
    if (n_samples == 0) return STATER_OK;
    const size_t HW = (size_t)width * height;
    cudaError_t e;
    if (precision == STATER_F64)
        e = dispatch_g<AccF64>(n_features, HW, (int)n_samples, samples, count, (double *)state, (cudaStream_t)stream);
    else if (precision == STATER_F32)
        e = lev_accumulate_f32_launch(n_features, HW, n_samples, samples, count, (float *)state, (cudaStream_t)stream);
    else
        return set_error(STATER_ERR_INVALID, "stater_lev_accumulate: bad precision");
    return cuda_status(e, "stater_lev_accumulate launch");
}

stater_status stater_lev_solve(int32_t width, int32_t height, int32_t n_features, stater_precision precision,
                               const void *state, double lambda, void *beta, void *m2C, void *r2,
                               stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || n_features < 0 || !state || !beta || !m2C || !r2 || !(lambda >= 0.0))
        return set_error(STATER_ERR_INVALID, "stater_lev_solve: bad arguments");
    if (n_features > kLevMaxG)
        return set_error(STATER_ERR_UNSUPPORTED, "stater_lev_solve: at most 8 feature channels");
    const size_t HW = (size_t)width * height;
    cudaError_t e;
    if (precision == STATER_F64)
        e = dispatch_g<SolveF64>(n_features, HW, state, lambda, beta, m2C, r2, (cudaStream_t)stream);
    else if (precision == STATER_F32)
        e = dispatch_g<SolveF32>(n_features, HW, state, lambda, beta, m2C, r2, (cudaStream_t)stream);
    else
        return set_error(STATER_ERR_INVALID, "stater_lev_solve: bad precision");
    return cuda_status(e, "stater_lev_solve launch");
}

}  // extern "C"
