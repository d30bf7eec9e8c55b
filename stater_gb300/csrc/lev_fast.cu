// FP32 LEV accumulation with blocked compensation: every thread sums 8 samples'
// pivot-shifted cross-products in plain FP32 registers, then folds the block
// into a compensated (hi, lo) pair per sum kept in shared memory
// (hi + lo is the running total; lo carries what the FP32 addition of hi lost).
// State planes: hi [NS][HW] followed by lo [NS][HW]; n and the pivot live in
// the hi planes. The FP64 solve (lev.cu) reads hi + lo.
#include "common.cuh"

namespace stater {
namespace {

__host__ __device__ constexpr int lev_nstate_f(int G) { return 1 + 2 * (G + 3) + G * (G + 1) / 2 + 3 * G + 3; }

constexpr int kBlockSamples = 8;
constexpr int kThreads = 128;

template <int G>
__global__ void __launch_bounds__(kThreads) lev_acc_f32(size_t HW, int S, const float *__restrict__ samples,
                                                        const int32_t *__restrict__ count, float *state) {
    constexpr int P0 = G + 3;
    constexpr int NS = lev_nstate_f(G);
    constexpr int oS = 1 + P0;
    constexpr int NSUM = NS - oS;  // S, Sff, Sfy, Syy
    extern __shared__ float sm[];
    float *hi = sm;
    float *lo = sm + (size_t)NSUM * kThreads;
    const int t = threadIdx.x;
    const size_t p = (size_t)blockIdx.x * kThreads + t;
    if (p >= HW) return;  // no block-wide synchronisation below
    float n = state[p];
    float piv[P0];
#pragma unroll
    for (int a = 0; a < P0; a++) piv[a] = state[(size_t)(1 + a) * HW + p];
#pragma unroll
    for (int q = 0; q < NSUM; q++) {
        hi[q * kThreads + t] = state[(size_t)(oS + q) * HW + p];
        lo[q * kThreads + t] = state[(size_t)(NS + oS + q) * HW + p];
    }
    const int cnt = count ? min(max(count[p], 0), S) : S;
    const size_t NCH = 5 + G;
    const float *sp = samples + p;
    for (int s0 = 0; s0 < cnt; s0 += kBlockSamples) {
        float part[NSUM];
#pragma unroll
        for (int q = 0; q < NSUM; q++) part[q] = 0.f;
        const int s1 = min(cnt, s0 + kBlockSamples);
        for (int s = s0; s < s1; s++, sp += NCH * HW) {
            float v[P0];
#pragma unroll
            for (int g = 0; g < G; g++) v[g] = __ldg(sp + (size_t)(5 + g) * HW);
#pragma unroll
            for (int c = 0; c < 3; c++) v[G + c] = __ldg(sp + (size_t)c * HW);
            if (n == 0.f) {
#pragma unroll
                for (int a = 0; a < P0; a++) piv[a] = v[a];
            }
            n += 1.f;
            float z[P0];
#pragma unroll
            for (int a = 0; a < P0; a++) {
                z[a] = v[a] - piv[a];
                part[a] += z[a];
            }
            int q = P0;
#pragma unroll
            for (int a = 0; a < G; a++)
#pragma unroll
                for (int b = a; b < G; b++, q++) part[q] = fmaf(z[a], z[b], part[q]);
#pragma unroll
            for (int a = 0; a < G; a++)
#pragma unroll
                for (int c = 0; c < 3; c++, q++) part[q] = fmaf(z[a], z[G + c], part[q]);
#pragma unroll
            for (int c = 0; c < 3; c++, q++) part[q] = fmaf(z[G + c], z[G + c], part[q]);
        }
#pragma unroll
        for (int q = 0; q < NSUM; q++) {
            const float h = hi[q * kThreads + t];
            const float y = part[q] + lo[q * kThreads + t];
            const float s = h + y;
            lo[q * kThreads + t] = y - (s - h);
            hi[q * kThreads + t] = s;
        }
    }
    state[p] = n;
#pragma unroll
    for (int a = 0; a < P0; a++) state[(size_t)(1 + a) * HW + p] = piv[a];
#pragma unroll
    for (int q = 0; q < NSUM; q++) {
        state[(size_t)(oS + q) * HW + p] = hi[q * kThreads + t];
        state[(size_t)(NS + oS + q) * HW + p] = lo[q * kThreads + t];
    }
}

template <int G>
cudaError_t run_g(size_t HW, int S, const float *samples, const int32_t *count, float *state, cudaStream_t s) {
    constexpr int NSUM = lev_nstate_f(G) - (1 + (G + 3));
    const size_t smem = sizeof(float) * 2 * NSUM * kThreads;
    cudaError_t e = cudaFuncSetAttribute(lev_acc_f32<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    lev_acc_f32<G><<<(unsigned)((HW + kThreads - 1) / kThreads), kThreads, smem, s>>>(HW, S, samples, count, state);
    return cudaGetLastError();
}

}  // namespace

cudaError_t lev_accumulate_f32_launch(int G, size_t HW, int S, const float *samples, const int32_t *count,
                                      float *state, cudaStream_t s) {
    switch (G) {
        case 0: return run_g<0>(HW, S, samples, count, state, s);
        case 1: return run_g<1>(HW, S, samples, count, state, s);
        case 2: return run_g<2>(HW, S, samples, count, state, s);
        case 3: return run_g<3>(HW, S, samples, count, state, s);
        case 4: return run_g<4>(HW, S, samples, count, state, s);
        case 5: return run_g<5>(HW, S, samples, count, state, s);
        case 6: return run_g<6>(HW, S, samples, count, state, s);
        case 7: return run_g<7>(HW, S, samples, count, state, s);
        case 8: return run_g<8>(HW, S, samples, count, state, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace stater
