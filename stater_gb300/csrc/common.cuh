// Shared device/host helpers of libstater.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "stater.h"

namespace stater {

// ---- error plumbing (runtime.cu) -------------------------------------------
stater_status set_error(stater_status s, const std::string &msg);
stater_status clear_error();
stater_status cuda_status(cudaError_t e, const char *what);
// Device scratch owned by the library: one grow-only buffer per (device, slot),
// reused across calls on the same stream order. Returns nullptr on failure.
void *scratch(int slot, size_t bytes, cudaStream_t stream);
// Device copy of the t-critical table for alpha (FP32 and FP64 copies).
const void *tcrit_table_device(double alpha, bool f64, cudaStream_t stream);
int tcrit_intervals();
int sm_count();

#define STATER_CHECK_LAUNCH(what)                                         \
    do {                                                                  \
        cudaError_t _e = cudaGetLastError();                              \
        if (_e != cudaSuccess) return ::stater::cuda_status(_e, what);    \
    } while (0)

// ---- layout -----------------------------------------------------------------
constexpr int kNQ = STATER_NQ;

// stats slab [K][7][3][HW]
__host__ __device__ inline size_t stat_index(int k, int q, int c, size_t HW) {
    return ((size_t)(k * kNQ + q) * 3 + c) * HW;
}

// ---- transforms ---------------------------------------------------------------
struct TransformSet {
    int32_t kind[STATER_MAX_TRANSFORMS];
    float lambda[STATER_MAX_TRANSFORMS];
};

template <typename T>
__device__ __forceinline__ T transform_exact(int kind, float lambda, T x);

template <>
__device__ __forceinline__ double transform_exact<double>(int kind, float lambda, double x) {
    switch (kind) {
        case STATER_TK_LOG1P: return log1p(x);
        case STATER_TK_SQRT: return sqrt(x);
        case STATER_TK_CBRT: return cbrt(x);
        case STATER_TK_ASINH: return asinh(x);
        case STATER_TK_BOXCOX: {
            const double l = (double)lambda;
            if (l == 1.0) return x;
            return (pow(x, l) - 1.0) / l;
        }
        default: return x;
    }
}

template <>
__device__ __forceinline__ float transform_exact<float>(int kind, float lambda, float x) {
    switch (kind) {
        case STATER_TK_LOG1P: return log1pf(x);
        case STATER_TK_SQRT: return sqrtf(x);
        case STATER_TK_CBRT: return cbrtf(x);
        case STATER_TK_ASINH: return asinhf(x);
        case STATER_TK_BOXCOX:
            if (lambda == 1.f) return x;
            return (powf(x, lambda) - 1.f) / lambda;
        default: return x;
    }
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ------------------------
struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ inline void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__host__ __device__ inline U4 philox4x32_10(U4 ctr, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, ctr.x, hi0, lo0);
        mulhilo32(0xCD9E8D57u, ctr.z, hi1, lo1);
        U4 n;
        n.x = hi1 ^ ctr.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ ctr.w ^ k1;
        n.w = lo0;
        ctr = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return ctr;
}

// [0, 1) with 24 random bits; (0, 1) variant for logarithms.
__host__ __device__ inline float u01(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }
__host__ __device__ inline float u01_open(uint32_t v) {
    return ((float)(v >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

}  // namespace stater
