// One sample's contribution to the film: pbrt-v3 FilmTile::AddSample with the
// box filter of radius 0.5 (core/film.h:152-190). Shared by the film kernel and
// the accumulation kernels, which add the film sums of transform 0's samples
// as they read them. Every operation is rounded on its own (explicit _rn
// intrinsics), so the sums are the same in FMA-contracting and exact units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace stater {

struct FilmTarget {
    int W, H;
    float max_lum;
    float *sum;     // [3][HW] own samples, in order
    float *weight;  // [HW]
    float *spill;   // [4][HW] edge samples of neighbouring pixels (R, G, B, weight)
};

struct FilmAcc {
    float s0, s1, s2, w;
};

__device__ __forceinline__ void film_load(const FilmTarget &F, size_t HW, size_t p, FilmAcc &a) {
    a.s0 = F.sum[p];
    a.s1 = F.sum[HW + p];
    a.s2 = F.sum[2 * HW + p];
    a.w = F.weight[p];
}

__device__ __forceinline__ void film_store(const FilmTarget &F, size_t HW, size_t p, const FilmAcc &a) {
    F.sum[p] = a.s0;
    F.sum[HW + p] = a.s1;
    F.sum[2 * HW + p] = a.s2;
    F.weight[p] = a.w;
}

// A sample at pFilm = (x + u, y + v) lies in the box filter's support of pixels
// ceil(x + u - 1) .. floor(x + u): also the left (right) neighbour exactly when
// u == 0 (u == 1), the same in y.
__device__ __forceinline__ void film_spill(const FilmTarget &F, size_t p, float r, float g, float b, float u, float v) {
    const size_t HW = (size_t)F.W * F.H;
    const int x = (int)(p % (size_t)F.W), y = (int)(p / (size_t)F.W);
    const int dx0 = u == 0.0f ? -1 : 0, dx1 = u == 1.0f ? 1 : 0;
    const int dy0 = v == 0.0f ? -1 : 0, dy1 = v == 1.0f ? 1 : 0;
    for (int dy = dy0; dy <= dy1; dy++) {
        for (int dx = dx0; dx <= dx1; dx++) {
            const int qx = x + dx, qy = y + dy;
            if ((dx == 0 && dy == 0) || qx < 0 || qy < 0 || qx >= F.W || qy >= F.H) continue;
            const size_t q = (size_t)qy * F.W + qx;
            atomicAdd(F.spill + q, r);
            atomicAdd(F.spill + HW + q, g);
            atomicAdd(F.spill + 2 * HW + q, b);
            atomicAdd(F.spill + 3 * HW + q, 1.0f);
        }
    }
}

__device__ __forceinline__ void film_add(const FilmTarget &F, size_t p, float r, float g, float b, float u, float v,
                                         FilmAcc &a) {
    // L *= maxSampleLuminance / L.y() above the limit (RGBSpectrum::y, core/spectrum.h:483-486)
    const float lum = __fadd_rn(__fadd_rn(__fmul_rn(0.212671f, r), __fmul_rn(0.715160f, g)), __fmul_rn(0.072169f, b));
    if (lum > F.max_lum) {
        const float f = __fdiv_rn(F.max_lum, lum);
        r = __fmul_rn(r, f);
        g = __fmul_rn(g, f);
        b = __fmul_rn(b, f);
    }
    a.s0 = __fadd_rn(a.s0, r);
    a.s1 = __fadd_rn(a.s1, g);
    a.s2 = __fadd_rn(a.s2, b);
    a.w = __fadd_rn(a.w, 1.0f);
    if (u == 0.0f || u == 1.0f || v == 0.0f || v == 1.0f) film_spill(F, p, r, g, b, u, v);
}

}  // namespace stater
