// Kernel parameter blocks shared by the FP64 (plain) and FP32 denoise forms.
#pragma once

#include "common.cuh"

namespace stater {

constexpr float kS2Floor = 1e-30f;  // variance floor inside ln(s^2)

template <typename T>
struct GBuf {
    int count;
    const T *planes[STATER_MAX_GBUFFERS];
    int channels[STATER_MAX_GBUFFERS];
    T dr[STATER_MAX_GBUFFERS];
};

template <typename T>
struct VarsParams {
    int W, H, K, max_moment, R;
    T ds, z;
    const int32_t *n;
    const T *m2[STATER_MAX_TRANSFORMS];
    const T *m3[STATER_MAX_TRANSFORMS];
    const T *m4[STATER_MAX_TRANSFORMS];
    const T *cx[STATER_MAX_TRANSFORMS];
    const T *cy[STATER_MAX_TRANSFORMS];
    const T *m2c_in;
    GBuf<T> gb;
    T *jb[STATER_MAX_TRANSFORMS];
    T *lnS2[STATER_MAX_TRANSFORMS];
    T *se2[STATER_MAX_TRANSFORMS];
    T *m2C[STATER_MAX_TRANSFORMS];
    T *varD[STATER_MAX_TRANSFORMS];
    T *varCD[STATER_MAX_TRANSFORMS];
    T *s2;   // scratch [K][3][HW]
    T *s2c;  // scratch [K][3][HW]
};

template <typename T>
struct FilmParams {
    int W, H, K, R, mt_mode, use_levc, lut_n, discr_source;
    T ds;
    const int32_t *n;
    const T *film;
    const T *mean[STATER_MAX_TRANSFORMS];
    const T *varD[STATER_MAX_TRANSFORMS];
    const T *varCD[STATER_MAX_TRANSFORMS];
    const T *m2s[STATER_MAX_TRANSFORMS];  // STATER_DISCR_SAMPLE: m2C (use_levc) or m2
    const T *jb[STATER_MAX_TRANSFORMS];
    const T *lut;
    GBuf<T> gb;
    T *discr[STATER_MAX_TRANSFORMS];
    T *filmD;
    uint32_t *bits;
    T *ediv;  // scratch [K][3][HW]
};

template <typename T>
inline bool fill_gbuf(GBuf<T> &g, const stater_gbuffers &in) {
    if (in.count < 0 || in.count > STATER_MAX_GBUFFERS) return false;
    g.count = in.count;
    for (int i = 0; i < STATER_MAX_GBUFFERS; i++) {
        g.planes[i] = i < in.count ? (const T *)in.planes[i] : nullptr;
        g.channels[i] = i < in.count ? in.channels[i] : 0;
        g.dr[i] = i < in.count ? (T)in.dr_factor[i] : T(0);
        if (i < in.count && (!in.planes[i] || (in.channels[i] != 1 && in.channels[i] != 3))) return false;
    }
    return true;
}

// FP32 form entry points (denoise_fast.cu).
stater_status denoise_vars_f32(const stater_denoise_vars_args *a, cudaStream_t s);
stater_status denoise_film_f32(const stater_denoise_film_args *a, cudaStream_t s);
// The batched denoise stages of jobs already accumulated, with their film
// images made, enqueued once on s (serving engine; denoise_fast.cu).
stater_status batch_denoise_once(const stater_batch_job *jobs, int n, cudaStream_t s, void *staging,
                                 size_t staging_bytes);

}  // namespace stater
