// Film path of the reference renderer: pbrt-v3's FilmTile::AddSample with the
// box filter of radius 0.5 that the statistics integrator enforces
// (core/film.h:152-190, core/api.cpp:1713-1739) and Film::UpdateImage
// (core/film.cpp:187-222) with the RGB -> XYZ -> RGB round trip of
// core/spectrum.h:66-76. Its output is the `film` buffer that denoiseFilm
// filters for the untransformed set (estimator.cpp:432).
//
// Compiled with -fmad=false: every product and sum is rounded on its own, in the
// order the reference writes them, so the film matches its x86 build bit for bit.
#include "common.cuh"
#include "film_common.cuh"

namespace stater {
namespace {

// spectrum.h:72-76 (RGBToXYZ), 66-70 (XYZToRGB), 483-486 (RGBSpectrum::y).
__device__ __forceinline__ void rgb_to_xyz(float r, float g, float b, float &x, float &y, float &z) {
    x = 0.412453f * r + 0.357580f * g + 0.180423f * b;
    y = 0.212671f * r + 0.715160f * g + 0.072169f * b;
    z = 0.019334f * r + 0.119193f * g + 0.950227f * b;
}
__device__ __forceinline__ void xyz_to_rgb(float x, float y, float z, float &r, float &g, float &b) {
    r = 3.240479f * x - 1.537150f * y - 0.498535f * z;
    g = -0.969256f * x + 1.875991f * y + 0.041556f * z;
    b = 0.055648f * x - 0.204043f * y + 1.057311f * z;
}

struct FilmParams {
    int S, NCH;
    const float *__restrict__ samples;
    const int32_t *__restrict__ count;
    FilmTarget F;
};

// One thread per pixel, samples in order; edge samples also go to the
// neighbours' spill planes (film_common.cuh).
__global__ void __launch_bounds__(256) film_add_kernel(FilmParams P) {
    const size_t HW = (size_t)P.F.W * P.F.H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    const int cnt = P.count ? min(max(P.count[p], 0), P.S) : P.S;
    FilmAcc a;
    film_load(P.F, HW, p, a);
    const size_t stride = (size_t)P.NCH * HW;
    const float *sp = P.samples + p;
    for (int s = 0; s < cnt; s++, sp += stride)
        film_add(P.F, p, __ldg(sp), __ldg(sp + HW), __ldg(sp + 2 * HW), __ldg(sp + 3 * HW), __ldg(sp + 4 * HW), a);
    film_store(P.F, HW, p, a);
}

// Film::UpdateImage without splats (the statistics integrator splats nothing).
// MergeFilmTile adds each tile's XYZ-converted sum to the cleared pixel
// (film.cpp:140-149): own samples and edge samples from neighbours are two such
// terms here.
__global__ void __launch_bounds__(256) film_update_kernel(size_t HW, const float *__restrict__ sum,
                                                          const float *__restrict__ weight,
                                                          const float *__restrict__ spill, float scale,
                                                          float *__restrict__ rgb) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    float ax, ay, az, bx = 0.f, by = 0.f, bz = 0.f, w = weight[p];
    rgb_to_xyz(sum[p], sum[HW + p], sum[2 * HW + p], ax, ay, az);
    float sw = 0.f;
    if (spill) {
        rgb_to_xyz(spill[p], spill[HW + p], spill[2 * HW + p], bx, by, bz);
        sw = spill[3 * HW + p];
    }
    const float X = (0.0f + ax) + bx, Y = (0.0f + ay) + by, Z = (0.0f + az) + bz;
    float r, g, b;
    xyz_to_rgb(X, Y, Z, r, g, b);
    w = w + sw;
    if (w != 0.0f) {
        const float inv = 1.0f / w;
        r = r * inv;
        g = g * inv;
        b = b * inv;
        r = 0.0f < r ? r : 0.0f;
        g = 0.0f < g ? g : 0.0f;
        b = 0.0f < b ? b : 0.0f;
    }
    rgb[p] = r * scale;
    rgb[HW + p] = g * scale;
    rgb[2 * HW + p] = b * scale;
}

}  // namespace
}  // namespace stater

using namespace stater;

extern "C" {

stater_status stater_film_add_samples(const stater_film_args *a, stater_stream stream) {
    clear_error();
    if (!a || a->width <= 0 || a->height <= 0 || a->n_samples < 0 || a->n_features < 0 ||
        a->n_features > STATER_MAX_FEATURES || !a->contrib_sum || !a->weight_sum || !a->spill ||
        (a->n_samples > 0 && !a->samples))
        return set_error(STATER_ERR_INVALID, "stater_film_add_samples: bad arguments");
    if (!(a->max_sample_luminance > 0.0f))
        return set_error(STATER_ERR_INVALID, "stater_film_add_samples: max_sample_luminance must be > 0");
    if (a->n_samples == 0) return STATER_OK;
    FilmParams P;
    P.S = a->n_samples;
    P.NCH = 5 + a->n_features;
    P.samples = a->samples;
    P.count = a->count;
    P.F.W = a->width;
    P.F.H = a->height;
    P.F.max_lum = a->max_sample_luminance;
    P.F.sum = a->contrib_sum;
    P.F.weight = a->weight_sum;
    P.F.spill = a->spill;
    const size_t HW = (size_t)a->width * a->height;
    film_add_kernel<<<(unsigned)((HW + 255) / 256), 256, 0, (cudaStream_t)stream>>>(P);
    return cuda_status(cudaGetLastError(), "stater_film_add_samples launch");
}

stater_status stater_film_update_image(int32_t width, int32_t height, const float *contrib_sum,
                                       const float *weight_sum, const float *spill, float scale,
                                       float *rgb, stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || !contrib_sum || !weight_sum || !rgb)
        return set_error(STATER_ERR_INVALID, "stater_film_update_image: bad arguments");
    const size_t HW = (size_t)width * height;
    film_update_kernel<<<(unsigned)((HW + 255) / 256), 256, 0, (cudaStream_t)stream>>>(HW, contrib_sum, weight_sum,
                                                                                      spill, scale, rgb);
    return cuda_status(cudaGetLastError(), "stater_film_update_image launch");
}

}  // extern "C"
