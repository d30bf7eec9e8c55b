// denoiseVars / denoiseFilm over the reference's own buffer layout.
//
// The reference's Estimator owns pitched cv::cuda::GpuMat images (cudaMallocPitch)
// and hands the denoiser PtrStepSzb tables {data, step, rows, cols}
// (estimator.cpp:26-81): an RGB statistics buffer is one image of interleaved
// float3 (CV_32FC3), n, jb and one-channel G-buffers are one-channel images, and
// element (c, x, y) of a buffer with C channels lies at data + y * step +
// (x * C + c) * element size. These entry points take the caller's buffers in
// that layout unchanged. One gather launch copies every input buffer of the call
// into planar scratch, the planar kernels run on it, and one scatter launch
// copies every output buffer back into the caller's layout. The filters are
// bound by FP32 issue and shared memory, not by HBM (they read each input once
// from L2 per halo row), so the two copy passes (about 1 GB of traffic per
// 1080p call with five transforms) cost a fraction of a millisecond; the planar
// kernels and their results are the same bits either way.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace stater {
namespace {

constexpr int kMaxJobs = 80;

struct CopyJob {
    const unsigned char *src;
    unsigned char *dst;
    int64_t step;   // bytes per row of the pitched side
    int channels;   // interleaved channels of the pitched side
    int elem;       // bytes per element (4 or 8)
};

struct CopyJobs {
    int count, W, H;
    int to_planar;  // 1: pitched -> planar (gather), 0: planar -> pitched (scatter)
    CopyJob job[kMaxJobs];
};

template <typename E>
__device__ __forceinline__ void copy_pixel(const CopyJob &j, int x, int y, size_t HW, size_t p, int to_planar) {
    const size_t poff = (size_t)y * (size_t)j.step + (size_t)x * j.channels * sizeof(E);
    for (int c = 0; c < j.channels; c++) {
        if (to_planar)
            ((E *)j.dst)[(size_t)c * HW + p] = *(const E *)(j.src + poff + c * sizeof(E));
        else
            *(E *)(j.dst + poff + c * sizeof(E)) = ((const E *)j.src)[(size_t)c * HW + p];
    }
}

__global__ void layout_copy_kernel(const __grid_constant__ CopyJobs J) {
    const size_t HW = (size_t)J.W * J.H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW || (int)blockIdx.y >= J.count) return;
    const CopyJob &j = J.job[blockIdx.y];
    const int y = (int)(p / (size_t)J.W), x = (int)(p - (size_t)y * J.W);
    if (j.elem == 8)
        copy_pixel<unsigned long long>(j, x, y, HW, p, J.to_planar);
    else
        copy_pixel<unsigned int>(j, x, y, HW, p, J.to_planar);
}

// Collects the buffers of one call: pitched pointer, channels, step, element
// size; assigns each its planar slice of one scratch block.
struct Plan {
    struct Item {
        const void *pitched;
        int channels, elem;
        int64_t step;
        size_t offset;  // bytes into the scratch block
    };
    std::vector<Item> in, out;
    size_t bytes = 0;
    size_t HW;
    explicit Plan(size_t hw) : HW(hw) {}
    void *add(std::vector<Item> &v, const void *p, int channels, int elem, int64_t step) {
        if (!p) return nullptr;
        bytes = (bytes + 255) & ~(size_t)255;
        v.push_back(Item{p, channels, elem, step, bytes});
        bytes += (size_t)channels * elem * HW;
        return (void *)(uintptr_t)(v.back().offset + 1);  // placeholder, resolved by at()
    }
};

void *resolve(void *placeholder, unsigned char *base) {
    return placeholder ? base + ((size_t)(uintptr_t)placeholder - 1) : nullptr;
}

stater_status launch_copies(const std::vector<Plan::Item> &items, unsigned char *base, int W, int H, bool to_planar,
                            cudaStream_t s, const char *what) {
    const size_t HW = (size_t)W * H;
    for (size_t first = 0; first < items.size(); first += kMaxJobs) {
        CopyJobs J;
        J.W = W;
        J.H = H;
        J.to_planar = to_planar ? 1 : 0;
        J.count = (int)std::min(items.size() - first, (size_t)kMaxJobs);
        for (int i = 0; i < J.count; i++) {
            const Plan::Item &it = items[first + i];
            unsigned char *planar = base + it.offset;
            J.job[i].src = to_planar ? (const unsigned char *)it.pitched : planar;
            J.job[i].dst = to_planar ? planar : (unsigned char *)it.pitched;
            J.job[i].step = it.step;
            J.job[i].channels = it.channels;
            J.job[i].elem = it.elem;
        }
        dim3 grid((unsigned)((HW + 255) / 256), (unsigned)J.count);
        layout_copy_kernel<<<grid, 256, 0, s>>>(J);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_status(e, what);
    }
    return STATER_OK;
}

stater_status check_layout(const stater_pitched_layout *L, int W, int elem, const char *fn) {
    if (!L) return set_error(STATER_ERR_INVALID, std::string(fn) + ": null layout");
    if (L->rgb_step < (int64_t)3 * W * elem || L->rgb_step % elem != 0)
        return set_error(STATER_ERR_INVALID, std::string(fn) + ": rgb_step below 3 * width * element size or "
                                                               "not a multiple of the element size");
    if (L->scalar_step < (int64_t)W * elem || L->scalar_step % elem != 0)
        return set_error(STATER_ERR_INVALID, std::string(fn) + ": scalar_step below width * element size or "
                                                               "not a multiple of the element size");
    if (L->n_step < (int64_t)W * 4 || L->n_step % 4 != 0)
        return set_error(STATER_ERR_INVALID, std::string(fn) + ": n_step below 4 * width or not a multiple of 4");
    return STATER_OK;
}

}  // namespace
}  // namespace stater

using namespace stater;

extern "C" stater_status stater_denoise_vars_pitched(const stater_denoise_vars_args *a,
                                                     const stater_pitched_layout *L, stater_stream stream) {
    clear_error();
    const char *fn = "stater_denoise_vars_pitched";
    if (!a) return set_error(STATER_ERR_INVALID, "stater_denoise_vars_pitched: null args");
    if (a->precision != STATER_F32 && a->precision != STATER_F64)
        return set_error(STATER_ERR_INVALID, "stater_denoise_vars_pitched: bad precision");
    if (a->width <= 0 || a->height <= 0 || a->n_buffers < 1 || a->n_buffers > STATER_MAX_TRANSFORMS ||
        a->gbuffers.count < 0 || a->gbuffers.count > STATER_MAX_GBUFFERS)
        return set_error(STATER_ERR_INVALID, "stater_denoise_vars_pitched: bad geometry");
    const int elem = a->precision == STATER_F64 ? 8 : 4;
    stater_status st = check_layout(L, a->width, elem, fn);
    if (st != STATER_OK) return st;
    const int W = a->width, H = a->height, K = a->n_buffers;
    Plan plan((size_t)W * H);
    stater_denoise_vars_args b = *a;  // planar copy of the call
    b.n = (const int32_t *)plan.add(plan.in, a->n, 1, 4, L->n_step);
    for (int k = 0; k < K; k++) {
        b.m2[k] = plan.add(plan.in, a->m2[k], 3, elem, L->rgb_step);
        b.m3[k] = plan.add(plan.in, a->m3[k], 3, elem, L->rgb_step);
        b.m4[k] = a->max_moment >= 4 ? plan.add(plan.in, a->m4[k], 3, elem, L->rgb_step) : nullptr;
        b.c2X[k] = a->max_moment >= 5 ? plan.add(plan.in, a->c2X[k], 3, elem, L->rgb_step) : nullptr;
        b.c2Y[k] = a->max_moment >= 5 ? plan.add(plan.in, a->c2Y[k], 3, elem, L->rgb_step) : nullptr;
    }
    b.m2C_in = plan.add(plan.in, a->m2C_in, 3, elem, L->rgb_step);
    for (int g = 0; g < a->gbuffers.count; g++) {
        const int ch = a->gbuffers.channels[g];
        b.gbuffers.planes[g] = plan.add(plan.in, a->gbuffers.planes[g], ch, elem, ch == 1 ? L->scalar_step : L->rgb_step);
    }
    for (int k = 0; k < K; k++) {
        b.jb[k] = plan.add(plan.out, a->jb[k], 1, elem, L->scalar_step);
        b.lnS2[k] = plan.add(plan.out, a->lnS2[k], 3, elem, L->rgb_step);
        b.se2[k] = plan.add(plan.out, a->se2[k], 3, elem, L->rgb_step);
        b.m2C[k] = plan.add(plan.out, a->m2C[k], 3, elem, L->rgb_step);
        b.varD[k] = plan.add(plan.out, a->varD[k], 3, elem, L->rgb_step);
        b.varCD[k] = plan.add(plan.out, a->varCD[k], 3, elem, L->rgb_step);
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *base = (unsigned char *)scratch(20, plan.bytes, s);
    if (!base) return set_error(STATER_ERR_NOMEM, "stater_denoise_vars_pitched: scratch allocation failed");
    // resolve the planar slices
    b.n = (const int32_t *)resolve((void *)b.n, base);
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        b.m2[k] = resolve((void *)b.m2[k], base);
        b.m3[k] = resolve((void *)b.m3[k], base);
        b.m4[k] = resolve((void *)b.m4[k], base);
        b.c2X[k] = resolve((void *)b.c2X[k], base);
        b.c2Y[k] = resolve((void *)b.c2Y[k], base);
        b.jb[k] = resolve(b.jb[k], base);
        b.lnS2[k] = resolve(b.lnS2[k], base);
        b.se2[k] = resolve(b.se2[k], base);
        b.m2C[k] = resolve(b.m2C[k], base);
        b.varD[k] = resolve(b.varD[k], base);
        b.varCD[k] = resolve(b.varCD[k], base);
    }
    b.m2C_in = resolve((void *)b.m2C_in, base);
    for (int g = 0; g < STATER_MAX_GBUFFERS; g++) b.gbuffers.planes[g] = resolve((void *)b.gbuffers.planes[g], base);
    st = launch_copies(plan.in, base, W, H, true, s, "stater_denoise_vars_pitched gather");
    if (st != STATER_OK) return st;
    st = stater_denoise_vars(&b, stream);
    if (st != STATER_OK) return st;
    return launch_copies(plan.out, base, W, H, false, s, "stater_denoise_vars_pitched scatter");
}

extern "C" stater_status stater_denoise_film_pitched(const stater_denoise_film_args *a,
                                                     const stater_pitched_layout *L, stater_stream stream) {
    clear_error();
    const char *fn = "stater_denoise_film_pitched";
    if (!a) return set_error(STATER_ERR_INVALID, "stater_denoise_film_pitched: null args");
    if (a->precision != STATER_F32 && a->precision != STATER_F64)
        return set_error(STATER_ERR_INVALID, "stater_denoise_film_pitched: bad precision");
    if (a->width <= 0 || a->height <= 0 || a->n_buffers < 1 || a->n_buffers > STATER_MAX_TRANSFORMS ||
        a->gbuffers.count < 0 || a->gbuffers.count > STATER_MAX_GBUFFERS)
        return set_error(STATER_ERR_INVALID, "stater_denoise_film_pitched: bad geometry");
    const int elem = a->precision == STATER_F64 ? 8 : 4;
    stater_status st = check_layout(L, a->width, elem, fn);
    if (st != STATER_OK) return st;
    const int W = a->width, H = a->height, K = a->n_buffers;
    const bool sample = a->discr_source == STATER_DISCR_SAMPLE;
    Plan plan((size_t)W * H);
    stater_denoise_film_args b = *a;
    b.n = (const int32_t *)plan.add(plan.in, a->n, 1, 4, L->n_step);
    b.film = plan.add(plan.in, a->film, 3, elem, L->rgb_step);
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        const bool on = k < K;
        b.mean[k] = on && k > 0 ? plan.add(plan.in, a->mean[k], 3, elem, L->rgb_step) : nullptr;
        b.varD[k] = on && !sample && !a->use_levc ? plan.add(plan.in, a->varD[k], 3, elem, L->rgb_step) : nullptr;
        b.varCD[k] = on && !sample && a->use_levc ? plan.add(plan.in, a->varCD[k], 3, elem, L->rgb_step) : nullptr;
        b.m2[k] = on && sample && !a->use_levc ? plan.add(plan.in, a->m2[k], 3, elem, L->rgb_step) : nullptr;
        b.m2C[k] = on && sample && a->use_levc ? plan.add(plan.in, a->m2C[k], 3, elem, L->rgb_step) : nullptr;
        b.jb[k] = on && a->mt_mode == STATER_MT_JB ? plan.add(plan.in, a->jb[k], 1, elem, L->scalar_step) : nullptr;
    }
    for (int g = 0; g < a->gbuffers.count; g++) {
        const int ch = a->gbuffers.channels[g];
        b.gbuffers.planes[g] = plan.add(plan.in, a->gbuffers.planes[g], ch, elem, ch == 1 ? L->scalar_step : L->rgb_step);
    }
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++)
        b.discr[k] = k < K ? plan.add(plan.out, a->discr[k], 3, elem, L->rgb_step) : nullptr;
    b.filmD = plan.add(plan.out, a->filmD, 3, elem, L->rgb_step);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *base = (unsigned char *)scratch(21, plan.bytes, s);
    if (!base) return set_error(STATER_ERR_NOMEM, "stater_denoise_film_pitched: scratch allocation failed");
    b.n = (const int32_t *)resolve((void *)b.n, base);
    b.film = resolve((void *)b.film, base);
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        b.mean[k] = resolve((void *)b.mean[k], base);
        b.varD[k] = resolve((void *)b.varD[k], base);
        b.varCD[k] = resolve((void *)b.varCD[k], base);
        b.m2[k] = resolve((void *)b.m2[k], base);
        b.m2C[k] = resolve((void *)b.m2C[k], base);
        b.jb[k] = resolve((void *)b.jb[k], base);
        b.discr[k] = resolve(b.discr[k], base);
    }
    b.filmD = resolve(b.filmD, base);
    for (int g = 0; g < STATER_MAX_GBUFFERS; g++) b.gbuffers.planes[g] = resolve((void *)b.gbuffers.planes[g], base);
    st = launch_copies(plan.in, base, W, H, true, s, "stater_denoise_film_pitched gather");
    if (st != STATER_OK) return st;
    st = stater_denoise_film(&b, stream);
    if (st != STATER_OK) return st;
    return launch_copies(plan.out, base, W, H, false, s, "stater_denoise_film_pitched scatter");
}

extern "C" stater_status stater_calc_target_spp_pitched(const stater_target_spp_args *a,
                                                        const stater_pitched_layout *L, stater_stream stream) {
    clear_error();
    if (!a) return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_pitched: null args");
    if (a->precision != STATER_F32 && a->precision != STATER_F64)
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_pitched: bad precision");
    if (a->width <= 0 || a->height <= 0)
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_pitched: bad geometry");
    const int elem = a->precision == STATER_F64 ? 8 : 4;
    stater_status st = check_layout(L, a->width, elem, "stater_calc_target_spp_pitched");
    if (st != STATER_OK) return st;
    const int W = a->width, H = a->height;
    const bool sample = a->as_source == STATER_AS_SAMPLE;
    Plan plan((size_t)W * H);
    stater_target_spp_args b = *a;
    b.n = (const int32_t *)plan.add(plan.in, a->n, 1, 4, L->n_step);
    b.m2 = sample ? plan.add(plan.in, a->m2, 3, elem, L->rgb_step) : nullptr;
    b.varD = sample ? nullptr : plan.add(plan.in, a->varD, 3, elem, L->rgb_step);
    b.mean = plan.add(plan.in, a->mean, 3, elem, L->rgb_step);
    b.targetspp = (int32_t *)plan.add(plan.out, a->targetspp, 1, 4, L->n_step);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *base = (unsigned char *)scratch(22, plan.bytes, s);
    if (!base) return set_error(STATER_ERR_NOMEM, "stater_calc_target_spp_pitched: scratch allocation failed");
    b.n = (const int32_t *)resolve((void *)b.n, base);
    b.m2 = resolve((void *)b.m2, base);
    b.varD = resolve((void *)b.varD, base);
    b.mean = resolve((void *)b.mean, base);
    b.targetspp = (int32_t *)resolve((void *)b.targetspp, base);
    st = launch_copies(plan.in, base, W, H, true, s, "stater_calc_target_spp_pitched gather");
    if (st != STATER_OK) return st;
    st = stater_calc_target_spp_ex(&b, stream);
    if (st != STATER_OK) return st;
    return launch_copies(plan.out, base, W, H, false, s, "stater_calc_target_spp_pitched scatter");
}
