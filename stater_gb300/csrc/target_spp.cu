// calcTargetSPP (estimator.cpp:498-513 call site): next-round sample budget per
// pixel. Compiled with -fmad=false. The image-wide sum of the per-pixel error
// estimates uses a fixed reduction tree (256 threads x 4 values per 1024-entry
// block: v0+v1+v2+v3 per thread, then pairwise halving 128..1; block sums
// reduced again the same way), so the result does not depend on scheduling and
// equals the CPU restatement bit for bit.
#include <cmath>
#include <mutex>
#include <string>

#include "common.cuh"

namespace stater {
namespace {

template <typename T>
__global__ void tspp_error_kernel(size_t HW, const int32_t *__restrict__ n, const T *__restrict__ varD,
                                  const T *__restrict__ mean, double eps, double *e) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    const int nn = n[p];
    if (nn < 2) {
        e[p] = 0.0;
        return;
    }
    const double nd = (double)nn;
    double acc = 0.0;
    for (int c = 0; c < 3; c++) {
        double v = (double)varD[(size_t)c * HW + p] / nd;
        if (mean) {
            const double m = (double)mean[(size_t)c * HW + p];
            v = v / (m * m + eps);
        }
        acc = acc + v;
    }
    e[p] = acc;
}

// AS_MODE=0 ("ASN"): the error estimate from the pixel's sample variance m2 / (n - 1).
template <typename T>
__global__ void tspp_error_sample_kernel(size_t HW, const int32_t *__restrict__ n, const T *__restrict__ m2,
                                         const T *__restrict__ mean, double eps, double *e) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    const int nn = n[p];
    if (nn < 2) {
        e[p] = 0.0;
        return;
    }
    const double nd = (double)nn;
    double acc = 0.0;
    for (int c = 0; c < 3; c++) {
        const double var = (double)m2[(size_t)c * HW + p] / (nd - 1.0);
        double v = var / nd;
        if (mean) {
            const double m = (double)mean[(size_t)c * HW + p];
            v = v / (m * m + eps);
        }
        acc = acc + v;
    }
    e[p] = acc;
}

__global__ void tree_block_kernel(const double *__restrict__ in, long long len, double *out) {
    __shared__ double part[256];
    const int t = threadIdx.x;
    const long long base = (long long)blockIdx.x * 1024;
    double v[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const long long idx = base + t + 256LL * r;
        v[r] = idx < len ? in[idx] : 0.0;
    }
    part[t] = ((v[0] + v[1]) + v[2]) + v[3];
    __syncthreads();
    for (int s = 128; s >= 1; s >>= 1) {
        if (t < s) part[t] = part[t] + part[t + s];
        __syncthreads();
    }
    if (t == 0) out[blockIdx.x] = part[0];
}

__global__ void tspp_target_kernel(size_t HW, int spp, const int32_t *__restrict__ n, const double *__restrict__ e,
                                   const double *__restrict__ total_ptr, int tmin, int tmax, int32_t *target) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= HW) return;
    const double total = *total_ptr;
    const double budget = (double)spp * (double)HW;
    double t;
    if (n[p] < 2)
        t = (double)tmax;
    else if (!(total > 0.0))
        t = (double)spp;
    else
        t = rint(budget * e[p] / total);
    if (t < tmin) t = tmin;
    if (t > tmax) t = tmax;
    target[p] = (int32_t)t;
}

}  // namespace
}  // namespace stater

using namespace stater;

extern "C" stater_status stater_calc_target_spp(int32_t width, int32_t height, int32_t spp, stater_precision precision,
                                                const int32_t *n, const void *varD, const void *mean, double eps,
                                                int32_t tmin, int32_t tmax, int32_t *targetspp, stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || spp < 0 || !n || !varD || !targetspp || tmin < 0 || tmax < tmin ||
        !(eps >= 0.0))
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t HW = (size_t)width * height;
    const size_t nb1 = (HW + 1023) / 1024;
    double *e = (double *)scratch(2, sizeof(double) * (HW + 2 * nb1 + 2), s);
    if (!e) return set_error(STATER_ERR_NOMEM, "stater_calc_target_spp: scratch allocation failed");
    double *bufA = e + HW, *bufB = bufA + nb1 + 1;
    const unsigned grid = (unsigned)((HW + 255) / 256);
    if (precision == STATER_F64)
        tspp_error_kernel<double><<<grid, 256, 0, s>>>(HW, n, (const double *)varD, (const double *)mean, eps, e);
    else if (precision == STATER_F32)
        tspp_error_kernel<float><<<grid, 256, 0, s>>>(HW, n, (const float *)varD, (const float *)mean, eps, e);
    else
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp: bad precision");
    STATER_CHECK_LAUNCH("tspp_error_kernel");
    const double *cur = e;
    long long len = (long long)HW;
    double *dst = bufA;
    if (len == 1) {
        cudaError_t ce = cudaMemcpyAsync(bufA, e, sizeof(double), cudaMemcpyDeviceToDevice, s);
        if (ce != cudaSuccess) return cuda_status(ce, "stater_calc_target_spp copy");
        cur = bufA;
    }
    while (len > 1) {
        const long long nb = (len + 1023) / 1024;
        tree_block_kernel<<<(unsigned)nb, 256, 0, s>>>(cur, len, dst);
        STATER_CHECK_LAUNCH("tree_block_kernel");
        cur = dst;
        dst = (dst == bufA) ? bufB : bufA;
        len = nb;
    }
    tspp_target_kernel<<<grid, 256, 0, s>>>(HW, spp, n, e, cur, tmin, tmax, targetspp);
    STATER_CHECK_LAUNCH("tspp_target_kernel");
    return STATER_OK;
}

extern "C" stater_status stater_calc_target_spp_ex(const stater_target_spp_args *a, stater_stream stream) {
    clear_error();
    if (!a) return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_ex: null args");
    if (a->as_source == STATER_AS_DENOISED)
        return stater_calc_target_spp(a->width, a->height, a->spp, a->precision, a->n, a->varD, a->mean, a->eps,
                                      a->tmin, a->tmax, a->targetspp, stream);
    if (a->as_source != STATER_AS_SAMPLE)
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_ex: as_source must be 0 or 1");
    if (a->width <= 0 || a->height <= 0 || a->spp < 0 || !a->n || !a->m2 || !a->targetspp || a->tmin < 0 ||
        a->tmax < a->tmin || !(a->eps >= 0.0))
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_ex: bad arguments");
    if (a->precision != STATER_F64 && a->precision != STATER_F32)
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_ex: bad precision");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t HW = (size_t)a->width * a->height;
    const size_t nb1 = (HW + 1023) / 1024;
    double *e = (double *)scratch(2, sizeof(double) * (HW + 2 * nb1 + 2), s);
    if (!e) return set_error(STATER_ERR_NOMEM, "stater_calc_target_spp_ex: scratch allocation failed");
    double *bufA = e + HW, *bufB = bufA + nb1 + 1;
    const unsigned grid = (unsigned)((HW + 255) / 256);
    if (a->precision == STATER_F64)
        tspp_error_sample_kernel<double><<<grid, 256, 0, s>>>(HW, a->n, (const double *)a->m2,
                                                              (const double *)a->mean, a->eps, e);
    else
        tspp_error_sample_kernel<float><<<grid, 256, 0, s>>>(HW, a->n, (const float *)a->m2, (const float *)a->mean,
                                                             a->eps, e);
    STATER_CHECK_LAUNCH("tspp_error_sample_kernel");
    const double *cur = e;
    long long len = (long long)HW;
    double *dst = bufA;
    if (len == 1) {
        cudaError_t ce = cudaMemcpyAsync(bufA, e, sizeof(double), cudaMemcpyDeviceToDevice, s);
        if (ce != cudaSuccess) return cuda_status(ce, "stater_calc_target_spp_ex copy");
        cur = bufA;
    }
    while (len > 1) {
        const long long nb = (len + 1023) / 1024;
        tree_block_kernel<<<(unsigned)nb, 256, 0, s>>>(cur, len, dst);
        STATER_CHECK_LAUNCH("tree_block_kernel");
        cur = dst;
        dst = (dst == bufA) ? bufB : bufA;
        len = nb;
    }
    tspp_target_kernel<<<grid, 256, 0, s>>>(HW, a->spp, a->n, e, cur, a->tmin, a->tmax, a->targetspp);
    STATER_CHECK_LAUNCH("tspp_target_kernel");
    return STATER_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of calcTargetSPP.
//
// Some callers cannot allocate device memory at the point where they need the
// next round's sample budget: a renderer whose device memory is carved up by its
// own pool allocator, or a plugin host that forbids cudaMalloc/cudaFree on its
// worker threads because those calls synchronise the whole device. For them the
// scratch of this entry point (the per-pixel error estimates and the reduction
// partials) lives in a fixed-size array compiled into the library, reserved on
// every GPU that loads libstater until the process exits.
//
// The first call on each device looks up the array's device address
// (cudaGetSymbolAddress, with that device current); make that first call before
// any stream capture begins. All calls share the one array, so calls whose work
// overlaps on the GPU (different streams, no ordering between them) race.
// ---------------------------------------------------------------------------
namespace stater {
namespace {

constexpr size_t kNoAllocMaxPixels = (size_t)1 << 21;  // 2,097,152 pixels: covers 1920x1080
constexpr size_t kNoAllocBlocks = (kNoAllocMaxPixels + 1023) / 1024;
constexpr size_t kNoAllocDoubles = kNoAllocMaxPixels + 2 * (kNoAllocBlocks + 1);

// 16.8 MB: errors [kNoAllocMaxPixels], then two ping-pong reduction buffers.
static __device__ __align__(256) double g_tspp_scratch[kNoAllocDoubles];

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[64] = {nullptr};

}  // namespace

// Forgets the cached address of the array on device `dev` (stater_release_cache):
// after a device reset the module is loaded again, possibly elsewhere, so the
// next call must look the address up afresh.
void noalloc_forget_device(int dev) {
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (dev >= 0 && dev < 64) g_noalloc_ptr[dev] = nullptr;
}

}  // namespace stater

extern "C" stater_status stater_calc_target_spp_noalloc(int32_t width, int32_t height, int32_t spp,
                                                        stater_precision precision, const int32_t *n,
                                                        const void *varD, const void *mean, double eps,
                                                        int32_t tmin, int32_t tmax, int32_t *targetspp,
                                                        stater_stream stream) {
    clear_error();
    if (width <= 0 || height <= 0 || spp < 0 || !n || !varD || !targetspp || tmin < 0 || tmax < tmin ||
        !(eps >= 0.0))
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_noalloc: bad arguments");
    const size_t HW = (size_t)width * height;
    if (HW > kNoAllocMaxPixels)
        return set_error(STATER_ERR_INVALID,
                         "stater_calc_target_spp_noalloc: width*height = " + std::to_string(HW) +
                             " exceeds the fixed scratch of " + std::to_string(kNoAllocMaxPixels) + " pixels");
    if (precision != STATER_F64 && precision != STATER_F32)
        return set_error(STATER_ERR_INVALID, "stater_calc_target_spp_noalloc: bad precision");
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_status(ce, "stater_calc_target_spp_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= 64)
        return set_error(STATER_ERR_UNSUPPORTED, "stater_calc_target_spp_noalloc: device index above 63");
    double *scr;
    {
        // First call on this device (with it current): resolve the device address
        // of the array. The host-side symbol is only a stand-in and must never be
        // handed to a kernel.
        std::lock_guard<std::mutex> lk(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            ce = cudaGetSymbolAddress(&p, g_tspp_scratch);
            if (ce != cudaSuccess) return cuda_status(ce, "stater_calc_target_spp_noalloc: cudaGetSymbolAddress");
            g_noalloc_ptr[dev] = (double *)p;
        }
        scr = g_noalloc_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    // Every scratch word this call reads is written earlier in the same call, so
    // the contents left by a previous call need no clearing.
    double *e = scr;
    double *bufA = scr + kNoAllocMaxPixels;
    double *bufB = bufA + kNoAllocBlocks + 1;
    const unsigned grid = (unsigned)((HW + 255) / 256);
    if (precision == STATER_F64)
        tspp_error_kernel<double><<<grid, 256, 0, s>>>(HW, n, (const double *)varD, (const double *)mean, eps, e);
    else
        tspp_error_kernel<float><<<grid, 256, 0, s>>>(HW, n, (const float *)varD, (const float *)mean, eps, e);
    STATER_CHECK_LAUNCH("tspp_error_kernel");
    const double *cur = e;
    long long len = (long long)HW;
    double *dst = bufA;
    if (len == 1) {
        ce = cudaMemcpyAsync(bufA, e, sizeof(double), cudaMemcpyDeviceToDevice, s);
        if (ce != cudaSuccess) return cuda_status(ce, "stater_calc_target_spp_noalloc copy");
        cur = bufA;
    }
    while (len > 1) {
        const long long nb = (len + 1023) / 1024;
        tree_block_kernel<<<(unsigned)nb, 256, 0, s>>>(cur, len, dst);
        STATER_CHECK_LAUNCH("tree_block_kernel");
        cur = dst;
        dst = (dst == bufA) ? bufB : bufA;
        len = nb;
    }
    tspp_target_kernel<<<grid, 256, 0, s>>>(HW, spp, n, e, cur, tmin, tmax, targetspp);
    STATER_CHECK_LAUNCH("tspp_target_kernel");
    return STATER_OK;
}
