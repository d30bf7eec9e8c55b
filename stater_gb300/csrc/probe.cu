// FP32 throughput probe: the denominator of the filters' roofline. The windowed
// filters of stage 2 are FP32 ALU work on CUDA cores (no tensor-core shape, not
// HBM-bound), so their fraction is taken against the FP32 rate this GPU reaches
// with its own FMA instructions: every thread runs kChains independent
// dependency chains of FMAs (enough independent work to fill the pipes), either
// scalar fma.rn.f32 or packed fma.rn.f32x2, and the caller times the launch.
// Operands stay away from overflow and denormals (x <- x * a + b with |a| < 1).
#include <cuda_runtime.h>

#include "common.cuh"
#include "packed_f32x2.cuh"

namespace stater {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) fma_probe_f32(int iters, float a, float b, float *sink) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (float)(threadIdx.x + c) * 1e-3f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++)
#pragma unroll
            for (int c = 0; c < kChains; c++) x[c] = fmaf(x[c], a, b);
    }
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) acc += x[c];
    if (acc == 123.456f) sink[blockIdx.x] = acc;  // keeps the chains alive
}

__global__ void __launch_bounds__(kThreads) fma_probe_f32x2(int iters, float a, float b, float *sink) {
    F2 x[kChains];
    const F2 av = f2_pack(a, a), bv = f2_pack(b, b);
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = f2_pack((float)(threadIdx.x + c) * 1e-3f, (float)(threadIdx.x - c) * 1e-3f);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++)
#pragma unroll
            for (int c = 0; c < kChains; c++) x[c] = vfma(x[c], av, bv);
    }
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        float lo, hi;
        f2_unpack(x[c], lo, hi);
        acc += lo + hi;
    }
    if (acc == 123.456f) sink[blockIdx.x] = acc;
}

}  // namespace
}  // namespace stater

using namespace stater;

extern "C" stater_status stater_fp32_peak_probe(int32_t blocks, int32_t iters, int32_t packed, float *sink,
                                                double *flops, stater_stream stream) {
    clear_error();
    if (blocks <= 0 || iters <= 0 || !sink || (packed != 0 && packed != 1))
        return set_error(STATER_ERR_INVALID, "stater_fp32_peak_probe: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (packed)
        fma_probe_f32x2<<<blocks, kThreads, 0, s>>>(iters, 0.999f, 1e-3f, sink);
    else
        fma_probe_f32<<<blocks, kThreads, 0, s>>>(iters, 0.999f, 1e-3f, sink);
    STATER_CHECK_LAUNCH("fma_probe");
    if (flops) *flops = 2.0 * (packed ? 2.0 : 1.0) * (double)blocks * kThreads * kChains * 16.0 * (double)iters;
    return STATER_OK;
}
