// Inline-PTX helpers for the TMA-fed kernels: mbarrier init / arrive /
// bounded wait, and tiled tensor loads (cp.async.bulk.tensor) that complete on
// an mbarrier. Every wait is bounded: the pipeline waits (consumers for a full
// stage, the producer for a free one) by the limit the kernel is given
// (kWaitLimit polls unless stater_debug_set_pipeline_waits lowered it), the
// producer's final wait for the copies it issued always by kWaitLimit. A
// pipeline wait that gives up returns false and the kernel ORs kErrTimeout into
// the library's device error word; a final wait that gives up ORs kErrDrain
// (copies may still have been in flight when the CTA ended). stater_synchronize
// reports either as STATER_ERR_TIMEOUT.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace stater {

int *device_error_word();
// Pipeline-wait limit and producer stall flag of the TMA-fed kernels
// (stater_debug_set_pipeline_waits; defaults kWaitLimit and 0).
uint32_t pipeline_wait_limit();
int pipeline_stall();
bool encode_tensor_map_2d_f32(CUtensorMap *map, const void *base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                              uint32_t box_rows);
// 3-D float tensor [d2][d1][d0] (d0 contiguous), box {b0, b1, b2}.
bool encode_tensor_map_3d_f32(CUtensorMap *map, const void *base, uint64_t d0, uint64_t d1, uint64_t d2, uint32_t b0,
                              uint32_t b1, uint32_t b2);

namespace tma {

constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int kErrTimeout = 1;
constexpr int kErrDrain = 2;

static __device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

static __device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

static __device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar)) : "memory");
}

static __device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// Bounded wait (at most `limit` polls) for the phase with parity `parity` to complete.
static __device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit = kWaitLimit) {
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

static __device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

static __device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                                   uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace tma
}  // namespace stater
