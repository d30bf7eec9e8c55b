// Two FP32 values in one 64-bit register, operated on by the packed FP32
// instructions of sm_100-class GPUs (add/sub/mul/fma .rn.f32x2). Each half is
// rounded exactly as the scalar .rn instruction rounds it, so a computation
// written once over the value type V (float or F2) gives the same bits per
// element either way, while the packed form issues one instruction per pair.
//
// The scalar overloads use the explicitly rounded intrinsics (__fadd_rn, ...),
// which the compiler never contracts into FMAs: the operation sequence is the
// one written, in both forms.
#pragma once
#include <cstdint>

namespace stater {

struct F2 {
    uint64_t v;  // low half: the first element
};

__device__ __forceinline__ F2 f2_pack(float lo, float hi) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(F2 x, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x.v));
}
template <int H>
__device__ __forceinline__ float f2_get(F2 x) {
    float lo, hi;
    f2_unpack(x, lo, hi);
    return H == 0 ? lo : hi;
}
template <int H>
__device__ __forceinline__ void f2_set(F2 &x, float v) {
    float lo, hi;
    f2_unpack(x, lo, hi);
    x = H == 0 ? f2_pack(v, hi) : f2_pack(lo, v);
}
// two consecutive floats of shared memory (8-byte aligned)
__device__ __forceinline__ F2 f2_load(const float *p) {
    F2 r;
    r.v = *reinterpret_cast<const uint64_t *>(p);
    return r;
}

__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

__device__ __forceinline__ F2 vadd(F2 a, F2 b) {
    F2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ F2 vsub(F2 a, F2 b) {
    F2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ F2 vmul(F2 a, F2 b) {
    F2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ F2 vfma(F2 a, F2 b, F2 c) {
    F2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return d;
}

template <typename V>
__device__ __forceinline__ V vconst(float c);
template <>
__device__ __forceinline__ float vconst<float>(float c) {
    return c;
}
template <>
__device__ __forceinline__ F2 vconst<F2>(float c) {
    return f2_pack(c, c);
}

// Element-wise application of a scalar function (hardware approximations,
// comparisons and selects have no packed form).
template <typename Fn>
__device__ __forceinline__ float vmap(float x, Fn f) {
    return f(x);
}
template <typename Fn>
__device__ __forceinline__ F2 vmap(F2 x, Fn f) {
    float a, b;
    f2_unpack(x, a, b);
    return f2_pack(f(a), f(b));
}
template <typename Fn>
__device__ __forceinline__ float vmap(float x, float y, Fn f) {
    return f(x, y);
}
template <typename Fn>
__device__ __forceinline__ F2 vmap(F2 x, F2 y, Fn f) {
    float a, b, c, d;
    f2_unpack(x, a, b);
    f2_unpack(y, c, d);
    return f2_pack(f(a, c), f(b, d));
}
template <typename Fn>
__device__ __forceinline__ float vmap(float x, float y, float z, Fn f) {
    return f(x, y, z);
}
template <typename Fn>
__device__ __forceinline__ F2 vmap(F2 x, F2 y, F2 z, Fn f) {
    float a, b, c, d, e, g;
    f2_unpack(x, a, b);
    f2_unpack(y, c, d);
    f2_unpack(z, e, g);
    return f2_pack(f(a, c, e), f(b, d, g));
}

}  // namespace stater
