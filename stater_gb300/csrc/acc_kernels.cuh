// Stage-1 kernels: per-pixel online moments of radiance under K transforms.
//
// One thread owns one (pixel, transform) pair: threadIdx.x walks pixels,
// threadIdx.y is the transform. The K threads of a pixel read the same sample
// words, so every sample plane is fetched from HBM once and served to the other
// transforms from L1. Moments live in registers for the whole call and are
// written back once, so the state crosses HBM twice per call regardless of the
// number of samples. Sample planes [S][5+G][HW] make every load a coalesced
// 128-byte row per warp.
//
// The update is the reference's (StatTile::AddStatSampleM1..M4C,
// src/statistics/estimator.h:226-305): n is incremented first, m2 updated
// before m3 uses it, m4 after m3, c2X/c2Y with the updated mean and the float
// offset inPxP - 0.5f, m1 += sqrt(d (d - dN)). EXACT divides by n (bitwise the
// reference's arithmetic when compiled with -fmad=false); FAST multiplies by a
// reciprocal shared by all moments of the sample.
#pragma once

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "film_common.cuh"
#include "packed_f32x2.cuh"

namespace stater {

struct AccParams {
    size_t HW;   // sample columns (pixels, or entries of pix)
    size_t HWs;  // pixels of the statistics planes (W*H)
    const int32_t *pix;  // nullable: sample column i belongs to pixel pix[i]
    int S, G, K, NCH;
    const float *__restrict__ samples;
    const int32_t *__restrict__ count;
    TransformSet ts;
    int32_t *n;
    void *stats;
    void *gmean;
    // Optional film sums (film.sum == nullptr: off), added by the transform-0
    // threads from the samples they read anyway.
    FilmTarget film;
    // Feature channels whose running means transform k's threads keep
    // (featmap[k][j] < 0: none); chosen on the host so that the cheap
    // transforms' threads carry them (acc_assign_features).
    int8_t featmap[STATER_MAX_TRANSFORMS][STATER_MAX_FEATURES];
    int maxf;  // largest number of channels one transform keeps
    // TMA-fed kernel: the transform of warp w (a permutation of 0..K-1 that
    // spreads the costly transforms over the SM's schedulers)
    int8_t wt[STATER_MAX_TRANSFORMS];
};

// Issue cost of one sample's update per transform kind in the FAST form:
// instructions a warp issues for one sample of its 64 columns (the shared part
// of 32 -- three loads, the reciprocal of n and the moment updates -- plus the
// transform's own), and the extras of the film sums and of one feature channel.
inline int acc_kind_cost(int kind) {
    switch (kind) {
        case STATER_TK_IDENTITY: return 32;
        case STATER_TK_SQRT: return 38;
        case STATER_TK_CBRT: return 53;
        case STATER_TK_LOG1P: return 80;
        case STATER_TK_ASINH: return 101;
        default: return 200;  // Box-Cox: libm exp and log per value
    }
}
constexpr int kAccFilmCost = 27;
constexpr int kAccFeatureCost = 3;

// Where the K transforms' warps and the feature channels go in the TMA-fed
// kernel. Warp w of a CTA issues on the SM's scheduler w % 4, so two warps
// whose indices differ by 4 share one; the CTA's time is set by its busiest
// scheduler. The plan tries every order of the transforms over the warps
// (K! orders, K <= 8) and, for each, hands the feature channels one by one to
// the transform on the least busy scheduler (at most ceil(G/K) each, to bound
// the registers a warp keeps); it keeps the order whose busiest scheduler has
// the least work. Plans are cached per (transform kinds, G, film).
struct AccPlan {
    int8_t wt[STATER_MAX_TRANSFORMS];                            // warp -> transform
    int8_t featmap[STATER_MAX_TRANSFORMS][STATER_MAX_FEATURES];  // transform -> its feature channels
    int maxf;
};

// Returns the busiest scheduler's load; *shared receives the consumer load on
// the scheduler of the producer warp (warp K).
inline int acc_plan_eval(const int *cost, int K, int G, const int8_t *wt, AccPlan *out, int *shared = nullptr) {
    int sched[4] = {0, 0, 0, 0}, cnt[STATER_MAX_TRANSFORMS] = {0};
    int where[STATER_MAX_TRANSFORMS];
    for (int w = 0; w < K; w++) {
        where[wt[w]] = w % 4;
        sched[w % 4] += cost[wt[w]];
    }
    const int cap = (G + K - 1) / K;
    int maxc = 0;
    if (out)
        for (int k = 0; k < STATER_MAX_TRANSFORMS; k++)
            for (int j = 0; j < STATER_MAX_FEATURES; j++) out->featmap[k][j] = -1;
    for (int g = 0; g < G; g++) {
        int best = -1;
        for (int k = 0; k < K; k++) {
            if (cnt[k] >= cap) continue;
            if (best < 0 || sched[where[k]] < sched[where[best]] ||
                (sched[where[k]] == sched[where[best]] && cost[k] < cost[best]))
                best = k;
        }
        if (out) out->featmap[best][cnt[best]] = (int8_t)g;
        cnt[best]++;
        sched[where[best]] += kAccFeatureCost;
        if (cnt[best] > maxc) maxc = cnt[best];
    }
    if (out) out->maxf = maxc;
    if (shared) *shared = sched[K % 4];
    return std::max(std::max(sched[0], sched[1]), std::max(sched[2], sched[3]));
}

inline AccPlan acc_plan(const int *kinds, int K, int G, bool film) {
    int cost[STATER_MAX_TRANSFORMS];
    for (int k = 0; k < K; k++) cost[k] = acc_kind_cost(kinds[k]) + (k == 0 && film ? kAccFilmCost : 0);
    int8_t order[STATER_MAX_TRANSFORMS], best[STATER_MAX_TRANSFORMS];
    for (int k = 0; k < K; k++) order[k] = best[k] = (int8_t)k;
    // among orders with the same busiest scheduler, the one with the most work
    // beside the producer warp (mostly waiting): measured at 1080p, the
    // costliest transform there ran 2.5% faster than on a scheduler of its own
    int best_shared = 0;
    int best_load = acc_plan_eval(cost, K, G, order, nullptr, &best_shared);
    while (std::next_permutation(order, order + K)) {
        int sh = 0;
        const int l = acc_plan_eval(cost, K, G, order, nullptr, &sh);
        if (l < best_load || (l == best_load && sh > best_shared)) {
            best_load = l;
            best_shared = sh;
            std::copy(order, order + K, best);
        }
    }
    AccPlan plan;
    for (int w = 0; w < STATER_MAX_TRANSFORMS; w++) plan.wt[w] = (int8_t)(w < K ? best[w] : w);
    acc_plan_eval(cost, K, G, best, &plan);
    return plan;
}

// The plan for P's transforms (cached), written into P. Returns the largest
// number of feature channels one transform keeps.
inline int acc_assign_features(AccParams &P) {
    struct Entry {
        int kinds[STATER_MAX_TRANSFORMS];
        int K, G;
        bool film;
        AccPlan plan;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;  // at most 64 sets; beyond, entries are overwritten in turn
    static size_t next_slot = 0;
    const bool film = P.film.sum != nullptr;
    AccPlan plan;
    bool found = false;
    {
        std::lock_guard<std::mutex> lock(mu);
        for (const Entry &e : cache)
            if (e.K == P.K && e.G == P.G && e.film == film &&
                std::equal(e.kinds, e.kinds + P.K, P.ts.kind)) {
                plan = e.plan;
                found = true;
                break;
            }
    }
    if (!found) {
        plan = acc_plan(P.ts.kind, P.K, P.G, film);
        std::lock_guard<std::mutex> lock(mu);
        Entry e;
        std::copy(P.ts.kind, P.ts.kind + P.K, e.kinds);
        e.K = P.K;
        e.G = P.G;
        e.film = film;
        e.plan = plan;
        if (cache.size() < 64)
            cache.push_back(e);
        else
            cache[next_slot++ % cache.size()] = e;
    }
    std::copy(plan.wt, plan.wt + STATER_MAX_TRANSFORMS, P.wt);
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++)
        std::copy(plan.featmap[k], plan.featmap[k] + STATER_MAX_FEATURES, P.featmap[k]);
    return plan.maxf;
}

// Compact FP32 forms used by the FAST mode, written once over the value type V
// (float, or F2 = two pixels in one register with packed arithmetic) from
// explicitly rounded operations and the hardware approximations, so the
// scalar and packed kernels give the same bits. No addition or subtraction
// takes a product as an operand (such pairs are written as FMAs): the code
// generator may fuse a packed multiply into a following packed add, never a
// scalar one with explicit rounding, so the sequence leaves it nothing to
// fuse. Accurate to about 1e-6 relative (a few 1e-7 for log1p and asinh),
// checked against the FP64 oracle:
//   log1p: 2 atanh(t), t = x/(2+x), by its Taylor series t + t^3/3 + t^5/5
//          for x < 1/4 (t < 1/9; truncation below 4e-7 relative), else
//          log2(1+x) ln 2 with the hardware log2;
//   asinh: for |x| < 1/4 its Taylor series x - x^3/6 + 3x^5/40 - 5x^7/112
//          (truncation below 5e-7 relative), else log2(|x| + sqrt(x^2 + 1)) ln 2
//          (2|x| where x^2 overflows), odd;
//   cbrt:  2^(log2|x| / 3) with the hardware log2 and exp2, odd (0 at 0,
//          infinite at infinity: the hardware's log2(0) = -inf, exp2(-inf) = 0);
//   sqrt:  the hardware square root (0 at 0, NaN below 0).
// The hardware log2/exp2/sqrt approximations are the special-function unit's,
// whose issue rate is an eighth of the FMA pipe's: each costs as much as
// several arithmetic instructions, so each form uses as few as its accuracy
// allows.
// Divisions are a multiplication by the hardware reciprocal.
__device__ __forceinline__ float fast_log2(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float fast_exp2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float fast_rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float fast_rsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float fast_sqrt(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr float kLn2f = 0.69314718055994531f;

template <typename V>
__device__ __forceinline__ V log1p_compact(V x) {
    const V t = vmul(x, vmap(vadd(vconst<V>(2.f), x), fast_rcp));
    const V t2 = vmul(t, t);
    V q = vfma(t2, vconst<V>(2.f / 5.f), vconst<V>(2.f / 3.f));
    q = vfma(t2, q, vconst<V>(2.f));
    const V small = vmul(t, q);  // 2 t (1 + t^2/3 + t^4/5)
    const V large = vmul(vmap(vadd(vconst<V>(1.f), x), fast_log2), vconst<V>(kLn2f));
    return vmap(x, small, large, [](float a, float s, float l) { return a < 0.25f ? s : l; });
}
template <typename V>
__device__ __forceinline__ V asinh_compact(V x) {
    const V a = vmap(x, [](float v) { return fabsf(v); });
    const V a2 = vmul(a, a);
    V q = vfma(a2, vconst<V>(-5.f / 112.f), vconst<V>(3.f / 40.f));
    q = vfma(a2, q, vconst<V>(-1.f / 6.f));
    q = vfma(a2, q, vconst<V>(1.f));
    const V small = vmul(a, q);
    const V w = vfma(a, a, vconst<V>(1.f));
    // a + sqrt(a^2 + 1) > 2a; where a^2 overflows (a above 1.8e19) the sum is
    // inf * 0 = NaN, and the maximum (which drops a NaN operand) gives 2a
    const V arg = vmap(vfma(w, vmap(w, fast_rsqrt), a), vmul(a, vconst<V>(2.f)),
                       [](float t, float t2) { return fmaxf(t, t2); });
    const V large = vmul(vmap(arg, fast_log2), vconst<V>(kLn2f));
    const V mag = vmap(a, small, large, [](float m, float s, float l) { return m < 0.25f ? s : l; });
    return vmap(mag, x, [](float m, float v) { return copysignf(m, v); });
}
template <typename V>
__device__ __forceinline__ V cbrt_compact(V x) {
    const V l = vmap(x, [](float v) { return fast_log2(fabsf(v)); });
    const V y = vmap(vmul(l, vconst<V>(1.f / 3.f)), fast_exp2);
    return vmap(y, x, [](float r, float v) { return copysignf(r, v); });
}
template <typename V>
__device__ __forceinline__ V sqrt_compact(V x) {
    return vmap(x, fast_sqrt);
}

// FAST transform of one radiance value (V = float or F2).
template <typename V, int KIND>
__device__ __forceinline__ V fast_transform(float lambda, V x) {
    switch (KIND) {
        case STATER_TK_LOG1P: return log1p_compact(x);
        case STATER_TK_SQRT: return sqrt_compact(x);
        case STATER_TK_CBRT: return cbrt_compact(x);
        case STATER_TK_ASINH: return asinh_compact(x);
        case STATER_TK_BOXCOX:
            // expm1(l ln x)/l: no cancellation for small l
            return vmap(x, [lambda](float v) { return lambda == 1.f ? v : expm1f(lambda * logf(v)) / lambda; });
        default: return x;
    }
}

// Transform of one radiance value. EXACT: the libm-accurate functions (and the
// reference's (x^l - 1)/l for Box-Cox). FAST (FP32 only): the compact forms.
template <typename T, bool FAST, int KIND>
__device__ __forceinline__ T acc_transform(float lambda, T x) {
    if (!FAST || sizeof(T) == 8) {
        return transform_exact<T>(KIND, lambda, x);
    } else {
        return (T)fast_transform<float, KIND>(lambda, (float)x);
    }
}

// FAST update of one channel's moments by one sample. rn = 1/n, dN = d/n.
// For a pixel's first sample (n = 1, moments 0) the sequence gives mean = x
// and leaves every moment exactly 0 for finite x: every increment carries the
// factor e = d - dN, the single rounding of d - d = 0. This takes the hardware
// reciprocal of 1 to be exactly 1 (checked on the GPU by the first-sample test
// of the edge-case suite). The reference's order: m2 updated first, m3 with the new
// m2 (d (d^2 - dN^2) = d (d - dN)(d + dN)), m4 with the new m3 and m2,
// c2X/c2Y with the new mean, m1 += sqrt(d (d - dN)). The transforms end in a
// select or a sign operation, so x itself is never a product.
template <typename V, int MAXMOM>
__device__ __forceinline__ void meng_fast(V x, V rn, V xD, V yD, V &mean, V &m2, V &m3, V &m4, V &cx, V &cy,
                                          V &m1) {
    const V d = vsub(x, mean);
    mean = vfma(d, rn, mean);
    if (MAXMOM >= 2) {
        const V e = vfma(d, vmul(rn, vconst<V>(-1.f)), d);  // d - dN
        m2 = vfma(d, e, m2);
        if (MAXMOM >= 3) {
            // m3 + d (d - dN)(d + dN) - 3 dN m2 = m3 + d ((d - dN)(d + dN) - 3 rn m2):
            // four operations (the multiples of rn are shared by the channels)
            const V s = vfma(m2, vmul(rn, vconst<V>(-3.f)), vmul(e, vfma(d, rn, d)));
            const V m3n = vfma(d, s, m3);
            if (MAXMOM >= 4) {
                const V dN = vmul(d, rn);
                const V dN2 = vmul(dN, dN);
                // d^3 - dN^3 = (d - dN)(d^2 + d dN + dN^2): exactly 0 with e at n = 1
                const V c3 = vmul(e, vfma(d, d, vfma(d, dN, dN2)));
                m4 = vadd(m4, vfma(d, c3, vfma(vmul(vconst<V>(-4.f), dN), m3n, vmul(vmul(vconst<V>(-6.f), dN2), m2))));
            }
            m3 = m3n;
        }
        if (MAXMOM >= 5) {
            const V xm = vsub(x, mean);
            cx = vfma(xm, xD, cx);
            cy = vfma(xm, yD, cy);
            m1 = vadd(m1, vmap(vmul(d, e), [](float q) { return __fsqrt_rn(q); }));
        }
    }
}

// EXACT update of one transform's moments for one channel: the reference's
// arithmetic (division by n; compiled with -fmad=false).
template <typename T, int MAXMOM>
__device__ __forceinline__ void acc_update1(T x, uint32_t nn, float xD, float yD, T &mean, T &m2, T &m3, T &m4,
                                            T &cx, T &cy, T &m1) {
    const T nT = (T)nn;
    const T d = x - mean;
    const T dN = d / nT;
    if (MAXMOM <= 1) {
        mean = mean + dN;
    } else if (MAXMOM == 2) {
        mean = mean + dN;
        m2 = m2 + d * (d - dN);
    } else {
        const T d2 = d * d;
        const T dN2 = dN * dN;
        mean = mean + dN;
        m2 = m2 + d * (d - dN);
        m3 = m3 + ((T)-3.f * dN * m2 + d * (d2 - dN2));
        if (MAXMOM >= 4) m4 = m4 + (((T)-4.f * dN * m3 - (T)6.f * dN2 * m2) + d * (d * d2 - dN * dN2));
        if (MAXMOM >= 5) {
            cx = cx + (x - mean) * (T)xD;
            cy = cy + (x - mean) * (T)yD;
            m1 = m1 + sqrt(d * (d - dN));
        }
    }
}

// One sample's update of one transform's moments (3 channels). `cur` holds
// R, G, B and, with MAXMOM >= 5, the in-pixel offsets u, v. FAST: rn_out
// receives 1/nn for the feature means.
template <typename T, bool FAST, int MAXMOM, int KIND>
__device__ __forceinline__ void acc_update(const float *cur, uint32_t nn, float lam, T (&mean)[3], T (&m2)[3],
                                           T (&m3)[3], T (&m4)[3], T (&cx)[3], T (&cy)[3], T (&m1)[3], T &rn_out) {
    if constexpr (FAST && sizeof(T) == 4) {
        const float rn = fast_rcp((float)nn);
        rn_out = rn;
        float xD = 0.f, yD = 0.f;
        if (MAXMOM >= 5) {
            xD = __fsub_rn(cur[3], 0.5f);
            yD = __fsub_rn(cur[4], 0.5f);
        }
#pragma unroll
        for (int c = 0; c < 3; c++)
            meng_fast<float, MAXMOM>(fast_transform<float, KIND>(lam, cur[c]), rn, xD, yD, mean[c], m2[c], m3[c],
                                     m4[c], cx[c], cy[c], m1[c]);
    } else {
        rn_out = T(0);
        float xD = 0.f, yD = 0.f;
        if (MAXMOM >= 5) {
            xD = cur[3] - 0.5f;
            yD = cur[4] - 0.5f;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const T x = acc_transform<T, false, KIND>(lam, (T)cur[c]);
            acc_update1<T, MAXMOM>(x, nn, xD, yD, mean[c], m2[c], m3[c], m4[c], cx[c], cy[c], m1[c]);
        }
    }
}

// Running mean of a feature channel (AddSampleM1 of a G-buffer tile). FAST:
// fm + (v - fm) / n with the reciprocal, fused; EXACT: the division.
template <typename T, bool FAST>
__device__ __forceinline__ void feat_update(float v, uint32_t nn, T rn, T &fm) {
    if constexpr (FAST && sizeof(T) == 4) {
        fm = vfma(vsub(v, fm), rn, fm);
    } else {
        const T d = (T)v - fm;
        const T dN = d / (T)nn;
        fm = fm + dN;
    }
}

template <typename T, bool FAST, int MAXMOM, int MAXF, int KIND>
__device__ __forceinline__ void acc_loop(const AccParams &P, size_t i, size_t p, int k, int cnt, uint32_t n0,
                                         float lam, T (&mean)[3], T (&m2)[3], T (&m3)[3], T (&m4)[3], T (&cx)[3],
                                         T (&cy)[3], T (&m1)[3], T (&fm)[MAXF > 0 ? MAXF : 1], bool film,
                                         FilmAcc &fa) {
    const size_t HW = P.HW;  // sample column stride
    const float *sp = P.samples + i;
    const size_t sstride = (size_t)P.NCH * HW;
    constexpr int NL = MAXMOM >= 5 ? 5 : 3;
    // The next sample's loads are issued before the current one is processed.
    float nxt[NL];
    if (cnt > 0) {
#pragma unroll
        for (int c = 0; c < NL; c++) nxt[c] = __ldg(sp + (size_t)c * HW);
    }
    for (int s = 0; s < cnt; s++) {
        float cur[NL];
#pragma unroll
        for (int c = 0; c < NL; c++) cur[c] = nxt[c];
        const float *spc = sp + (size_t)s * sstride;
        if (s + 1 < cnt) {
#pragma unroll
            for (int c = 0; c < NL; c++) nxt[c] = __ldg(spc + sstride + (size_t)c * HW);
        }
        const uint32_t nn = n0 + (uint32_t)s + 1u;
        if (film) {
            const float u = NL >= 5 ? cur[NL >= 5 ? 3 : 0] : __ldg(spc + 3 * HW);
            const float v = NL >= 5 ? cur[NL >= 5 ? 4 : 0] : __ldg(spc + 4 * HW);
            film_add(P.film, p, cur[0], cur[1], cur[2], u, v, fa);
        }
        T rn;
        acc_update<T, FAST, MAXMOM, KIND>(cur, nn, lam, mean, m2, m3, m4, cx, cy, m1, rn);
#pragma unroll
        for (int jf = 0; jf < MAXF; jf++) {
            const int g = P.featmap[k][jf];
            if (g >= 0) feat_update<T, FAST>(__ldg(spc + (size_t)(5 + g) * HW), nn, rn, fm[jf]);
        }
    }
}

template <typename T, bool FAST, int MAXMOM, int MAXF>
__global__ void __launch_bounds__(256) acc_kernel(AccParams P) {
    // sample column i, pixel p (the same unless a pixel index is given)
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = threadIdx.y;
    size_t p = i;
    bool valid = i < P.HW;
    if (valid && P.pix) {
        const int32_t q = P.pix[i];
        valid = q >= 0 && (size_t)q < P.HWs;
        p = valid ? (size_t)q : 0;
    }
    // per-pixel counts beyond the S sample planes are clamped (never read past them)
    const int cnt = valid ? (P.count ? min(max(P.count[i], 0), P.S) : P.S) : 0;
    // Every transform's thread reads n before the transform-0 thread of the same
    // pixel may write the updated count back.
    const uint32_t n0 = cnt > 0 ? (uint32_t)P.n[p] : 0u;
    __syncthreads();
    if (cnt == 0) return;  // nothing to add: the pixel's state is neither read nor written
    const size_t HW = P.HWs;  // statistics plane stride
    T *st = (T *)P.stats;
    T *gm = (T *)P.gmean;

    T mean[3], m2[3], m3[3], m4[3], cx[3], cy[3], m1[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        mean[c] = st[stat_index(k, STATER_Q_MEAN, c, HW) + p];
        m2[c] = MAXMOM >= 2 ? st[stat_index(k, STATER_Q_M2, c, HW) + p] : T(0);
        m3[c] = MAXMOM >= 3 ? st[stat_index(k, STATER_Q_M3, c, HW) + p] : T(0);
        m4[c] = MAXMOM >= 4 ? st[stat_index(k, STATER_Q_M4, c, HW) + p] : T(0);
        cx[c] = MAXMOM >= 5 ? st[stat_index(k, STATER_Q_C2X, c, HW) + p] : T(0);
        cy[c] = MAXMOM >= 5 ? st[stat_index(k, STATER_Q_C2Y, c, HW) + p] : T(0);
        m1[c] = MAXMOM >= 5 ? st[stat_index(k, STATER_Q_M1, c, HW) + p] : T(0);
    }
    T fm[MAXF > 0 ? MAXF : 1];
#pragma unroll
    for (int j = 0; j < MAXF; j++) {
        const int g = P.featmap[k][j];
        fm[j] = g >= 0 ? gm[(size_t)g * HW + p] : T(0);
    }
    const float lam = P.ts.lambda[k];
    // the film sums ride along with transform 0 (warp-uniform: k = threadIdx.y)
    const bool film = k == 0 && P.film.sum != nullptr;
    FilmAcc fa{0.f, 0.f, 0.f, 0.f};
    if (film) film_load(P.film, HW, p, fa);
    // one specialised sample loop per transform kind (warp-uniform)
    switch (P.ts.kind[k]) {
#define STATER_ACC_CASE(KD)                                                                                   \
    case KD:                                                                                                  \
        acc_loop<T, FAST, MAXMOM, MAXF, KD>(P, i, p, k, cnt, n0, lam, mean, m2, m3, m4, cx, cy, m1, fm, film, fa); \
        break;
        STATER_ACC_CASE(STATER_TK_LOG1P)
        STATER_ACC_CASE(STATER_TK_SQRT)
        STATER_ACC_CASE(STATER_TK_CBRT)
        STATER_ACC_CASE(STATER_TK_ASINH)
        STATER_ACC_CASE(STATER_TK_BOXCOX)
        default: acc_loop<T, FAST, MAXMOM, MAXF, STATER_TK_IDENTITY>(P, i, p, k, cnt, n0, lam, mean, m2, m3, m4,
                                                                     cx, cy, m1, fm, film, fa);
#undef STATER_ACC_CASE
    }
    if (film) film_store(P.film, HW, p, fa);

#pragma unroll
    for (int c = 0; c < 3; c++) {
        st[stat_index(k, STATER_Q_MEAN, c, HW) + p] = mean[c];
        if (MAXMOM >= 2) st[stat_index(k, STATER_Q_M2, c, HW) + p] = m2[c];
        if (MAXMOM >= 3) st[stat_index(k, STATER_Q_M3, c, HW) + p] = m3[c];
        if (MAXMOM >= 4) st[stat_index(k, STATER_Q_M4, c, HW) + p] = m4[c];
        if (MAXMOM >= 5) {
            st[stat_index(k, STATER_Q_C2X, c, HW) + p] = cx[c];
            st[stat_index(k, STATER_Q_C2Y, c, HW) + p] = cy[c];
            st[stat_index(k, STATER_Q_M1, c, HW) + p] = m1[c];
        }
    }
#pragma unroll
    for (int j = 0; j < MAXF; j++) {
        const int g = P.featmap[k][j];
        if (g >= 0) gm[(size_t)g * HW + p] = fm[j];
    }
    if (k == 0) P.n[p] = (int32_t)(n0 + (uint32_t)cnt);
}

inline int acc_threads_x(int K) {
    int tx = (256 / K) & ~31;
    return tx < 32 ? 32 : tx;
}

template <typename T, bool FAST, int MAXMOM, int MAXF>
cudaError_t launch_acc_mf(const AccParams &P, cudaStream_t s) {
    const int tx = acc_threads_x(P.K);
    dim3 block(tx, P.K);
    dim3 grid((unsigned)((P.HW + tx - 1) / tx));
    acc_kernel<T, FAST, MAXMOM, MAXF><<<grid, block, 0, s>>>(P);
    return cudaGetLastError();
}

template <typename T, bool FAST, int MAXMOM>
cudaError_t launch_acc_m(const AccParams &P, cudaStream_t s) {
    const int per = P.maxf;
    if (per == 0) return launch_acc_mf<T, FAST, MAXMOM, 0>(P, s);
    if (per <= 2) return launch_acc_mf<T, FAST, MAXMOM, 2>(P, s);
    if (per <= 4) return launch_acc_mf<T, FAST, MAXMOM, 4>(P, s);
    if (per <= 8) return launch_acc_mf<T, FAST, MAXMOM, 8>(P, s);
    return launch_acc_mf<T, FAST, MAXMOM, 16>(P, s);
}

template <typename T, bool FAST>
cudaError_t launch_acc(const AccParams &P, int max_moment, cudaStream_t s) {
    switch (max_moment) {
        case 1: return launch_acc_m<T, FAST, 1>(P, s);
        case 2: return launch_acc_m<T, FAST, 2>(P, s);
        case 3: return launch_acc_m<T, FAST, 3>(P, s);
        case 4: return launch_acc_m<T, FAST, 4>(P, s);
        default: return launch_acc_m<T, FAST, 5>(P, s);
    }
}

}  // namespace stater
