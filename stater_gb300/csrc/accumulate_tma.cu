// FP32 accumulation fed by the Tensor Memory Accelerator.
//
// The sample planes [S][5+G][HW] are viewed as a 2-D tensor of S*(5+G) rows by
// HW columns. A CTA owns kPx = 64 consecutive sample columns; one producer
// thread streams stages of kSB samples x (5+G) channels x kPx columns (one or
// a few boxes of whole samples) into a kStages-deep ring in shared memory
// with cp.async.bulk.tensor, completing on per-stage mbarriers. One consumer
// warp per transform reads the stages (the transform-0 warp also adds the film
// sums; which warp keeps which transform comes from the host's plan, which
// spreads the costly transforms over the SM's four schedulers); each lane owns two neighbouring columns and keeps both pixels'
// moments in the halves of 64-bit registers, updated by the packed FP32
// instructions (one issue per pair) with 8-byte shared-memory loads. The
// update is the same operation sequence as the plain FAST kernel's (the
// value-type-generic meng_fast / fast_transform), so both give the same bits.
// The samples of one column beyond its neighbour's count go through the
// scalar form.
//
// Every sample byte crosses HBM once, and kStages boxes per CTA are always in
// flight, independent of the consumers' register use.
//
// Every wait is bounded. A pipeline wait that gives up records kErrTimeout in
// the library's device error word (reported by stater_synchronize), releases
// what it holds and lets the CTA finish. Before it exits, the producer always
// waits for the last boxes it issued to land (on success as well: consumers
// that gave up may already have left), by the full kWaitLimit; if that wait
// gives up too it records kErrDrain.
#include <cuda.h>

#include "acc_kernels.cuh"
#include "tma_common.cuh"

namespace stater {
namespace {

using namespace tma;

#ifndef STATER_TMA_SAMPLES_PER_STAGE
#define STATER_TMA_SAMPLES_PER_STAGE 12
#endif
#ifndef STATER_TMA_STAGES
#define STATER_TMA_STAGES 2
#endif
#ifndef STATER_TMA_MAX_REGS
#define STATER_TMA_MAX_REGS 96
#endif
#ifndef STATER_TMA_UNROLL
#define STATER_TMA_UNROLL 1
#endif
constexpr int kPx = 64;                            // sample columns per CTA (two per consumer lane)
constexpr int kSB = STATER_TMA_SAMPLES_PER_STAGE;  // samples per stage
constexpr int kStages = STATER_TMA_STAGES;         // ring depth
constexpr int kUnroll = STATER_TMA_UNROLL;         // unroll of the packed loop (1: unrolling measured slower)

struct TmaAccParams {
    AccParams P;
    int *err;
    int spb;              // samples per TMA box (a divisor of kSB; a box has at most 256 rows)
    uint32_t wait_limit;  // polls of a pipeline wait
    int stall;            // 1: the producer issues nothing (test hook: the consumers' waits run out)
};

// Film sums of a column pair (low half: the lane's first column).
struct Film2 {
    F2 s0, s1, s2, w;
};

// Moments, feature means and film sums of a lane's two columns.
template <int MAXF>
struct PairState {
    F2 mean[3], m2[3], m3[3], m4[3], cx[3], cy[3], m1[3];
    F2 fm[MAXF > 0 ? MAXF : 1];
    Film2 fa;
};

// film_add of two pixels' samples, element for element the same rounding,
// except the weight: it gains exactly 1 per sample (integers below 2^24), so
// the caller adds the number of samples once per stage.
// The luminance (separately rounded products) is taken element-wise: packed,
// its multiplies could be fused into the adds.
__device__ __forceinline__ float film_lum(float r, float g, float b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(0.212671f, r), __fmul_rn(0.715160f, g)), __fmul_rn(0.072169f, b));
}
__device__ __forceinline__ void film_add2(const FilmTarget &F, size_t pa, size_t pb, F2 r, F2 g, F2 b, F2 u, F2 v,
                                          Film2 &a) {
    float la, lb;
    {
        float ra, rb, ga, gb, ba, bb;
        f2_unpack(r, ra, rb);
        f2_unpack(g, ga, gb);
        f2_unpack(b, ba, bb);
        la = film_lum(ra, ga, ba);
        lb = film_lum(rb, gb, bb);
    }
    if (la > F.max_lum || lb > F.max_lum) {
        float ra, rb, ga, gb, ba, bb;
        f2_unpack(r, ra, rb);
        f2_unpack(g, ga, gb);
        f2_unpack(b, ba, bb);
        if (la > F.max_lum) {
            const float f = __fdiv_rn(F.max_lum, la);
            ra = __fmul_rn(ra, f);
            ga = __fmul_rn(ga, f);
            ba = __fmul_rn(ba, f);
        }
        if (lb > F.max_lum) {
            const float f = __fdiv_rn(F.max_lum, lb);
            rb = __fmul_rn(rb, f);
            gb = __fmul_rn(gb, f);
            bb = __fmul_rn(bb, f);
        }
        r = f2_pack(ra, rb);
        g = f2_pack(ga, gb);
        b = f2_pack(ba, bb);
    }
    a.s0 = vadd(a.s0, r);
    a.s1 = vadd(a.s1, g);
    a.s2 = vadd(a.s2, b);
    float ua, ub, va, vb;
    f2_unpack(u, ua, ub);
    f2_unpack(v, va, vb);
    const bool ea = ua == 0.0f || ua == 1.0f || va == 0.0f || va == 1.0f;
    const bool eb = ub == 0.0f || ub == 1.0f || vb == 0.0f || vb == 1.0f;
    if (ea || eb) {
        float ra, rb, ga, gb, ba, bb;
        f2_unpack(r, ra, rb);
        f2_unpack(g, ga, gb);
        f2_unpack(b, ba, bb);
        if (ea) film_spill(F, pa, ra, ga, ba, ua, va);
        if (eb) film_spill(F, pb, rb, gb, bb, ub, vb);
    }
}

// One sample of one column of the pair (H: 0 the lane's first column, 1 its
// second), in the scalar form, with n = nn: the operations of acc_update's
// FAST form, one channel at a time (fewer values live than unpacking the
// whole state first). The column is a template argument: a runtime index into
// the lane's per-column arrays would place them in local memory.
template <int MAXMOM, int MAXF, int KIND, int H>
__device__ __forceinline__ void sample_one(const AccParams &P, const float *row, uint32_t nn,
                                           const int (&foff)[MAXF > 0 ? MAXF : 1], size_t p, float lam, bool film,
                                           PairState<MAXF> &S) {
    auto get = [](F2 x) { return f2_get<H>(x); };
    auto put = [](F2 &x, float v) { f2_set<H>(x, v); };
    row += H;
    if (film) {
        FilmAcc fa{get(S.fa.s0), get(S.fa.s1), get(S.fa.s2), get(S.fa.w)};
        film_add(P.film, p, row[0], row[kPx], row[2 * kPx], row[3 * kPx], row[4 * kPx], fa);
        put(S.fa.s0, fa.s0);
        put(S.fa.s1, fa.s1);
        put(S.fa.s2, fa.s2);
        put(S.fa.w, fa.w);
    }
    const float rn = fast_rcp((float)nn);
    float xD = 0.f, yD = 0.f;
    if (MAXMOM >= 5) {
        xD = __fsub_rn(row[3 * kPx], 0.5f);
        yD = __fsub_rn(row[4 * kPx], 0.5f);
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float mean = get(S.mean[c]), m2 = get(S.m2[c]), m3 = get(S.m3[c]), m4 = get(S.m4[c]);
        float cx = get(S.cx[c]), cy = get(S.cy[c]), m1 = get(S.m1[c]);
        meng_fast<float, MAXMOM>(fast_transform<float, KIND>(lam, row[c * kPx]), rn, xD, yD, mean, m2, m3, m4, cx,
                                 cy, m1);
        put(S.mean[c], mean);
        if (MAXMOM >= 2) put(S.m2[c], m2);
        if (MAXMOM >= 3) put(S.m3[c], m3);
        if (MAXMOM >= 4) put(S.m4[c], m4);
        if (MAXMOM >= 5) {
            put(S.cx[c], cx);
            put(S.cy[c], cy);
            put(S.m1[c], m1);
        }
    }
#pragma unroll
    for (int jf = 0; jf < MAXF; jf++) {
        if (foff[jf] >= 0) {
            float f = get(S.fm[jf]);
            feat_update<float, true>(row[foff[jf]], nn, rn, f);
            put(S.fm[jf], f);
        }
    }
}

// The consumer loop of one transform kind (the kind is hoisted out of the
// sample loop: one specialised loop per kind, chosen once per warp; FILM: the
// warp also adds the film sums). Returns false when a wait gave up.
template <int MAXMOM, int MAXF, int KIND, bool FILM>
__device__ __forceinline__ bool tma_consume(const AccParams &P, uint32_t wait_limit, const float *stages,
                                            int stage_floats, uint64_t *full, uint64_t *empty, int nchunks,
                                            const int (&cnt)[2],
                                            const uint32_t (&n0)[2], const size_t (&p)[2],
                                            const int (&foff)[MAXF > 0 ? MAXF : 1], int lane, float lam,
                                            PairState<MAXF> &S) {
    const int NCH = P.NCH;
    constexpr int NL = MAXMOM >= 5 ? 5 : 3;
    for (int c = 0; c < nchunks; c++) {
        const int sidx = c % kStages;
        if (!mbar_wait(&full[sidx], (c / kStages) & 1, wait_limit)) return false;
        const float *stage = stages + (size_t)sidx * stage_floats + 2 * lane;
        const int ja = min(kSB, max(0, cnt[0] - c * kSB));
        const int jb = min(kSB, max(0, cnt[1] - c * kSB));
        const int jlo = min(ja, jb);
        if (jlo > 0) {
            // both columns: n as floats (exact below 2^24), advanced by one per sample
            F2 nf = f2_pack((float)(n0[0] + (uint32_t)(c * kSB)), (float)(n0[1] + (uint32_t)(c * kSB)));
#pragma unroll kUnroll
            for (int j = 0; j < jlo; j++) {
                const float *row = stage + (size_t)j * NCH * kPx;
                F2 cur[NL];
#pragma unroll
                for (int q = 0; q < NL; q++) cur[q] = f2_load(row + q * kPx);
                nf = vadd(nf, vconst<F2>(1.f));
                const F2 rn = vmap(nf, fast_rcp);
                // in-pixel offsets u, v: loaded with the radiance for M5, else only for the film
                F2 u = vconst<F2>(0.f), v = vconst<F2>(0.f), xD = vconst<F2>(0.f), yD = vconst<F2>(0.f);
                if constexpr (MAXMOM >= 5) {
                    u = cur[NL - 2];
                    v = cur[NL - 1];
                    xD = vsub(u, vconst<F2>(0.5f));
                    yD = vsub(v, vconst<F2>(0.5f));
                } else if constexpr (FILM) {
                    u = f2_load(row + 3 * kPx);
                    v = f2_load(row + 4 * kPx);
                }
                if constexpr (FILM) film_add2(P.film, p[0], p[1], cur[0], cur[1], cur[2], u, v, S.fa);
#pragma unroll
                for (int ch = 0; ch < 3; ch++)
                    meng_fast<F2, MAXMOM>(fast_transform<F2, KIND>(lam, cur[ch]), rn, xD, yD, S.mean[ch], S.m2[ch],
                                          S.m3[ch], S.m4[ch], S.cx[ch], S.cy[ch], S.m1[ch]);
#pragma unroll
                for (int jf = 0; jf < MAXF; jf++)
                    if (foff[jf] >= 0) S.fm[jf] = vfma(vsub(f2_load(row + foff[jf]), S.fm[jf]), rn, S.fm[jf]);
            }
            if constexpr (FILM) S.fa.w = vadd(S.fa.w, vconst<F2>((float)jlo));
        }
        // the column with more samples in this stage takes the rest alone
        if (ja > jb) {
            for (int j = jlo; j < ja; j++)
                sample_one<MAXMOM, MAXF, KIND, 0>(P, stage + (size_t)j * NCH * kPx, n0[0] + (uint32_t)(c * kSB + j) + 1u,
                                                  foff, p[0], lam, FILM, S);
        } else if (jb > ja) {
            for (int j = jlo; j < jb; j++)
                sample_one<MAXMOM, MAXF, KIND, 1>(P, stage + (size_t)j * NCH * kPx, n0[1] + (uint32_t)(c * kSB + j) + 1u,
                                                  foff, p[1], lam, FILM, S);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sidx]);
    }
    return true;
}

// Registers per thread: 96 keeps 3 CTAs of K = 5 (6 warps each, the producer
// included) resident per SM, as the shared-memory ring does; measured on
// GB300, a bound of 104 or 112 already leaves only 2 resident and the kernel
// runs about 14% slower: the few values spilled at 96 cost less than the lost
// CTA. The larger states (4 or more moments, 8 or more
// feature channels per transform) get 224, one CTA per SM. The bound is given
// per thread rather than as resident blocks of the largest CTA (288 threads).
constexpr int acc_tma_max_regs(int maxmom, int maxf) {
    return (maxmom >= 4 || maxf >= 8) ? 224 : STATER_TMA_MAX_REGS;
}

template <int MAXMOM, int MAXF>
__global__ void __launch_bounds__(32 * STATER_MAX_TRANSFORMS + 32) __maxnreg__(acc_tma_max_regs(MAXMOM, MAXF))
    acc_tma_kernel(const __grid_constant__ CUtensorMap map, TmaAccParams TP) {
    const AccParams &P = TP.P;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages];
    __shared__ int s_maxcnt;
    const int NCH = P.NCH;
    const int stage_floats = kSB * NCH * kPx;
    float *stages = reinterpret_cast<float *>(smem_raw);
    const int nconsumer_warps = P.K;  // one warp per transform
    const int tid = threadIdx.x;
    const int warp = tid / 32, lane = tid % 32;
    const bool producer = warp == P.K;
    const size_t c0 = (size_t)blockIdx.x * kPx;  // first sample column of the CTA
    const size_t HW = P.HWs;                     // statistics plane stride

    if (tid == 0) {
        for (int i = 0; i < kStages; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], nconsumer_warps);
        }
        s_maxcnt = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // the lane's sample columns i = c0 + 2 lane + h and their pixels p (the same
    // unless a pixel index is given); a column without samples neither reads
    // nor writes its pixel's state
    size_t p[2];
    int cnt[2];
    uint32_t n0[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const size_t i = c0 + 2 * lane + h;
        p[h] = i;
        bool inr = !producer && i < P.HW;
        if (inr && P.pix) {
            const int32_t q = P.pix[i];
            inr = q >= 0 && (size_t)q < P.HWs;
            p[h] = inr ? (size_t)q : 0;
        }
        cnt[h] = inr ? (P.count ? min(max(P.count[i], 0), P.S) : P.S) : 0;
        // Every transform's thread reads n before the transform-0 thread of the
        // same pixel may write the updated count back (the barrier below orders them).
        n0[h] = cnt[h] > 0 ? (uint32_t)P.n[p[h]] : 0u;
    }
    // Number of samples this CTA needs: the largest count among its columns.
    if (warp == 0) {
        int c = max(cnt[0], cnt[1]);
        for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
        if (lane == 0) s_maxcnt = c;
    }
    __syncthreads();
    const int maxcnt = s_maxcnt;
    const int nchunks = (maxcnt + kSB - 1) / kSB;

    if (producer) {
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)stage_floats * 4u;
            int issued = 0;
            bool ok = true;
            for (int c = 0; c < nchunks && ok && !TP.stall; c++) {
                const int st = c % kStages;
                if (c >= kStages) ok = mbar_wait(&empty[st], ((c / kStages) - 1) & 1, TP.wait_limit);
                if (!ok) break;
                mbar_arrive_expect_tx(&full[st], bytes);
                for (int b = 0; b < kSB; b += TP.spb)
                    tma_load_2d(stages + (size_t)st * stage_floats + (size_t)b * NCH * kPx, &map, (int)c0,
                                (c * kSB + b) * NCH, &full[st]);
                issued = c + 1;
            }
            if (!ok) atomicOr(TP.err, kErrTimeout);
            // the last kStages boxes issued (each on its own stage, at its final
            // phase) must have landed before the CTA may end
            bool drained = true;
            for (int c = max(0, issued - kStages); c < issued; c++)
                drained = mbar_wait(&full[c % kStages], (c / kStages) & 1) && drained;
            if (!drained) atomicOr(TP.err, kErrDrain);
        }
        return;
    }

    // consumers: warp = the plan's transform P.wt[warp], lane = column pair
    const int k = P.wt[warp];
    float *st = (float *)P.stats;
    float *gm = (float *)P.gmean;
    const bool va = cnt[0] > 0, vb = cnt[1] > 0;
    PairState<MAXF> S;
    auto ld2 = [&](const float *base) {
        return f2_pack(va ? base[p[0]] : 0.f, vb ? base[p[1]] : 0.f);
    };
#pragma unroll
    for (int c = 0; c < 3; c++) {
        S.mean[c] = ld2(st + stat_index(k, STATER_Q_MEAN, c, HW));
        S.m2[c] = MAXMOM >= 2 ? ld2(st + stat_index(k, STATER_Q_M2, c, HW)) : vconst<F2>(0.f);
        S.m3[c] = MAXMOM >= 3 ? ld2(st + stat_index(k, STATER_Q_M3, c, HW)) : vconst<F2>(0.f);
        S.m4[c] = MAXMOM >= 4 ? ld2(st + stat_index(k, STATER_Q_M4, c, HW)) : vconst<F2>(0.f);
        S.cx[c] = MAXMOM >= 5 ? ld2(st + stat_index(k, STATER_Q_C2X, c, HW)) : vconst<F2>(0.f);
        S.cy[c] = MAXMOM >= 5 ? ld2(st + stat_index(k, STATER_Q_C2Y, c, HW)) : vconst<F2>(0.f);
        S.m1[c] = MAXMOM >= 5 ? ld2(st + stat_index(k, STATER_Q_M1, c, HW)) : vconst<F2>(0.f);
    }
    // feature channels this transform's warp keeps: their row offsets in a stage
    int foff[MAXF > 0 ? MAXF : 1];
#pragma unroll
    for (int j = 0; j < MAXF; j++) {
        const int g = P.featmap[k][j];
        foff[j] = g >= 0 ? (5 + g) * kPx : -1;
        S.fm[j] = g >= 0 ? ld2(gm + (size_t)g * HW) : vconst<F2>(0.f);
    }
    const int kind = P.ts.kind[k];
    const float lam = P.ts.lambda[k];
    // film sums ride along with the transform-0 warp
    const bool film = k == 0 && P.film.sum != nullptr;
    S.fa = Film2{vconst<F2>(0.f), vconst<F2>(0.f), vconst<F2>(0.f), vconst<F2>(0.f)};
    if (film) {
        FilmAcc a{0.f, 0.f, 0.f, 0.f}, b{0.f, 0.f, 0.f, 0.f};
        if (va) film_load(P.film, HW, p[0], a);
        if (vb) film_load(P.film, HW, p[1], b);
        S.fa = Film2{f2_pack(a.s0, b.s0), f2_pack(a.s1, b.s1), f2_pack(a.s2, b.s2), f2_pack(a.w, b.w)};
    }
    bool ok;
    switch (kind) {
#define STATER_TMA_CASE(KD)                                                                                           \
    case KD:                                                                                                          \
        ok = tma_consume<MAXMOM, MAXF, KD, false>(P, TP.wait_limit, stages, stage_floats, full, empty, nchunks, cnt, n0, \
                                                  p, foff, lane, lam, S);                                              \
        break;
        STATER_TMA_CASE(STATER_TK_LOG1P)
        STATER_TMA_CASE(STATER_TK_SQRT)
        STATER_TMA_CASE(STATER_TK_CBRT)
        STATER_TMA_CASE(STATER_TK_ASINH)
        STATER_TMA_CASE(STATER_TK_BOXCOX)
#undef STATER_TMA_CASE
        default:
            ok = film ? tma_consume<MAXMOM, MAXF, STATER_TK_IDENTITY, true>(P, TP.wait_limit, stages, stage_floats, full,
                                                                            empty, nchunks, cnt, n0, p, foff, lane,
                                                                            lam, S)
                      : tma_consume<MAXMOM, MAXF, STATER_TK_IDENTITY, false>(P, TP.wait_limit, stages, stage_floats,
                                                                             full, empty, nchunks, cnt, n0, p, foff,
                                                                             lane, lam, S);
    }
    if (!ok) {
        if (lane == 0) atomicOr(TP.err, kErrTimeout);
        return;
    }
    auto st2 = [&](float *base, F2 v) {
        float lo, hi;
        f2_unpack(v, lo, hi);
        if (va) base[p[0]] = lo;
        if (vb) base[p[1]] = hi;
    };
#pragma unroll
    for (int c = 0; c < 3; c++) {
        st2(st + stat_index(k, STATER_Q_MEAN, c, HW), S.mean[c]);
        if (MAXMOM >= 2) st2(st + stat_index(k, STATER_Q_M2, c, HW), S.m2[c]);
        if (MAXMOM >= 3) st2(st + stat_index(k, STATER_Q_M3, c, HW), S.m3[c]);
        if (MAXMOM >= 4) st2(st + stat_index(k, STATER_Q_M4, c, HW), S.m4[c]);
        if (MAXMOM >= 5) {
            st2(st + stat_index(k, STATER_Q_C2X, c, HW), S.cx[c]);
            st2(st + stat_index(k, STATER_Q_C2Y, c, HW), S.cy[c]);
            st2(st + stat_index(k, STATER_Q_M1, c, HW), S.m1[c]);
        }
    }
#pragma unroll
    for (int j = 0; j < MAXF; j++)
        if (foff[j] >= 0) st2(gm + (size_t)P.featmap[k][j] * HW, S.fm[j]);
    if (film) {
        float s0[2], s1[2], s2[2], w[2];
        f2_unpack(S.fa.s0, s0[0], s0[1]);
        f2_unpack(S.fa.s1, s1[0], s1[1]);
        f2_unpack(S.fa.s2, s2[0], s2[1]);
        f2_unpack(S.fa.w, w[0], w[1]);
        if (va) film_store(P.film, HW, p[0], FilmAcc{s0[0], s1[0], s2[0], w[0]});
        if (vb) film_store(P.film, HW, p[1], FilmAcc{s0[1], s1[1], s2[1], w[1]});
    }
    if (k == 0) {
        if (va) P.n[p[0]] = (int32_t)(n0[0] + (uint32_t)cnt[0]);
        if (vb) P.n[p[1]] = (int32_t)(n0[1] + (uint32_t)cnt[1]);
    }
}

template <int MAXMOM, int MAXF>
cudaError_t launch_tma_mf(const CUtensorMap &map, const TmaAccParams &TP, cudaStream_t s) {
    const size_t smem = (size_t)kStages * kSB * TP.P.NCH * kPx * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(acc_tma_kernel<MAXMOM, MAXF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((TP.P.HW + kPx - 1) / kPx);
    acc_tma_kernel<MAXMOM, MAXF><<<grid, 32 * TP.P.K + 32, smem, s>>>(map, TP);
    return cudaGetLastError();
}

template <int MAXMOM>
cudaError_t launch_tma_m(const CUtensorMap &map, const TmaAccParams &TP, cudaStream_t s) {
    const int per = TP.P.maxf;
    if (per == 0) return launch_tma_mf<MAXMOM, 0>(map, TP, s);
    if (per <= 2) return launch_tma_mf<MAXMOM, 2>(map, TP, s);
    if (per <= 4) return launch_tma_mf<MAXMOM, 4>(map, TP, s);
    if (per <= 8) return launch_tma_mf<MAXMOM, 8>(map, TP, s);
    return launch_tma_mf<MAXMOM, 16>(map, TP, s);
}

}  // namespace

// Returns cudaErrorNotSupported when the sample planes do not meet the TMA
// rules (row pitch a multiple of 16 bytes, 16-byte aligned base), the stages
// do not fit in shared memory, or the film is asked for with a transform 0
// other than the identity: the caller then uses the plain kernel.
cudaError_t launch_acc_tma_f32(const AccParams &P, int max_moment, cudaStream_t s) {
    if ((P.HW % 4) != 0 || ((uintptr_t)P.samples % 16) != 0) return cudaErrorNotSupported;
    // the film sums ride along with an identity transform 0 only
    if (P.film.sum && P.ts.kind[0] != STATER_TK_IDENTITY) return cudaErrorNotSupported;
    const size_t smem = (size_t)kStages * kSB * P.NCH * kPx * sizeof(float);
    if (smem > 200 * 1024) return cudaErrorNotSupported;
    // a stage is loaded as kSB / spb boxes of spb whole samples, at most 256 rows each
    int spb = kSB;
    while (spb * P.NCH > 256 || kSB % spb != 0) spb--;
    if (spb < 1) return cudaErrorNotSupported;
    const uint64_t rows = (uint64_t)P.S * P.NCH;
    CUtensorMap map;
    if (!encode_tensor_map_2d_f32(&map, P.samples, P.HW, rows, kPx, (uint32_t)(spb * P.NCH)))
        return cudaErrorNotSupported;
    TmaAccParams TP;
    TP.P = P;
    TP.spb = spb;
    TP.err = device_error_word();
    if (!TP.err) return cudaErrorMemoryAllocation;
    TP.wait_limit = pipeline_wait_limit();
    TP.stall = pipeline_stall();
    switch (max_moment) {
        case 1: return launch_tma_m<1>(map, TP, s);
        case 2: return launch_tma_m<2>(map, TP, s);
        case 3: return launch_tma_m<3>(map, TP, s);
        case 4: return launch_tma_m<4>(map, TP, s);
        default: return launch_tma_m<5>(map, TP, s);
    }
}

}  // namespace stater
