// FP32 accumulation fed by the Tensor Memory Accelerator.
//
// The sample planes [S][5+G][HW] are viewed as a 2-D tensor of S*(5+G) rows by
// HW columns. A CTA owns kPx consecutive pixels; one producer thread streams
// boxes of kSB samples x (5+G) channels x kPx pixels into a kStages-deep ring
// of shared-memory stages with cp.async.bulk.tensor, completing on per-stage
// mbarriers; kPx x K consumer threads (one per pixel and transform, as in the
// plain kernel) read the stage, update their moments in registers and release
// the stage. Every sample byte crosses HBM once and kStages boxes per CTA are
// always in flight, independent of the consumers' register use.
//
// Every wait is bounded. A wait that gives up records kErrTimeout in the
// library's device error word (reported by stater_synchronize), releases what
// it holds and lets the CTA finish; the producer first waits, again bounded,
// for the boxes it has issued.
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
constexpr int kPx = 32;                                // pixels per CTA (one warp-wide row of consumers per transform)
constexpr int kSB = STATER_TMA_SAMPLES_PER_STAGE;      // samples per stage
constexpr int kStages = STATER_TMA_STAGES;             // ring depth

struct TmaAccParams {
    AccParams P;
    int *err;
};

// The consumer loop of one transform kind (the kind is hoisted out of the
// sample loop: one specialised loop per kind, chosen once per warp). Returns
// false when a wait gave up.
template <int MAXMOM, int MAXF, int KIND>
__device__ __forceinline__ bool tma_consume(const AccParams &P, const float *stages, int stage_floats, uint64_t *full,
                                            uint64_t *empty, int nchunks, int cnt, uint32_t n0, int k, int lane,
                                            size_t p, float lam, float (&mean)[3], float (&m2)[3], float (&m3)[3],
                                            float (&m4)[3], float (&cx)[3], float (&cy)[3], float (&m1)[3],
                                            float (&fm)[MAXF > 0 ? MAXF : 1], bool film, FilmAcc &fa) {
    const int NCH = P.NCH;
    constexpr int NL = MAXMOM >= 5 ? 5 : 3;
    for (int c = 0; c < nchunks; c++) {
        const int sidx = c % kStages;
        if (!mbar_wait(&full[sidx], (c / kStages) & 1)) return false;
        const float *stage = stages + (size_t)sidx * stage_floats;
        const int jn = min(kSB, cnt - c * kSB);
        int j0 = 0;
        if (c == 0 && n0 == 0u && jn > 0) {
            // the pixel's first sample: mean = x, the feature means take the sample
            const float *row = stage + lane;
            float cur[NL];
#pragma unroll
            for (int q = 0; q < NL; q++) cur[q] = row[q * kPx];
            if (film) film_add(P.film, p, cur[0], cur[1], cur[2], row[3 * kPx], row[4 * kPx], fa);
            acc_first<KIND>(cur, lam, mean);
#pragma unroll
            for (int jf = 0; jf < MAXF; jf++) {
                const int g = P.featmap[k][jf];
                if (g >= 0) feat_update<float, true>(row[(5 + g) * kPx], 1u, 1.f, fm[jf]);
            }
            j0 = 1;
        }
        for (int j = j0; j < jn; j++) {
            const float *row = stage + (size_t)j * NCH * kPx + lane;
            float cur[NL];
#pragma unroll
            for (int q = 0; q < NL; q++) cur[q] = row[q * kPx];
            const uint32_t nn = n0 + (uint32_t)(c * kSB + j) + 1u;
            if (film) film_add(P.film, p, cur[0], cur[1], cur[2], row[3 * kPx], row[4 * kPx], fa);
            float rn;
            acc_update<float, true, MAXMOM, KIND, true>(cur, nn, lam, mean, m2, m3, m4, cx, cy, m1, rn);
#pragma unroll
            for (int jf = 0; jf < MAXF; jf++) {
                const int g = P.featmap[k][jf];
                if (g >= 0) feat_update<float, true>(row[(5 + g) * kPx], nn, rn, fm[jf]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sidx]);
    }
    return true;
}

template <int MAXMOM, int MAXF>
__global__ void __launch_bounds__(kPx *STATER_MAX_TRANSFORMS + 32)
    acc_tma_kernel(const __grid_constant__ CUtensorMap map, TmaAccParams TP) {
    const AccParams &P = TP.P;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages];
    __shared__ int s_maxcnt;
    const int NCH = P.NCH;
    const int stage_floats = kSB * NCH * kPx;
    float *stages = reinterpret_cast<float *>(smem_raw);
    const int nconsumer_warps = P.K;  // kPx == 32: one warp per transform
    const int tid = threadIdx.x;
    const int warp = tid / 32, lane = tid % 32;
    const bool producer = warp == P.K;
    const size_t p0 = (size_t)blockIdx.x * kPx;  // first sample column of the CTA
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
    // sample column i, pixel p (the same unless a pixel index is given); a
    // column without samples neither reads nor writes its pixel's state
    const size_t i = p0 + lane;
    size_t p = i;
    bool inr = !producer && i < P.HW;
    if (inr && P.pix) {
        const int32_t q = P.pix[i];
        inr = q >= 0 && (size_t)q < P.HWs;
        p = inr ? (size_t)q : 0;
    }
    const int cnt = inr ? (P.count ? min(max(P.count[i], 0), P.S) : P.S) : 0;
    const bool valid = cnt > 0;
    // Every transform's thread reads n before the transform-0 thread of the same
    // pixel may write the updated count back (the barrier below orders them).
    const uint32_t n0 = valid ? (uint32_t)P.n[p] : 0u;
    // Number of samples this CTA needs: the largest count among its pixels.
    if (warp == 0) {
        int c = cnt;
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
            for (int c = 0; c < nchunks && ok; c++) {
                const int st = c % kStages;
                if (c >= kStages) ok = mbar_wait(&empty[st], ((c / kStages) - 1) & 1);
                if (!ok) break;
                mbar_arrive_expect_tx(&full[st], bytes);
                tma_load_2d(stages + (size_t)st * stage_floats, &map, (int)p0, c * kSB * NCH, &full[st]);
                issued = c + 1;
            }
            if (!ok) {
                atomicExch(TP.err, kErrTimeout);
                // wait (bounded) for the boxes still in flight before leaving
                for (int c = max(0, issued - kStages); c < issued; c++) mbar_wait(&full[c % kStages], (c / kStages) & 1);
            }
        }
        return;
    }

    // consumers: thread (pixel, transform)
    const int k = warp;
    float *st = (float *)P.stats;
    float *gm = (float *)P.gmean;
    float mean[3], m2[3], m3[3], m4[3], cx[3], cy[3], m1[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        mean[c] = valid ? st[stat_index(k, STATER_Q_MEAN, c, HW) + p] : 0.f;
        m2[c] = (MAXMOM >= 2 && valid) ? st[stat_index(k, STATER_Q_M2, c, HW) + p] : 0.f;
        m3[c] = (MAXMOM >= 3 && valid) ? st[stat_index(k, STATER_Q_M3, c, HW) + p] : 0.f;
        m4[c] = (MAXMOM >= 4 && valid) ? st[stat_index(k, STATER_Q_M4, c, HW) + p] : 0.f;
        cx[c] = (MAXMOM >= 5 && valid) ? st[stat_index(k, STATER_Q_C2X, c, HW) + p] : 0.f;
        cy[c] = (MAXMOM >= 5 && valid) ? st[stat_index(k, STATER_Q_C2Y, c, HW) + p] : 0.f;
        m1[c] = (MAXMOM >= 5 && valid) ? st[stat_index(k, STATER_Q_M1, c, HW) + p] : 0.f;
    }
    float fm[MAXF > 0 ? MAXF : 1];
#pragma unroll
    for (int j = 0; j < MAXF; j++) {
        const int g = P.featmap[k][j];
        fm[j] = (g >= 0 && valid) ? gm[(size_t)g * HW + p] : 0.f;
    }
    const int kind = P.ts.kind[k];
    const float lam = P.ts.lambda[k];
    // film sums ride along with the transform-0 warp
    const bool film = k == 0 && valid && P.film.sum != nullptr;
    FilmAcc fa{0.f, 0.f, 0.f, 0.f};
    if (film) film_load(P.film, HW, p, fa);
    bool ok;
    switch (kind) {
#define STATER_TMA_CASE(KD)                                                                                      \
    case KD:                                                                                                     \
        ok = tma_consume<MAXMOM, MAXF, KD>(P, stages, stage_floats, full, empty, nchunks, cnt, n0, k, lane, p, lam, \
                                           mean, m2, m3, m4, cx, cy, m1, fm, film, fa);                            \
        break;
        STATER_TMA_CASE(STATER_TK_LOG1P)
        STATER_TMA_CASE(STATER_TK_SQRT)
        STATER_TMA_CASE(STATER_TK_CBRT)
        STATER_TMA_CASE(STATER_TK_ASINH)
        STATER_TMA_CASE(STATER_TK_BOXCOX)
        default:
            ok = tma_consume<MAXMOM, MAXF, STATER_TK_IDENTITY>(P, stages, stage_floats, full, empty, nchunks, cnt, n0,
                                                               k, lane, p, lam, mean, m2, m3, m4, cx, cy, m1, fm,
                                                               film, fa);
#undef STATER_TMA_CASE
    }
    if (!ok) {
        if (lane == 0) atomicExch(TP.err, kErrTimeout);
        return;
    }
    if (!valid) return;
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
    if (film) film_store(P.film, HW, p, fa);
    if (k == 0) P.n[p] = (int32_t)(n0 + (uint32_t)cnt);
}

template <int MAXMOM, int MAXF>
cudaError_t launch_tma_mf(const CUtensorMap &map, const TmaAccParams &TP, cudaStream_t s) {
    const size_t smem = (size_t)kStages * kSB * TP.P.NCH * kPx * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(acc_tma_kernel<MAXMOM, MAXF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((TP.P.HW + kPx - 1) / kPx);
    acc_tma_kernel<MAXMOM, MAXF><<<grid, kPx * TP.P.K + 32, smem, s>>>(map, TP);
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
// rules (row pitch a multiple of 16 bytes, 16-byte aligned base): the caller
// then uses the plain kernel.
cudaError_t launch_acc_tma_f32(const AccParams &P, int max_moment, cudaStream_t s) {
    if ((P.HW % 4) != 0 || ((uintptr_t)P.samples % 16) != 0) return cudaErrorNotSupported;
    const size_t smem = (size_t)kStages * kSB * P.NCH * kPx * sizeof(float);
    if (smem > 200 * 1024) return cudaErrorNotSupported;
    const uint64_t rows = (uint64_t)P.S * P.NCH;
    CUtensorMap map;
    if (!encode_tensor_map_2d_f32(&map, P.samples, P.HW, rows, kPx, (uint32_t)(kSB * P.NCH)))
        return cudaErrorNotSupported;
    TmaAccParams TP;
    TP.P = P;
    TP.err = device_error_word();
    if (!TP.err) return cudaErrorMemoryAllocation;
    switch (max_moment) {
        case 1: return launch_tma_m<1>(map, TP, s);
        case 2: return launch_tma_m<2>(map, TP, s);
        case 3: return launch_tma_m<3>(map, TP, s);
        case 4: return launch_tma_m<4>(map, TP, s);
        default: return launch_tma_m<5>(map, TP, s);
    }
}

}  // namespace stater
