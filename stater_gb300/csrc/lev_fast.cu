// FP32 LEV accumulation with blocked compensation: a thread sums 8 samples'
// pivot-shifted cross-products in plain FP32 registers, then folds the block
// into a compensated (hi, lo) pair per sum kept in shared memory
// (hi + lo is the running total; lo carries what the FP32 addition of hi lost).
// kParts threads (two) share a pixel, each keeping its share of the sums: the
// per-thread state stays small enough for many resident warps, while each
// thread's loads and pivot shifts serve half the sums (four parts: 11.3 ms,
// two: 9.2 ms, one: 12.3 ms at 1080p / 512 spp; the sums are the same bits).
// State planes: hi [NS][HW] followed by lo [NS][HW]; n and the pivot live in
// the hi planes. The FP64 solve (lev.cu) reads hi + lo.
#include "common.cuh"
#include "tma_common.cuh"

namespace stater {
namespace {

__host__ __device__ constexpr int lev_nstate_f(int G) { return 1 + 2 * (G + 3) + G * (G + 1) / 2 + 3 * G + 3; }

constexpr int kBlockSamples = 8;
constexpr int kPx = 32;    // pixels per CTA (one warp row per part of the sums)
#ifndef STATER_LEV_PARTS
#define STATER_LEV_PARTS 2
#endif
constexpr int kParts = STATER_LEV_PARTS;  // threads per pixel (1 to 4), each keeping a share of the sums

__host__ __device__ constexpr int lev_nsum(int G) { return lev_nstate_f(G) - (1 + (G + 3)); }
__host__ __device__ constexpr int lev_part(int G) { return (lev_nsum(G) + kParts - 1) / kParts; }

// The sums of one pixel are split across kParts threads (threadIdx.y): part J
// keeps sums [QLO, QHI) of the order S_a, S_ab (a <= b < G), S_ay, S_yy. All
// parts read the same sample words (one HBM fetch, the others from L1) and
// compute the same pivot-shifted values; part 0 also keeps n and the pivot.
template <int G, int QLO, int QHI>
__device__ __forceinline__ void lev_part_loop(size_t HW, int cnt, const float *__restrict__ sp, float &n, float (&piv)[G + 3],
                                              float *hi, float *lo, int slot) {
    constexpr int P0 = G + 3;
    constexpr int NQ = QHI - QLO;
    const size_t NCH = 5 + G;
    for (int s0 = 0; s0 < cnt; s0 += kBlockSamples) {
        float part[NQ > 0 ? NQ : 1];
#pragma unroll
        for (int q = 0; q < NQ; q++) part[q] = 0.f;
        const int s1 = min(cnt, s0 + kBlockSamples);
        for (int s = s0; s < s1; s++, sp += NCH * HW) {
            float v[P0];
#pragma unroll
            for (int g = 0; g < G; g++) v[g] = __ldg(sp + (size_t)(5 + g) * HW);
#pragma unroll
            for (int c = 0; c < 3; c++) v[G + c] = __ldg(sp + (size_t)c * HW);
            if (n == 0.f) {
#pragma unroll
                for (int a = 0; a < P0; a++) piv[a] = v[a];
            }
            n += 1.f;
            float z[P0];
#pragma unroll
            for (int a = 0; a < P0; a++) z[a] = v[a] - piv[a];
            int q = 0;
#pragma unroll
            for (int a = 0; a < P0; a++, q++)
                if (q >= QLO && q < QHI) part[q - QLO] += z[a];
#pragma unroll
            for (int a = 0; a < G; a++)
#pragma unroll
                for (int b = a; b < G; b++, q++)
                    if (q >= QLO && q < QHI) part[q - QLO] = fmaf(z[a], z[b], part[q - QLO]);
#pragma unroll
            for (int a = 0; a < G; a++)
#pragma unroll
                for (int c = 0; c < 3; c++, q++)
                    if (q >= QLO && q < QHI) part[q - QLO] = fmaf(z[a], z[G + c], part[q - QLO]);
#pragma unroll
            for (int c = 0; c < 3; c++, q++)
                if (q >= QLO && q < QHI) part[q - QLO] = fmaf(z[G + c], z[G + c], part[q - QLO]);
        }
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            const float h = hi[q * kPx + slot];
            const float y = part[q] + lo[q * kPx + slot];
            const float t = h + y;
            lo[q * kPx + slot] = y - (t - h);
            hi[q * kPx + slot] = t;
        }
    }
}

template <int G>
__global__ void __launch_bounds__(kPx *kParts) lev_acc_f32(size_t HW, int S, const float *__restrict__ samples,
                                                          const int32_t *__restrict__ count, float *state) {
    constexpr int P0 = G + 3;
    constexpr int NS = lev_nstate_f(G);
    constexpr int oS = 1 + P0;
    constexpr int NSUM = lev_nsum(G);
    constexpr int QP = lev_part(G);
    extern __shared__ float sm[];
    const int lane = threadIdx.x, J = threadIdx.y;
    const size_t p = (size_t)blockIdx.x * kPx + lane;
    if (p >= HW) return;  // no block-wide synchronisation below
    // this part's hi / lo columns: [QP][kPx] each, parts one after another
    float *hi = sm + (size_t)J * 2 * QP * kPx;
    float *lo = hi + (size_t)QP * kPx;
    const int qlo = J * QP, qhi = min(NSUM, qlo + QP);
    float n = state[p];
    float piv[P0];
#pragma unroll
    for (int a = 0; a < P0; a++) piv[a] = state[(size_t)(1 + a) * HW + p];
    for (int q = qlo; q < qhi; q++) {
        hi[(q - qlo) * kPx + lane] = state[(size_t)(oS + q) * HW + p];
        lo[(q - qlo) * kPx + lane] = state[(size_t)(NS + oS + q) * HW + p];
    }
    const int cnt = count ? min(max(count[p], 0), S) : S;
    const float *sp = samples + p;
    switch (J) {
        case 0: lev_part_loop<G, 0, (QP < NSUM ? QP : NSUM)>(HW, cnt, sp, n, piv, hi, lo, lane); break;
        case 1: lev_part_loop<G, (QP < NSUM ? QP : NSUM), (2 * QP < NSUM ? 2 * QP : NSUM)>(HW, cnt, sp, n, piv, hi, lo, lane); break;
        case 2: lev_part_loop<G, (2 * QP < NSUM ? 2 * QP : NSUM), (3 * QP < NSUM ? 3 * QP : NSUM)>(HW, cnt, sp, n, piv, hi, lo, lane); break;
        default: lev_part_loop<G, (3 * QP < NSUM ? 3 * QP : NSUM), NSUM>(HW, cnt, sp, n, piv, hi, lo, lane);
    }
    if (J == 0) {
        // n and the pivot (set by a pixel's first sample) are the same in every part
        state[p] = n;
#pragma unroll
        for (int a = 0; a < P0; a++) state[(size_t)(1 + a) * HW + p] = piv[a];
    }
    for (int q = qlo; q < qhi; q++) {
        state[(size_t)(oS + q) * HW + p] = hi[(q - qlo) * kPx + lane];
        state[(size_t)(NS + oS + q) * HW + p] = lo[(q - qlo) * kPx + lane];
    }
}

// ---------------------------------------------------------------------------
// TMA-fed form: one producer thread streams, per stage, the radiance rows and
// the feature rows of kLSB samples x 32 pixels (two boxes of the 3-D view
// [S][5+G][HW], skipping the in-pixel offsets the regression does not read)
// into a ring of shared-memory stages; the kParts consumer warps read the
// stage instead of global memory. Same arithmetic and the same 8-sample
// compensation blocks as lev_acc_f32, so the state is bit-identical.
// ---------------------------------------------------------------------------
#ifndef STATER_LEV_SAMPLES_PER_STAGE
#define STATER_LEV_SAMPLES_PER_STAGE 4
#endif
#ifndef STATER_LEV_STAGES
#define STATER_LEV_STAGES 3
#endif
constexpr int kLSB = STATER_LEV_SAMPLES_PER_STAGE;  // samples per stage (divides the 8-sample blocks)
constexpr int kLStages = STATER_LEV_STAGES;

template <int G, int QLO, int QHI>
__device__ __forceinline__ bool lev_tma_consume(uint32_t wait_limit, const float *stages, int stage_floats,
                                                uint64_t *full, uint64_t *empty, int nchunks, int cnt, float &n,
                                                float (&piv)[G + 3], float *hi, float *lo, int lane) {
    using namespace tma;
    constexpr int P0 = G + 3;
    constexpr int NQ = QHI - QLO;
    static_assert(kBlockSamples % kLSB == 0, "compensation blocks are whole stages");
    constexpr int kStagesPerBlock = kBlockSamples / kLSB;
    float part[NQ > 0 ? NQ : 1];
#pragma unroll
    for (int q = 0; q < NQ; q++) part[q] = 0.f;
    for (int c = 0; c < nchunks; c++) {
        const int sidx = c % kLStages;
        if (!mbar_wait(&full[sidx], (c / kLStages) & 1, wait_limit)) return false;
        const float *rgb = stages + (size_t)sidx * stage_floats;  // [kLSB][3][kPx]
        const float *feat = rgb + kLSB * 3 * kPx;                 // [kLSB][G][kPx]
        const int jn = min(kLSB, cnt - c * kLSB);
        for (int j = 0; j < jn; j++) {
            float v[P0];
#pragma unroll
            for (int g = 0; g < G; g++) v[g] = feat[(j * G + g) * kPx + lane];
#pragma unroll
            for (int ch = 0; ch < 3; ch++) v[G + ch] = rgb[(j * 3 + ch) * kPx + lane];
            if (n == 0.f) {
#pragma unroll
                for (int a = 0; a < P0; a++) piv[a] = v[a];
            }
            n += 1.f;
            float z[P0];
#pragma unroll
            for (int a = 0; a < P0; a++) z[a] = v[a] - piv[a];
            int q = 0;
#pragma unroll
            for (int a = 0; a < P0; a++, q++)
                if (q >= QLO && q < QHI) part[q - QLO] += z[a];
#pragma unroll
            for (int a = 0; a < G; a++)
#pragma unroll
                for (int b = a; b < G; b++, q++)
                    if (q >= QLO && q < QHI) part[q - QLO] = fmaf(z[a], z[b], part[q - QLO]);
#pragma unroll
            for (int a = 0; a < G; a++)
#pragma unroll
                for (int ch = 0; ch < 3; ch++, q++)
                    if (q >= QLO && q < QHI) part[q - QLO] = fmaf(z[a], z[G + ch], part[q - QLO]);
#pragma unroll
            for (int ch = 0; ch < 3; ch++, q++)
                if (q >= QLO && q < QHI) part[q - QLO] = fmaf(z[G + ch], z[G + ch], part[q - QLO]);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sidx]);
        // fold at the end of each 8-sample block the pixel reached, and after its last sample
        const bool block_end = (c + 1) % kStagesPerBlock == 0 || c + 1 == nchunks;
        const bool pixel_end = jn > 0 && (c + 1) * kLSB >= cnt;
        if ((block_end && c * kLSB < cnt) || pixel_end) {
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const float h = hi[q * kPx + lane];
                const float y = part[q] + lo[q * kPx + lane];
                const float t = h + y;
                lo[q * kPx + lane] = y - (t - h);
                hi[q * kPx + lane] = t;
                part[q] = 0.f;
            }
        }
    }
    return true;
}

struct LevTmaParams {
    size_t HW;
    int S;
    const int32_t *count;
    float *state;
    int *err;
    uint32_t wait_limit;  // polls of a pipeline wait
    int stall;            // 1: the producer issues nothing (test hook: the consumers' waits run out)
};

template <int G>
__global__ void __launch_bounds__(kPx *(kParts + 1))
    lev_tma_f32(const __grid_constant__ CUtensorMap map_rgb, const __grid_constant__ CUtensorMap map_feat,
                LevTmaParams LP) {
    using namespace tma;
    constexpr int P0 = G + 3;
    constexpr int NS = lev_nstate_f(G);
    constexpr int oS = 1 + P0;
    constexpr int NSUM = lev_nsum(G);
    constexpr int QP = lev_part(G);
    constexpr int stage_floats = kLSB * (3 + G) * kPx;
    extern __shared__ __align__(128) float lsm[];
    float *stages = lsm;
    float *hilo = lsm + (size_t)kLStages * stage_floats;
    __shared__ __align__(8) uint64_t full[kLStages], empty[kLStages];
    __shared__ int s_maxcnt;
    const int lane = threadIdx.x % kPx, w = threadIdx.x / kPx;
    const bool producer = w == kParts;
    const size_t HW = LP.HW;
    const size_t p0 = (size_t)blockIdx.x * kPx, p = p0 + lane;
    const bool valid = p < HW;
    if (threadIdx.x == 0) {
        for (int i = 0; i < kLStages; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], kParts);
        }
        s_maxcnt = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (w == 0) {
        int c = 0;
        if (valid) c = LP.count ? min(max(LP.count[p], 0), LP.S) : LP.S;
        for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
        if (lane == 0) s_maxcnt = c;
    }
    __syncthreads();
    const int nchunks = (s_maxcnt + kLSB - 1) / kLSB;

    if (producer) {
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)stage_floats * 4u;
            int issued = 0;
            bool ok = true;
            for (int c = 0; c < nchunks && ok && !LP.stall; c++) {
                const int st = c % kLStages;
                if (c >= kLStages) ok = mbar_wait(&empty[st], ((c / kLStages) - 1) & 1, LP.wait_limit);
                if (!ok) break;
                mbar_arrive_expect_tx(&full[st], bytes);
                float *dst = stages + (size_t)st * stage_floats;
                tma_load_3d(dst, &map_rgb, (int)p0, 0, c * kLSB, &full[st]);
                if (G > 0) tma_load_3d(dst + kLSB * 3 * kPx, &map_feat, (int)p0, 5, c * kLSB, &full[st]);
                issued = c + 1;
            }
            if (!ok) atomicOr(LP.err, kErrTimeout);
            // the last boxes issued must have landed before the CTA may end (on
            // success too: consumers that gave up may already have left)
            bool drained = true;
            for (int c = max(0, issued - kLStages); c < issued; c++)
                drained = mbar_wait(&full[c % kLStages], (c / kLStages) & 1) && drained;
            if (!drained) atomicOr(LP.err, kErrDrain);
        }
        return;
    }

    const int J = w;
    float *hi = hilo + (size_t)J * 2 * QP * kPx;
    float *lo = hi + (size_t)QP * kPx;
    const int qlo = J * QP, qhi = min(NSUM, qlo + QP);
    float n = valid ? LP.state[p] : 0.f;
    float piv[P0];
#pragma unroll
    for (int a = 0; a < P0; a++) piv[a] = valid ? LP.state[(size_t)(1 + a) * HW + p] : 0.f;
    for (int q = qlo; q < qhi; q++) {
        hi[(q - qlo) * kPx + lane] = valid ? LP.state[(size_t)(oS + q) * HW + p] : 0.f;
        lo[(q - qlo) * kPx + lane] = valid ? LP.state[(size_t)(NS + oS + q) * HW + p] : 0.f;
    }
    const int cnt = valid ? (LP.count ? min(max(LP.count[p], 0), LP.S) : LP.S) : 0;
    bool ok;
    switch (J) {
        case 0: ok = lev_tma_consume<G, 0, (QP < NSUM ? QP : NSUM)>(LP.wait_limit, stages, stage_floats, full, empty, nchunks, cnt, n, piv, hi, lo, lane); break;
        case 1: ok = lev_tma_consume<G, (QP < NSUM ? QP : NSUM), (2 * QP < NSUM ? 2 * QP : NSUM)>(LP.wait_limit, stages, stage_floats, full, empty, nchunks, cnt, n, piv, hi, lo, lane); break;
        case 2: ok = lev_tma_consume<G, (2 * QP < NSUM ? 2 * QP : NSUM), (3 * QP < NSUM ? 3 * QP : NSUM)>(LP.wait_limit, stages, stage_floats, full, empty, nchunks, cnt, n, piv, hi, lo, lane); break;
        default: ok = lev_tma_consume<G, (3 * QP < NSUM ? 3 * QP : NSUM), NSUM>(LP.wait_limit, stages, stage_floats, full, empty, nchunks, cnt, n, piv, hi, lo, lane);
    }
    if (!ok) {
        if (lane == 0) atomicOr(LP.err, kErrTimeout);
        return;
    }
    if (!valid) return;
    if (J == 0) {
        LP.state[p] = n;
#pragma unroll
        for (int a = 0; a < P0; a++) LP.state[(size_t)(1 + a) * HW + p] = piv[a];
    }
    for (int q = qlo; q < qhi; q++) {
        LP.state[(size_t)(oS + q) * HW + p] = hi[(q - qlo) * kPx + lane];
        LP.state[(size_t)(NS + oS + q) * HW + p] = lo[(q - qlo) * kPx + lane];
    }
}

// cudaErrorNotSupported when the sample planes do not meet the TMA rules
// (W*H a multiple of 4 floats, 16-byte aligned base): the caller falls back.
template <int G>
cudaError_t run_tma_g(size_t HW, int S, const float *samples, const int32_t *count, float *state, cudaStream_t s) {
    using namespace tma;
    if ((HW % 4) != 0 || ((uintptr_t)samples % 16) != 0) return cudaErrorNotSupported;
    CUtensorMap mrgb, mfeat;
    const uint64_t NCH = 5 + G;
    if (!encode_tensor_map_3d_f32(&mrgb, samples, HW, NCH, (uint64_t)S, kPx, 3, kLSB)) return cudaErrorNotSupported;
    if (G > 0 && !encode_tensor_map_3d_f32(&mfeat, samples, HW, NCH, (uint64_t)S, kPx, G, kLSB))
        return cudaErrorNotSupported;
    if (G == 0) mfeat = mrgb;
    LevTmaParams LP{HW, S, count, state, device_error_word(), pipeline_wait_limit(), pipeline_stall()};
    if (!LP.err) return cudaErrorMemoryAllocation;
    const size_t smem = sizeof(float) * ((size_t)kLStages * kLSB * (3 + G) * kPx + 2 * (size_t)lev_part(G) * kPx * kParts);
    cudaError_t e = cudaFuncSetAttribute(lev_tma_f32<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    lev_tma_f32<G><<<(unsigned)((HW + kPx - 1) / kPx), kPx * (kParts + 1), smem, s>>>(mrgb, mfeat, LP);
    return cudaGetLastError();
}

template <int G>
cudaError_t run_g(size_t HW, int S, const float *samples, const int32_t *count, float *state, cudaStream_t s) {
    const size_t smem = sizeof(float) * 2 * lev_part(G) * kPx * kParts;
    cudaError_t e = cudaFuncSetAttribute(lev_acc_f32<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    lev_acc_f32<G><<<(unsigned)((HW + kPx - 1) / kPx), dim3(kPx, kParts), smem, s>>>(HW, S, samples, count, state);
    return cudaGetLastError();
}

}  // namespace

cudaError_t lev_accumulate_f32_launch(int G, size_t HW, int S, const float *samples, const int32_t *count,
                                      float *state, cudaStream_t s) {
    cudaError_t e = cudaErrorNotSupported;
    switch (G) {
        case 0: e = run_tma_g<0>(HW, S, samples, count, state, s); break;
        case 1: e = run_tma_g<1>(HW, S, samples, count, state, s); break;
        case 2: e = run_tma_g<2>(HW, S, samples, count, state, s); break;
        case 3: e = run_tma_g<3>(HW, S, samples, count, state, s); break;
        case 4: e = run_tma_g<4>(HW, S, samples, count, state, s); break;
        case 5: e = run_tma_g<5>(HW, S, samples, count, state, s); break;
        case 6: e = run_tma_g<6>(HW, S, samples, count, state, s); break;
        case 7: e = run_tma_g<7>(HW, S, samples, count, state, s); break;
        case 8: e = run_tma_g<8>(HW, S, samples, count, state, s); break;
        default: break;
    }
    if (e != cudaErrorNotSupported) return e;
    cudaGetLastError();
    switch (G) {
        case 0: return run_g<0>(HW, S, samples, count, state, s);
        case 1: return run_g<1>(HW, S, samples, count, state, s);
        case 2: return run_g<2>(HW, S, samples, count, state, s);
        case 3: return run_g<3>(HW, S, samples, count, state, s);
        case 4: return run_g<4>(HW, S, samples, count, state, s);
        case 5: return run_g<5>(HW, S, samples, count, state, s);
        case 6: return run_g<6>(HW, S, samples, count, state, s);
        case 7: return run_g<7>(HW, S, samples, count, state, s);
        case 8: return run_g<8>(HW, S, samples, count, state, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace stater
