// Stage 2, FP32 form. Same formulas as the plain FP64 form (denoise.cu), laid
// out for the GPU:
//  * per-pixel statistics (lnS2, se2, s2, s2C, jb) in one elementwise pass;
//  * the windowed filters stream the halo rows of a 32 x TY output tile through
//    a shared-memory ring holding every transform's planes, so the range weight
//    of a neighbour is computed once for all transforms (row-ring kernels, up to
//    5 transforms and 7 feature channels); other configurations, and calls that
//    ask for the decision bits, use per-transform kernels that stage the whole
//    (32+2R) x (TY+2R) halo of one transform at a time. Both give the same bits;
//  * the Welch decisions of all transforms are combined in a per-pixel bit mask
//    in shared memory (one bit per window position), so the film pass touches
//    only accepted neighbours;
//  * the Welch df always lies in [min(n_i, n_j) - 1, n_i + n_j - 2], and the
//    critical value decreases with df, so the test is decided from two
//    per-pair bounds (tables indexed by integer df) and only the narrow band
//    between them evaluates the exact df and the interpolated quantile. The
//    exact branch falls back to FP64 when the summed variance is near zero.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <map>
#include <tuple>
#include <vector>

#include "denoise_params.cuh"

namespace stater {

namespace {

constexpr int kTX2 = 32;
constexpr int kMaxFeatCh = 24;
constexpr int kDfMax = 4096;
constexpr float kLog2e = 1.4426950408889634f;

struct FeatSet {
    int nch;
    const float *plane[kMaxFeatCh];
    float mul[kMaxFeatCh];    // sqrt(-dr log2 e) of the owning G-buffer (dr <= 0)
};

bool make_featset(FeatSet &f, const stater_gbuffers &g, size_t HW) {
    f.nch = 0;
    if (g.count < 0 || g.count > STATER_MAX_GBUFFERS) return false;
    for (int i = 0; i < g.count; i++) {
        if (!g.planes[i] || (g.channels[i] != 1 && g.channels[i] != 3)) return false;
        for (int c = 0; c < g.channels[i]; c++) {
            if (f.nch >= kMaxFeatCh) return false;
            f.plane[f.nch] = (const float *)g.planes[i] + (size_t)c * HW;
            if (!(g.dr_factor[i] <= 0.f)) return false;
            f.mul[f.nch] = sqrtf(-g.dr_factor[i] * kLog2e);
            f.nch++;
        }
    }
    return true;
}

struct FastVars {
    int W, H, K, R, max_moment, levc;
    float ds2, z, z2;
    const int32_t *n;
    const float *m2[STATER_MAX_TRANSFORMS];
    const float *m3[STATER_MAX_TRANSFORMS];
    const float *m4[STATER_MAX_TRANSFORMS];
    const float *cx[STATER_MAX_TRANSFORMS];
    const float *cy[STATER_MAX_TRANSFORMS];
    const float *m2c_in;
    FeatSet feat;
    float *jb[STATER_MAX_TRANSFORMS];
    float *lnS2[STATER_MAX_TRANSFORMS];
    float *se2[STATER_MAX_TRANSFORMS];
    float *m2C[STATER_MAX_TRANSFORMS];
    float *varD[STATER_MAX_TRANSFORMS];
    float *varCD[STATER_MAX_TRANSFORMS];
    float *s2, *s2c;  // scratch [K][3][HW]
};

struct FastFilm {
    int W, H, K, R, mt_mode, use_levc, lut_n, discr_source;
    float ds2;
    const int32_t *n;
    const float *film;
    const float *mean[STATER_MAX_TRANSFORMS];
    const float *var[STATER_MAX_TRANSFORMS];  // varCD or varD; m2C or m2 with STATER_DISCR_SAMPLE
    const float *jb[STATER_MAX_TRANSFORMS];
    const float *lut;    // [lut_n + 1] t2 over u
    const float *tlo;    // [kDfMax + 1] lower envelope of t2 at integer df
    const float *thi;    // [kDfMax + 1] upper envelope
    float z2lo;          // lower bound of t2 beyond kDfMax
    FeatSet feat;
    float *discr[STATER_MAX_TRANSFORMS];
    float *filmD;
    uint32_t *bits;
    int8_t order[STATER_MAX_TRANSFORMS];  // ring kernel: slot -> transform tested in that position
};

// ---------------------------------------------------------------------------
// Per-pixel variance statistics.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void vars_stats_body(const FastVars &P, size_t p, int k) {
    const size_t HW = (size_t)P.W * P.H;
    if (p >= HW) return;
    const int nn = P.n[p];
    const float n = (float)nn;
    const float z = P.z;
    float jbsum = 0.f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const size_t o = (size_t)c * HW + p;
        const size_t so = ((size_t)k * 3 + c) * HW + p;
        if (nn < 2) {
            P.s2[so] = 0.f;
            P.s2c[so] = 0.f;
            P.lnS2[k][o] = 0.f;
            P.se2[k][o] = 0.f;
            P.m2C[k][o] = 0.f;
            continue;
        }
        const float M2 = P.m2[k][o];
        const float M3 = P.m3[k][o];
        const float s2 = M2 / (n - 1.f);
        const float cB = n > z + 1.f ? n / (n - z) : 1.f;
        float kurt = 3.f;
        if (P.max_moment >= 4 && M2 > 0.f) kurt = (n * P.m4[k][o] / M2) / M2;
        float m2c = M2;
        if (k == 0 && P.m2c_in) {
            m2c = P.m2c_in[o];
        } else if (P.max_moment >= 5) {
            const float cx = P.cx[k][o], cy = P.cy[k][o];
            m2c = fmaxf(M2 - 12.f * (cx * cx + cy * cy) / n, 0.f);
        }
        P.s2[so] = s2;
        P.s2c[so] = m2c / (n - 1.f);
        P.m2C[k][o] = m2c;
        P.lnS2[k][o] = logf(cB * fmaxf(s2, kS2Floor));
        P.se2[k][o] = cB * cB * (kurt - (n - 3.f) / n) / (n - 1.f);
        if (M2 > 0.f) {
            const float r = M3 / M2;
            float jbc = n * r * r / M2;
            if (P.max_moment >= 4) jbc += 0.25f * (kurt - 3.f) * (kurt - 3.f);
            jbsum += n / 6.f * jbc;
        }
    }
    P.jb[k][p] = nn < 2 ? 0.f : jbsum;
}

__global__ void vars_stats_f32(FastVars P) {
    vars_stats_body(P, (size_t)blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__device__ __forceinline__ void load_penalty(float *dst, const int32_t *__restrict__ n, int W, int H, int x0,
                                             int y0, int R, int hw, int hh) {
    const int A = hw * hh;
    for (int idx = threadIdx.x; idx < A; idx += blockDim.x) {
        const int hy = idx / hw, hx = idx - hy * hw;
        const int gx = x0 - R + hx, gy = y0 - R + hy;
        bool ok = false;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) ok = __ldg(n + (size_t)gy * W + gx) >= 2;
        dst[idx] = ok ? 0.f : -INFINITY;
    }
}

// ---------------------------------------------------------------------------
// Tiles: 32 x 8 output pixels per CTA of 128 threads; a warp covers one
// 32-pixel row (conflict-free shared-memory rows) and each thread owns two
// vertically adjacent pixels, so every neighbour row it loads serves both.
// Feature planes are staged pre-scaled by sqrt(-dr log2 e), so the range
// weight is exp2(ds log2e |dp|^2 - sum_f (f_i - f_j)^2).
// ---------------------------------------------------------------------------
// Preferred tile: RB pixels per thread (vertical) x TR thread rows per CTA.
#ifndef STATER_TILE_RB
#define STATER_TILE_RB 1
#endif
#ifndef STATER_TILE_TR
#define STATER_TILE_TR 8
#endif

__device__ __forceinline__ void load_feat_scaled(float *dst, const float *__restrict__ src, float mul, int W, int H,
                                                 int x0, int y0, int R, int hw, int hh) {
    const int A = hw * hh;
    for (int idx = threadIdx.x; idx < A; idx += blockDim.x) {
        const int hy = idx / hw, hx = idx - hy * hw;
        const int gx = x0 - R + hx, gy = y0 - R + hy;
        dst[idx] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? __fmul_rn(__ldg(src + (size_t)gy * W + gx), mul) : 0.f;
    }
}

__device__ __forceinline__ void load_halo_scaled(float *dst, const float *__restrict__ src, float mul, int W, int H,
                                                 int x0, int y0, int R, int hw, int hh) {
    const int A = hw * hh;
    for (int idx = threadIdx.x; idx < A; idx += blockDim.x) {
        const int hy = idx / hw, hx = idx - hy * hw;
        const int gx = x0 - R + hx, gy = y0 - R + hy;
        dst[idx] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? __fmul_rn(__ldg(src + (size_t)gy * W + gx), mul) : 0.f;
    }
}

template <int MF>
__device__ __forceinline__ float range_arg2(const float (&fi)[MF > 0 ? MF : 1], const float *feat, int A, int h,
                                            int nf, float sp) {
    float a = sp;
#pragma unroll
    for (int f = 0; f < MF; f++) {
        if (f < nf) {
            const float d = fi[f] - feat[f * A + h];
            a = fmaf(-d, d, a);
        }
    }
    return a;
}

__device__ __forceinline__ float fast_exp2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ZPIX: se2 does not depend on the transform or channel (no kurtosis tracked),
// so one z^2 se2 plane serves every test.
template <bool LEVC, bool ZPIX, int MF, int kRows, int kThreadRows>
__global__ void __launch_bounds__(kTX2 *kThreadRows) vars_filter_f32(FastVars P) {
    constexpr int kTY = kRows * kThreadRows;
    extern __shared__ float smem[];
    const int R = P.R, hw = kTX2 + 2 * R, hh = kTY + 2 * R, A = hw * hh;
    const int nf = P.feat.nch;
    float *vpen = smem;  // 0 for a usable neighbour, -inf otherwise (added to the weight exponent)
    float *feat = smem + A;
    float *zpix = feat + nf * A;            // ZPIX: [A]
    float *ln = zpix + (ZPIX ? A : 0);      // [3][A]
    float *zs = ln + 3 * A;                 // !ZPIX: [3][A]
    float *sv = zs + (ZPIX ? 0 : 3 * A);    // [3][A]
    float *svc = sv + 3 * A;                // LEVC: [3][A]

    const int x0 = blockIdx.x * kTX2, y0 = blockIdx.y * kTY;
    const int lx = threadIdx.x % kTX2, tr = threadIdx.x / kTX2;
    const int x = x0 + lx;
    const size_t HW = (size_t)P.W * P.H;

    load_penalty(vpen, P.n, P.W, P.H, x0, y0, R, hw, hh);
    for (int f = 0; f < nf; f++)
        load_feat_scaled(feat + f * A, P.feat.plane[f], P.feat.mul[f], P.W, P.H, x0, y0, R, hw, hh);
    if (ZPIX) load_halo_scaled(zpix, P.se2[0], P.z2, P.W, P.H, x0, y0, R, hw, hh);
    __syncthreads();

    int ci[kRows];
    bool vi[kRows], in[kRows];
    size_t gi[kRows];
    float fi[kRows][MF > 0 ? MF : 1], zpi[kRows];
#pragma unroll
    for (int q = 0; q < kRows; q++) {
        const int ly = tr * kRows + q, y = y0 + ly;
        in[q] = x < P.W && y < P.H;
        gi[q] = (size_t)y * P.W + x;
        ci[q] = (ly + R) * hw + (lx + R);
        vi[q] = in[q] && vpen[ci[q]] == 0.f;
        zpi[q] = ZPIX ? zpix[ci[q]] : 0.f;
#pragma unroll
        for (int f = 0; f < MF; f++) fi[q][f] = f < nf ? feat[f * A + ci[q]] : 0.f;
    }

    for (int k = 0; k < P.K; k++) {
        __syncthreads();
        for (int c = 0; c < 3; c++) {
            const size_t off = ((size_t)k * 3 + c) * HW;
            load_halo_scaled(ln + c * A, P.lnS2[k] + (size_t)c * HW, 1.f, P.W, P.H, x0, y0, R, hw, hh);
            if (!ZPIX) load_halo_scaled(zs + c * A, P.se2[k] + (size_t)c * HW, P.z2, P.W, P.H, x0, y0, R, hw, hh);
            load_halo_scaled(sv + c * A, P.s2 + off, 1.f, P.W, P.H, x0, y0, R, hw, hh);
            if (LEVC) load_halo_scaled(svc + c * A, P.s2c + off, 1.f, P.W, P.H, x0, y0, R, hw, hh);
        }
        __syncthreads();
        float li[kRows][3], zi[kRows][3], aw[kRows][3], av[kRows][3], avc[kRows][3];
#pragma unroll
        for (int q = 0; q < kRows; q++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                li[q][c] = ln[c * A + ci[q]];
                zi[q][c] = ZPIX ? zpi[q] : zs[c * A + ci[q]];
                aw[q][c] = av[q][c] = avc[q][c] = 0.f;
            }
        for (int r = -R; r <= R + kRows - 1; r++) {
            const int row = (tr * kRows + R + r) * hw + lx + R;
            float spq[kRows];
            bool use[kRows];
#pragma unroll
            for (int q = 0; q < kRows; q++) {
                const int dy = r - q;
                use[q] = vi[q] && dy >= -R && dy <= R;
                spq[q] = __fmul_rn(P.ds2, (float)(dy * dy));
            }
#pragma unroll 4
            for (int dx = -R; dx <= R; dx++) {
                const int h = row + dx;
                const float dxs = fmaf(P.ds2, (float)(dx * dx), vpen[h]);
                float lj[3], zj[3], vj[3], vcj[3];
                const float zpj = ZPIX ? zpix[h] : 0.f;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    lj[c] = ln[c * A + h];
                    zj[c] = ZPIX ? zpj : zs[c * A + h];
                    vj[c] = sv[c * A + h];
                    vcj[c] = LEVC ? svc[c * A + h] : 0.f;
                }
#pragma unroll
                for (int q = 0; q < kRows; q++) {
                    if (!use[q]) continue;
                    const float e = range_arg2<MF>(fi[q], feat, A, h, nf, __fadd_rn(spq[q], dxs));
                    if (e < -127.f) continue;  // weight 0: adds nothing; skipped as in the ring kernel
                    const float w = fast_exp2(e);
                    const float zz = __fadd_rn(zi[q][0], zj[0]);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float dl = li[q][c] - lj[c];
                        const float t = fmaf(-dl, dl, ZPIX ? zz : __fadd_rn(zi[q][c], zj[c]));
                        // an accepted neighbour adds its weight (a rejected one adds nothing)
                        if (t >= 0.f) {
                            aw[q][c] += w;
                            av[q][c] = fmaf(w, vj[c], av[q][c]);
                            if (LEVC) avc[q][c] = fmaf(w, vcj[c], avc[q][c]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kRows; q++) {
            if (!in[q]) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float vd = vi[q] ? av[q][c] / aw[q][c] : 0.f;
                P.varD[k][(size_t)c * HW + gi[q]] = vd;
                P.varCD[k][(size_t)c * HW + gi[q]] = vi[q] ? (LEVC ? avc[q][c] / aw[q][c] : vd) : 0.f;
            }
        }
    }
}

__device__ __forceinline__ void film_discr_body(const FastFilm &P, size_t p, int k) {
    const size_t HW = (size_t)P.W * P.H;
    if (p >= HW) return;
    const int nn = P.n[p];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const size_t o = (size_t)c * HW + p;
        // CASCADE_MODE: the denoised variance, or the pixel's own sample variance
        const float v = P.discr_source == STATER_DISCR_SAMPLE ? P.var[k][o] / ((float)nn - 1.f) : P.var[k][o];
        P.discr[k][o] = nn < 2 ? 0.f : v / (float)nn;
    }
}

__global__ void film_discr_f32(FastFilm P) {
    film_discr_body(P, (size_t)blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__device__ __forceinline__ float lut_interp_f32(const float *lut, int N, float u) {
    u = fminf(u, 1.f);
    const float f = u * (float)N;
    int m = (int)f;
    if (m > N - 1) m = N - 1;
    const float frac = f - (float)m;
    const float a = __ldg(lut + m), b = __ldg(lut + m + 1);
    return fmaf(frac, b - a, a);
}

__device__ __forceinline__ double lut_interp_f64(const float *lut, int N, double u) {
    if (u > 1.0) u = 1.0;
    const double f = u * (double)N;
    int m = (int)f;
    if (m > N - 1) m = N - 1;
    const double frac = f - (double)m;
    const double a = __ldg(lut + m), b = __ldg(lut + m + 1);
    return a + frac * (b - a);
}

// Exact Welch decision for one channel (accept = 1).
__device__ __noinline__ int welch_exact(float diff, float di, float dj, int ni, int nj, const float *lut, int N) {
    const float s = di + dj;
    if (s < 1e-18f) {
        // Variance ratios near zero: evaluate df in FP64.
        const double sd = (double)di + (double)dj;
        if (!(sd > 0.0)) return diff == 0.f;
        const double e = (double)di * di / (double)(ni - 1) + (double)dj * dj / (double)(nj - 1);
        const double t2 = lut_interp_f64(lut, N, e / (sd * sd));
        return (double)diff * diff <= t2 * sd;
    }
    const float e = di * di / (float)(ni - 1) + dj * dj / (float)(nj - 1);
    const float t2 = lut_interp_f32(lut, N, e / (s * s));
    return diff * diff <= t2 * s;
}

// Mask layout: per pixel, per window row, ceil((2R+1)/32) words: bit dx+R of
// row dy+R is set while the neighbour is still accepted. Rows are handled as
// one 64-bit register value (2R+1 <= 41 bits).
template <int MF, int kRows, int kThreadRows>
__global__ void __launch_bounds__(kTX2 *kThreadRows) film_filter_f32(FastFilm P) {
    constexpr int kTY = kRows * kThreadRows;
    constexpr int kThreads = kTX2 * kThreadRows;
    extern __shared__ float smem[];
    const int R = P.R, D = 2 * R + 1, wpr = (D + 31) / 32, fwords = (D * D + 31) / 32;
    const int hw = kTX2 + 2 * R, hh = kTY + 2 * R, A = hw * hh;
    const int nf = P.feat.nch;
    const int t = threadIdx.x;
    uint32_t *mask = (uint32_t *)smem;                          // [kRows][D][wpr][kThreads]
    int *nval = (int *)(mask + kRows * D * wpr * kThreads);     // [A]
    float *feat = (float *)(nval + A);                          // [nf][A]
    float *mu = feat + nf * A;                                  // [3][A] (film in the last pass)
    float *dd = mu + 3 * A;                                     // [3][A]
    __shared__ int s_nmin, s_nmax;

    const int x0 = blockIdx.x * kTX2, y0 = blockIdx.y * kTY;
    const int lx = t % kTX2, tr = t / kTX2;
    const int x = x0 + lx;
    const size_t HW = (size_t)P.W * P.H;
    auto mask_at = [&](int q, int row, int w) -> uint32_t & { return mask[((q * D + row) * wpr + w) * kThreads + t]; };
    auto load_row = [&](int q, int row) -> uint64_t {
        uint64_t v = mask_at(q, row, 0);
        if (wpr > 1) v |= (uint64_t)mask_at(q, row, 1) << 32;
        return v;
    };
    auto and_row = [&](int q, int row, uint64_t v) {
        mask_at(q, row, 0) &= (uint32_t)v;
        if (wpr > 1) mask_at(q, row, 1) &= (uint32_t)(v >> 32);
    };

    if (t == 0) {
        s_nmin = 0x7fffffff;
        s_nmax = 0;
    }
    for (int q = 0; q < kRows; q++)
        for (int row = 0; row < D; row++)
            for (int w = 0; w < wpr; w++) mask_at(q, row, w) = 0xFFFFFFFFu;
    __syncthreads();
    {
        int lmin = 0x7fffffff, lmax = 0;
        for (int idx = t; idx < A; idx += blockDim.x) {
            const int hy = idx / hw, hx = idx - hy * hw;
            const int gx = x0 - R + hx, gy = y0 - R + hy;
            int v = 0;
            if (gx >= 0 && gx < P.W && gy >= 0 && gy < P.H) {
                v = __ldg(P.n + (size_t)gy * P.W + gx);
                if (v < 2) v = 0;
            }
            nval[idx] = v;
            if (v >= 2) {
                lmin = min(lmin, v);
                lmax = max(lmax, v);
            }
        }
        atomicMin(&s_nmin, lmin);
        atomicMax(&s_nmax, lmax);
    }
    for (int f = 0; f < nf; f++)
        load_feat_scaled(feat + f * A, P.feat.plane[f], P.feat.mul[f], P.W, P.H, x0, y0, R, hw, hh);
    __syncthreads();
    // All valid n in the halo equal: the df bounds are the same for every pair.
    const bool uni = s_nmin == s_nmax;
    float tlo_u = 0.f, thi_u = 0.f;
    if (uni) {
        const int dfl = 2 * s_nmin - 2, dfh = s_nmin - 1;
        tlo_u = dfl > kDfMax ? P.z2lo : __ldg(P.tlo + dfl);
        thi_u = __ldg(P.thi + (dfh > kDfMax ? kDfMax : dfh));
    }

    int ci[kRows], ni[kRows], ksel[kRows];
    bool in[kRows];
    size_t gi[kRows];
#pragma unroll
    for (int q = 0; q < kRows; q++) {
        const int ly = tr * kRows + q, y = y0 + ly;
        in[q] = x < P.W && y < P.H;
        gi[q] = (size_t)y * P.W + x;
        ci[q] = (ly + R) * hw + (lx + R);
        ni[q] = in[q] ? nval[ci[q]] : 0;
        ksel[q] = -1;
        if (in[q] && P.mt_mode == STATER_MT_JB && ni[q] >= 2) {
            ksel[q] = 0;
            float best = P.jb[0][gi[q]];
            for (int k = 1; k < P.K; k++) {
                const float v = P.jb[k][gi[q]];
                if (v < best) {
                    best = v;
                    ksel[q] = k;
                }
            }
        }
    }

    for (int k = 0; k < P.K; k++) {
        __syncthreads();
        const float *mean = k == 0 ? P.film : P.mean[k];
        for (int c = 0; c < 3; c++) {
            load_halo_scaled(mu + c * A, mean + (size_t)c * HW, 1.f, P.W, P.H, x0, y0, R, hw, hh);
            load_halo_scaled(dd + c * A, P.discr[k] + (size_t)c * HW, 1.f, P.W, P.H, x0, y0, R, hw, hh);
        }
        __syncthreads();
        float mi[kRows][3], di[kRows][3];
        bool act[kRows], andm[kRows];
#pragma unroll
        for (int q = 0; q < kRows; q++) {
            act[q] = in[q] && ni[q] >= 2;
            andm[q] = ksel[q] < 0 || ksel[q] == k;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                mi[q][c] = mu[c * A + ci[q]];
                di[q][c] = dd[c * A + ci[q]];
            }
            if (P.bits && in[q])
                for (int w = 0; w < fwords; w++) P.bits[(gi[q] * P.K + k) * (size_t)fwords + w] = 0u;
        }
        // Only transforms that feed the mask may skip pairs an earlier transform rejected.
        const bool skip_rejected = (P.bits == nullptr) && P.mt_mode == STATER_MT_ALL && k > 0;
        for (int r = -R; r <= R + kRows - 1; r++) {
            const int row = (tr * kRows + R + r) * hw + lx + R;
            bool use[kRows];
            uint64_t prev[kRows], cur[kRows];
#pragma unroll
            for (int q = 0; q < kRows; q++) {
                const int dy = r - q;
                use[q] = act[q] && dy >= -R && dy <= R;
                cur[q] = 0ull;
                prev[q] = ~0ull;
                if (use[q] && skip_rejected) prev[q] = load_row(q, dy + R);
            }
#pragma unroll 2
            for (int dx = -R; dx <= R; dx++) {
                const int h = row + dx;
                const int nj = nval[h];
                const int b = dx + R;
                float mj[3], dj[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    mj[c] = mu[c * A + h];
                    dj[c] = dd[c * A + h];
                }
#pragma unroll
                for (int q = 0; q < kRows; q++) {
                    if (!use[q]) continue;
                    float tlo = tlo_u, thi = thi_u;
                    if (!uni) {
                        // per-pair bounds (only when n varies inside the halo)
                        const int njc = max(nj, 2);
                        const int dfl = ni[q] + njc - 2, dfh = min(ni[q], njc) - 1;
                        tlo = dfl > kDfMax ? P.z2lo : __ldg(P.tlo + dfl);
                        thi = __ldg(P.thi + (dfh > kDfMax ? kDfMax : dfh));
                    }
                    // qq <= tlo s accepts, qq > thi s rejects, in between the exact
                    // df decides; s = 0 accepts exactly when the means are equal.
                    bool acc = true, amb = false;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float diff = mi[q][c] - mj[c];
                        const float s = di[q][c] + dj[c];
                        const float qq = diff * diff;
                        const bool lo = qq <= tlo * s;
                        const bool hi = qq <= thi * s;
                        acc = acc && hi;
                        amb = amb || (hi && !lo);
                    }
                    bool a = acc && nj >= 2 && ((prev[q] >> b) & 1ull);
                    if (a && amb) {
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const float diff = mi[q][c] - mj[c];
                            const float s = di[q][c] + dj[c];
                            const float qq = diff * diff;
                            if (!(qq <= tlo * s) && qq <= thi * s)
                                a = a && welch_exact(diff, di[q][c], dj[c], ni[q], nj, P.lut, P.lut_n);
                        }
                    }
                    if (dx == 0 && r == q) a = true;
                    cur[q] |= (uint64_t)a << b;
                }
            }
#pragma unroll
            for (int q = 0; q < kRows; q++) {
                if (!use[q]) continue;
                const int dy = r - q;
                if (andm[q]) and_row(q, dy + R, cur[q]);
                if (P.bits) {
                    uint32_t *fb = P.bits + (gi[q] * P.K + k) * (size_t)fwords;
                    for (int b = 0; b < D; b++) {
                        if ((cur[q] >> b) & 1ull) {
                            const int fbit = (dy + R) * D + b;
                            fb[fbit >> 5] |= 1u << (fbit & 31);
                        }
                    }
                }
            }
        }
    }

    __syncthreads();
    for (int c = 0; c < 3; c++) load_halo_scaled(mu + c * A, P.film + (size_t)c * HW, 1.f, P.W, P.H, x0, y0, R, hw, hh);
    __syncthreads();
    float fi[kRows][MF > 0 ? MF : 1];
#pragma unroll
    for (int q = 0; q < kRows; q++)
#pragma unroll
        for (int f = 0; f < MF; f++) fi[q][f] = f < nf ? feat[f * A + ci[q]] : 0.f;
#pragma unroll
    for (int q = 0; q < kRows; q++) {
        if (!in[q]) continue;
        if (ni[q] < 2) {
            for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + gi[q]] = mu[c * A + ci[q]];
            continue;
        }
        float sw = 0.f, sf[3] = {0.f, 0.f, 0.f};
        for (int dy = -R; dy <= R; dy++) {
            const int row = (tr * kRows + q + R + dy) * hw + lx + R;
            const float sdy = __fmul_rn(P.ds2, (float)(dy * dy));
            const uint64_t m = load_row(q, dy + R);
#pragma unroll 4
            for (int dx = -R; dx <= R; dx++) {
                const int h = row + dx;
                const float e = range_arg2<MF>(fi[q], feat, A, h, nf, fmaf(P.ds2, (float)(dx * dx), sdy));
                const float wt = ((m >> (dx + R)) & 1ull) ? fast_exp2(e) : 0.f;
                sw += wt;
#pragma unroll
                for (int c = 0; c < 3; c++) sf[c] = fmaf(wt, mu[c * A + h], sf[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + gi[q]] = sf[c] / sw;
    }
}

// ---------------------------------------------------------------------------
// Row-ring forms: every transform per neighbour, one range weight.
//
// The halo rows of a 32 x TY tile stream through a ring of TY + 1 shared-memory
// rows. A ring row holds, as float4 fields in structure-of-arrays order (lane
// l reads column l: conflict-free 128-bit loads), everything the filter reads
// at that row: the scaled features and the validity of the pixel, and for every
// transform the planes of its test and its weighted sums. At window row dy the
// TY thread rows read the consecutive halo rows dy .. dy + TY - 1 while the CTA
// loads halo row dy + TY into the one free slot: one barrier per window row.
// The range weight of a neighbour is computed once and applied to every
// transform (the per-transform accumulators live in registers), and the
// operations and their order per transform are those of the per-transform
// kernels above, so both give the same bits.
// Features: up to kRingMF channels, validity (or n) in field kRingMF.
// ---------------------------------------------------------------------------
constexpr int kRingMF = 7;
constexpr int kRingFW = 2;  // float4 fields of features + validity

__device__ __forceinline__ float4 f4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

// Feature fields of one halo pixel: scaled features, then `last` in field 7.
__device__ __forceinline__ void ring_feat_fields(const FeatSet &fs, bool inb, size_t g, float last, float4 &a,
                                                 float4 &b) {
    float v[8];
#pragma unroll
    for (int f = 0; f < kRingMF; f++) v[f] = (inb && f < fs.nch) ? __fmul_rn(__ldg(fs.plane[f] + g), fs.mul[f]) : 0.f;
    v[7] = last;
    a = f4(v[0], v[1], v[2], v[3]);
    b = f4(v[4], v[5], v[6], v[7]);
}

// Vars ring fields per transform k: {lnS2 x3, z^2 se2 (ZPIX) | c0}, {s2 x3, 0 | c1},
// [{s2C x3, 0 | c2}] with c = z^2 se2 per channel when it depends on it.
// With one z^2 se2 per pixel and no LEVC sums (PACKED) the records are packed
// instead: the six values of every transform slot k < KMAX (lnS2 x3, s2 x3)
// back to back, then the pixel's z^2 se2: ceil((6 KMAX + 1) / 4) records, 8
// for 5 transforms where the per-transform form takes 10 (one shared load in
// six fewer per neighbour of nonzero weight; where every neighbour's records
// are loaded, the filter is bound by its shared loads).
template <bool LEVC, bool ZPIX>
struct VarsRing {
    static constexpr bool PACKED = ZPIX && !LEVC;
    static constexpr int TW = (LEVC || !ZPIX) ? 3 : 2;
};

// Ring records of a vars job (KMAX: the ring kernel's transform slots).
__host__ __device__ constexpr int vars_ring_nrec(int K, int KMAX, bool levc, bool zpix) {
    return kRingFW + ((zpix && !levc) ? (6 * KMAX + 4) / 4 : K * 3);
}

template <bool LEVC, bool ZPIX, int KMAX>
__device__ __forceinline__ float4 vars_ring_value(const FastVars &P, int rec, int col, int hrow, int x0, int y0) {
    constexpr int TW = VarsRing<LEVC, ZPIX>::TW;
    const size_t HW = (size_t)P.W * P.H;
    const int gy = y0 - P.R + hrow, gx = x0 - P.R + col;
    const bool inb = gx >= 0 && gx < P.W && gy >= 0 && gy < P.H;
    const size_t g = inb ? (size_t)gy * P.W + gx : 0;
    float4 v = f4(0.f, 0.f, 0.f, 0.f);
    if (rec < kRingFW) {
        float4 a, b;
        const float pen = (inb && __ldg(P.n + g) >= 2) ? 0.f : -INFINITY;
        ring_feat_fields(P.feat, inb, g, pen, a, b);
        v = rec == 0 ? a : b;
    } else if (VarsRing<LEVC, ZPIX>::PACKED) {
        if (inb) {
            float e[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int f = (rec - kRingFW) * 4 + i, k = f / 6, sub = f - 6 * k;
                float x = 0.f;
                if (f < 6 * KMAX && k < P.K)
                    x = sub < 3 ? __ldg(P.lnS2[k] + (size_t)sub * HW + g)
                                : __ldg(P.s2 + ((size_t)k * 3 + (sub - 3)) * HW + g);
                else if (f == 6 * KMAX)
                    x = __fmul_rn(__ldg(P.se2[0] + g), P.z2);
                e[i] = x;
            }
            v = f4(e[0], e[1], e[2], e[3]);
        }
    } else if (inb) {
        const int kr = rec - kRingFW, k = kr / TW, sub = kr - k * TW;
        const float *src = sub == 0 ? P.lnS2[k] : (sub == 1 ? P.s2 + (size_t)k * 3 * HW : P.s2c + (size_t)k * 3 * HW);
        const bool zero = sub == 2 && !LEVC;
        v.x = zero ? 0.f : __ldg(src + g);
        v.y = zero ? 0.f : __ldg(src + HW + g);
        v.z = zero ? 0.f : __ldg(src + 2 * HW + g);
        if (ZPIX)
            v.w = sub == 0 ? __fmul_rn(__ldg(P.se2[0] + g), P.z2) : 0.f;
        else
            v.w = __fmul_rn(__ldg(P.se2[k] + (size_t)sub * HW + g), P.z2);
    }
    return v;
}

// Ring row loaders. A CTA loads one halo row of nrec x hw fields; with the
// pipelined form each thread fetches its (at most kRingPer) fields into
// registers before the window row's arithmetic and stores them after it, so
// the loads' latency is hidden behind the arithmetic.
constexpr int kRingPer = 5;

template <typename ValueFn>
__device__ __forceinline__ void ring_load_now(float4 *ring, int slot, int hrow, int hw, int nrec, ValueFn value) {
    for (int idx = threadIdx.x; idx < nrec * hw; idx += blockDim.x) {
        const int rec = idx / hw, col = idx - rec * hw;
        ring[((size_t)slot * nrec + rec) * hw + col] = value(rec, col, hrow);
    }
}

template <typename ValueFn>
__device__ __forceinline__ void ring_fetch(float4 (&pend)[kRingPer], int hrow, int hw, int nrec, ValueFn value) {
#pragma unroll
    for (int i = 0; i < kRingPer; i++) {
        const int idx = threadIdx.x + i * blockDim.x;
        if (idx < nrec * hw) {
            const int rec = idx / hw;
            pend[i] = value(rec, idx - rec * hw, hrow);
        }
    }
}

__device__ __forceinline__ void ring_store(const float4 (&pend)[kRingPer], float4 *ring, int slot, int hw, int nrec) {
#pragma unroll
    for (int i = 0; i < kRingPer; i++) {
        const int idx = threadIdx.x + i * blockDim.x;
        if (idx < nrec * hw) ring[(size_t)slot * nrec * hw + idx] = pend[i];
    }
}

template <bool LEVC, bool ZPIX, int KMAX, int TY>
__device__ __forceinline__ void vars_ring_body(const FastVars &P, int bx, int by) {
    constexpr int TW = VarsRing<LEVC, ZPIX>::TW;
    constexpr bool PACKED = VarsRing<LEVC, ZPIX>::PACKED;
    constexpr int NQ = (6 * KMAX + 4) / 4;  // packed records
    constexpr int ZREC = (6 * KMAX) / 4, ZCOMP = (6 * KMAX) % 4;
    constexpr int NS = TY + 1;
    extern __shared__ float4 ring[];
    const int R = P.R, hw = kTX2 + 2 * R, hh = TY + 2 * R;
    const int K = P.K, nf = P.feat.nch;
    const int nrec = vars_ring_nrec(K, KMAX, LEVC, ZPIX);
    const int x0 = bx * kTX2, y0 = by * TY;
    const int lx = threadIdx.x % kTX2, tr = threadIdx.x / kTX2;
    const int x = x0 + lx, y = y0 + tr;
    const bool in = x < P.W && y < P.H;
    const size_t HW = (size_t)P.W * P.H;
    const size_t gi = in ? (size_t)y * P.W + x : 0;

    // (the variance filter is not bound by the latency of these loads: they
    // are stored as they arrive; fetching the next row into registers during
    // the window row's arithmetic measured slower, at 128 registers)
    auto value = [&](int rec, int col, int hrow) {
        return vars_ring_value<LEVC, ZPIX, KMAX>(P, rec, col, hrow, x0, y0);
    };
    for (int hrow = 0; hrow < TY; hrow++) ring_load_now(ring, hrow % NS, hrow, hw, nrec, value);

    // centre values, read as the per-transform kernel stages them
    const bool vi = in && __ldg(P.n + gi) >= 2;
    float fi[kRingMF];
#pragma unroll
    for (int f = 0; f < kRingMF; f++) fi[f] = (in && f < nf) ? __fmul_rn(__ldg(P.feat.plane[f] + gi), P.feat.mul[f]) : 0.f;
    float li[KMAX][3], zi[KMAX][3], aw[KMAX][3], av[KMAX][3], avc[KMAX][3];
    const float zp = (ZPIX && in) ? __fmul_rn(__ldg(P.se2[0] + gi), P.z2) : 0.f;
#pragma unroll
    for (int k = 0; k < KMAX; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const bool ok = in && k < K;
            li[k][c] = ok ? __ldg(P.lnS2[k] + (size_t)c * HW + gi) : 0.f;
            zi[k][c] = ZPIX ? zp : (ok ? __fmul_rn(__ldg(P.se2[k] + (size_t)c * HW + gi), P.z2) : 0.f);
            aw[k][c] = av[k][c] = avc[k][c] = 0.f;
        }
    __syncthreads();

    for (int r = -R; r <= R; r++) {
        const int next = R + r + TY;
        if (next < hh) ring_load_now(ring, next % NS, next, hw, nrec, value);
        if (vi) {
            const float4 *rp = ring + (size_t)((tr + R + r) % NS) * nrec * hw + lx + R;
            const float spq = __fmul_rn(P.ds2, (float)(r * r));
#pragma unroll 2
            for (int dx = -R; dx <= R; dx++) {
                const float4 F0 = rp[dx], F1 = rp[hw + dx];
                const float fj[kRingMF] = {F0.x, F0.y, F0.z, F0.w, F1.x, F1.y, F1.z};
                const float dxs = fmaf(P.ds2, (float)(dx * dx), F1.w);
                float e = __fadd_rn(spq, dxs);
#pragma unroll
                for (int f = 0; f < kRingMF; f++) {
                    if (f < nf) {
                        const float d = fi[f] - fj[f];
                        e = fmaf(-d, d, e);
                    }
                }
                // Below -127 the weight exp2(e) is 0 (2^-127 is subnormal, flushed
                // to zero), and a neighbour of weight 0 adds nothing (its records
                // are finite: the statistics of a pixel with n < 2 are zeros), so
                // its records are not loaded; a warp whose lanes all have such a
                // neighbour skips them. The test on e does not wait for exp2.
                if (e < -127.f) continue;
                const float w = fast_exp2(e);
                // the packed records of the neighbour (PACKED: lnS2 and s2 of every slot, then z)
                float q[PACKED ? 4 * NQ : 1];
                if constexpr (PACKED) {
                    const float4 *qp = rp + (size_t)kRingFW * hw + dx;
#pragma unroll
                    for (int i = 0; i < NQ; i++) {
                        const float4 Q = qp[(size_t)i * hw];
                        q[4 * i] = Q.x;
                        q[4 * i + 1] = Q.y;
                        q[4 * i + 2] = Q.z;
                        q[4 * i + 3] = Q.w;
                    }
                }
                // per-pixel z (ZPIX): the threshold sum z_i + z_j is the same for
                // every transform (every record carries the same z_j)
                float zz = 0.f;
                if constexpr (PACKED)
                    zz = __fadd_rn(zp, q[4 * ZREC + ZCOMP]);
                else if constexpr (ZPIX)
                    zz = __fadd_rn(zp, rp[(size_t)kRingFW * hw + dx].w);
#pragma unroll
                for (int k = 0; k < KMAX; k++) {
                    if (k >= K) break;
                    float lj[3], vj[3], vcj[3] = {0.f, 0.f, 0.f}, zj[3] = {0.f, 0.f, 0.f};
                    if constexpr (PACKED) {
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            lj[c] = q[6 * k + c];
                            vj[c] = q[6 * k + 3 + c];
                        }
                    } else {
                        const float4 *tp = rp + (size_t)(kRingFW + k * TW) * hw + dx;
                        const float4 T0 = tp[0], T1 = tp[hw];
                        const float4 T2 = TW == 3 ? tp[2 * hw] : f4(0.f, 0.f, 0.f, 0.f);
                        lj[0] = T0.x; lj[1] = T0.y; lj[2] = T0.z;
                        vj[0] = T1.x; vj[1] = T1.y; vj[2] = T1.z;
                        vcj[0] = T2.x; vcj[1] = T2.y; vcj[2] = T2.z;
                        zj[0] = T0.w; zj[1] = T1.w; zj[2] = T2.w;
                    }
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float dl = li[k][c] - lj[c];
                        const float t = fmaf(-dl, dl, ZPIX ? zz : __fadd_rn(zi[k][c], zj[c]));
                        if (t >= 0.f) {  // the same updates as the per-transform kernel
                            aw[k][c] += w;
                            av[k][c] = fmaf(w, vj[c], av[k][c]);
                            if (LEVC) avc[k][c] = fmaf(w, vcj[c], avc[k][c]);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!in) return;
#pragma unroll
    for (int k = 0; k < KMAX; k++) {
        if (k >= K) break;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float vd = vi ? av[k][c] / aw[k][c] : 0.f;
            P.varD[k][(size_t)c * HW + gi] = vd;
            P.varCD[k][(size_t)c * HW + gi] = vi ? (LEVC ? avc[k][c] / aw[k][c] : vd) : 0.f;
        }
    }
}

template <bool LEVC, bool ZPIX, int KMAX, int TY>
__global__ void __launch_bounds__(kTX2 *TY) vars_ring_f32(FastVars P) {
    vars_ring_body<LEVC, ZPIX, KMAX, TY>(P, blockIdx.x, blockIdx.y);
}

// Film ring fields: features with n (as float) in field 7, {film x3, 0}, and per
// transform {mean x3, discr_0}, {discr_1, discr_2, 0, 0}.
__device__ __forceinline__ float4 film_ring_value(const FastFilm &P, int rec, int col, int hrow, int x0, int y0) {
    const size_t HW = (size_t)P.W * P.H;
    const int gy = y0 - P.R + hrow, gx = x0 - P.R + col;
    const bool inb = gx >= 0 && gx < P.W && gy >= 0 && gy < P.H;
    const size_t g = inb ? (size_t)gy * P.W + gx : 0;
    float4 v = f4(0.f, 0.f, 0.f, 0.f);
    if (rec < kRingFW) {
        float4 a, b;
        int nv = inb ? __ldg(P.n + g) : 0;
        if (nv < 2) nv = 0;
        ring_feat_fields(P.feat, inb, g, (float)nv, a, b);
        v = rec == 0 ? a : b;
    } else if (inb) {
        const int kr = rec - kRingFW;
        if (kr == 0) {
            v = f4(__ldg(P.film + g), __ldg(P.film + HW + g), __ldg(P.film + 2 * HW + g), 0.f);
        } else {
            const int k = P.order[(kr - 1) >> 1], sub = (kr - 1) & 1;
            const float *mean = k == 0 ? P.film : P.mean[k];
            if (sub == 0)
                v = f4(__ldg(mean + g), __ldg(mean + HW + g), __ldg(mean + 2 * HW + g), __ldg(P.discr[k] + g));
            else
                v = f4(__ldg(P.discr[k] + HW + g), __ldg(P.discr[k] + 2 * HW + g), 0.f, 0.f);
        }
    }
    return v;
}

// The film filter in two passes per window row. Pass A tests, for all 2R + 1
// neighbours of the row in lockstep, only the upper df bound of the first
// transform in test order (the JB choice in STATER_MT_JB mode): a neighbour it
// rejects is rejected by the full test too, and on the benchmark's radiance it
// rejects most of them. Each lane keeps the survivors as bits of a 64-bit mask.
// Pass B walks each lane's own survivors in increasing dx and runs the full
// test (every transform in test order, the exact df only in the band between
// the bounds) and, for accepted ones, the range weight and the film sums.
// Lanes therefore no longer idle while a neighbour of another lane goes through
// all transforms, and every pixel still sums its accepted neighbours in the
// same order (rows, then dx), so filmD is bitwise that of the per-transform
// kernel.
template <int KMAX, int TY, bool JB>
__device__ __forceinline__ void film_ring_body(const FastFilm &P, int bx, int by) {
    constexpr int NS = TY + 1;
    extern __shared__ float4 ring[];
    __shared__ int s_nmin, s_nmax;
    const int R = P.R, hw = kTX2 + 2 * R, hh = TY + 2 * R;
    const int K = P.K, nf = P.feat.nch;
    const int nrec = kRingFW + 1 + 2 * K;
    const int x0 = bx * kTX2, y0 = by * TY;
    const int t = threadIdx.x, lx = t % kTX2, tr = t / kTX2;
    const int x = x0 + lx, y = y0 + tr;
    const bool in = x < P.W && y < P.H;
    const size_t HW = (size_t)P.W * P.H;
    const size_t gi = in ? (size_t)y * P.W + x : 0;

    if (t == 0) {
        s_nmin = 0x7fffffff;
        s_nmax = 0;
    }
    __syncthreads();
    {
        // range of the valid counts in the halo: uniform counts share one pair of df bounds
        int lmin = 0x7fffffff, lmax = 0;
        for (int idx = t; idx < hw * hh; idx += blockDim.x) {
            const int hy = idx / hw, hx = idx - hy * hw;
            const int gx = x0 - R + hx, gy = y0 - R + hy;
            if (gx >= 0 && gx < P.W && gy >= 0 && gy < P.H) {
                const int v = __ldg(P.n + (size_t)gy * P.W + gx);
                if (v >= 2) {
                    lmin = min(lmin, v);
                    lmax = max(lmax, v);
                }
            }
        }
        atomicMin(&s_nmin, lmin);
        atomicMax(&s_nmax, lmax);
    }
    auto value = [&](int rec, int col, int hrow) { return film_ring_value(P, rec, col, hrow, x0, y0); };
    const bool pipelined = nrec * hw <= kRingPer * (int)blockDim.x;
    float4 pend[kRingPer];
    for (int hrow = 0; hrow < TY; hrow++) ring_load_now(ring, hrow % NS, hrow, hw, nrec, value);

    int ni = in ? __ldg(P.n + gi) : 0;
    if (ni < 2) ni = 0;
    const bool act = in && ni >= 2;
    // slots hold the transforms in test order; ksel is the slot of the JB choice
    int ksel = -1;
    if (JB && act) {
        int kbest = 0;
        float best = __ldg(P.jb[0] + gi);
        for (int k = 1; k < K; k++) {
            const float v = __ldg(P.jb[k] + gi);
            if (v < best) {
                best = v;
                kbest = k;
            }
        }
        for (int sl = 0; sl < K; sl++)
            if (P.order[sl] == kbest) ksel = sl;
    }
    float fi[kRingMF];
#pragma unroll
    for (int f = 0; f < kRingMF; f++) fi[f] = (in && f < nf) ? __fmul_rn(__ldg(P.feat.plane[f] + gi), P.feat.mul[f]) : 0.f;
    float mi[KMAX][3], di[KMAX][3];
#pragma unroll
    for (int sl = 0; sl < KMAX; sl++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const bool ok = in && sl < K;
            const int k = ok ? P.order[sl] : 0;
            const float *mean = k == 0 ? P.film : P.mean[k];
            mi[sl][c] = ok ? __ldg(mean + (size_t)c * HW + gi) : 0.f;
            di[sl][c] = ok ? __ldg(P.discr[k] + (size_t)c * HW + gi) : 0.f;
        }
    // the slot pass A tests and its centre values
    const int slotA = JB ? max(ksel, 0) : 0;
    float mA[3], dA[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        mA[c] = mi[0][c];
        dA[c] = di[0][c];
        if (JB) {
#pragma unroll
            for (int sl = 1; sl < KMAX; sl++)
                if (sl == slotA) {
                    mA[c] = mi[sl][c];
                    dA[c] = di[sl][c];
                }
        }
    }
    __syncthreads();
    const bool uni = s_nmin == s_nmax;
    float tlo_u = 0.f, thi_u = 0.f;
    if (uni) {
        const int dfl = 2 * s_nmin - 2, dfh = s_nmin - 1;
        tlo_u = dfl > kDfMax ? P.z2lo : __ldg(P.tlo + dfl);
        thi_u = __ldg(P.thi + (dfh > kDfMax ? kDfMax : dfh));
    }
    auto bounds = [&](int nj, float &tlo, float &thi) {
        tlo = tlo_u;
        thi = thi_u;
        if (!uni) {
            const int njc = max(nj, 2);
            const int dfl = ni + njc - 2, dfh = min(ni, njc) - 1;
            tlo = dfl > kDfMax ? P.z2lo : __ldg(P.tlo + dfl);
            thi = __ldg(P.thi + (dfh > kDfMax ? kDfMax : dfh));
        }
    };

    float sw = 0.f, sf[3] = {0.f, 0.f, 0.f};
    for (int r = -R; r <= R; r++) {
        const int next = R + r + TY;
        if (next < hh) {
            if (pipelined)
                ring_fetch(pend, next, hw, nrec, value);
            else
                ring_load_now(ring, next % NS, next, hw, nrec, value);
        }
        if (act) {
            const float4 *rp = ring + (size_t)((tr + R + r) % NS) * nrec * hw + lx + R;
            // pass A: the upper-bound test of slot A for every neighbour of the row
            uint64_t cand = 0;
            {
                const float4 *ap = rp + (size_t)(kRingFW + 1 + 2 * slotA) * hw;
                for (int dx = -R; dx <= R; dx++) {
                    float thi = thi_u;
                    if (!uni) {
                        float tlo;
                        bounds((int)rp[hw + dx].w, tlo, thi);
                    }
                    const float4 T0 = ap[dx], T1 = ap[hw + dx];
                    const float mj[3] = {T0.x, T0.y, T0.z}, dj[3] = {T0.w, T1.x, T1.y};
                    bool hi = true;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float diff = mA[c] - mj[c];
                        const float sv = dA[c] + dj[c];
                        hi = hi && diff * diff <= thi * sv;
                    }
                    cand |= (uint64_t)hi << (dx + R);
                }
            }
            if (r == 0) cand |= 1ull << R;  // the centre is always kept
            // pass B: the lane's survivors, in increasing dx
            const float sdy = __fmul_rn(P.ds2, (float)(r * r));
            while (cand) {
                const int dx = __ffsll((long long)cand) - 1 - R;
                cand &= cand - 1;
                const float4 F1 = rp[hw + dx];
                const int nj = (int)F1.w;
                bool a = nj >= 2;
                float tlo, thi;
                bounds(nj, tlo, thi);
#pragma unroll
                for (int k = 0; k < KMAX; k++) {
                    if (k >= K) break;
                    if (!a || (JB && ksel != k)) continue;
                    const float4 *tp = rp + (size_t)(kRingFW + 1 + 2 * k) * hw + dx;
                    const float4 T0 = tp[0], T1 = tp[hw];
                    const float mj[3] = {T0.x, T0.y, T0.z}, dj[3] = {T0.w, T1.x, T1.y};
                    // qq <= tlo s accepts, qq > thi s rejects, in between the exact df decides
                    bool acc = true, amb = false;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float diff = mi[k][c] - mj[c];
                        const float sv = di[k][c] + dj[c];
                        const float qq = diff * diff;
                        const bool lo = qq <= tlo * sv;
                        const bool hi = qq <= thi * sv;
                        acc = acc && hi;
                        amb = amb || (hi && !lo);
                    }
                    if (acc && amb) {
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const float diff = mi[k][c] - mj[c];
                            const float sv = di[k][c] + dj[c];
                            const float qq = diff * diff;
                            if (!(qq <= tlo * sv) && qq <= thi * sv)
                                acc = acc && welch_exact(diff, di[k][c], dj[c], ni, nj, P.lut, P.lut_n);
                        }
                    }
                    a = acc;
                }
                if (dx == 0 && r == 0) a = true;
                if (a) {
                    const float4 F0 = rp[dx];
                    const float fj[kRingMF] = {F0.x, F0.y, F0.z, F0.w, F1.x, F1.y, F1.z};
                    float e = fmaf(P.ds2, (float)(dx * dx), sdy);
#pragma unroll
                    for (int f = 0; f < kRingMF; f++) {
                        if (f < nf) {
                            const float d = fi[f] - fj[f];
                            e = fmaf(-d, d, e);
                        }
                    }
                    const float wt = fast_exp2(e);
                    const float4 Fm = rp[(size_t)kRingFW * hw + dx];
                    sw += wt;
                    sf[0] = fmaf(wt, Fm.x, sf[0]);
                    sf[1] = fmaf(wt, Fm.y, sf[1]);
                    sf[2] = fmaf(wt, Fm.z, sf[2]);
                }
            }
        }
        if (pipelined && next < hh) ring_store(pend, ring, next % NS, hw, nrec);
        __syncthreads();
    }
    if (!in) return;
    if (!act) {
        for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + gi] = __ldg(P.film + (size_t)c * HW + gi);
        return;
    }
#pragma unroll
    for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + gi] = sf[c] / sw;
}

template <int KMAX, int TY, bool JB>
__global__ void __launch_bounds__(kTX2 *TY, 16 / TY) film_ring_f32(FastFilm P) {
    film_ring_body<KMAX, TY, JB>(P, blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct DfTables {
    float *lo = nullptr, *hi = nullptr;
    float z2lo = 0.f;
};
std::mutex g_df_mutex;
std::map<std::pair<int, double>, DfTables> g_df_tables;

// t2 at integer df from the u-table (same interpolation as the test), widened
// by 1e-5 relative so that the bounds never exclude a value the exact branch
// could produce.
const DfTables *df_tables(double alpha, cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_df_mutex);
    DfTables &t = g_df_tables[std::make_pair(dev, alpha)];
    if (!t.lo) {
        const int N = tcrit_intervals();
        std::vector<double> lut(N + 1);
        stater_tcrit2_table(alpha, lut.data());
        auto interp = [&](double u) {
            if (u > 1.0) u = 1.0;
            const double f = u * N;
            int m = (int)f;
            if (m > N - 1) m = N - 1;
            return lut[m] + (f - m) * (lut[m + 1] - lut[m]);
        };
        std::vector<float> lo(kDfMax + 1), hi(kDfMax + 1);
        for (int df = 0; df <= kDfMax; df++) {
            const double v = interp(df < 1 ? 1.0 : 1.0 / df);
            lo[df] = (float)(v * (1.0 - 1e-5));
            hi[df] = (float)(v * (1.0 + 1e-5));
        }
        t.z2lo = (float)(lut[0] * (1.0 - 1e-5));
        if (cudaMalloc(&t.lo, sizeof(float) * lo.size()) != cudaSuccess ||
            cudaMalloc(&t.hi, sizeof(float) * hi.size()) != cudaSuccess) {
            cudaGetLastError();
            t.lo = t.hi = nullptr;
            return nullptr;
        }
        cudaMemcpy(t.lo, lo.data(), sizeof(float) * lo.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(t.hi, hi.data(), sizeof(float) * hi.size(), cudaMemcpyHostToDevice);
    }
    (void)s;
    return &t;
}

size_t vars_smem(int R, int nf, bool levc, bool zpix, int RB, int TR) {
    const size_t A = (size_t)(kTX2 + 2 * R) * (RB * TR + 2 * R);
    return A * sizeof(float) * (1 + nf + 6 + (zpix ? 1 : 3) + (levc ? 3 : 0));
}

size_t film_smem(int R, int nf, int RB, int TR) {
    const size_t A = (size_t)(kTX2 + 2 * R) * (RB * TR + 2 * R);
    const int D = 2 * R + 1, wpr = (D + 31) / 32;
    return (size_t)RB * D * wpr * kTX2 * TR * 4 + A * sizeof(float) * (1 + nf + 6);
}

// Tile shapes tried in order (the preferred one first, then smaller ones for large radii).
constexpr int kTileCfg[3][2] = {{STATER_TILE_RB, STATER_TILE_TR}, {1, 4}, {1, 2}};

constexpr size_t kSmemLimit = 227 * 1024;

int mf_bucket(int nf) { return nf == 0 ? 0 : nf <= 4 ? 4 : nf <= 8 ? 8 : nf <= 16 ? 16 : 24; }

// Row-ring kernels: up to 5 transforms and kRingMF feature channels; TY = 8
// output rows per tile when the ring fits two CTAs per SM, else TY = 4.
constexpr size_t kRingSmemMax = 113 * 1024;

int ring_kmax(int K) { return K <= 1 ? 1 : K <= 3 ? 3 : K <= 5 ? 5 : 0; }

size_t ring_smem(int R, int nrec, int TY) { return (size_t)(TY + 1) * nrec * (kTX2 + 2 * R) * sizeof(float4); }
// stater_debug_set_vars_ring_form: a forced tile height of the variance ring
// (0: the tuner's; -1: the per-transform kernel instead of the ring)
std::atomic<int> g_vars_form{0};

int ring_ty(int R, int nrec) {
    if (ring_smem(R, nrec, 8) <= kRingSmemMax) return 8;
    if (ring_smem(R, nrec, 4) <= kRingSmemMax) return 4;
    return 0;
}

// ---------------------------------------------------------------------------
// Tile-height autotuner of the row-ring filters. The tile height TY trades the
// halo rows a CTA streams per output row ((TY + 2R) / TY) against occupancy (a
// TY = 16 ring takes one CTA per SM; TY = 4 and 8 take two). The best choice
// depends on the radius, the transform count and the image size (small images
// have few tiles per SM), so the first call of each shape class times every
// height whose ring fits in shared memory (4, 8, 16), with CUDA events on the
// call's own stream, and caches the fastest per device. Results do not depend
// on TY (every pixel sums its neighbours in the same order), so tuning changes
// speed only. Calls made while their stream is being captured into a graph,
// or with the autotuner switched off (stater_set_autotune), use the default
// height (8 where two CTAs fit per SM, else 4).
// ---------------------------------------------------------------------------
struct TuneKey {
    int dev, filter, km, nrec, R, variant, size_class;
    bool operator<(const TuneKey &o) const {
        return std::tie(dev, filter, km, nrec, R, variant, size_class) <
               std::tie(o.dev, o.filter, o.km, o.nrec, o.R, o.variant, o.size_class);
    }
};
std::mutex g_tune_mutex;
std::map<TuneKey, int> g_tuned;
std::atomic<int> g_autotune{1};

int size_class(size_t px) { return px <= ((size_t)1 << 18) ? 0 : px <= ((size_t)1 << 20) ? 1 : 2; }

bool ring_fits(int R, int nrec, int ty) { return ring_smem(R, nrec, ty) <= kSmemLimit; }

bool stream_capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
        cudaGetLastError();
        return true;  // cannot tell: do not synchronise
    }
    return st != cudaStreamCaptureStatusNone;
}

// The cached height of a shape class, else the default (never tunes, never
// synchronises).
int cached_ring_ty(int filter, int km, int nrec, int R, int variant, size_t px) {
    int dev = 0;
    cudaGetDevice(&dev);
    const TuneKey key{dev, filter, km, nrec, R, variant, size_class(px)};
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tuned.find(key);
    return it != g_tuned.end() ? it->second : ring_ty(R, nrec);
}

// launch(ty) enqueues the filter with tile height ty on s and returns its error.
template <typename LaunchFn>
int pick_ring_ty(int filter, int km, int nrec, int R, int variant, size_t px, cudaStream_t s, LaunchFn launch) {
    int dev = 0;
    cudaGetDevice(&dev);
    const TuneKey key{dev, filter, km, nrec, R, variant, size_class(px)};
    {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) return it->second;
    }
    const int def = ring_ty(R, nrec);
    if (!g_autotune.load() || stream_capturing(s)) return def;
    int cands[3], nc = 0;
    for (int ty : {4, 8, 16})
        if (ring_fits(R, nrec, ty)) cands[nc++] = ty;
    int best = def;
    if (nc > 1) {
        float best_ms = 1e30f;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int i = 0; i < nc; i++) {
            if (launch(cands[i]) != cudaSuccess) {  // warm-up (shared-memory attribute, caches)
                cudaGetLastError();
                continue;
            }
            cudaEventRecord(e0, s);
            launch(cands[i]);
            cudaEventRecord(e1, s);
            float ms = 1e30f;
            if (cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
            cudaGetLastError();
            if (ms < best_ms) {
                best_ms = ms;
                best = cands[i];
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_tuned[key] = best;
    return best;
}

template <typename KernelT>
cudaError_t set_smem(KernelT kern, size_t bytes) {
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

// Frees the df-bound tables of device `dev` (stater_release_cache).
void df_tables_release(int dev) {
    std::lock_guard<std::mutex> lk(g_df_mutex);
    for (auto it = g_df_tables.begin(); it != g_df_tables.end();) {
        if (it->first.first == dev) {
            cudaFree(it->second.lo);
            cudaFree(it->second.hi);
            it = g_df_tables.erase(it);
        } else {
            ++it;
        }
    }
}

// Kernel parameters of one FP32 denoiseVars call (scratch pointers s2 / s2c
// left to the caller).
stater_status fill_fast_vars(const stater_denoise_vars_args *a, FastVars &P) {
    P.W = a->width;
    P.H = a->height;
    P.K = a->n_buffers;
    P.R = a->filter_radius;
    P.max_moment = a->max_moment;
    P.levc = (a->max_moment >= 5 || a->m2C_in) ? 1 : 0;
    P.ds2 = a->ds_factor * kLog2e;
    P.z = a->var_z;
    P.z2 = a->var_z * a->var_z;
    P.n = a->n;
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        P.m2[k] = (const float *)a->m2[k];
        P.m3[k] = (const float *)a->m3[k];
        P.m4[k] = (const float *)a->m4[k];
        P.cx[k] = (const float *)a->c2X[k];
        P.cy[k] = (const float *)a->c2Y[k];
        P.jb[k] = (float *)a->jb[k];
        P.lnS2[k] = (float *)a->lnS2[k];
        P.se2[k] = (float *)a->se2[k];
        P.m2C[k] = (float *)a->m2C[k];
        P.varD[k] = (float *)a->varD[k];
        P.varCD[k] = (float *)a->varCD[k];
    }
    P.m2c_in = (const float *)a->m2C_in;
    P.s2 = P.s2c = nullptr;
    if (!make_featset(P.feat, a->gbuffers, (size_t)P.W * P.H))
        return set_error(STATER_ERR_INVALID, "stater_denoise_vars: bad gbuffers (at most 24 channels, dr_factor <= 0)");
    return STATER_OK;
}

stater_status denoise_vars_f32(const stater_denoise_vars_args *a, cudaStream_t s) {
    FastVars P;
    stater_status st = fill_fast_vars(a, P);
    if (st != STATER_OK) return st;
    const size_t HW = (size_t)P.W * P.H;
    float *scr = (float *)scratch(0, sizeof(float) * 2 * 3 * P.K * HW, s);
    if (!scr) return set_error(STATER_ERR_NOMEM, "stater_denoise_vars: scratch allocation failed");
    P.s2 = scr;
    P.s2c = scr + (size_t)3 * P.K * HW;

    dim3 g1((unsigned)((HW + 127) / 128), P.K);
    vars_stats_f32<<<g1, 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("vars_stats_f32");

    const bool zp = P.max_moment < 4;
    {
        const int km = ring_kmax(P.K);
        const int nrec = vars_ring_nrec(P.K, km, P.levc != 0, zp);
        if (km > 0 && ring_ty(P.R, nrec) > 0 && P.feat.nch <= kRingMF && g_vars_form.load() >= 0) {
            auto launch = [&](int ty) {
                cudaError_t e = cudaErrorInvalidValue;
                const size_t sm = ring_smem(P.R, nrec, ty);
                dim3 grid((P.W + kTX2 - 1) / kTX2, (P.H + ty - 1) / ty);
#define STATER_RING_VARS(LV, ZV, KV, TV)                                                   \
    if ((P.levc != 0) == LV && zp == ZV && km == KV && ty == TV) {                          \
        e = set_smem(vars_ring_f32<LV, ZV, KV, TV>, sm);                                    \
        if (e == cudaSuccess) vars_ring_f32<LV, ZV, KV, TV><<<grid, kTX2 * TV, sm, s>>>(P); \
    }
#define STATER_RING_VARS_K(LV, ZV, TV) \
    STATER_RING_VARS(LV, ZV, 1, TV) STATER_RING_VARS(LV, ZV, 3, TV) STATER_RING_VARS(LV, ZV, 5, TV)
#define STATER_RING_VARS_T(TV)                                                                   \
    STATER_RING_VARS_K(true, true, TV) STATER_RING_VARS_K(true, false, TV)                        \
    STATER_RING_VARS_K(false, true, TV) STATER_RING_VARS_K(false, false, TV)
                STATER_RING_VARS_T(16)
                STATER_RING_VARS_T(8)
                STATER_RING_VARS_T(4)
#undef STATER_RING_VARS_T
#undef STATER_RING_VARS_K
#undef STATER_RING_VARS
                return e == cudaSuccess ? cudaGetLastError() : e;
            };
            const int variant = (P.levc ? 1 : 0) + (zp ? 2 : 0) + (P.feat.nch > 0 ? 4 : 0);
            int ty = pick_ring_ty(0, km, nrec, P.R, variant, HW, s, launch);
            const int forced = g_vars_form.load();
            if (forced != 0 && ring_fits(P.R, nrec, forced)) ty = forced;
            cudaError_t e = launch(ty);
            if (e != cudaSuccess) return cuda_status(e, "vars_ring_f32");
            return STATER_OK;
        }
    }
    int cfg = 0;
    while (cfg < 3 && vars_smem(P.R, P.feat.nch, P.levc != 0, zp, kTileCfg[cfg][0], kTileCfg[cfg][1]) > kSmemLimit) cfg++;
    if (cfg == 3) return set_error(STATER_ERR_UNSUPPORTED, "stater_denoise_vars: radius too large for FP32 tiles");
    const int RB = kTileCfg[cfg][0], TR = kTileCfg[cfg][1];
    const size_t sm = vars_smem(P.R, P.feat.nch, P.levc != 0, zp, RB, TR);
    dim3 grid((P.W + kTX2 - 1) / kTX2, (P.H + RB * TR - 1) / (RB * TR));
    const int mf = mf_bucket(P.feat.nch);
    cudaError_t e = cudaSuccess;
#define STATER_VARS_LAUNCH(LV, ZV, MFV, RBV, TRV)                                                      \
    if ((P.levc != 0) == LV && zp == ZV && mf == MFV && RB == RBV && TR == TRV) {                      \
        e = set_smem(vars_filter_f32<LV, ZV, MFV, RBV, TRV>, sm);                                      \
        if (e == cudaSuccess) vars_filter_f32<LV, ZV, MFV, RBV, TRV><<<grid, kTX2 * TRV, sm, s>>>(P);  \
    }
#define STATER_VARS_LAUNCH_M(LV, ZV, RBV, TRV)                                                          \
    STATER_VARS_LAUNCH(LV, ZV, 0, RBV, TRV) STATER_VARS_LAUNCH(LV, ZV, 4, RBV, TRV)                      \
    STATER_VARS_LAUNCH(LV, ZV, 8, RBV, TRV) STATER_VARS_LAUNCH(LV, ZV, 16, RBV, TRV)                     \
    STATER_VARS_LAUNCH(LV, ZV, 24, RBV, TRV)
#define STATER_VARS_LAUNCH_T(RBV, TRV)                                                                  \
    STATER_VARS_LAUNCH_M(true, false, RBV, TRV) STATER_VARS_LAUNCH_M(false, false, RBV, TRV)             \
    STATER_VARS_LAUNCH_M(true, true, RBV, TRV) STATER_VARS_LAUNCH_M(false, true, RBV, TRV)
    STATER_VARS_LAUNCH_T(STATER_TILE_RB, STATER_TILE_TR)
    if (cfg == 1) { STATER_VARS_LAUNCH_T(1, 4) }
    if (cfg == 2) { STATER_VARS_LAUNCH_T(1, 2) }
#undef STATER_VARS_LAUNCH_T
#undef STATER_VARS_LAUNCH_M
#undef STATER_VARS_LAUNCH
    if (e != cudaSuccess) return cuda_status(e, "vars_filter_f32 smem attribute");
    STATER_CHECK_LAUNCH("vars_filter_f32");
    return STATER_OK;
}

// Kernel parameters of one FP32 denoiseFilm call, tables included.
stater_status fill_fast_film(const stater_denoise_film_args *a, FastFilm &P, cudaStream_t s) {
    P.W = a->width;
    P.H = a->height;
    P.K = a->n_buffers;
    P.R = a->filter_radius;
    P.mt_mode = a->mt_mode;
    P.use_levc = a->use_levc;
    P.discr_source = a->discr_source;
    P.lut_n = tcrit_intervals();
    P.ds2 = a->ds_factor * kLog2e;
    P.n = a->n;
    P.film = (const float *)a->film;
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        P.mean[k] = (const float *)a->mean[k];
        P.var[k] = (const float *)(a->discr_source == STATER_DISCR_SAMPLE ? (a->use_levc ? a->m2C[k] : a->m2[k])
                                                                          : (a->use_levc ? a->varCD[k] : a->varD[k]));
        P.jb[k] = (const float *)a->jb[k];
        P.discr[k] = (float *)a->discr[k];
    }
    P.filmD = (float *)a->filmD;
    P.bits = a->accept_bits;
    {
        // a permutation of 0..K-1, else the reverse index order
        bool seen[STATER_MAX_TRANSFORMS] = {false}, perm = true, zero = true;
        for (int sl = 0; sl < P.K; sl++) {
            const int k = a->test_order[sl];
            if (k != 0) zero = false;
            if (k < 0 || k >= P.K || seen[k]) perm = false;
            else seen[k] = true;
        }
        if (!perm && !zero)
            return set_error(STATER_ERR_INVALID, "stater_denoise_film: test_order is not a permutation");
        for (int sl = 0; sl < STATER_MAX_TRANSFORMS; sl++)
            P.order[sl] = (int8_t)(sl < P.K ? (perm && !(zero && P.K > 1) ? a->test_order[sl] : P.K - 1 - sl) : 0);
    }
    const size_t HW = (size_t)P.W * P.H;
    if (!make_featset(P.feat, a->gbuffers, HW))
        return set_error(STATER_ERR_INVALID, "stater_denoise_film: bad gbuffers (at most 24 channels, dr_factor <= 0)");
    P.lut = (const float *)tcrit_table_device((double)a->alpha, false, s);
    const DfTables *dt = df_tables((double)a->alpha, s);
    if (!P.lut || !dt) return set_error(STATER_ERR_NOMEM, "stater_denoise_film: table allocation failed");
    P.tlo = dt->lo;
    P.thi = dt->hi;
    P.z2lo = dt->z2lo;
    return STATER_OK;
}

stater_status denoise_film_f32(const stater_denoise_film_args *a, cudaStream_t s) {
    FastFilm P;
    stater_status st = fill_fast_film(a, P, s);
    if (st != STATER_OK) return st;
    const size_t HW = (size_t)P.W * P.H;

    dim3 g1((unsigned)((HW + 127) / 128), P.K);
    film_discr_f32<<<g1, 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("film_discr_f32");

    {
        const int km = ring_kmax(P.K);
        const int nrec = kRingFW + 1 + 2 * P.K;
        if (km > 0 && ring_ty(P.R, nrec) > 0 && P.feat.nch <= kRingMF && !P.bits) {
            const bool jb = P.mt_mode == STATER_MT_JB;
            auto launch = [&](int ty) {
                const size_t sm = ring_smem(P.R, nrec, ty);
                dim3 grid((P.W + kTX2 - 1) / kTX2, (P.H + ty - 1) / ty);
                cudaError_t e = cudaErrorInvalidValue;
#define STATER_RING_FILM(KV, TV, JV)                                                          \
    if (km == KV && ty == TV && jb == JV) {                                                    \
        e = set_smem(film_ring_f32<KV, TV, JV>, sm);                                           \
        if (e == cudaSuccess) film_ring_f32<KV, TV, JV><<<grid, kTX2 * TV, sm, s>>>(P);        \
    }
#define STATER_RING_FILM_T(TV, JV) STATER_RING_FILM(1, TV, JV) STATER_RING_FILM(3, TV, JV) STATER_RING_FILM(5, TV, JV)
                STATER_RING_FILM_T(16, false) STATER_RING_FILM_T(8, false) STATER_RING_FILM_T(4, false)
                STATER_RING_FILM_T(16, true) STATER_RING_FILM_T(8, true) STATER_RING_FILM_T(4, true)
#undef STATER_RING_FILM_T
#undef STATER_RING_FILM
                return e == cudaSuccess ? cudaGetLastError() : e;
            };
            const int variant = (jb ? 1 : 0) + (P.feat.nch > 0 ? 4 : 0);
            const int ty = pick_ring_ty(1, km, nrec, P.R, variant, HW, s, launch);
            cudaError_t e = launch(ty);
            if (e != cudaSuccess) return cuda_status(e, "film_ring_f32");
            return STATER_OK;
        }
    }
    int cfg = 0;
    while (cfg < 3 && film_smem(P.R, P.feat.nch, kTileCfg[cfg][0], kTileCfg[cfg][1]) > kSmemLimit) cfg++;
    if (cfg == 3) return set_error(STATER_ERR_UNSUPPORTED, "stater_denoise_film: radius too large for FP32 tiles");
    const int RB = kTileCfg[cfg][0], TR = kTileCfg[cfg][1];
    const size_t sm = film_smem(P.R, P.feat.nch, RB, TR);
    dim3 grid((P.W + kTX2 - 1) / kTX2, (P.H + RB * TR - 1) / (RB * TR));
    const int mf = mf_bucket(P.feat.nch);
    cudaError_t e = cudaSuccess;
#define STATER_FILM_LAUNCH(MFV, RBV, TRV)                                                    \
    if (mf == MFV && RB == RBV && TR == TRV) {                                               \
        e = set_smem(film_filter_f32<MFV, RBV, TRV>, sm);                                    \
        if (e == cudaSuccess) film_filter_f32<MFV, RBV, TRV><<<grid, kTX2 * TRV, sm, s>>>(P); \
    }
#define STATER_FILM_LAUNCH_T(RBV, TRV)                                                              \
    STATER_FILM_LAUNCH(0, RBV, TRV) STATER_FILM_LAUNCH(4, RBV, TRV) STATER_FILM_LAUNCH(8, RBV, TRV) \
    STATER_FILM_LAUNCH(16, RBV, TRV) STATER_FILM_LAUNCH(24, RBV, TRV)
    STATER_FILM_LAUNCH_T(STATER_TILE_RB, STATER_TILE_TR)
    if (cfg == 1) { STATER_FILM_LAUNCH_T(1, 4) }
    if (cfg == 2) { STATER_FILM_LAUNCH_T(1, 2) }
#undef STATER_FILM_LAUNCH_T
#undef STATER_FILM_LAUNCH
    if (e != cudaSuccess) return cuda_status(e, "film_filter_f32 smem attribute");
    STATER_CHECK_LAUNCH("film_filter_f32");
    return STATER_OK;
}

}  // namespace stater

extern "C" stater_status stater_set_autotune(int32_t enable) {
    using namespace stater;
    clear_error();
    if (enable != 0 && enable != 1) return set_error(STATER_ERR_INVALID, "stater_set_autotune: 0 or 1");
    g_autotune.store(enable);
    if (!enable) {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        g_tuned.clear();
    }
    return STATER_OK;
}

extern "C" int32_t stater_tuned_tile_height(int32_t filter, int32_t n_transforms, int32_t width, int32_t height,
                                            int32_t filter_radius) {
    using namespace stater;
    int dev = 0;
    cudaGetDevice(&dev);
    const int km = ring_kmax(n_transforms);
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    for (const auto &kv : g_tuned)
        if (kv.first.dev == dev && kv.first.filter == filter && kv.first.km == km && kv.first.R == filter_radius &&
            kv.first.size_class == size_class((size_t)width * height) &&
            kv.first.nrec == (filter == 1 ? kRingFW + 1 + 2 * n_transforms : kv.first.nrec))
            return kv.second;
    return 0;
}

extern "C" stater_status stater_debug_set_vars_ring_form(int32_t tile_height) {
    using namespace stater;
    clear_error();
    if (!(tile_height == -1 || tile_height == 0 || tile_height == 4 || tile_height == 8 || tile_height == 16))
        return set_error(STATER_ERR_INVALID, "stater_debug_set_vars_ring_form: tile height not -1, 0, 4, 8 or 16");
    g_vars_form.store(tile_height);
    return STATER_OK;
}

extern "C" stater_status stater_test_order(const stater_transform *transforms, int32_t n_transforms,
                                           int32_t *order) {
    using namespace stater;
    clear_error();
    if (!transforms || !order || n_transforms < 1 || n_transforms > STATER_MAX_TRANSFORMS)
        return set_error(STATER_ERR_INVALID, "stater_test_order: bad arguments");
    auto rank = [&](int k) {
        if (k == 0) return 100;  // the untransformed set last
        // measured on the benchmark's radiance (means around 0.4): the strongly
        // compressing transforms reject first; log1p is nearly linear there
        const float lam = transforms[k].lambda;
        switch (transforms[k].kind) {
            case STATER_TK_ASINH: return 0;
            case STATER_TK_CBRT: return 1;
            case STATER_TK_BOXCOX: return lam < 0.5f ? 1 : (lam < 1.f ? 2 : 5);
            case STATER_TK_SQRT: return 2;
            case STATER_TK_LOG1P: return 3;
            default: return 6;
        }
    };
    int idx[STATER_MAX_TRANSFORMS];
    for (int k = 0; k < n_transforms; k++) idx[k] = k;
    // stable insertion sort by rank, then by descending index
    for (int i = 1; i < n_transforms; i++) {
        const int v = idx[i];
        int j = i - 1;
        while (j >= 0 && (rank(idx[j]) > rank(v) || (rank(idx[j]) == rank(v) && idx[j] < v))) {
            idx[j + 1] = idx[j];
            j--;
        }
        idx[j + 1] = v;
    }
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) order[k] = k < n_transforms ? idx[k] : 0;
    return STATER_OK;
}


// ---------------------------------------------------------------------------
// Batches: many small images through one launch per stage.
//
// A small image (256x256 is 256 ring tiles of 32x8) fills a fraction of the
// GPU and pays a launch and a tail per stage. A batch runs the jobs' stages
// together: every job's accumulation (with the film sums) and film image on
// one stream, then each denoise stage as ONE launch covering the tiles of all
// jobs that share a kernel instantiation (transform-count class, LEV / moment
// variant, multi-transform mode, radius): a CTA finds its job by binary search
// over the per-job tile offsets and runs the same tile code as the
// single-image kernels, so each job's results are bitwise those of its
// single-image calls. The first run of a batch tunes each class's tile height
// on the real data and then records the whole sequence into a CUDA graph;
// later runs replay the graph (one launch for the host). The serving engine
// uses the same tables for one-shot groups of small jobs, allocated and freed
// in stream order (batch_denoise_once).
// ---------------------------------------------------------------------------
namespace stater {
namespace {

__device__ __forceinline__ int batch_job(const int *__restrict__ start, int njobs, int t) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(start + mid) <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// start[j]: first block of job j (blocks of 128 pixels), start[njobs] = total
__global__ void vars_stats_batch(const FastVars *__restrict__ jobs, const int *__restrict__ start, int njobs) {
    const int j = batch_job(start, njobs, blockIdx.x);
    const FastVars &P = jobs[j];
    if ((int)blockIdx.y >= P.K) return;
    vars_stats_body(P, (size_t)(blockIdx.x - __ldg(start + j)) * blockDim.x + threadIdx.x, blockIdx.y);
}

__global__ void film_discr_batch(const FastFilm *__restrict__ jobs, const int *__restrict__ start, int njobs) {
    const int j = batch_job(start, njobs, blockIdx.x);
    const FastFilm &P = jobs[j];
    if ((int)blockIdx.y >= P.K) return;
    film_discr_body(P, (size_t)(blockIdx.x - __ldg(start + j)) * blockDim.x + threadIdx.x, blockIdx.y);
}

// The CTA's job parameters, copied from the job table into shared memory: the
// ring bodies read them from there as the single-image kernels read theirs
// from the parameter space, rather than keeping global-memory copies of them
// in registers (which spilled).
template <typename Params>
__device__ __forceinline__ void load_job_params(const Params *__restrict__ src, Params &dst) {
    static_assert(sizeof(Params) % 4 == 0, "parameter block of whole words");
    const int *s = reinterpret_cast<const int *>(src);
    int *d = reinterpret_cast<int *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(Params) / 4); i += blockDim.x) d[i] = __ldg(s + i);
    __syncthreads();
}

// jobs: the class's jobs only; start[j]: first ring tile of job j
template <bool LEVC, bool ZPIX, int KMAX, int TY>
__global__ void __launch_bounds__(kTX2 *TY) vars_ring_batch(const FastVars *__restrict__ jobs,
                                                            const int *__restrict__ start, int njobs) {
    __shared__ FastVars P;
    const int j = batch_job(start, njobs, blockIdx.x);
    load_job_params(jobs + j, P);
    const int tx = (P.W + kTX2 - 1) / kTX2, local = blockIdx.x - __ldg(start + j);
    vars_ring_body<LEVC, ZPIX, KMAX, TY>(P, local % tx, local / tx);
}

template <int KMAX, int TY, bool JB>
__global__ void __launch_bounds__(kTX2 *TY, 16 / TY) film_ring_batch(const FastFilm *__restrict__ jobs,
                                                                    const int *__restrict__ start, int njobs) {
    __shared__ FastFilm P;
    const int j = batch_job(start, njobs, blockIdx.x);
    load_job_params(jobs + j, P);
    const int tx = (P.W + kTX2 - 1) / kTX2, local = blockIdx.x - __ldg(start + j);
    film_ring_body<KMAX, TY, JB>(P, local % tx, local / tx);
}

constexpr int kTys[3] = {4, 8, 16};
int ty_index(int ty) { return ty == 4 ? 0 : ty == 8 ? 1 : 2; }

// Jobs of one ring instantiation, with the tile offsets of every height.
struct RingClass {
    int filter;  // 0: variance filter, 1: film filter
    int km, nrec, R;
    bool levc, zp, jb, feats;
    std::vector<int> jobs;
    size_t pixels = 0;
    int ty = 0;
    int ntiles[3] = {0, 0, 0};
    size_t off_params = 0, off_start[3] = {0, 0, 0};  // into the device block
    const void *d_params = nullptr;
    const int *d_start[3] = {nullptr, nullptr, nullptr};
};

// Host plan of a batch: parameter blocks, classes and one device block
// holding every table (built once, uploaded with one copy).
struct BatchPlan {
    std::vector<FastVars> vars;
    std::vector<FastFilm> film;
    std::vector<RingClass> classes;
    std::vector<unsigned char> host;  // the device block's contents
    size_t off_vars = 0, off_film = 0, off_pix = 0, bytes = 0;
    int pix_blocks = 0, kmax = 1;
    unsigned char *dev = nullptr;
    FastVars *d_vars = nullptr;
    FastFilm *d_film = nullptr;
    const int *d_pix_start = nullptr;
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Validates the jobs and lays out the plan; s2 scratch (2 x 3 x K x HW floats
// per job) starts at s2base. Device pointers are filled by plan_bind.
stater_status plan_build(const stater_batch_job *jobs, int n, float *s2base, BatchPlan &B, bool need_acc) {
    std::vector<int> pix_start;
    B.vars.resize(n);
    B.film.resize(n);
    size_t off = 0;
    int blocks = 0;
    for (int j = 0; j < n; j++) {
        const stater_batch_job &J = jobs[j];
        const stater_accumulate_args &A = J.acc;
        if ((need_acc && (A.precision != STATER_F32 || A.mode != STATER_ACC_FAST || !A.film_contrib_sum ||
                          A.pixel_index)) ||
            J.vars.precision != STATER_F32 || J.film.precision != STATER_F32 || !J.film_rgb)
            return set_error(STATER_ERR_INVALID, "stater_batch_create: a batch runs the FP32 form with film sums, "
                                                 "film_rgb and no pixel index");
        if (J.vars.width != A.width || J.vars.height != A.height || J.film.width != A.width ||
            J.film.height != A.height || J.vars.n_buffers != A.n_transforms || J.film.n_buffers != A.n_transforms ||
            J.film.accept_bits)
            return set_error(STATER_ERR_INVALID, "stater_batch_create: the stages of a job disagree");
        stater_status st = fill_fast_vars(&J.vars, B.vars[j]);
        if (st != STATER_OK) return st;
        st = fill_fast_film(&J.film, B.film[j], nullptr);
        if (st != STATER_OK) return st;
        FastVars &V = B.vars[j];
        const size_t HW = (size_t)V.W * V.H;
        V.s2 = s2base + off;
        V.s2c = V.s2 + (size_t)3 * V.K * HW;
        off += (size_t)2 * 3 * V.K * HW;
        pix_start.push_back(blocks);
        blocks += (int)((HW + 127) / 128);
        B.kmax = std::max(B.kmax, V.K);
        const bool zp = V.max_moment < 4;
        const int kmv = ring_kmax(V.K), nrv = vars_ring_nrec(V.K, kmv, V.levc != 0, zp);
        const FastFilm &F = B.film[j];
        const int nrf = kRingFW + 1 + 2 * F.K;
        if (!(kmv > 0 && ring_ty(V.R, nrv) > 0 && V.feat.nch <= kRingMF && ring_ty(F.R, nrf) > 0 &&
              F.feat.nch <= kRingMF))
            return set_error(STATER_ERR_UNSUPPORTED, "stater_batch_create: a job needs more than 5 transforms, 7 "
                                                     "feature channels or more than the ring's shared memory");
        for (int f = 0; f < 2; f++) {
            RingClass key;
            key.filter = f;
            key.km = kmv;
            key.nrec = f == 0 ? nrv : nrf;
            key.R = f == 0 ? V.R : F.R;
            key.levc = f == 0 && V.levc;
            key.zp = f == 0 && zp;
            key.jb = f == 1 && F.mt_mode == STATER_MT_JB;
            key.feats = (f == 0 ? V.feat.nch : F.feat.nch) > 0;
            RingClass *found = nullptr;
            for (auto &c : B.classes)
                if (c.filter == key.filter && c.km == key.km && c.nrec == key.nrec && c.R == key.R &&
                    c.levc == key.levc && c.zp == key.zp && c.jb == key.jb && c.feats == key.feats)
                    found = &c;
            if (!found) {
                B.classes.push_back(key);
                found = &B.classes.back();
            }
            found->jobs.push_back(j);
            found->pixels += HW;
        }
    }
    pix_start.push_back(blocks);
    B.pix_blocks = blocks;
    // device block: job tables, pixel offsets, per class parameter blocks and tile offsets
    size_t o = 0;
    auto take = [&](size_t b) {
        o = align_up(o, 256);
        const size_t r = o;
        o += b;
        return r;
    };
    B.off_vars = take(sizeof(FastVars) * n);
    B.off_film = take(sizeof(FastFilm) * n);
    B.off_pix = take(sizeof(int) * pix_start.size());
    std::vector<std::vector<int>> starts;
    for (auto &c : B.classes) {
        const size_t sz = c.filter == 0 ? sizeof(FastVars) : sizeof(FastFilm);
        c.off_params = take(sz * c.jobs.size());
        for (int t = 0; t < 3; t++) {
            std::vector<int> st;
            int total = 0;
            for (int j : c.jobs) {
                st.push_back(total);
                const int W = c.filter == 0 ? B.vars[j].W : B.film[j].W, H = c.filter == 0 ? B.vars[j].H : B.film[j].H;
                total += ((W + kTX2 - 1) / kTX2) * ((H + kTys[t] - 1) / kTys[t]);
            }
            st.push_back(total);
            c.ntiles[t] = total;
            c.off_start[t] = take(sizeof(int) * st.size());
            starts.push_back(st);
        }
    }
    B.bytes = align_up(o, 256);
    B.host.assign(B.bytes, 0);
    std::memcpy(B.host.data() + B.off_vars, B.vars.data(), sizeof(FastVars) * n);
    std::memcpy(B.host.data() + B.off_film, B.film.data(), sizeof(FastFilm) * n);
    std::memcpy(B.host.data() + B.off_pix, pix_start.data(), sizeof(int) * pix_start.size());
    size_t si = 0;
    for (auto &c : B.classes) {
        const size_t sz = c.filter == 0 ? sizeof(FastVars) : sizeof(FastFilm);
        for (size_t i = 0; i < c.jobs.size(); i++)
            std::memcpy(B.host.data() + c.off_params + i * sz,
                        c.filter == 0 ? (const void *)&B.vars[c.jobs[i]] : (const void *)&B.film[c.jobs[i]], sz);
        for (int t = 0; t < 3; t++, si++)
            std::memcpy(B.host.data() + c.off_start[t], starts[si].data(), sizeof(int) * starts[si].size());
    }
    return STATER_OK;
}

void plan_bind(BatchPlan &B, unsigned char *dev) {
    B.dev = dev;
    B.d_vars = (FastVars *)(dev + B.off_vars);
    B.d_film = (FastFilm *)(dev + B.off_film);
    B.d_pix_start = (const int *)(dev + B.off_pix);
    for (auto &c : B.classes) {
        c.d_params = dev + c.off_params;
        for (int t = 0; t < 3; t++) c.d_start[t] = (const int *)(dev + c.off_start[t]);
    }
}

cudaError_t launch_ring_class(const RingClass &c, int ty, cudaStream_t s) {
    const int t = ty_index(ty);
    const int total = c.ntiles[t];
    const int *start = c.d_start[t];
    const size_t sm = ring_smem(c.R, c.nrec, ty);
    const int nj = (int)c.jobs.size();
    cudaError_t e = cudaErrorInvalidValue;
    if (c.filter == 0) {
        const FastVars *P = (const FastVars *)c.d_params;
#define STATER_BATCH_VARS(LV, ZV, KV, TV)                                                                \
    if (c.levc == LV && c.zp == ZV && c.km == KV && ty == TV) {                                            \
        e = set_smem(vars_ring_batch<LV, ZV, KV, TV>, sm);                                                 \
        if (e == cudaSuccess) vars_ring_batch<LV, ZV, KV, TV><<<total, kTX2 * TV, sm, s>>>(P, start, nj); \
    }
#define STATER_BATCH_VARS_K(LV, ZV, TV) \
    STATER_BATCH_VARS(LV, ZV, 1, TV) STATER_BATCH_VARS(LV, ZV, 3, TV) STATER_BATCH_VARS(LV, ZV, 5, TV)
#define STATER_BATCH_VARS_T(TV)                                                       \
    STATER_BATCH_VARS_K(true, true, TV) STATER_BATCH_VARS_K(true, false, TV)          \
    STATER_BATCH_VARS_K(false, true, TV) STATER_BATCH_VARS_K(false, false, TV)
        STATER_BATCH_VARS_T(16)
        STATER_BATCH_VARS_T(8)
        STATER_BATCH_VARS_T(4)
#undef STATER_BATCH_VARS_T
#undef STATER_BATCH_VARS_K
#undef STATER_BATCH_VARS
    } else {
        const FastFilm *P = (const FastFilm *)c.d_params;
#define STATER_BATCH_FILM(KV, TV, JV)                                                             \
    if (c.km == KV && ty == TV && c.jb == JV) {                                                    \
        e = set_smem(film_ring_batch<KV, TV, JV>, sm);                                             \
        if (e == cudaSuccess) film_ring_batch<KV, TV, JV><<<total, kTX2 * TV, sm, s>>>(P, start, nj); \
    }
#define STATER_BATCH_FILM_T(TV, JV) STATER_BATCH_FILM(1, TV, JV) STATER_BATCH_FILM(3, TV, JV) STATER_BATCH_FILM(5, TV, JV)
        STATER_BATCH_FILM_T(16, false) STATER_BATCH_FILM_T(8, false) STATER_BATCH_FILM_T(4, false)
        STATER_BATCH_FILM_T(16, true) STATER_BATCH_FILM_T(8, true) STATER_BATCH_FILM_T(4, true)
#undef STATER_BATCH_FILM_T
#undef STATER_BATCH_FILM
    }
    return e == cudaSuccess ? cudaGetLastError() : e;
}

// The batched denoise stages: variance statistics, variance filter, Welch
// discriminators, film filter. tune: let the classes' tile heights be tuned.
stater_status plan_enqueue_denoise(BatchPlan &B, int n, cudaStream_t s, bool tune) {
    {
        dim3 g((unsigned)B.pix_blocks, (unsigned)B.kmax);
        vars_stats_batch<<<g, 128, 0, s>>>(B.d_vars, B.d_pix_start, n);
        STATER_CHECK_LAUNCH("vars_stats_batch");
    }
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            dim3 g((unsigned)B.pix_blocks, (unsigned)B.kmax);
            film_discr_batch<<<g, 128, 0, s>>>(B.d_film, B.d_pix_start, n);
            STATER_CHECK_LAUNCH("film_discr_batch");
        }
        for (auto &c : B.classes) {
            if (c.filter != pass) continue;
            int ty = c.ty;
            if (!tune && !ty) {
                const int variant = 64 + (c.filter == 0 ? (c.levc ? 1 : 0) + (c.zp ? 2 : 0) : (c.jb ? 1 : 0)) +
                                    (c.feats ? 4 : 0);
                ty = c.ty = cached_ring_ty(c.filter, c.km, c.nrec, c.R, variant, c.pixels);
            }
            if (tune) {
                const int variant = 64 + (c.filter == 0 ? (c.levc ? 1 : 0) + (c.zp ? 2 : 0) : (c.jb ? 1 : 0)) +
                                    (c.feats ? 4 : 0);
                ty = pick_ring_ty(c.filter, c.km, c.nrec, c.R, variant, c.pixels, s,
                                  [&](int t) { return launch_ring_class(c, t, s); });
                c.ty = ty;
            }
            cudaError_t e = launch_ring_class(c, ty, s);
            if (e != cudaSuccess) return cuda_status(e, "batched ring filter");
        }
    }
    return STATER_OK;
}

}  // namespace
}  // namespace stater

struct stater_batch {
    int dev = 0;
    int reset = 0;
    std::vector<stater_batch_job> jobs;
    stater::BatchPlan plan;
    unsigned char *dev_block = nullptr;
    float *s2 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t capture = nullptr;
};

namespace stater {
namespace {

void batch_free(stater_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->capture) cudaStreamDestroy(b->capture);
    cudaFree(b->dev_block);
    cudaFree(b->s2);
}

// Enqueues one run of the batch on s.
stater_status batch_enqueue(stater_batch *b, cudaStream_t s, bool tune) {
    const int n = (int)b->jobs.size();
    for (int j = 0; j < n; j++) {
        const stater_batch_job &J = b->jobs[j];
        const size_t HW = (size_t)J.acc.width * J.acc.height;
        if (b->reset) {
            cudaMemsetAsync(J.acc.n, 0, sizeof(int32_t) * HW, s);
            cudaMemsetAsync(J.acc.stats, 0, sizeof(float) * (size_t)J.acc.n_transforms * STATER_NQ * 3 * HW, s);
            if (J.acc.gmean && J.acc.n_features > 0)
                cudaMemsetAsync(J.acc.gmean, 0, sizeof(float) * (size_t)J.acc.n_features * HW, s);
            cudaMemsetAsync(J.acc.film_contrib_sum, 0, sizeof(float) * 3 * HW, s);
            cudaMemsetAsync(J.acc.film_weight_sum, 0, sizeof(float) * HW, s);
            cudaMemsetAsync(J.acc.film_spill, 0, sizeof(float) * 4 * HW, s);
        }
        stater_status st = stater_accumulate(&J.acc, (stater_stream)s);
        if (st != STATER_OK) return st;
        st = stater_film_update_image(J.acc.width, J.acc.height, J.acc.film_contrib_sum, J.acc.film_weight_sum,
                                      J.acc.film_spill, J.film_scale, J.film_rgb, (stater_stream)s);
        if (st != STATER_OK) return st;
    }
    return plan_enqueue_denoise(b->plan, n, s, tune);
}

size_t s2_floats(const stater_batch_job *jobs, int n) {
    size_t f = 0;
    for (int j = 0; j < n; j++)
        f += (size_t)2 * 3 * std::max(jobs[j].acc.n_transforms, 1) * jobs[j].acc.width * jobs[j].acc.height;
    return f;
}

}  // namespace

// Serving engine: the batched denoise stages of a group of small jobs whose
// samples are already accumulated and whose film images are made, enqueued on
// s once (no graph). Tables and scratch are allocated and freed in stream
// order; `staging` (pinned host memory of staging_bytes) carries the tables
// and must stay untouched until the stream has passed this point.
stater_status batch_denoise_once(const stater_batch_job *jobs, int n, cudaStream_t s, void *staging,
                                 size_t staging_bytes) {
    BatchPlan B;
    const size_t s2b = align_up(sizeof(float) * s2_floats(jobs, n), 256);
    stater_status st = plan_build(jobs, n, nullptr, B, false);
    if (st != STATER_OK) return st;
    if (B.bytes > staging_bytes)
        return set_error(STATER_ERR_UNSUPPORTED, "batch_denoise_once: tables exceed the staging buffer");
    unsigned char *dev = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&dev, B.bytes + s2b, s);
    if (e != cudaSuccess) return cuda_status(e, "batch_denoise_once: tables");
    // rebuild with the scratch placed after the tables
    BatchPlan B2;
    st = plan_build(jobs, n, (float *)(dev + B.bytes), B2, false);
    if (st != STATER_OK) {
        cudaFreeAsync(dev, s);
        return st;
    }
    std::memcpy(staging, B2.host.data(), B2.bytes);
    e = cudaMemcpyAsync(dev, staging, B2.bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        cudaFreeAsync(dev, s);
        return cuda_status(e, "batch_denoise_once: table upload");
    }
    plan_bind(B2, dev);
    // no tuning here: it would synchronise the serving engine's scheduler thread
    st = plan_enqueue_denoise(B2, n, s, false);
    cudaFreeAsync(dev, s);
    return st;
}

}  // namespace stater

using namespace stater;

extern "C" stater_status stater_batch_create(const stater_batch_job *jobs, int32_t n_jobs, int32_t reset,
                                             stater_batch **out) {
    clear_error();
    if (!jobs || n_jobs < 1 || !out || (reset != 0 && reset != 1))
        return set_error(STATER_ERR_INVALID, "stater_batch_create: bad arguments");
    *out = nullptr;
    auto *b = new stater_batch();
    cudaGetDevice(&b->dev);
    b->reset = reset;
    b->jobs.assign(jobs, jobs + n_jobs);
    auto fail = [&](stater_status st) {
        batch_free(b);
        delete b;
        return st;
    };
    cudaError_t ce = cudaMalloc(&b->s2, sizeof(float) * std::max<size_t>(s2_floats(jobs, n_jobs), 1));
    if (ce != cudaSuccess) return fail(cuda_status(ce, "stater_batch_create: scratch"));
    stater_status st = plan_build(jobs, n_jobs, b->s2, b->plan, true);
    if (st != STATER_OK) return fail(st);
    if ((ce = cudaMalloc(&b->dev_block, b->plan.bytes)) != cudaSuccess ||
        (ce = cudaMemcpy(b->dev_block, b->plan.host.data(), b->plan.bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(cuda_status(ce, "stater_batch_create: job tables"));
    plan_bind(b->plan, b->dev_block);
    *out = b;
    return STATER_OK;
}

extern "C" stater_status stater_batch_run(stater_batch *b, stater_stream stream) {
    clear_error();
    if (!b) return set_error(STATER_ERR_INVALID, "stater_batch_run: null batch");
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != b->dev) return set_error(STATER_ERR_INVALID, "stater_batch_run: the batch belongs to another device");
    cudaStream_t s = (cudaStream_t)stream;
    if (b->exec) return cuda_status(cudaGraphLaunch(b->exec, s), "stater_batch_run: graph launch");
    if (stream_capturing(s))
        return set_error(STATER_ERR_INVALID, "stater_batch_run: the first run of a batch must not be captured");
    // first run: eager, with the tile heights tuned on the real data, then the
    // same sequence is recorded for the later runs
    stater_status st = batch_enqueue(b, s, true);
    if (st != STATER_OK) return st;
    cudaError_t e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "stater_batch_run: capture stream");
    e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_status(e, "stater_batch_run: begin capture");
    st = batch_enqueue(b, b->capture, false);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->capture, &g);
    if (st != STATER_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_status(e, "stater_batch_run: end capture");
    b->graph = g;
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) {
        b->exec = nullptr;
        return cuda_status(e, "stater_batch_run: graph instantiate");
    }
    return STATER_OK;
}

extern "C" stater_status stater_batch_destroy(stater_batch *b) {
    clear_error();
    if (!b) return STATER_OK;
    cudaDeviceSynchronize();
    batch_free(b);
    delete b;
    return STATER_OK;
}
