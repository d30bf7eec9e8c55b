// Stage 2, FP32 form. Same formulas as the plain FP64 form (denoise.cu), laid
// out for the GPU:
//  * per-pixel statistics (lnS2, se2, s2, s2C, jb) in one elementwise pass;
//  * each windowed filter works on a 16 x TY output tile whose (16+2R) x (TY+2R)
//    halo of every needed plane is staged in shared memory once per transform,
//    so each HBM byte is read once per tile and every neighbour access is an
//    on-chip load;
//  * the Welch decisions of all transforms are combined in a per-pixel bit mask
//    in shared memory (one bit per window position), so the film pass touches
//    only accepted neighbours;
//  * the Welch df always lies in [min(n_i, n_j) - 1, n_i + n_j - 2], and the
//    critical value decreases with df, so the test is decided from two
//    per-pair bounds (tables indexed by integer df) and only the narrow band
//    between them evaluates the exact df and the interpolated quantile. The
//    exact branch falls back to FP64 when the summed variance is near zero.
#include <cmath>
#include <mutex>
#include <map>
#include <vector>

#include "denoise_params.cuh"

namespace stater {

namespace {

constexpr int kTX = 16;
constexpr int kMaxFeatCh = 24;
constexpr int kDfMax = 4096;
constexpr float kLog2e = 1.4426950408889634f;

struct FeatSet {
    int nch;
    const float *plane[kMaxFeatCh];
    float scale[kMaxFeatCh];  // dr * log2(e) of the owning G-buffer
};

bool make_featset(FeatSet &f, const stater_gbuffers &g, size_t HW) {
    f.nch = 0;
    if (g.count < 0 || g.count > STATER_MAX_GBUFFERS) return false;
    for (int i = 0; i < g.count; i++) {
        if (!g.planes[i] || (g.channels[i] != 1 && g.channels[i] != 3)) return false;
        for (int c = 0; c < g.channels[i]; c++) {
            if (f.nch >= kMaxFeatCh) return false;
            f.plane[f.nch] = (const float *)g.planes[i] + (size_t)c * HW;
            f.scale[f.nch] = g.dr_factor[i] * kLog2e;
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
    int W, H, K, R, mt_mode, use_levc, lut_n;
    float ds2;
    const int32_t *n;
    const float *film;
    const float *mean[STATER_MAX_TRANSFORMS];
    const float *var[STATER_MAX_TRANSFORMS];  // varCD or varD
    const float *jb[STATER_MAX_TRANSFORMS];
    const float *lut;    // [lut_n + 1] t2 over u
    const float *tlo;    // [kDfMax + 1] lower envelope of t2 at integer df
    const float *thi;    // [kDfMax + 1] upper envelope
    float z2lo;          // lower bound of t2 beyond kDfMax
    FeatSet feat;
    float *discr[STATER_MAX_TRANSFORMS];
    float *filmD;
    uint32_t *bits;
};

// ---------------------------------------------------------------------------
// Per-pixel variance statistics.
// ---------------------------------------------------------------------------
__global__ void vars_stats_f32(FastVars P) {
    const size_t HW = (size_t)P.W * P.H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
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

// Stages the halo of `src` ((TX+2R) x (TY+2R) around the tile) into dst;
// out-of-image entries get `fill`.
__device__ __forceinline__ void load_halo(float *dst, const float *__restrict__ src, int W, int H, int x0,
                                          int y0, int R, int hw, int hh, float fill) {
    const int A = hw * hh;
    for (int idx = threadIdx.x; idx < A; idx += blockDim.x) {
        const int hy = idx / hw, hx = idx - hy * hw;
        const int gx = x0 - R + hx, gy = y0 - R + hy;
        dst[idx] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? __ldg(src + (size_t)gy * W + gx) : fill;
    }
}

__device__ __forceinline__ void load_valid(int *dst, const int32_t *__restrict__ n, int W, int H, int x0, int y0,
                                           int R, int hw, int hh) {
    const int A = hw * hh;
    for (int idx = threadIdx.x; idx < A; idx += blockDim.x) {
        const int hy = idx / hw, hx = idx - hy * hw;
        const int gx = x0 - R + hx, gy = y0 - R + hy;
        int v = 0;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            v = __ldg(n + (size_t)gy * W + gx);
            if (v < 2) v = 0;
        }
        dst[idx] = v;
    }
}

// ---------------------------------------------------------------------------
// Variance filter (varD, varCD).
// ---------------------------------------------------------------------------
template <int TY, bool LEVC, int MF>
__global__ void __launch_bounds__(kTX *TY) vars_filter_f32(FastVars P) {
    extern __shared__ float smem[];
    const int R = P.R, hw = kTX + 2 * R, hh = TY + 2 * R, A = hw * hh;
    const int nf = P.feat.nch;
    int *valid = (int *)smem;
    float *feat = smem + A;
    float *ln = feat + (size_t)nf * A;
    float *se = ln + 3 * A;
    float *sv = se + 3 * A;
    float *svc = sv + 3 * A;

    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * TY;
    const int lx = threadIdx.x % kTX, ly = threadIdx.x / kTX;
    const int x = x0 + lx, y = y0 + ly;
    const bool inside = x < P.W && y < P.H;
    const size_t HW = (size_t)P.W * P.H;
    const size_t i = (size_t)y * P.W + x;
    const int ci = (ly + R) * hw + (lx + R);

    load_valid(valid, P.n, P.W, P.H, x0, y0, R, hw, hh);
    for (int f = 0; f < nf; f++) load_halo(feat + (size_t)f * A, P.feat.plane[f], P.W, P.H, x0, y0, R, hw, hh, 0.f);
    __syncthreads();
    float fi[MF > 0 ? MF : 1];
#pragma unroll
    for (int f = 0; f < MF; f++) fi[f] = f < nf ? feat[(size_t)f * A + ci] : 0.f;
    const bool vi = inside && valid[ci] != 0;

    for (int k = 0; k < P.K; k++) {
        __syncthreads();
        for (int c = 0; c < 3; c++) {
            const size_t off = ((size_t)k * 3 + c) * HW;
            load_halo(ln + c * A, P.lnS2[k] + (size_t)c * HW, P.W, P.H, x0, y0, R, hw, hh, 0.f);
            load_halo(se + c * A, P.se2[k] + (size_t)c * HW, P.W, P.H, x0, y0, R, hw, hh, 0.f);
            load_halo(sv + c * A, P.s2 + off, P.W, P.H, x0, y0, R, hw, hh, 0.f);
            if (LEVC) load_halo(svc + c * A, P.s2c + off, P.W, P.H, x0, y0, R, hw, hh, 0.f);
        }
        __syncthreads();
        if (!inside) continue;
        if (!vi) {
            for (int c = 0; c < 3; c++) {
                P.varD[k][(size_t)c * HW + i] = 0.f;
                P.varCD[k][(size_t)c * HW + i] = 0.f;
            }
            continue;
        }
        float li[3], si[3], aw[3] = {0.f, 0.f, 0.f}, av[3] = {0.f, 0.f, 0.f}, avc[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            li[c] = ln[c * A + ci];
            si[c] = se[c * A + ci];
        }
        for (int dy = -R; dy <= R; dy++) {
            const int row = (ly + R + dy) * hw + lx + R;
            const float sdy = P.ds2 * (float)(dy * dy);
            for (int dx = -R; dx <= R; dx++) {
                const int h = row + dx;
                if (valid[h] == 0) continue;
                float arg = fmaf(P.ds2, (float)(dx * dx), sdy);
#pragma unroll
                for (int f = 0; f < MF; f++) {
                    if (f < nf) {
                        const float d = fi[f] - feat[(size_t)f * A + h];
                        arg = fmaf(P.feat.scale[f] * d, d, arg);
                    }
                }
                const float w = exp2f(arg);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float dl = li[c] - ln[c * A + h];
                    if (dl * dl <= P.z2 * (si[c] + se[c * A + h])) {
                        aw[c] += w;
                        av[c] = fmaf(w, sv[c * A + h], av[c]);
                        if (LEVC) avc[c] = fmaf(w, svc[c * A + h], avc[c]);
                    }
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float vd = av[c] / aw[c];
            P.varD[k][(size_t)c * HW + i] = vd;
            P.varCD[k][(size_t)c * HW + i] = LEVC ? avc[c] / aw[c] : vd;
        }
    }
}

// ---------------------------------------------------------------------------
// Welch discriminator and the film filter.
// ---------------------------------------------------------------------------
__global__ void film_discr_f32(FastFilm P) {
    const size_t HW = (size_t)P.W * P.H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (p >= HW) return;
    const int nn = P.n[p];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const size_t o = (size_t)c * HW + p;
        P.discr[k][o] = nn < 2 ? 0.f : P.var[k][o] / (float)nn;
    }
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

template <int TY, int MF>
__global__ void __launch_bounds__(kTX *TY) film_filter_f32(FastFilm P) {
    extern __shared__ float smem[];
    constexpr int NT = kTX * TY;
    const int R = P.R, D = 2 * R + 1, words = (D * D + 31) / 32;
    const int hw = kTX + 2 * R, hh = TY + 2 * R, A = hw * hh;
    const int nf = P.feat.nch;
    uint32_t *mask = (uint32_t *)smem;                 // [words][NT]
    int *nval = (int *)(mask + (size_t)words * NT);    // [A]
    float *feat = (float *)(nval + A);                 // [nf][A]
    float *mu = feat + (size_t)nf * A;                 // [3][A] (film in the last pass)
    float *dd = mu + 3 * A;                            // [3][A]

    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * TY;
    const int t = threadIdx.x;
    const int lx = t % kTX, ly = t / kTX;
    const int x = x0 + lx, y = y0 + ly;
    const bool inside = x < P.W && y < P.H;
    const size_t HW = (size_t)P.W * P.H;
    const size_t i = (size_t)y * P.W + x;
    const int ci = (ly + R) * hw + (lx + R);

    for (int w = 0; w < words; w++) mask[(size_t)w * NT + t] = 0xFFFFFFFFu;
    load_valid(nval, P.n, P.W, P.H, x0, y0, R, hw, hh);
    for (int f = 0; f < nf; f++) load_halo(feat + (size_t)f * A, P.feat.plane[f], P.W, P.H, x0, y0, R, hw, hh, 0.f);
    __syncthreads();
    const int ni = inside ? nval[ci] : 0;
    int ksel = -1;
    if (inside && P.mt_mode == STATER_MT_JB && ni >= 2) {
        ksel = 0;
        float best = P.jb[0][i];
        for (int k = 1; k < P.K; k++) {
            const float v = P.jb[k][i];
            if (v < best) {
                best = v;
                ksel = k;
            }
        }
    }

    for (int k = 0; k < P.K; k++) {
        __syncthreads();
        const float *mean = k == 0 ? P.film : P.mean[k];
        for (int c = 0; c < 3; c++) {
            load_halo(mu + c * A, mean + (size_t)c * HW, P.W, P.H, x0, y0, R, hw, hh, 0.f);
            load_halo(dd + c * A, P.discr[k] + (size_t)c * HW, P.W, P.H, x0, y0, R, hw, hh, 0.f);
        }
        __syncthreads();
        if (!inside) continue;
        if (ni < 2) {
            if (P.bits)
                for (int w = 0; w < words; w++) P.bits[(i * P.K + k) * (size_t)words + w] = 0u;
            continue;
        }
        float mi[3], di[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            mi[c] = mu[c * A + ci];
            di[c] = dd[c * A + ci];
        }
        const bool and_into_mask = ksel < 0 || ksel == k;
        uint32_t cur = 0u;
        int bit = 0, word = 0;
        for (int dy = -R; dy <= R; dy++) {
            const int row = (ly + R + dy) * hw + lx + R;
            for (int dx = -R; dx <= R; dx++, bit++) {
                const int h = row + dx;
                const int nj = nval[h];
                int a = 0;
                if (nj >= 2) {
                    a = 1;
                    if (dx != 0 || dy != 0) {
                        const int dfl = ni + nj - 2;
                        const int dfh = min(ni, nj) - 1;
                        const float tlo = dfl > kDfMax ? P.z2lo : __ldg(P.tlo + dfl);
                        const float thi = __ldg(P.thi + (dfh > kDfMax ? kDfMax : dfh));
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const float dj = dd[c * A + h];
                            const float diff = mi[c] - mu[c * A + h];
                            const float s = di[c] + dj;
                            const float q = diff * diff;
                            if (!(s > 0.f)) {
                                if (diff != 0.f) a = 0;
                            } else if (q <= tlo * s) {
                            } else if (q > thi * s) {
                                a = 0;
                            } else {
                                a &= welch_exact(diff, di[c], dj, ni, nj, P.lut, P.lut_n);
                            }
                        }
                    }
                }
                cur |= (uint32_t)a << (bit & 31);
                if ((bit & 31) == 31 || bit == D * D - 1) {
                    if (and_into_mask) mask[(size_t)word * NT + t] &= cur;
                    if (P.bits) P.bits[(i * P.K + k) * (size_t)words + word] = cur;
                    cur = 0u;
                    word++;
                }
            }
        }
    }

    __syncthreads();
    for (int c = 0; c < 3; c++) load_halo(mu + c * A, P.film + (size_t)c * HW, P.W, P.H, x0, y0, R, hw, hh, 0.f);
    __syncthreads();
    if (!inside) return;
    if (ni < 2) {
        for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + i] = mu[c * A + ci];
        return;
    }
    float fi[MF > 0 ? MF : 1];
#pragma unroll
    for (int f = 0; f < MF; f++) fi[f] = f < nf ? feat[(size_t)f * A + ci] : 0.f;
    float sw = 0.f, sf[3] = {0.f, 0.f, 0.f};
    int bit = 0;
    for (int dy = -R; dy <= R; dy++) {
        const int row = (ly + R + dy) * hw + lx + R;
        const float sdy = P.ds2 * (float)(dy * dy);
        for (int dx = -R; dx <= R; dx++, bit++) {
            const uint32_t m = mask[(size_t)(bit >> 5) * NT + t];
            if (!((m >> (bit & 31)) & 1u)) continue;
            const int h = row + dx;
            if (nval[h] < 2) continue;
            float arg = fmaf(P.ds2, (float)(dx * dx), sdy);
#pragma unroll
            for (int f = 0; f < MF; f++) {
                if (f < nf) {
                    const float d = fi[f] - feat[(size_t)f * A + h];
                    arg = fmaf(P.feat.scale[f] * d, d, arg);
                }
            }
            const float w = exp2f(arg);
            sw += w;
#pragma unroll
            for (int c = 0; c < 3; c++) sf[c] = fmaf(w, mu[c * A + h], sf[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) P.filmD[(size_t)c * HW + i] = sf[c] / sw;
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

size_t vars_smem(int R, int TY, int nf) {
    const size_t A = (size_t)(kTX + 2 * R) * (TY + 2 * R);
    return A * sizeof(float) * (1 + nf + 12);
}

size_t film_smem(int R, int TY, int nf) {
    const size_t A = (size_t)(kTX + 2 * R) * (TY + 2 * R);
    const int D = 2 * R + 1, words = (D * D + 31) / 32;
    return (size_t)words * kTX * TY * 4 + A * sizeof(float) * (1 + nf + 6);
}

constexpr size_t kSmemLimit = 227 * 1024;

int mf_bucket(int nf) { return nf == 0 ? 0 : nf <= 4 ? 4 : nf <= 8 ? 8 : nf <= 16 ? 16 : 24; }

template <typename KernelT>
cudaError_t set_smem(KernelT kern, size_t bytes) {
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

stater_status denoise_vars_f32(const stater_denoise_vars_args *a, cudaStream_t s) {
    FastVars P;
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
    const size_t HW = (size_t)P.W * P.H;
    if (!make_featset(P.feat, a->gbuffers, HW))
        return set_error(STATER_ERR_INVALID, "stater_denoise_vars: bad gbuffers (at most 24 channels)");
    float *scr = (float *)scratch(0, sizeof(float) * 2 * 3 * P.K * HW, s);
    if (!scr) return set_error(STATER_ERR_NOMEM, "stater_denoise_vars: scratch allocation failed");
    P.s2 = scr;
    P.s2c = scr + (size_t)3 * P.K * HW;

    dim3 g1((unsigned)((HW + 127) / 128), P.K);
    vars_stats_f32<<<g1, 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("vars_stats_f32");

    int TY = 16;
    size_t sm = vars_smem(P.R, TY, P.feat.nch);
    if (sm > kSmemLimit) {
        TY = 8;
        sm = vars_smem(P.R, TY, P.feat.nch);
    }
    if (sm > kSmemLimit) return set_error(STATER_ERR_UNSUPPORTED, "stater_denoise_vars: radius too large for FP32 tiles");
    dim3 grid((P.W + kTX - 1) / kTX, (P.H + TY - 1) / TY);
    const int mf = mf_bucket(P.feat.nch);
    cudaError_t e = cudaSuccess;
#define STATER_VARS_LAUNCH(TYV, LV, MFV)                                           \
    if (TY == TYV && (P.levc != 0) == LV && mf == MFV) {                          \
        e = set_smem(vars_filter_f32<TYV, LV, MFV>, sm);                          \
        if (e == cudaSuccess) vars_filter_f32<TYV, LV, MFV><<<grid, kTX * TYV, sm, s>>>(P); \
    }
#define STATER_VARS_LAUNCH_MF(TYV, LV) \
    STATER_VARS_LAUNCH(TYV, LV, 0) STATER_VARS_LAUNCH(TYV, LV, 4) STATER_VARS_LAUNCH(TYV, LV, 8) \
    STATER_VARS_LAUNCH(TYV, LV, 16) STATER_VARS_LAUNCH(TYV, LV, 24)
    STATER_VARS_LAUNCH_MF(16, true)
    STATER_VARS_LAUNCH_MF(16, false)
    STATER_VARS_LAUNCH_MF(8, true)
    STATER_VARS_LAUNCH_MF(8, false)
#undef STATER_VARS_LAUNCH_MF
#undef STATER_VARS_LAUNCH
    if (e != cudaSuccess) return cuda_status(e, "vars_filter_f32 smem attribute");
    STATER_CHECK_LAUNCH("vars_filter_f32");
    return STATER_OK;
}

stater_status denoise_film_f32(const stater_denoise_film_args *a, cudaStream_t s) {
    FastFilm P;
    P.W = a->width;
    P.H = a->height;
    P.K = a->n_buffers;
    P.R = a->filter_radius;
    P.mt_mode = a->mt_mode;
    P.use_levc = a->use_levc;
    P.lut_n = tcrit_intervals();
    P.ds2 = a->ds_factor * kLog2e;
    P.n = a->n;
    P.film = (const float *)a->film;
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        P.mean[k] = (const float *)a->mean[k];
        P.var[k] = (const float *)(a->use_levc ? a->varCD[k] : a->varD[k]);
        P.jb[k] = (const float *)a->jb[k];
        P.discr[k] = (float *)a->discr[k];
    }
    P.filmD = (float *)a->filmD;
    P.bits = a->accept_bits;
    const size_t HW = (size_t)P.W * P.H;
    if (!make_featset(P.feat, a->gbuffers, HW))
        return set_error(STATER_ERR_INVALID, "stater_denoise_film: bad gbuffers (at most 24 channels)");
    P.lut = (const float *)tcrit_table_device((double)a->alpha, false, s);
    const DfTables *dt = df_tables((double)a->alpha, s);
    if (!P.lut || !dt) return set_error(STATER_ERR_NOMEM, "stater_denoise_film: table allocation failed");
    P.tlo = dt->lo;
    P.thi = dt->hi;
    P.z2lo = dt->z2lo;

    dim3 g1((unsigned)((HW + 127) / 128), P.K);
    film_discr_f32<<<g1, 128, 0, s>>>(P);
    STATER_CHECK_LAUNCH("film_discr_f32");

    int TY = 16;
    size_t sm = film_smem(P.R, TY, P.feat.nch);
    if (sm > kSmemLimit) {
        TY = 8;
        sm = film_smem(P.R, TY, P.feat.nch);
    }
    if (sm > kSmemLimit) return set_error(STATER_ERR_UNSUPPORTED, "stater_denoise_film: radius too large for FP32 tiles");
    dim3 grid((P.W + kTX - 1) / kTX, (P.H + TY - 1) / TY);
    const int mf = mf_bucket(P.feat.nch);
    cudaError_t e = cudaSuccess;
#define STATER_FILM_LAUNCH(TYV, MFV)                                          \
    if (TY == TYV && mf == MFV) {                                             \
        e = set_smem(film_filter_f32<TYV, MFV>, sm);                          \
        if (e == cudaSuccess) film_filter_f32<TYV, MFV><<<grid, kTX * TYV, sm, s>>>(P); \
    }
    STATER_FILM_LAUNCH(16, 0) STATER_FILM_LAUNCH(16, 4) STATER_FILM_LAUNCH(16, 8)
    STATER_FILM_LAUNCH(16, 16) STATER_FILM_LAUNCH(16, 24)
    STATER_FILM_LAUNCH(8, 0) STATER_FILM_LAUNCH(8, 4) STATER_FILM_LAUNCH(8, 8)
    STATER_FILM_LAUNCH(8, 16) STATER_FILM_LAUNCH(8, 24)
#undef STATER_FILM_LAUNCH
    if (e != cudaSuccess) return cuda_status(e, "film_filter_f32 smem attribute");
    STATER_CHECK_LAUNCH("film_filter_f32");
    return STATER_OK;
}

}  // namespace stater
