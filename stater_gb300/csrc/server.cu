// Serving engine: continuous admission of denoise jobs onto stream slots.
//
// One scheduler thread owns the device work of all jobs. Each admitted job gets
// a slot (a non-blocking CUDA stream) and one stream-ordered allocation
// (cudaMallocAsync from the device's memory pool) holding its sample chunk,
// moment buffers and outputs. A job is a small state machine: its rounds are
// enqueued on its stream, and a CUDA event marks the point where the scheduler
// must look again (the next round needs the largest per-pixel sample target of
// the previous one; the last round ends with the device-to-host copy of the
// denoised film). Between events the scheduler only polls, so work of all slots
// runs concurrently on the device and new jobs are admitted the moment a slot
// and enough memory are free.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "denoise_params.cuh"

namespace stater {
namespace {

using Clock = std::chrono::steady_clock;

constexpr int kTmin = 16, kTmax = 1024;
constexpr double kEps = 1e-4;


__global__ void widen_kernel(size_t n, const float *in, double *out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

// Adaptive rounds visit the pixels grouped by the number of sample steps their
// target still needs (descending), so that the samples still due at any point
// belong to a prefix of the order and each step covers only that prefix (a
// 32-pixel group no longer runs to the largest target among its neighbours).
// Within a group the pixels keep their image order (a stable counting sort), so
// the columns of a warp are mostly neighbouring pixels and the statistics
// planes are read and written in long runs.
constexpr int kBins = 1025;  // targets 0..kTmax (bounds the step count and the act table)

int sort_bins(int chunk) { return (kTmax + chunk - 1) / chunk + 1; }

__device__ __forceinline__ int steps_of(int t, int chunk, int nbins) {
    return min((t + chunk - 1) / chunk, nbins - 1);
}

// Per block of 256 pixels: how many pixels need each number of steps; the
// largest target of the image (*tmax zeroed before).
__global__ void __launch_bounds__(256) target_count_kernel(size_t HW, const int32_t *target, int chunk, int nbins,
                                                           int32_t *block_hist, int32_t *tmax) {
    extern __shared__ int cnt[];
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) cnt[b] = 0;
    __syncthreads();
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    int t = 0;
    if (p < HW) {
        t = min(max(target[p], 0), kTmax);
        atomicAdd(&cnt[steps_of(t, chunk, nbins)], 1);
    }
    for (int o = 16; o > 0; o >>= 1) t = max(t, __shfl_xor_sync(0xffffffffu, t, o));
    if ((threadIdx.x & 31) == 0 && t > 0) atomicMax(tmax, t);
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) block_hist[(size_t)b * gridDim.x + blockIdx.x] = cnt[b];
}

// One CTA of 1024 threads, in place: the per-block counts become the first
// position of every (step count, block) group in the order (step counts
// descending, blocks ascending); act[c] = the pixels that need more than c
// steps, c = 0..nbins. Each thread scans a contiguous run of blocks.
__global__ void __launch_bounds__(1024) target_offsets_kernel(int nblocks, int nbins, int32_t *hist_base,
                                                              int32_t *act) {
    __shared__ int warp_sum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int seg = (nblocks + 1023) / 1024;
    const int i0 = min(nblocks, (int)threadIdx.x * seg), i1 = min(nblocks, i0 + seg);
    int running = 0;
    for (int b = nbins - 1; b >= 0; b--) {
        int32_t *row = hist_base + (size_t)b * nblocks;
        int v = 0;
        for (int i = i0; i < i1; i++) v += row[i];
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = warp_sum[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_sum[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        int pos = running + x - v + (warp > 0 ? warp_sum[warp - 1] : 0);
        for (int i = i0; i < i1; i++) {
            const int c = row[i];
            row[i] = pos;
            pos += c;
        }
        running += warp_sum[31];
        if (threadIdx.x == 0 && b >= 1) act[b - 1] = running;  // pixels with at least b steps
        __syncthreads();  // warp_sum is rewritten by the next step count
    }
    if (threadIdx.x == 0) {
        act[nbins - 1] = 0;
        act[nbins] = 0;
    }
}

// Every pixel's place: its group's first position plus its rank among the
// group's pixels of the block in image order.
__global__ void __launch_bounds__(256) target_place_kernel(size_t HW, const int32_t *target, int chunk, int nbins,
                                                           const int32_t *base, int32_t *order, int32_t *tsorted) {
    extern __shared__ int wcnt[];  // [8][nbins]
    for (int i = threadIdx.x; i < 8 * nbins; i += blockDim.x) wcnt[i] = 0;
    __syncthreads();
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < HW;
    const int t = valid ? min(max(target[p], 0), kTmax) : 0;
    const int key = valid ? steps_of(t, chunk, nbins) : -1;
    const unsigned same = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lrank = __popc(same & ((1u << lane) - 1u));
    if (valid && lrank == 0) wcnt[warp * nbins + key] = __popc(same);
    __syncthreads();
    if (!valid) return;
    int r = lrank;
    for (int w = 0; w < warp; w++) r += wcnt[w * nbins + key];
    const int pos = base[(size_t)key * gridDim.x + blockIdx.x] + r;
    order[pos] = (int32_t)p;
    tsorted[pos] = t;
}

// Per column of step `done`: samples due (0 for padding beyond the active
// prefix) and the pixel's next sample index.
__global__ void sorted_step_kernel(int ncols, const int32_t *order, const int32_t *tsorted, const int32_t *n,
                                   int done, int chunk, int32_t *counts, int32_t *first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncols) return;
    counts[i] = max(0, min(tsorted[i] - done, chunk));
    first[i] = n[order[i]];
}


size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Layout {
    size_t HW, T, K, G, chunk;
    size_t off_n, off_counts, off_target, off_max, off_order, off_tsorted, off_first, off_hist, off_act,
        off_stats, off_gmean, off_film, off_rgb, off_rgb64, off_jb, off_out6, off_filmD, off_samples, total;
};

int chunk_for(const stater_job_desc &d, int chunk_spp) {
    const size_t HW = (size_t)d.width * d.height;
    const size_t per = (size_t)(5 + d.n_features) * HW * 4;
    // automatic (chunk_spp <= 0): 128 samples per step for adaptive jobs, whose
    // many short steps read and write the moment state each time (a 1080p job
    // of 4 rounds: 68 ms at 32, 52 ms at 128), 32 for one-round jobs (larger
    // steps cost the mixed serving trace a few percent through larger footprints)
    int c = chunk_spp > 0 ? chunk_spp : (d.rounds > 1 ? 128 : 32);
    // no more than a round can take: spp for one round, up to kTmax per pixel in adaptive rounds
    c = std::max(1, std::min(c, d.rounds > 1 ? std::max(d.spp, kTmax) : d.spp));
    // at most 16 GiB of sample planes per step: a 3840x2160 job still takes 32
    // samples per step (each step also reads and writes the whole moment state)
    while (c > 1 && (size_t)c * per > ((size_t)16 << 30)) c /= 2;
    return c;
}

Layout layout(const stater_job_desc &d, int precision, int chunk_spp) {
    Layout L;
    L.HW = (size_t)d.width * d.height;
    L.T = precision == STATER_F64 ? 8 : 4;
    L.K = d.n_transforms;
    L.G = d.n_features;
    L.chunk = chunk_for(d, chunk_spp);
    size_t o = 0;
    auto take = [&](size_t b) {
        const size_t r = o;
        o += align256(b);
        return r;
    };
    L.off_n = take(4 * L.HW);
    L.off_counts = take(4 * (L.HW + 4));
    L.off_target = take(4 * L.HW);
    L.off_max = take(4);
    L.off_order = take(4 * (L.HW + 4));
    L.off_tsorted = take(4 * (L.HW + 4));
    L.off_first = take(4 * (L.HW + 4));
    const size_t nblk = (L.HW + 255) / 256;
    L.off_hist = take(4 * (size_t)sort_bins((int)L.chunk) * nblk);
    L.off_act = take(4 * (kBins + 2));
    L.off_stats = take(L.K * STATER_NQ * 3 * L.HW * L.T);
    L.off_gmean = take(std::max<size_t>(L.G, 1) * L.HW * L.T);
    L.off_film = take(8 * L.HW * 4);  // film sums: contrib[3], weight, spill[4]
    L.off_rgb = take(3 * L.HW * 4);
    L.off_rgb64 = take(L.T == 8 ? 3 * L.HW * 8 : 0);
    L.off_jb = take(L.K * L.HW * L.T);
    L.off_out6 = take(6 * L.K * 3 * L.HW * L.T);
    L.off_filmD = take(3 * L.HW * L.T);
    L.off_samples = take(L.chunk * (5 + L.G) * (L.HW + 4) * 4);  // + 4 columns: a padded active prefix
    L.total = o;
    return L;
}

// Scratch the library's denoise and target-SPP calls keep per stream.
size_t scratch_bytes(const Layout &L) {
    const size_t vars = 2 * 3 * L.K * L.HW * L.T;
    const size_t film = L.T == 8 ? 3 * L.K * L.HW * 8 : 0;
    const size_t tspp = 8 * (L.HW + 2 * ((L.HW + 1023) / 1024) + 2);
    return vars + film + tspp;
}

struct Job {
    int64_t id = 0;
    stater_job_desc d{};
    Layout L{};
    int state = STATER_JOB_QUEUED;
    int slot = -1;
    int round = 0;
    bool final_enqueued = false;
    double footprint = 0;
    unsigned char *base = nullptr;
    cudaEvent_t ev = nullptr;
    std::shared_ptr<int> group_left;  // fused group: jobs of the group not finished yet
    // A pageable result buffer is filled from the slot's pinned staging once the
    // job's GPU work is done: a device-to-host copy into pageable memory would
    // run through the driver's synchronous staging (and fault in the caller's
    // fresh pages) on the scheduler thread, up to 20 ms for a 1080p result.
    bool out_pinned = true;
    float *out_stage = nullptr;
    Clock::time_point t_submit, t_done;
    double latency_ms = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    int32_t *hmax = nullptr;  // pinned: largest target of the last round
    int32_t *hact = nullptr;  // pinned: active prefix length of each step of the next round
    void *staging = nullptr;  // pinned: job tables of a fused group
    float *out = nullptr;     // pinned: results bound for pageable buffers (grown while the slot is idle)
    size_t out_cap = 0;       // floats
    bool busy = false;
};

// Small single-round jobs admitted together run as one group on one slot: each
// job's samples are generated and accumulated on the slot's stream, then the
// denoise stages of the whole group run as one launch per stage (the batched
// kernels of stater_batch), so small images no longer pay a launch and a tail
// per stage each. Results are bitwise those of the same job run alone.
constexpr size_t kFuseMaxPixels = (size_t)512 * 512;
constexpr int kFuseMaxJobs = 16;
constexpr size_t kStagingBytes = (size_t)1 << 20;

}  // namespace
}  // namespace stater

using namespace stater;

struct stater_server {
    stater_server_config cfg{};
    int device = 0;
    double budget = 0, used = 0, peak = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Job>> queue;
    std::vector<std::shared_ptr<Job>> active;
    std::map<int64_t, std::shared_ptr<Job>> jobs;
    int64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    std::vector<double> latencies;
    int64_t submitted = 0, completed = 0, failed = 0;
    double pixels_done = 0;
    bool have_first = false;
    Clock::time_point first_submit, last_done;

    void run();
    bool start(Job &j);
    bool start_group(std::vector<std::shared_ptr<Job>> &group);
    bool fusable(const Job &j) const;
    bool enqueue_round(Job &j, int samples, bool uniform);
    bool enqueue_after_round(Job &j);
    void finish(Job &j, bool ok);
};

namespace {

stater_precision prec_of(const stater_server *s) { return (stater_precision)s->cfg.precision; }

double group_footprint(const std::vector<std::shared_ptr<Job>> &g) {
    double f = 0;
    for (auto &j : g) f += j->footprint;
    return f;
}

void fill_gbuffers(stater_gbuffers &g, const Job &j) {
    std::memset(&g, 0, sizeof(g));
    const int G = j.d.n_features;
    const size_t plane = j.L.HW * j.L.T;
    unsigned char *gm = j.base + j.L.off_gmean;
    const float sig[3] = {0.02f, 0.1f, 0.1f};
    const int first[3] = {0, 3, 6}, chans[3] = {3, 3, 1};
    for (int i = 0; i < 3; i++) {
        if (first[i] + chans[i] > G) break;
        g.planes[g.count] = gm + first[i] * plane;
        g.channels[g.count] = chans[i];
        g.dr_factor[g.count] = -0.5f / (sig[i] * sig[i]);
        g.count++;
    }
}

}  // namespace

bool stater_server::enqueue_round(Job &j, int samples, bool uniform) {
    const Slot &sl = slots[j.slot];
    cudaStream_t s = sl.stream;
    const Layout &L = j.L;
    int32_t *n = (int32_t *)(j.base + L.off_n);
    int32_t *counts = (int32_t *)(j.base + L.off_counts);
    float *smp = (float *)(j.base + L.off_samples);
    const int32_t *order = (const int32_t *)(j.base + L.off_order);
    int32_t *first = (int32_t *)(j.base + L.off_first);
    for (int done = 0, step = 0; done < samples; done += (int)L.chunk, step++) {
        const int S = std::min((int)L.chunk, samples - done);
        // adaptive round: the active prefix of the sorted order, padded to 4 columns
        int ncols = 0;
        if (!uniform) {
            const int active = sl.hact[step];
            if (active <= 0) break;
            ncols = std::min((int)L.HW + 4, (active + 3) / 4 * 4);
            sorted_step_kernel<<<(unsigned)((ncols + 255) / 256), 256, 0, s>>>(ncols, order, (const int32_t *)(j.base + L.off_tsorted),
                                                                              n, done, S, counts, first);
            if (cudaGetLastError() != cudaSuccess) return false;
        }
        stater_generate_args g{};
        g.width = j.d.width;
        g.height = j.d.height;
        g.n_samples = S;
        g.n_features = j.d.n_features;
        g.seed = j.d.seed;
        g.region = 8;
        g.mean_mu = -1.f;
        g.mean_sigma = 1.f;
        g.noise_sigma = 0.5f;
        g.firefly_prob = 1e-3f;
        g.firefly_scale = 1e3f;
        g.first_index = uniform ? n : first;  // every pixel continues its own sample sequence
        g.count = uniform ? nullptr : counts;  // only the samples the accumulation will read
        g.samples = smp;
        if (!uniform) {
            g.pixel_index = order;
            g.n_active = ncols;
        }
        if (stater_generate_samples(&g, (stater_stream)s) != STATER_OK) return false;
        stater_accumulate_args a{};
        a.width = j.d.width;
        a.height = j.d.height;
        a.n_samples = S;
        a.n_features = j.d.n_features;
        a.samples = smp;
        a.count = uniform ? nullptr : counts;
        a.n_transforms = j.d.n_transforms;
        for (int k = 0; k < j.d.n_transforms; k++) a.transforms[k] = j.d.transforms[k];
        a.max_moment = j.d.max_moment;
        a.precision = prec_of(this);
        a.mode = prec_of(this) == STATER_F32 ? STATER_ACC_FAST : STATER_ACC_EXACT;
        a.n = n;
        a.stats = j.base + L.off_stats;
        a.gmean = j.base + L.off_gmean;
        float *fs = (float *)(j.base + L.off_film);
        a.film_contrib_sum = fs;
        a.film_weight_sum = fs + 3 * L.HW;
        a.film_spill = fs + 4 * L.HW;
        a.film_max_sample_luminance = INFINITY;
        if (!uniform) {
            a.pixel_index = order;
            a.n_active = ncols;
        }
        if (stater_accumulate(&a, (stater_stream)s) != STATER_OK) return false;
    }
    return true;
}

namespace {

// The denoiseVars and denoiseFilm arguments of a job over its device block
// (film = the FP32 film image; the FP64 form passes its widened copy).
void job_denoise_args(const Job &j, stater_precision prec, stater_denoise_vars_args &v,
                      stater_denoise_film_args &f) {
    const Layout &L = j.L;
    const size_t plane3 = 3 * L.HW * L.T;
    unsigned char *out6 = j.base + L.off_out6;
    auto out_of = [&](int which, int k) { return (void *)(out6 + ((size_t)which * L.K + k) * plane3); };
    unsigned char *stats = j.base + L.off_stats;
    auto moment = [&](int k, int q) { return (void *)(stats + ((size_t)k * STATER_NQ + q) * plane3); };
    stater_gbuffers gb;
    fill_gbuffers(gb, j);
    std::memset(&v, 0, sizeof(v));
    v.n_buffers = j.d.n_transforms;
    v.width = j.d.width;
    v.height = j.d.height;
    v.filter_radius = j.d.filter_radius;
    v.ds_factor = -0.5f / (j.d.filter_sd * j.d.filter_sd);
    v.var_z = j.d.var_z;
    v.max_moment = j.d.max_moment;
    v.precision = prec;
    v.n = (const int32_t *)(j.base + L.off_n);
    for (int k = 0; k < j.d.n_transforms; k++) {
        v.m2[k] = moment(k, STATER_Q_M2);
        v.m3[k] = moment(k, STATER_Q_M3);
        v.m4[k] = moment(k, STATER_Q_M4);
        v.c2X[k] = moment(k, STATER_Q_C2X);
        v.c2Y[k] = moment(k, STATER_Q_C2Y);
        v.jb[k] = j.base + L.off_jb + (size_t)k * L.HW * L.T;
        v.lnS2[k] = out_of(0, k);
        v.se2[k] = out_of(1, k);
        v.m2C[k] = out_of(2, k);
        v.varD[k] = out_of(3, k);
        v.varCD[k] = out_of(4, k);
    }
    v.gbuffers = gb;
    std::memset(&f, 0, sizeof(f));
    f.n_buffers = j.d.n_transforms;
    f.width = j.d.width;
    f.height = j.d.height;
    f.filter_radius = j.d.filter_radius;
    f.ds_factor = v.ds_factor;
    f.alpha = j.d.alpha;
    f.mt_mode = STATER_MT_ALL;
    f.use_levc = j.d.max_moment >= 5 ? 1 : 0;
    f.precision = prec;
    f.n = v.n;
    f.film = L.T == 8 ? (const void *)(j.base + L.off_rgb64) : (const void *)(j.base + L.off_rgb);
    for (int k = 0; k < j.d.n_transforms; k++) {
        f.mean[k] = moment(k, STATER_Q_MEAN);
        f.varD[k] = v.varD[k];
        f.varCD[k] = v.varCD[k];
        f.jb[k] = v.jb[k];
        f.discr[k] = out_of(5, k);
        f.m2[k] = v.m2[k];
        f.m2C[k] = v.m2C[k];
    }
    f.gbuffers = gb;
    f.filmD = j.base + L.off_filmD;
    stater_test_order(j.d.transforms, j.d.n_transforms, f.test_order);
}

}  // namespace

// After a round: denoise the variance; then either allot the next round's
// samples (and fetch their maximum) or filter the film and copy it out.
bool stater_server::enqueue_after_round(Job &j) {
    const Slot &sl = slots[j.slot];
    cudaStream_t s = sl.stream;
    const Layout &L = j.L;
    const size_t plane3 = 3 * L.HW * L.T;
    unsigned char *stats = j.base + L.off_stats;
    auto moment = [&](int k, int q) { return (void *)(stats + ((size_t)k * STATER_NQ + q) * plane3); };
    stater_denoise_vars_args v;
    stater_denoise_film_args f;
    job_denoise_args(j, prec_of(this), v, f);
    if (stater_denoise_vars(&v, (stater_stream)s) != STATER_OK) return false;
    j.round++;
    if (j.round < j.d.rounds) {
        int32_t *target = (int32_t *)(j.base + L.off_target);
        const int budget = j.d.round_spp > 0 ? j.d.round_spp : j.d.spp;
        if (stater_calc_target_spp(j.d.width, j.d.height, budget, prec_of(this), v.n, v.varD[0], moment(0, STATER_Q_MEAN),
                                   kEps, kTmin, kTmax, target, (stater_stream)s) != STATER_OK)
            return false;
        // pixels sorted by target; the largest target and each step's active prefix to the host
        int32_t *dmax = (int32_t *)(j.base + L.off_max);
        int32_t *hist = (int32_t *)(j.base + L.off_hist);
        int32_t *act = (int32_t *)(j.base + L.off_act);
        const unsigned blocks = (unsigned)((L.HW + 255) / 256);
        const int nbins = sort_bins((int)L.chunk);
        if (cudaMemsetAsync(dmax, 0, 4, s) != cudaSuccess) return false;
        target_count_kernel<<<blocks, 256, sizeof(int) * nbins, s>>>(L.HW, target, (int)L.chunk, nbins, hist, dmax);
        target_offsets_kernel<<<1, 1024, 0, s>>>((int)blocks, nbins, hist, act);
        target_place_kernel<<<blocks, 256, sizeof(int) * 8 * nbins, s>>>(L.HW, target, (int)L.chunk, nbins, hist,
                                                                       (int32_t *)(j.base + L.off_order),
                                                                       (int32_t *)(j.base + L.off_tsorted));
        if (cudaGetLastError() != cudaSuccess) return false;
        if (cudaMemcpyAsync(sl.hmax, dmax, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return false;
        if (cudaMemcpyAsync(sl.hact, act, 4 * (kBins + 2), cudaMemcpyDeviceToHost, s) != cudaSuccess) return false;
    } else {
        // Film::UpdateImage: the film image is the untransformed mean that denoiseFilm filters
        const float *fs = (const float *)(j.base + L.off_film);
        float *rgb = (float *)(j.base + L.off_rgb);
        if (stater_film_update_image(j.d.width, j.d.height, fs, fs + 3 * L.HW, fs + 4 * L.HW, 1.0f, rgb,
                                     (stater_stream)s) != STATER_OK)
            return false;
        if (L.T == 8) {
            widen_kernel<<<(unsigned)((3 * L.HW + 255) / 256), 256, 0, s>>>(3 * L.HW, rgb,
                                                                          (double *)(j.base + L.off_rgb64));
            if (cudaGetLastError() != cudaSuccess) return false;
        }
        if (stater_denoise_film(&f, (stater_stream)s) != STATER_OK) return false;
        if (j.d.out_host) {
            if (L.T == 4) {
                void *dst = j.out_stage ? (void *)j.out_stage : j.d.out_host;
                if (cudaMemcpyAsync(dst, f.filmD, 3 * L.HW * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
                    return false;
            } else {
                // plain FP64 form: the film is delivered as float32 like the FP32 form
                return false;
            }
        }
        j.final_enqueued = true;
    }
    return cudaEventRecord(j.ev, s) == cudaSuccess;
}

bool stater_server::fusable(const Job &j) const {
    return cfg.fuse_small_jobs && cfg.precision == STATER_F32 && j.d.rounds == 1 && j.L.HW <= kFuseMaxPixels &&
           j.d.n_transforms <= 5 && j.d.n_features <= 7;
}

// Pinned staging of the slot for the results of `jobs` bound for pageable
// buffers; the slot is idle, so its staging is free to grow.
bool stage_results(Slot &sl, const std::vector<Job *> &jobs) {
    size_t need = 0;
    for (Job *j : jobs)
        if (j->d.out_host && !j->out_pinned) need += 3 * j->L.HW;
    if (need > sl.out_cap) {
        if (sl.out) cudaFreeHost(sl.out);
        sl.out = nullptr;
        sl.out_cap = 0;
        if (cudaMallocHost((void **)&sl.out, need * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            sl.out = nullptr;
            return false;
        }
        sl.out_cap = need;
    }
    size_t o = 0;
    for (Job *j : jobs) {
        j->out_stage = nullptr;
        if (j->d.out_host && !j->out_pinned) {
            j->out_stage = sl.out + o;
            o += 3 * j->L.HW;
        }
    }
    return true;
}

bool stater_server::start_group(std::vector<std::shared_ptr<Job>> &group) {
    const int slot = group[0]->slot;
    Slot &sl = slots[slot];
    cudaStream_t s = sl.stream;
    {
        std::vector<Job *> js;
        for (auto &g : group) js.push_back(g.get());
        if (!stage_results(sl, js)) return false;
    }
    std::vector<stater_batch_job> bj(group.size());
    for (size_t i = 0; i < group.size(); i++) {
        Job &j = *group[i];
        if (cudaMallocAsync((void **)&j.base, j.L.total, s) != cudaSuccess) {
            cudaGetLastError();
            j.base = nullptr;
            return false;
        }
        if (cudaMemsetAsync(j.base, 0, j.L.off_samples, s) != cudaSuccess) return false;
        if (cudaEventCreateWithFlags(&j.ev, cudaEventDisableTiming) != cudaSuccess) return false;
        if (!enqueue_round(j, j.d.spp, true)) return false;
        const float *fs = (const float *)(j.base + j.L.off_film);
        float *rgb = (float *)(j.base + j.L.off_rgb);
        if (stater_film_update_image(j.d.width, j.d.height, fs, fs + 3 * j.L.HW, fs + 4 * j.L.HW, 1.0f, rgb,
                                     (stater_stream)s) != STATER_OK)
            return false;
        std::memset(&bj[i], 0, sizeof(bj[i]));
        bj[i].acc.width = j.d.width;
        bj[i].acc.height = j.d.height;
        bj[i].acc.n_transforms = j.d.n_transforms;
        bj[i].film_rgb = rgb;
        bj[i].film_scale = 1.0f;
        job_denoise_args(j, STATER_F32, bj[i].vars, bj[i].film);
    }
    if (batch_denoise_once(bj.data(), (int)bj.size(), s, sl.staging, kStagingBytes) != STATER_OK) return false;
    for (auto &jp : group) {
        Job &j = *jp;
        if (j.d.out_host &&
            cudaMemcpyAsync(j.out_stage ? (void *)j.out_stage : j.d.out_host, j.base + j.L.off_filmD, 3 * j.L.HW * 4,
                            cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return false;
        j.round = 1;
        j.final_enqueued = true;
        if (cudaEventRecord(j.ev, s) != cudaSuccess) return false;
    }
    return true;
}

bool stater_server::start(Job &j) {
    Slot &sl = slots[j.slot];
    if (!stage_results(sl, {&j})) return false;
    if (cudaMallocAsync((void **)&j.base, j.L.total, sl.stream) != cudaSuccess) {
        cudaGetLastError();
        j.base = nullptr;
        return false;
    }
    if (cudaMemsetAsync(j.base, 0, j.L.off_samples, sl.stream) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&j.ev, cudaEventDisableTiming) != cudaSuccess) return false;
    if (!enqueue_round(j, j.d.spp, true)) return false;
    return enqueue_after_round(j);
}

void stater_server::finish(Job &j, bool ok) {
    if (j.slot >= 0) {
        Slot &sl = slots[j.slot];
        if (j.base) cudaFreeAsync(j.base, sl.stream);
        if (!ok) cudaStreamSynchronize(sl.stream);
        // a fused group holds its slot until its last job is finished
        if (!j.group_left || --*j.group_left == 0) sl.busy = false;
    }
    if (j.ev) cudaEventDestroy(j.ev);
    j.ev = nullptr;
    j.base = nullptr;
    j.t_done = Clock::now();
    j.latency_ms = std::chrono::duration<double, std::milli>(j.t_done - j.t_submit).count();
    std::lock_guard<std::mutex> lk(mu);
    used -= j.footprint;
    j.state = ok ? STATER_JOB_DONE : STATER_JOB_FAILED;
    if (ok) {
        completed++;
        latencies.push_back(j.latency_ms);
        pixels_done += (double)j.L.HW;
        last_done = j.t_done;
    } else {
        failed++;
    }
    active.erase(std::remove_if(active.begin(), active.end(), [&](const std::shared_ptr<Job> &p) { return p.get() == &j; }),
                 active.end());
    cv_done.notify_all();
}

// Scheduler loop: admit queued jobs in arrival order while a slot is free and
// the head job's footprint fits under the budget, then advance every job whose
// event has completed.
void stater_server::run() {
    cudaSetDevice(device);
    while (true) {
        std::vector<std::shared_ptr<Job>> to_start;
        std::vector<std::vector<std::shared_ptr<Job>>> groups;
        {
            std::unique_lock<std::mutex> lk(mu);
            if (stop && queue.empty() && active.empty()) break;
            while (!queue.empty()) {
                auto &j = queue.front();
                int free_slot = -1;
                for (size_t i = 0; i < slots.size(); i++)
                    if (!slots[i].busy) {
                        free_slot = (int)i;
                        break;
                    }
                const bool fits = used + j->footprint <= budget || active.empty();
                if (free_slot < 0 || !fits) break;
                slots[free_slot].busy = true;
                // Small single-round jobs waiting together share a slot as one
                // group, but only as many as the free slots cannot take one by
                // one: a run of q such jobs at the head of the queue with f free
                // slots forms groups of ceil(q / f), so fusion never serialises
                // jobs that could run side by side.
                std::vector<std::shared_ptr<Job>> group;
                if (fusable(*j)) {
                    int nfree = 0, q = 0;
                    for (const auto &sl : slots) nfree += sl.busy ? 0 : 1;
                    nfree += 1;  // the slot just taken
                    for (const auto &qj : queue) {
                        if (!fusable(*qj) || q == kFuseMaxJobs * nfree) break;
                        q++;
                    }
                    const int gsize = std::min(kFuseMaxJobs, (q + nfree - 1) / nfree);
                    group.push_back(j);
                    queue.pop_front();
                    while (!queue.empty() && (int)group.size() < gsize && fusable(*queue.front()) &&
                           used + group_footprint(group) + queue.front()->footprint <= budget) {
                        group.push_back(queue.front());
                        queue.pop_front();
                    }
                } else {
                    group.push_back(j);
                    queue.pop_front();
                }
                auto left = group.size() > 1 ? std::make_shared<int>((int)group.size()) : nullptr;
                for (auto &g : group) {
                    g->slot = free_slot;
                    g->state = STATER_JOB_RUNNING;
                    g->group_left = left;
                    used += g->footprint;
                    active.push_back(g);
                }
                peak = std::max(peak, used);
                if (group.size() > 1 || fusable(*group[0]))
                    groups.push_back(group);
                else
                    to_start.push_back(group[0]);
            }
        }
        for (auto &j : to_start)
            if (!start(*j)) finish(*j, false);
        for (auto &g : groups)
            if (!start_group(g))
                for (auto &j : g) finish(*j, false);
        bool progressed = !to_start.empty() || !groups.empty();
        std::vector<std::shared_ptr<Job>> snapshot;
        {
            std::lock_guard<std::mutex> lk(mu);
            snapshot = active;
        }
        for (auto &j : snapshot) {
            if (!j->ev) continue;
            const cudaError_t q = cudaEventQuery(j->ev);
            if (q == cudaErrorNotReady) continue;
            progressed = true;
            if (q != cudaSuccess) {
                cudaGetLastError();
                finish(*j, false);
                continue;
            }
            if (j->final_enqueued) {
                if (j->out_stage) std::memcpy(j->d.out_host, j->out_stage, 3 * j->L.HW * sizeof(float));
                finish(*j, true);
                continue;
            }
            // the previous round's largest per-pixel target is now in pinned memory
            const int next = *slots[j->slot].hmax;
            bool ok = enqueue_round(*j, next, false) && enqueue_after_round(*j);
            if (!ok) finish(*j, false);
        }
        if (!progressed) {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait_for(lk, std::chrono::microseconds(50));
        }
    }
}

extern "C" {

double stater_job_footprint(const stater_job_desc *job, int32_t precision, int32_t chunk_spp) {
    if (!job) return 0;
    const Layout L = layout(*job, precision, chunk_spp);
    return (double)L.total + (double)scratch_bytes(L);
}

stater_status stater_server_create(const stater_server_config *cfg, stater_server **out) {
    clear_error();
    if (!cfg || !out || cfg->max_slots < 1 || cfg->max_slots > 64 ||
        (cfg->precision != STATER_F32 && cfg->precision != STATER_F64))
        return set_error(STATER_ERR_INVALID, "stater_server_create: bad configuration");
    auto *s = new stater_server();
    s->cfg = *cfg;
    if (s->cfg.chunk_spp < 0) s->cfg.chunk_spp = 0;  // 0: automatic per job
    cudaGetDevice(&s->device);
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    s->budget = cfg->hbm_budget_bytes > 0 ? cfg->hbm_budget_bytes : 0.8 * (double)free_b;
    // keep freed job memory in the pool instead of returning it to the driver
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    s->slots.resize(cfg->max_slots);
    for (auto &sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaMallocHost(&sl.hmax, sizeof(int32_t)) != cudaSuccess ||
            cudaMallocHost(&sl.hact, sizeof(int32_t) * (kBins + 2)) != cudaSuccess ||
            cudaMallocHost(&sl.staging, kStagingBytes) != cudaSuccess) {
            cudaGetLastError();
            delete s;
            return set_error(STATER_ERR_CUDA, "stater_server_create: stream or pinned allocation failed");
        }
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return STATER_OK;
}

stater_status stater_server_submit(stater_server *srv, const stater_job_desc *job, int64_t *job_id) {
    clear_error();
    if (!srv || !job || job->width <= 0 || job->height <= 0 || job->spp < 1 || job->rounds < 1 ||
        job->n_transforms < 1 || job->n_transforms > STATER_MAX_TRANSFORMS ||
        job->transforms[0].kind != STATER_TK_IDENTITY || job->n_features < 0 ||
        job->n_features > STATER_MAX_FEATURES || job->max_moment < 3 || job->max_moment > 5 ||
        job->filter_radius < 0 || job->filter_radius > STATER_MAX_RADIUS || !(job->filter_sd > 0.f) ||
        !(job->alpha > 0.f && job->alpha < 1.f) || job->round_spp < 0)
        return set_error(STATER_ERR_INVALID, "stater_server_submit: bad job description");
    if (srv->cfg.precision == STATER_F64 && job->out_host)
        return set_error(STATER_ERR_UNSUPPORTED, "stater_server_submit: host output is float32 (serve in STATER_F32)");
    auto j = std::make_shared<Job>();
    j->d = *job;
    if (job->out_host) {
        cudaPointerAttributes pa;
        const cudaError_t e = cudaPointerGetAttributes(&pa, job->out_host);
        if (e != cudaSuccess) cudaGetLastError();
        // a result in pageable memory is copied there by the host, from staging
        if (e == cudaSuccess && pa.type == cudaMemoryTypeDevice)
            return set_error(STATER_ERR_INVALID, "stater_server_submit: out_host is device memory");
        j->out_pinned = e == cudaSuccess && pa.type == cudaMemoryTypeHost;
    }
    j->L = layout(*job, srv->cfg.precision, srv->cfg.chunk_spp);
    j->footprint = (double)j->L.total + (double)scratch_bytes(j->L);
    j->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (j->footprint > srv->budget)
            return set_error(STATER_ERR_NOMEM, "stater_server_submit: the job alone exceeds the memory budget");
        j->id = srv->next_id++;
        srv->jobs[j->id] = j;
        srv->queue.push_back(j);
        srv->submitted++;
        if (!srv->have_first) {
            srv->have_first = true;
            srv->first_submit = j->t_submit;
        }
    }
    srv->cv_work.notify_all();
    if (job_id) *job_id = j->id;
    return STATER_OK;
}

stater_status stater_server_poll(stater_server *srv, int64_t job_id, int32_t *state, double *latency_ms) {
    clear_error();
    if (!srv) return set_error(STATER_ERR_INVALID, "stater_server_poll: null server");
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(job_id);
    if (it == srv->jobs.end()) return set_error(STATER_ERR_INVALID, "stater_server_poll: unknown job");
    if (state) *state = it->second->state;
    if (latency_ms) *latency_ms = it->second->latency_ms;
    return STATER_OK;
}

stater_status stater_server_wait(stater_server *srv, int64_t job_id, double timeout_s) {
    clear_error();
    if (!srv) return set_error(STATER_ERR_INVALID, "stater_server_wait: null server");
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(job_id);
    if (it == srv->jobs.end()) return set_error(STATER_ERR_INVALID, "stater_server_wait: unknown job");
    auto j = it->second;
    const bool ok = srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        return j->state == STATER_JOB_DONE || j->state == STATER_JOB_FAILED;
    });
    if (!ok) return set_error(STATER_ERR_TIMEOUT, "stater_server_wait: job not finished in time");
    if (j->state == STATER_JOB_FAILED) return set_error(STATER_ERR_CUDA, "stater_server_wait: job failed");
    return STATER_OK;
}

stater_status stater_server_drain(stater_server *srv, double timeout_s) {
    clear_error();
    if (!srv) return set_error(STATER_ERR_INVALID, "stater_server_drain: null server");
    std::unique_lock<std::mutex> lk(srv->mu);
    const bool ok = srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                          [&] { return srv->queue.empty() && srv->active.empty(); });
    return ok ? STATER_OK : set_error(STATER_ERR_TIMEOUT, "stater_server_drain: jobs still running");
}

stater_status stater_server_stats_get(stater_server *srv, stater_server_stats *out) {
    clear_error();
    if (!srv || !out) return set_error(STATER_ERR_INVALID, "stater_server_stats_get: null argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = srv->submitted;
    out->completed = srv->completed;
    out->failed = srv->failed;
    out->running = (int64_t)srv->active.size();
    out->queued = (int64_t)srv->queue.size();
    out->peak_footprint_bytes = srv->peak;
    if (!srv->latencies.empty()) {
        std::vector<double> v = srv->latencies;
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) {
            const double pos = q * (double)(v.size() - 1);
            const size_t i = (size_t)pos;
            const double f = pos - (double)i;
            return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
        };
        out->latency_p50_ms = pct(0.50);
        out->latency_p99_ms = pct(0.99);
        double sum = 0;
        for (double x : v) sum += x;
        out->latency_mean_ms = sum / (double)v.size();
        const double span = std::chrono::duration<double>(srv->last_done - srv->first_submit).count();
        out->mpix_per_s = span > 0 ? srv->pixels_done / span / 1e6 : 0;
    }
    return STATER_OK;
}

stater_status stater_server_destroy(stater_server *srv) {
    clear_error();
    if (!srv) return STATER_OK;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    if (srv->worker.joinable()) srv->worker.join();
    for (auto &sl : srv->slots) {
        if (sl.stream) {
            cudaStreamSynchronize(sl.stream);
            cudaStreamDestroy(sl.stream);
        }
        if (sl.hmax) cudaFreeHost(sl.hmax);
        if (sl.hact) cudaFreeHost(sl.hact);
        if (sl.staging) cudaFreeHost(sl.staging);
        if (sl.out) cudaFreeHost(sl.out);
    }
    delete srv;
    return STATER_OK;
}

}  // extern "C"
