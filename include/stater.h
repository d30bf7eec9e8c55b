/*
 * stater: GB300-native (sm_103a) statistics hot path of StatER.
 *
 * C ABI of libstater.so. Plain pointers and sizes only; every call returns a
 * stater_status and never aborts. All image buffers are planar: a "plane" holds
 * W*H elements with pixel p = y*W + x, and an RGB statistics buffer ("float3
 * buffer" in the reference) is three consecutive planes (R, G, B). Element type
 * of the statistics buffers is chosen per call by `precision`: STATER_F64 is the
 * plain FP64 form, STATER_F32 the FP32 form. Sample counts are int32, as the
 * reference's t?-b?-film-n buffer (estimator.h:477).
 *
 * Reference boundary replaced (paths inside the StatER tree):
 *   cv::cuda::stat_denoiser::setup()               src/statistics/estimator.h:383
 *   cv::cuda::stat_denoiser::denoiseVars<float3>   src/statistics/estimator.cpp:374-414
 *   cv::cuda::stat_denoiser::denoiseFilm           src/statistics/estimator.cpp:421-457
 *   cv::cuda::stat_denoiser::calcTargetSPP<float3> src/statistics/estimator.cpp:502-511
 *   cv::cuda::stat_denoiser::synchronize           src/statistics/estimator.cpp:516
 *   cv::cuda::stat_denoiser::printMacroConfiguration src/statistics/estimator.cpp:520
 * and, moved from the CPU onto the GPU:
 *   StatTile::AddTransformSample* / AddSample*     src/statistics/estimator.h:226-324
 *   Estimator::MergeTransformTile / MergeTile      src/statistics/estimator.cpp:267-324
 *   Estimator::CalcMeanVars (calcMatMeanVar)       src/statistics/estimator.cpp:462-496
 */
#ifndef STATER_H
#define STATER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STATER_ABI_VERSION 2
#define STATER_MAX_TRANSFORMS 8 /* buffers b0..b7 per statistics type */
#define STATER_MAX_GBUFFERS 8
#define STATER_MAX_FEATURES 16
#define STATER_MAX_RADIUS 20   /* the reference default filterradius */

typedef struct CUstream_st *stater_stream; /* a cudaStream_t; NULL = legacy default stream */

typedef enum {
    STATER_OK = 0,
    STATER_ERR_INVALID = 1,     /* bad argument (message in stater_last_error) */
    STATER_ERR_CUDA = 2,        /* a CUDA call failed */
    STATER_ERR_NOMEM = 3,       /* device scratch could not be allocated */
    STATER_ERR_UNSUPPORTED = 4, /* configuration outside what this build handles */
    STATER_ERR_TIMEOUT = 5      /* a bounded device wait gave up */
} stater_status;

typedef enum { STATER_F32 = 0, STATER_F64 = 1 } stater_precision;

/* Monotone transforms applied to radiance samples. Transform 0 of every job must
 * be STATER_TK_IDENTITY: it is the untransformed "t0 / film" set of the reference. */
typedef enum {
    STATER_TK_IDENTITY = 0,
    STATER_TK_LOG1P = 1,
    STATER_TK_SQRT = 2,
    STATER_TK_CBRT = 3,
    STATER_TK_ASINH = 4,
    STATER_TK_BOXCOX = 5 /* (x^lambda - 1) / lambda, identity at lambda == 1 (estimator.h:43-76) */
} stater_transform_kind;

/* Moment planes of one transform, in this order, 3 planes each. */
typedef enum {
    STATER_Q_MEAN = 0, STATER_Q_M2 = 1, STATER_Q_M3 = 2, STATER_Q_M4 = 3,
    STATER_Q_C2X = 4, STATER_Q_C2Y = 5, STATER_Q_M1 = 6, STATER_NQ = 7
} stater_moment;

/* How the Welch decisions of several transforms combine in denoiseFilm; the
 * values are those of the reference's FILM_MULTI_TRANSFORM_MODE switch
 * (src/statistics/statpbrt.h:27-29, estimator.cpp:446-448). */
typedef enum {
    STATER_MT_ALL = 2, /* neighbour kept only if every transform accepts it */
    STATER_MT_JB = 3   /* only the transform with the lowest Jarque-Bera score at the centre */
} stater_mt_mode;

/* Variance behind the Welch discriminator of denoiseFilm: the reference's
 * CASCADE_MODE build switch (scripts/alternate-builds/build-asm+m.sh sets 0 for
 * the "M" variant; MC and MCL keep the default 1). The cascade feeds the
 * denoised variances of denoiseVars into the mean filter; without it, each pixel
 * uses its own sample variance (denoiseVars is then needed only for adaptive
 * sampling, as the comment in build-asm+m.sh notes). */
typedef enum {
    STATER_DISCR_DENOISED = 0, /* CASCADE_MODE=1: varCD with use_levc, else varD */
    STATER_DISCR_SAMPLE = 1    /* CASCADE_MODE=0: m2C / (n - 1) with use_levc, else m2 / (n - 1) */
} stater_discr_source;

/* Variance behind the adaptive-sampling error estimate of calcTargetSPP: the
 * reference's AS_MODE build switch ("ASM" by default, "ASN" with AS_MODE=0 in
 * scripts/alternate-builds/build-asn+mcl.sh). calcTargetSPP receives both n, m2
 * and varD (estimator.cpp:502-511); ASM uses the denoised variance, ASN the
 * pixel's own sample variance m2 / (n - 1). */
typedef enum {
    STATER_AS_DENOISED = 0, /* "ASM", AS_MODE=1 */
    STATER_AS_SAMPLE = 1    /* "ASN", AS_MODE=0 */
} stater_as_source;

typedef enum {
    STATER_ACC_EXACT = 0, /* the reference's operation order: x/n division, libm-accurate transforms */
    STATER_ACC_FAST = 1   /* FP32 only: reciprocal of n shared per sample, fast transforms */
} stater_acc_mode;

typedef struct {
    int32_t kind;   /* stater_transform_kind */
    float lambda;   /* Box-Cox lambda (float, as the reference's lambdas list) */
} stater_transform;

/* G-buffers used by a range kernel (estimator.cpp:10-18, 69-81): each entry is
 * `channels` (1 or 3) consecutive planes with the element type of the call. */
typedef struct {
    int32_t count;
    const void *planes[STATER_MAX_GBUFFERS];
    int32_t channels[STATER_MAX_GBUFFERS];
    float dr_factor[STATER_MAX_GBUFFERS]; /* -0.5 / sigma_r^2 */
} stater_gbuffers;

/* ---- lifetime ---------------------------------------------------------- */

/* stat_denoiser::setup(): selects the current device, checks that it is an
 * sm_103 part and prepares per-device state. Idempotent. */
stater_status stater_setup(void);
/* stat_denoiser::synchronize(stream). Also reports, once, STATER_ERR_TIMEOUT
 * when a bounded wait of a TMA-fed kernel gave up since the last call (the
 * affected call's results are incomplete; the message says whether the final
 * wait for copies in flight gave up too), and clears that state. */
stater_status stater_synchronize(stater_stream stream);
/* stat_denoiser::printMacroConfiguration(): prints the runtime configuration
 * that replaces the reference's compile-time macros. */
void stater_print_macro_configuration(void);
/* Message of the last failing call on this thread ("" if none). */
const char *stater_last_error(void);
int32_t stater_abi_version(void);
/* Test hook for the bounded waits of the TMA-fed pipelines (the FP32
 * stater_accumulate and stater_lev_accumulate kernels); no counterpart in the
 * reference, which has no such pipelines. wait_polls limits every pipeline wait
 * (0 = the default, 4,194,304 polls of mbarrier.try_wait); stall_producers = 1
 * makes their producers issue no copies, so that the consumers' waits run out
 * and the kernels end early, leaving STATER_ERR_TIMEOUT for stater_synchronize
 * (stalling requires wait_polls <= 65536). The producer's final wait for copies
 * it has issued always keeps the default limit. Settings are process-wide and
 * apply to launches made after the call. */
stater_status stater_debug_set_pipeline_waits(uint32_t wait_polls, int32_t stall_producers);
/* Tuning hook of the TMA-fed FP32 accumulation, no counterpart in the
 * reference: warp w of each CTA keeps the moments of transform order[w]
 * (order: a permutation of 0 .. n_transforms-1), for launches with that many
 * transforms made after the call, in place of the library's own placement.
 * Results are the same bits for every order. n_transforms = 0 restores the
 * library's placement. Process-wide. */
stater_status stater_debug_set_warp_order(const int32_t *order, int32_t n_transforms);
/* Tuning hook of the FP32 variance filter's row ring, no counterpart in the
 * reference: tile_height 4, 8 or 16 forces that tile height (where its ring
 * fits in shared memory) for the single-image calls made after this one;
 * -1 runs the per-transform kernel in place of the ring; 0 restores the
 * tuner. Results are the same bits in every form. Process-wide. */
stater_status stater_debug_set_vars_ring_form(int32_t tile_height);
/* FP32 throughput probe, no counterpart in the reference: launches `blocks`
 * CTAs of 256 threads, each thread running 8 independent chains of 16 * iters
 * FMAs (packed = 1: fma.rn.f32x2, two lanes per instruction), and returns in
 * *flops the floating-point operations launched (an FMA counts 2). Timing the
 * launch gives the FP32 rate the stage-2 filters are measured against. sink:
 * device float [blocks], written only if a chain reaches an impossible value. */
stater_status stater_fp32_peak_probe(int32_t blocks, int32_t iters, int32_t packed, float *sink, double *flops,
                                     stater_stream stream);
/* Page-locked host memory for sample buffers (no counterpart in the reference,
 * whose Estimator pins its host buffers through OpenCV's allocator,
 * estimator.h:382). The memory is mapped anonymously on huge pages where the
 * operating system offers transparent huge pages, zeroed and registered with
 * CUDA, so copies from it run at the host link's rate every time: with base
 * pages, copies of tens of GB varied between about 65 and 210 GB/s from run to
 * run on a GB300 host, and from huge pages held 210 GB/s. Free with
 * stater_host_free and the same size. */
stater_status stater_host_alloc(size_t bytes, void **out);
stater_status stater_host_free(void *ptr, size_t bytes);
/* Releases cached device scratch and tables of the current device and forgets
 * the cached device addresses of the library's fixed arrays. Call it before a
 * device reset (cudaDeviceReset) that is followed by further calls into the
 * library: the cached buffers and addresses do not survive the reset. */
stater_status stater_release_cache(void);

/* ---- stage 1: moment accumulation ------------------------------------- */

/* Per-sample statistics update of StatTile (estimator.h:226-324), for a whole
 * image at once. Samples are float32 planes [S][5+G][W*H]: R, G, B, the
 * in-pixel position u, v (inPxP, statpath.cpp:339) and G feature channels.
 * For pixel p only the first count[p] sample planes are used (count == NULL:
 * all S). Statistics persist in the caller's buffers, so later calls continue
 * the same online update, as the reference's tiles do across iterations
 * (statpath.cpp:133-150). n is incremented once per sample.
 *   stats: precision-typed [K][7][3][W*H] (transform, moment, channel, pixel)
 *   gmean: precision-typed [G][W*H] running mean of every feature channel
 *          (AddSampleM1 of the G-buffer tiles, statpath.cpp:366-379); may be NULL if G == 0
 * max_moment: 1..5 as the reference's "maxmoment" (statpath.cpp:36-60; 5 = M4 + c2X, c2Y, m1).
 * FP32 with STATER_ACC_FAST reads the planes through the Tensor Memory
 * Accelerator when the column count is a multiple of 4 and `samples` is
 * 16-byte aligned, and through plain loads otherwise; both forms give the same
 * bits. */
typedef struct {
    int32_t width, height;
    int32_t n_samples;          /* S */
    int32_t n_features;         /* G */
    const float *samples;
    const int32_t *count;       /* nullable */
    int32_t n_transforms;       /* K */
    stater_transform transforms[STATER_MAX_TRANSFORMS];
    int32_t max_moment;
    stater_precision precision;
    int32_t mode;               /* stater_acc_mode */
    int32_t *n;
    void *stats;
    void *gmean;
    /* Optional film (film_contrib_sum == NULL: off): the same sums as
     * stater_film_add_samples, taken from the samples this call reads anyway. */
    float *film_contrib_sum;    /* [3][W*H] */
    float *film_weight_sum;     /* [W*H] */
    float *film_spill;          /* [4][W*H] */
    float film_max_sample_luminance; /* INFINITY = off */
    /* Optional pixel index (NULL: sample column i is pixel i): the sample planes
     * are [S][5+G][n_active] and column i, with count[i] samples, belongs to
     * pixel pixel_index[i]. Columns with samples must name distinct pixels;
     * columns with count 0 (padding) and indices outside the image are skipped.
     * Lets a caller pack only the pixels that still need samples, e.g. sorted
     * by their adaptive target so that each launch covers a dense prefix. */
    const int32_t *pixel_index;
    int32_t n_active;
} stater_accumulate_args;
stater_status stater_accumulate(const stater_accumulate_args *a, stater_stream stream);

/* Seeded synthetic sample source (stands in for the renderer): writes sample
 * planes [S][5+G][W*H] for sample indices first_index[p] + s (first_index may be
 * NULL = 0), counter-based (Philox4x32-10) so that any sample of any pixel can be
 * regenerated. Radiance = per-region lognormal mean x lognormal(0, sigma) with
 * firefly_prob fireflies scaled by firefly_scale; u,v uniform; features piecewise
 * constant per region plus small jitter, or, with lev_r2 > 0, uniform per sample
 * with radiance linear in the features (target R^2 = lev_r2). */
typedef struct {
    int32_t width, height, n_samples, n_features;
    uint64_t seed;
    int32_t region;             /* side of the square regions sharing a mean (1 = per pixel) */
    float mean_mu, mean_sigma;  /* per-region mean ~ LogNormal(mean_mu, mean_sigma) */
    float noise_sigma;          /* per-sample factor ~ LogNormal(0, noise_sigma) */
    float firefly_prob, firefly_scale;
    float lev_r2;               /* 0 = off */
    const int32_t *first_index; /* nullable */
    const int32_t *count;       /* nullable: only the first count[p] samples of pixel p are written */
    float *samples;
    /* Optional pixel index as in stater_accumulate_args: column i of the planes
     * [S][5+G][n_active] holds the samples of pixel pixel_index[i]; first_index
     * and count are then per column. */
    const int32_t *pixel_index;
    int32_t n_active;
} stater_generate_args;
stater_status stater_generate_samples(const stater_generate_args *a, stater_stream stream);

/* Estimator::MergeTransformTile / MergeTile (estimator.cpp:267-324): copies CPU
 * tile records into the image planes. records: raw StatTilePixel<Vec3> of the
 * reference's float build (320 bytes: uint64 n at 0, t0 at 64, t1 at 192, seven
 * float3 each), for every tile in order, pixels row-major in the tile. bounds:
 * int32 [n_tiles][4] = x0, y0, x1, y1 (exclusive). Writes n and FP32 stats
 * [n_sets][7][3][W*H]: n_sets = 2 (transform tile) writes all seven quantities of
 * t0 and t1; n_sets = 1 (plain tile) writes t0's mean, M2, M3 and M4 and leaves
 * its c2X, c2Y and m1 planes as they are, as MergeTile does. Device pointers. */
stater_status stater_merge_tiles(int32_t width, int32_t height, int32_t n_tiles,
                                 const int32_t *bounds, const void *records, int32_t n_sets,
                                 int32_t *n, float *stats, stater_stream stream);

/* Pairwise combine of two moment sets of the same geometry (Chan et al.;
 * Pebay 2008): A <- A (+) B, for merging independently accumulated rounds or
 * partial tiles. stats as in stater_accumulate. */
stater_status stater_merge_moments(int32_t width, int32_t height, int32_t n_transforms,
                                   int32_t max_moment, stater_precision precision, int32_t *nA,
                                   void *statsA, const int32_t *nB, const void *statsB,
                                   stater_stream stream);

/* ---- stage 2: denoising ------------------------------------------------- */

/* stat_denoiser::denoiseVars<float3> (estimator.cpp:374-414). For every
 * transform b < n_buffers (pointer tables indexed by b, each an RGB buffer):
 * per-pixel Jarque-Bera score jb (one plane per buffer, BUF_LIST estimator.h:467),
 * Bonett lnS2 and se2, LEV-corrected m2C, and the variance filter outputs varD and
 * varCD. m2C_in (nullable) replaces the c2X/c2Y correction of buffer 0 by an
 * external LEV result (stater_lev_solve). */
typedef struct {
    int32_t n_buffers;
    int32_t width, height;
    int32_t filter_radius;
    float ds_factor;            /* -0.5 / filtersd^2 (estimator.h:353) */
    float var_z;                /* "varzvalue" (statpath.cpp:1070), default 2.80703 */
    int32_t max_moment;
    stater_precision precision;
    const int32_t *n;
    const void *m2[STATER_MAX_TRANSFORMS];
    const void *m3[STATER_MAX_TRANSFORMS];
    const void *m4[STATER_MAX_TRANSFORMS];   /* used when max_moment >= 4 */
    const void *c2X[STATER_MAX_TRANSFORMS];  /* used when max_moment >= 5 */
    const void *c2Y[STATER_MAX_TRANSFORMS];
    const void *m2C_in;
    stater_gbuffers gbuffers;
    void *jb[STATER_MAX_TRANSFORMS];
    void *lnS2[STATER_MAX_TRANSFORMS];
    void *se2[STATER_MAX_TRANSFORMS];
    void *m2C[STATER_MAX_TRANSFORMS];
    void *varD[STATER_MAX_TRANSFORMS];
    void *varCD[STATER_MAX_TRANSFORMS];
} stater_denoise_vars_args;
stater_status stater_denoise_vars(const stater_denoise_vars_args *a, stater_stream stream);

/* stat_denoiser::denoiseFilm (estimator.cpp:421-457). Welch-discriminated
 * neighbourhood filter of the film. Buffer 0 uses `film` as its mean, as the
 * reference passes filmBuffer for the untransformed set; buffers b >= 1 use
 * mean[b]. Writes the per-pixel Welch discriminator discr[b] (squared standard
 * error of the mean) and filmD. accept_bits (nullable, debug): uint32
 * [W*H][n_buffers][ceil((2R+1)^2/32)], bit (dy+R)(2R+1)+(dx+R) set when
 * transform b accepts that neighbour. */
typedef struct {
    int32_t n_buffers;
    int32_t width, height;
    int32_t filter_radius;
    float ds_factor;
    float alpha;                /* two-sided level of the Welch test, e.g. 0.01 */
    int32_t mt_mode;            /* stater_mt_mode */
    int32_t use_levc;           /* 1: test with varCD, 0: with varD */
    stater_precision precision;
    const int32_t *n;
    const void *film;
    const void *mean[STATER_MAX_TRANSFORMS];  /* [0] unused */
    const void *varD[STATER_MAX_TRANSFORMS];
    const void *varCD[STATER_MAX_TRANSFORMS];
    const void *jb[STATER_MAX_TRANSFORMS];    /* used by STATER_MT_JB */
    stater_gbuffers gbuffers;
    void *discr[STATER_MAX_TRANSFORMS];
    void *filmD;
    uint32_t *accept_bits;
    /* Order in which the FP32 form tests the transforms of a neighbour (it stops
     * at the first rejection in STATER_MT_ALL mode; the result does not depend
     * on the order). A permutation of 0..n_buffers-1, or all zero for the
     * reverse index order. stater_test_order gives one from the transform kinds. */
    int32_t test_order[STATER_MAX_TRANSFORMS];
    /* stater_discr_source (0, the default, is the reference's default build) and
     * the buffers STATER_DISCR_SAMPLE reads: m2 (moments) without use_levc, the
     * m2C output of stater_denoise_vars with it. */
    int32_t discr_source;
    const void *m2[STATER_MAX_TRANSFORMS];
    const void *m2C[STATER_MAX_TRANSFORMS];
} stater_denoise_film_args;
stater_status stater_denoise_film(const stater_denoise_film_args *a, stater_stream stream);

/* The reference's own buffer layout (estimator.cpp:26-81): the Estimator owns
 * pitched cv::cuda::GpuMat images and passes the denoiser PtrStepSzb tables
 * {data, step, rows, cols}. An RGB buffer is one image of interleaved channels
 * (CV_32FC3 with STATER_F32, CV_64FC3 with STATER_F64); n, jb and one-channel
 * G-buffers are one-channel images. Element (c, x, y) of a buffer with C
 * channels is at data + y * step + (x * C + c) * element size. The pitched entry
 * points take the same argument blocks as the planar ones, with every buffer
 * pointer naming the caller's pitched image (`data` of its PtrStepSzb), and one
 * step per kind of buffer (cudaMallocPitch gives every image of the same row
 * width the same pitch). accept_bits stays a plain array. Results equal the
 * planar call's bit for bit. */
typedef struct {
    int64_t rgb_step;    /* bytes per row of every RGB buffer and 3-channel G-buffer (>= 3 W element size) */
    int64_t scalar_step; /* bytes per row of jb and 1-channel G-buffers (>= W element size) */
    int64_t n_step;      /* bytes per row of the int32 count image n (>= 4 W) */
} stater_pitched_layout;
/* stat_denoiser::denoiseVars<float3> over the layout above (estimator.cpp:374-414). */
stater_status stater_denoise_vars_pitched(const stater_denoise_vars_args *a, const stater_pitched_layout *layout,
                                          stater_stream stream);
/* stat_denoiser::denoiseFilm over the layout above (estimator.cpp:421-457). */
stater_status stater_denoise_film_pitched(const stater_denoise_film_args *a, const stater_pitched_layout *layout,
                                          stater_stream stream);

/* Tile-height autotuner of the FP32 window filters (no counterpart in the
 * reference, whose filters have fixed launch shapes). The first FP32
 * denoiseVars / denoiseFilm call of each shape class (filter, transform count,
 * radius, feature use, image-size class: up to 2^18, 2^20 or more pixels) on a
 * device times the row-ring kernels at tile heights 4, 8 and 16 rows, where the
 * ring fits in shared memory, on its own stream, synchronising it once, and
 * keeps the fastest for later calls. Results are bitwise the same at every
 * height. Calls on a stream being captured into a CUDA graph use the default
 * height and tune nothing. enable = 0 switches tuning off and forgets the
 * choices (all calls then use the default); 1 switches it back on. */
stater_status stater_set_autotune(int32_t enable);
/* The tile height chosen for a shape class on the current device (filter 0 =
 * denoiseVars, 1 = denoiseFilm), or 0 if none has been tuned yet. */
int32_t stater_tuned_tile_height(int32_t filter, int32_t n_transforms, int32_t width, int32_t height,
                                 int32_t filter_radius);

/* A test order for stater_denoise_film_args.test_order: the most compressing
 * transforms first (asinh, cbrt and Box-Cox with lambda < 1/2, sqrt, log1p,
 * other Box-Cox), the untransformed set (transform 0) last; they reject most
 * of the neighbours that any transform rejects, so the filter stops earlier. */
stater_status stater_test_order(const stater_transform *transforms, int32_t n_transforms, int32_t *order);

/* Squared two-sided Student-t critical values over u = 1/df: table[m] =
 * t_{1-alpha/2}(N/m)^2 (table[0] = z^2), m = 0..N, N = lut_intervals. The Welch
 * test of stater_denoise_film interpolates this table linearly in u. Host memory. */
int32_t stater_tcrit_lut_intervals(void);
stater_status stater_tcrit2_table(double alpha, double *table);
double stater_t_quantile(double p, double df);

/* stat_denoiser::calcTargetSPP<float3> (estimator.cpp:502-511): extra samples
 * for the next adaptive round. e_p = sum_c varD_c / n_p (divided by mean_c^2 +
 * eps when mean != NULL); target_p = clamp(rint(spp * W*H * e_p / sum e), tmin,
 * tmax), the sum by a fixed-order tree so that the result is deterministic.
 * varD and mean are RGB buffers of the call's precision. */
stater_status stater_calc_target_spp(int32_t width, int32_t height, int32_t spp,
                                     stater_precision precision, const int32_t *n,
                                     const void *varD, const void *mean, double eps,
                                     int32_t tmin, int32_t tmax, int32_t *targetspp,
                                     stater_stream stream);

/* calcTargetSPP with the reference's AS_MODE choice: as stater_calc_target_spp,
 * but the per-pixel variance is varD (as_source STATER_AS_DENOISED, "ASM") or
 * the sample variance m2 / (n - 1) (STATER_AS_SAMPLE, "ASN"); the buffer the
 * choice does not read may be NULL. */
typedef struct {
    int32_t width, height, spp;
    stater_precision precision;
    const int32_t *n;
    const void *m2;             /* RGB buffer, read by STATER_AS_SAMPLE */
    const void *varD;           /* RGB buffer, read by STATER_AS_DENOISED */
    const void *mean;           /* nullable: relative error (divide by mean^2 + eps) */
    double eps;
    int32_t tmin, tmax;
    int32_t as_source;          /* stater_as_source */
    int32_t *targetspp;
} stater_target_spp_args;
stater_status stater_calc_target_spp_ex(const stater_target_spp_args *a, stater_stream stream);
/* stat_denoiser::calcTargetSPP<float3> over the reference's pitched GpuMat layout
 * (stater_pitched_layout; estimator.cpp:502-511): n and targetspp are int32
 * images of n_step, m2, varD and mean RGB images of rgb_step. */
stater_status stater_calc_target_spp_pitched(const stater_target_spp_args *a, const stater_pitched_layout *layout,
                                             stater_stream stream);

/* No counterpart in the reference. The same computation as
 * stater_calc_target_spp for callers that cannot allocate device memory (pool
 * allocators that own the device, hosts that forbid the device-wide
 * synchronisation of cudaMalloc/cudaFree): its scratch is a fixed array inside
 * the library, 2,097,152 pixels at most (W*H above that returns
 * STATER_ERR_INVALID), about 16.8 MB held on every GPU that loads the library.
 * The first call on a device resolves the array's address and should come
 * before any stream capture; calls that overlap on the GPU share the array and
 * race. */
stater_status stater_calc_target_spp_noalloc(int32_t width, int32_t height, int32_t spp,
                                             stater_precision precision, const int32_t *n,
                                             const void *varD, const void *mean, double eps,
                                             int32_t tmin, int32_t tmax, int32_t *targetspp,
                                             stater_stream stream);

/* ---- film buffer --------------------------------------------------------- */

/* FilmTile::AddSample with the box filter of radius 0.5 (core/film.h:152-190;
 * the statistics integrator forces that filter, core/api.cpp:1713-1739) for
 * whole sample planes as stater_accumulate reads them (R, G, B, u, v first).
 * Radiance above max_sample_luminance (luminance per core/spectrum.h:483-486) is
 * scaled down to it, as FilmTile does (+inf: off, the reference's default). Each
 * pixel's own samples are summed in order into contrib_sum (RGB planes) and
 * weight_sum, which persist across calls like the reference's film tiles do
 * across iterations (statpath.cpp:144, 388). A sample on a pixel edge (u or v
 * exactly 0 or 1) also lies in the neighbour's filter support and is added to
 * that neighbour's spill planes (R, G, B, weight) by atomic adds, so several
 * edge samples landing on one pixel are summed in no fixed order. Zero the three
 * buffers to start a film (Film::Clear with fresh tiles). Device pointers. */
typedef struct {
    int32_t width, height;
    int32_t n_samples;          /* S */
    int32_t n_features;         /* G: sample planes [S][5+G][W*H] */
    const float *samples;
    const int32_t *count;       /* nullable: first count[p] samples of pixel p */
    float max_sample_luminance; /* FilmTile maxSampleLuminance; INFINITY = off */
    float *contrib_sum;         /* [3][W*H] */
    float *weight_sum;          /* [W*H] */
    float *spill;               /* [4][W*H] */
} stater_film_args;
stater_status stater_film_add_samples(const stater_film_args *a, stater_stream stream);

/* Film::UpdateImage (core/film.cpp:187-222) without splats: xyz = RGBToXYZ(own
 * sum) + RGBToXYZ(spill) (the MergeFilmTile sums, film.cpp:140-149), film RGB =
 * max(0, XYZToRGB(xyz) / weight) where the weight is non-zero, times scale. This
 * is the `film` input of stater_denoise_film. spill may be NULL. float RGB planes. */
stater_status stater_film_update_image(int32_t width, int32_t height, const float *contrib_sum,
                                       const float *weight_sum, const float *spill, float scale,
                                       float *rgb, stater_stream stream);

/* Estimator::CalcMeanVars / calcMatMeanVar (estimator.cpp:462-496):
 * meanVar = m2 / ((n - 1) * n) in float arithmetic. RGB buffers. */
stater_status stater_calc_mean_var(int32_t width, int32_t height, const int32_t *n,
                                   const float *m2, float *mean_var, stater_stream stream);

/* ---- stage 3: linear explained variance ------------------------------- */

/* Per-pixel regression of the three radiance channels on the G feature channels
 * plus an intercept. Accumulation keeps, per pixel, n, a pivot sample and the
 * pivot-shifted sums and cross-products (stater_lev_state_size values, planes
 * of W*H). STATER_F64 accumulates in FP64; STATER_F32 in FP32 with blocked
 * Kahan-compensated sums (hi and lo planes, 2 * state size). The solve is FP64:
 * ridge with lambda on the slopes, Cholesky. Outputs (precision-typed):
 * beta [3][G+1][W*H] (intercept first), m2C [3][W*H] = residual sum of squares,
 * r2 [3][W*H]. */
int32_t stater_lev_state_size(int32_t n_features, stater_precision precision);
stater_status stater_lev_accumulate(int32_t width, int32_t height, int32_t n_features,
                                    int32_t n_samples, const float *samples,
                                    const int32_t *count, stater_precision precision,
                                    void *state, stater_stream stream);
stater_status stater_lev_solve(int32_t width, int32_t height, int32_t n_features,
                               stater_precision precision, const void *state, double lambda,
                               void *beta, void *m2C, void *r2, stater_stream stream);

/* ---- batches: many images through one launch per stage ----------------- */

/* No counterpart in the reference, which makes one call per image per stage
 * (statpath.cpp:424-441). A batch takes, per image, the arguments of the calls
 * a caller would make for it (stater_accumulate with the film sums,
 * stater_film_update_image into film_rgb, stater_denoise_vars,
 * stater_denoise_film with film = film_rgb) and runs them together: the
 * accumulations and film images per image, then every denoise stage as one
 * launch over the tiles of all images that share a kernel form (transform-count
 * class, moment/LEV variant, multi-transform mode, radius). Each image's
 * outputs are bitwise those of its own calls. FP32 form only (STATER_F32,
 * STATER_ACC_FAST), up to 5 transforms and 7 range-kernel feature channels per
 * image, no pixel index, no accept bits.
 * The first stater_batch_run tunes each launch's tile height on the data (one
 * synchronisation of the stream) and records the sequence into a CUDA graph,
 * so later runs are one graph launch; it must not itself be captured. The
 * batch keeps the pointers it was given: every buffer must stay allocated, at
 * the same address, until stater_batch_destroy. With reset = 1 each run first
 * zeroes each image's n, statistics, feature means and film sums (a fresh
 * image per run); with 0 the runs keep adding samples like repeated calls. */
typedef struct {
    stater_accumulate_args acc;
    float *film_rgb;            /* [3][W*H]: Film::UpdateImage of the job's film sums */
    float film_scale;
    stater_denoise_vars_args vars;
    stater_denoise_film_args film;
} stater_batch_job;
typedef struct stater_batch stater_batch;
stater_status stater_batch_create(const stater_batch_job *jobs, int32_t n_jobs, int32_t reset, stater_batch **out);
stater_status stater_batch_run(stater_batch *batch, stater_stream stream);
/* Waits for the device, then frees the batch's tables and graph. */
stater_status stater_batch_destroy(stater_batch *batch);

/* ---- serving: continuous batching of denoise jobs ---------------------- */

/* A server owns `max_slots` CUDA streams on the current device and one
 * scheduler thread. Jobs are admitted in arrival order as soon as a slot is free
 * and their device-memory footprint fits under `hbm_budget_bytes` together with
 * the jobs already running, so jobs that arrive while others are on the GPU start
 * without waiting for them and their work overlaps on the device. Each job
 * generates its samples on the device (the seeded synthetic source), accumulates
 * them together with the film sums, makes the film image (Film::UpdateImage),
 * runs denoiseVars and denoiseFilm, and copies the denoised film to `out_host`. With rounds > 1 a job is rendered adaptively: after each round its
 * moment buffers stay on the device, calcTargetSPP allots the next round's
 * samples (round_spp on average per pixel, clamped to [16, 1024]) and the round's
 * samples continue every pixel's own sample sequence. Results are independent of
 * what else runs: a job gives the same output alone and in any mix. */
typedef struct stater_server stater_server;

typedef struct {
    int32_t max_slots;          /* concurrent jobs (streams), 1..64 */
    double hbm_budget_bytes;    /* admission limit; <= 0: 80% of the free memory at creation */
    int32_t precision;          /* STATER_F32 (serving form) or STATER_F64 (plain form) */
    int32_t chunk_spp;          /* samples generated and accumulated per step; 0: automatic, 128 for adaptive
                                 * jobs and 32 for one-round jobs; capped at what a round can take and at
                                 * 16 GiB of sample planes per job */
    /* 1: small single-round FP32 jobs (up to 512x512 pixels, 5 transforms) that
     * wait together are admitted as one group onto one slot, and their denoise
     * stages run as one launch per stage for the group (stater_batch); each
     * job's output is bitwise the same as when it runs alone. */
    int32_t fuse_small_jobs;
} stater_server_config;

typedef struct {
    int32_t width, height;
    int32_t spp;                /* samples per pixel of the first round */
    int32_t rounds;             /* 1 = one pass */
    int32_t round_spp;          /* average extra samples per pixel in each later round (0 = spp) */
    int32_t n_transforms;
    stater_transform transforms[STATER_MAX_TRANSFORMS];
    int32_t n_features;         /* feature channels generated; the range kernels use albedo (0-2, sigma 0.02),
                                   normal (3-5, 0.1) and depth (6, 0.1) when present */
    int32_t max_moment;         /* 3..5 */
    int32_t filter_radius;
    float filter_sd, alpha, var_z;
    uint64_t seed;
    float *out_host;            /* [3][H][W] float32, written when the job completes (may be NULL); page-locked
                                 * memory is written by the device copy, pageable memory from a page-locked
                                 * staging buffer of the engine once the job's GPU work is done; device memory
                                 * is refused (STATER_ERR_INVALID) */
} stater_job_desc;

typedef enum { STATER_JOB_QUEUED = 0, STATER_JOB_RUNNING = 1, STATER_JOB_DONE = 2, STATER_JOB_FAILED = 3 } stater_job_state;

typedef struct {
    int64_t submitted, completed, failed, running, queued;
    double latency_p50_ms, latency_p99_ms, latency_mean_ms;
    double mpix_per_s;          /* pixels of completed jobs / (last completion - first submission) */
    double peak_footprint_bytes;
} stater_server_stats;

stater_status stater_server_create(const stater_server_config *cfg, stater_server **out);
stater_status stater_server_submit(stater_server *srv, const stater_job_desc *job, int64_t *job_id);
stater_status stater_server_poll(stater_server *srv, int64_t job_id, int32_t *state, double *latency_ms);
/* Blocks until the job is done or failed, or timeout_s elapses (STATER_ERR_TIMEOUT). */
stater_status stater_server_wait(stater_server *srv, int64_t job_id, double timeout_s);
stater_status stater_server_drain(stater_server *srv, double timeout_s);
stater_status stater_server_stats_get(stater_server *srv, stater_server_stats *out);
/* Device bytes a job needs while it runs (the admission footprint). */
double stater_job_footprint(const stater_job_desc *job, int32_t precision, int32_t chunk_spp);
stater_status stater_server_destroy(stater_server *srv);

#ifdef __cplusplus
}
#endif
#endif
