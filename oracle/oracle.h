/*
 * CPU oracle for the StatER statistics hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the GPU library
 * (stater_gb300/csrc): only tests/, __graft_entry__.smoke() and the CPU-baseline
 * legs of bench.py may load it. Nothing in the product links or calls it.
 *
 * Stage 1 (moment accumulation, tile merge, meanVar) restates the reference's
 * own code and is pinned bit-for-bit against that code compiled in place
 * (oracle/build_ref.sh -> tests/golden/). Stages 2-3 (variance denoise, Welch
 * mean filter, LEV, target-SPP) have no source in the reference tree (the CUDA
 * denoiser lives in an absent submodule); they restate formulas written from the
 * reference's buffer semantics (README.md:290-346) and standard statistics
 * (Bonett's ln s^2 interval, Welch's t with Welch-Satterthwaite df, Jarque-Bera,
 * ridge least squares), each stated beside its function in oracle.c, and are
 * "parity unpinned" against the reference.
 *
 * Every function exists in an f64 form (the FP64 restatement, equivalent to a
 * PBRT_FLOAT_AS_DOUBLE build of the reference) and, where the reference computes
 * in FP32, an f32 form that follows the reference's float arithmetic exactly.
 *
 * Layouts (all planar, pixel p = y*W + x, HW = W*H):
 *   samples  float [S][5+G][HW]   channels R,G,B,u,v,f_0..f_{G-1}
 *   n        int32 [HW]           per-pixel sample count
 *   stats    T [K][7][3][HW]      moments mean,m2,m3,m4,c2X,c2Y,m1 per transform
 *   gmean    T [G][HW]            running mean of every feature channel
 */
#ifndef STATER_ORACLE_H
#define STATER_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_TK_IDENTITY = 0, ORC_TK_LOG1P = 1, ORC_TK_SQRT = 2, ORC_TK_CBRT = 3,
       ORC_TK_ASINH = 4, ORC_TK_BOXCOX = 5 };
enum { ORC_Q_MEAN = 0, ORC_Q_M2 = 1, ORC_Q_M3 = 2, ORC_Q_M4 = 3, ORC_Q_C2X = 4,
       ORC_Q_C2Y = 5, ORC_Q_M1 = 6, ORC_NQ = 7 };
enum { ORC_MT_ALL = 2, ORC_MT_JB = 3 };

typedef struct {
    int first_channel;  /* first feature channel of this G-buffer in gmean */
    int channels;       /* 1 or 3 */
    double dr_factor;   /* -0.5 / sigma_r^2 (estimator.cpp:10-18) */
} orc_gbuf;

double orc_transform_f64(int kind, double lambda, double x);
float orc_transform_f32(int kind, float lambda, float x);

/* Stage 1: StatTile::AddTransformSample* / AddSample* (estimator.h:226-324). */
void orc_accumulate_f64(int W, int H, int G, int S, const float *samples, const int32_t *count,
                        int K, const int32_t *tkind, const double *tlambda, int max_moment,
                        int32_t *n, double *stats, double *gmean, int nthreads);
void orc_accumulate_f32(int W, int H, int G, int S, const float *samples, const int32_t *count,
                        int K, const int32_t *tkind, const float *tlambda, int max_moment,
                        int32_t *n, float *stats, float *gmean, int nthreads);

/* Estimator::MergeTransformTile (estimator.cpp:301-324): AoS StatTilePixel<Vec3>
 * records (float build, 320 bytes each) -> planar n, stats[2][7][3][HW]. */
void orc_merge_transform_tiles_f32(int W, int H, int ntiles, const int32_t *bounds,
                                   const uint8_t *records, int32_t *n, float *stats);

/* Pairwise (Chan/Pebay) combine of two moment sets: A <- A (+) B. */
void orc_merge_moments_f64(int HW, int K, int max_moment, int32_t *nA, double *statsA,
                           const int32_t *nB, const double *statsB);

/* Student-t quantile t_p(nu) (nu <= 0 means the normal quantile). */
double orc_t_quantile(double p, double nu);
/* Squared two-sided critical value table over u = 1/df, nodes u_m = m/N, m=0..N. */
void orc_tcrit2_table(double alpha, int N, double *table);

/* Stage 2a+2b: denoiseVars. Outputs jb[K][HW], lnS2/se2/m2C/varD/varCD [K][3][HW].
 * m2c_ext (nullable): [3][HW] externally corrected m2 for transform 0 (LEV). */
void orc_denoise_vars_f64(int W, int H, int K, int max_moment, const int32_t *n,
                          const double *stats, int R, double ds_factor, double var_z,
                          int nG, const orc_gbuf *gbufs, const double *gmean,
                          const double *m2c_ext, double *jb, double *lnS2, double *se2,
                          double *m2C, double *varD, double *varCD, int nthreads);

/* Stage 2c: denoiseFilm. film [3][HW]; outputs discr [K][3][HW], filmD [3][HW].
 * discr_source 0: the discriminator uses varCD (use_levc) or varD; 1 (the
 * reference's CASCADE_MODE=0): m2C (use_levc, [K][3][HW]) or the m2 moments,
 * divided by n - 1.
 * accept_bits (nullable): uint32 [HW][K][words], words = ceil((2R+1)^2/32), bit
 * (dy+R)*(2R+1)+(dx+R) set when the pair test of transform k accepts neighbour
 * (dx,dy) (in-image, valid neighbours only). */
void orc_denoise_film_f64(int W, int H, int K, const int32_t *n, const double *stats,
                          const double *varD, const double *varCD, const double *jb,
                          int use_levc, int discr_source, const double *m2C, int mt_mode, int R,
                          double ds_factor,
                          int lut_n, const double *tcrit2, int nG, const orc_gbuf *gbufs,
                          const double *gmean, const double *film, double *discr,
                          double *filmD, uint32_t *accept_bits, int nthreads);

/* calcTargetSPP: next-round extra samples per pixel. as_source 0 ("ASM"): from
 * varD; 1 ("ASN", the reference's AS_MODE=0): from the sample variance m2/(n-1). */
void orc_calc_target_spp(int W, int H, int spp, const int32_t *n, const double *varD,
                         const double *mean, double eps, int tmin, int tmax, int32_t *target);
void orc_calc_target_spp_src(int W, int H, int spp, const int32_t *n, const double *varD,
                             const double *m2, int as_source, const double *mean, double eps, int tmin,
                             int tmax, int32_t *target);
/* Deterministic reduction used by calcTargetSPP: the values are summed in
 * blocks of 1024 (each block: 256 partial sums of 4 strided values, then a
 * pairwise halving tree), and the block sums again the same way until one value
 * is left; the GPU's reduction uses the same tree. */
double orc_tree_sum(const double *v, int64_t len);

/* Estimator::calcMatMeanVar (estimator.cpp:462-474), float arithmetic. */
void orc_calc_mean_var_f32(int HW, const int32_t *n, const float *m2, float *var);

/* Linear explained-variance regression on the feature channels (G + intercept).
 * state per pixel: [n][pivot 10][S 10][Sff G(G+1)/2][Sfy 3G][Syy 3] as doubles,
 * layout [LEV_NSTATE][HW]. */
int orc_lev_nstate(int G);
void orc_lev_accumulate_f64(int W, int H, int G, int S, const float *samples, const int32_t *count,
                            double *state, int nthreads);
void orc_lev_solve_f64(int W, int H, int G, const double *state, double lambda,
                       double *beta, double *m2C, double *r2, int nthreads);

/* Film path (core/film.h:152-190, core/film.cpp:140-149, 187-222). Buffers
 * float: contrib_sum [3][HW], weight_sum [HW], spill [4][HW] (R,G,B,weight of
 * samples lying on an edge shared with the pixel), rgb [3][HW]. */
void orc_film_constants(float *rgb_to_xyz, float *xyz_to_rgb, float *y_weight);
void orc_film_add_samples(int W, int H, int G, int S, const float *samples, const int32_t *count,
                          float max_lum, float *contrib_sum, float *weight_sum, float *spill);
void orc_film_update_image(int W, int H, const float *contrib_sum, const float *weight_sum,
                           const float *spill, float scale, float *rgb);

#ifdef __cplusplus
}
#endif
#endif
