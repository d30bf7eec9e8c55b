// Host-side mirror of the reference's Estimator (src/statistics/estimator.h:330-500,
// estimator.cpp) and of the renderer's Film as the statistics integrator uses it,
// over the C ABI of libstater (include/stater.h). A renderer that drives the
// reference's
//     Upload -> DenoiseVars -> DenoiseMeans -> CalcTargetSPPs -> Download -> Synchronize
// sequence (statpath.cpp:424-441) calls the same methods here; the per-sample
// statistics, which the reference accumulates in CPU tiles, are added on the GPU
// (AddSamples) or merged from the reference's own tile records
// (MergeTransformTiles).
//
// Buffers carry the reference's names, "t<type>-b<j>-film-<name>" for the
// untransformed set and "t<type>-b<j>-<name>" for the transformed set of Box-Cox
// index j (ALLOC_BUF, estimator.cpp:21-24; names of BUF_LIST / FILM_BUF_LIST,
// estimator.h:459-479), plus "filmD" and "targetspp", so that
// OutputBufferSelection writes and the replay reads the reference's files.
//
// Mapping onto the device layout (multi-transform build, FULL_MULTI_TRANSFORM):
// transform 0 of the configuration is the identity and holds the untransformed
// set, which the reference duplicates for every j; transform j + 1 holds the
// transformed set of index j. The G feature-channel means are the G-buffers'
// "film-mean" buffers of their own statistics types (albedo t6, normal t5,
// depth t4: StatTypeIndex, statpath.h:28-37).
//
// Errors: every failing library or CUDA call throws std::runtime_error with the
// library's message (the reference's methods return void and check nothing).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "buffer.hpp"
#include "stater.h"

namespace stater {
namespace host {

inline void check(stater_status s, const char *what) {
    if (s != STATER_OK) throw std::runtime_error(std::string(what) + ": " + stater_last_error());
}
inline void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// Pinned host memory, as the reference makes every cv::Mat page-locked
// (estimator.h:381).
inline std::shared_ptr<void> pinned_host(size_t bytes) {
    void *p = nullptr;
    check_cuda(cudaMallocHost(&p, bytes ? bytes : 1), "cudaMallocHost");
    std::memset(p, 0, bytes);
    return std::shared_ptr<void>(p, [](void *q) { cudaFreeHost(q); });
}

// Zero-initialised device allocation.
inline std::shared_ptr<void> device_alloc(size_t bytes) {
    void *p = nullptr;
    check_cuda(cudaMalloc(&p, bytes ? bytes : 1), "cudaMalloc");
    check_cuda(cudaMemset(p, 0, bytes), "cudaMemset");
    return std::shared_ptr<void>(p, [](void *q) { cudaFree(q); });
}

inline void upload(Buffer &b, cudaStream_t s) {
    if (!b.host || !b.device) return;
    check_cuda(cudaMemcpyAsync(b.device, b.host, b.bytes(), cudaMemcpyHostToDevice, s), "upload");
    b.host_dirty = false;
}
inline void download(Buffer &b, cudaStream_t s) {
    alloc_host(b, pinned_host);
    check_cuda(cudaMemcpyAsync(b.host, b.device, b.bytes(), cudaMemcpyDeviceToHost, s), "download");
}

// BUF_LIST (estimator.h:459-473) and the extra FILM_BUF_LIST entries (:475-479).
// Position q < 7 of BUF_LIST is moment q of the device statistics slab.
static const char *const kBufList[] = {"mean", "m2",   "m3",  "m4",   "c2X",  "c2Y",  "m1",
                                       "jb",   "lnS2", "se2", "m2C",  "varD", "varCD", "discr"};
constexpr int kNBufList = 14;

enum StatTypeIndex { Radiance = 0, StatDepth = 4, StatNormal = 5, StatAlbedo = 6 };

// The film of the statistics integrator: pbrt-v3 Film and its tiles with the box
// filter of radius 0.5 (core/film.h, core/film.cpp), sums on the device. Its
// `buffer` ("film", float RGB) is what Film::UpdateImage writes and what
// DenoiseMeans filters.
class Film {
  public:
    Film(int width, int height, int n_features, float max_sample_luminance = INFINITY, float scale = 1.f)
        : width(width), height(height), n_features(n_features), max_sample_luminance(max_sample_luminance),
          scale(scale) {
        const size_t HW = (size_t)width * height;
        sums_ = device_alloc(8 * HW * sizeof(float));  // contrib_sum[3], weight_sum, spill[4]
        rgb_ = device_alloc(3 * HW * sizeof(float));
        buffer.name = "film";
        buffer.width = width;
        buffer.height = height;
        buffer.channels = 3;
        buffer.elem = Elem::F32;
        buffer.device = rgb_.get();
    }
    // Film::Clear together with fresh tiles: the sums start again from zero.
    void Clear(cudaStream_t s) {
        check_cuda(cudaMemsetAsync(sums_.get(), 0, 8 * (size_t)width * height * sizeof(float), s), "Film::Clear");
    }
    // FilmTile::AddSample for every sample of device sample planes [S][5+G][H*W].
    void AddSamples(const float *samples, int n_samples, const int32_t *count, cudaStream_t s) {
        stater_film_args a;
        std::memset(&a, 0, sizeof(a));
        a.width = width;
        a.height = height;
        a.n_samples = n_samples;
        a.n_features = n_features;
        a.samples = samples;
        a.count = count;
        a.max_sample_luminance = max_sample_luminance;
        a.contrib_sum = contrib_sum();
        a.weight_sum = weight_sum();
        a.spill = spill();
        check(stater_film_add_samples(&a, (stater_stream)s), "Film::AddSamples");
    }
    void UpdateImage(cudaStream_t s) {
        check(stater_film_update_image(width, height, contrib_sum(), weight_sum(), spill(), scale,
                                       (float *)rgb_.get(), (stater_stream)s),
              "Film::UpdateImage");
    }

    float *contrib_sum() const { return sum_ptr(); }
    float *weight_sum() const { return sum_ptr() + 3 * (size_t)width * height; }
    float *spill() const { return sum_ptr() + 4 * (size_t)width * height; }

    const int width, height, n_features;
    const float max_sample_luminance, scale;
    Buffer buffer;

  private:
    float *sum_ptr() const { return (float *)sums_.get(); }
    std::shared_ptr<void> sums_, rgb_;
};

struct EstimatorConfig {
    // transforms[0] must be the identity (the untransformed set); the others are
    // the reference's "lambdas" in order (Box-Cox), or any stater_transform_kind.
    std::vector<stater_transform> transforms;
    int n_features = 7;
    int max_moment = 5;              // "maxmoment" (statpath.cpp:1056)
    int filter_radius = 20;          // "filterradius" (statpath.cpp:1072)
    float filter_sd = 10.f;          // "filtersd" (statpath.cpp:1071)
    float mean_z_value = 1.95996f;   // "meanzvalue": accepted and, as in the reference, without effect
    float var_z_value = 2.80703f;    // "varzvalue" (statpath.cpp:1070)
    double alpha = 0.01;             // two-sided level of the Welch test
    // The reference's build variants (scripts/alternate-builds/*.sh), as runtime
    // switches: MCL = cascade + use_levc (the reference's default build), MC =
    // cascade only, M = neither; ASM / ASN = as_source; MT-JB = mt_mode 3.
    int mt_mode = STATER_MT_ALL;     // FILM_MULTI_TRANSFORM_MODE
    bool use_levc = true;            // USE_LEVC (needs max_moment 5: c2X, c2Y)
    bool cascade = true;             // CASCADE_MODE
    int as_source = STATER_AS_DENOISED;  // AS_MODE: ASM (denoised varD) or ASN (sample variance)
    bool enable_as = false;          // "enableas": CalcTargetSPPs output downloaded
    bool denoise_film = true;        // "denoisefilm": film uploaded / filmD downloaded
    stater_precision precision = STATER_F32;
    int acc_mode = STATER_ACC_FAST;
    double target_eps = 1e-4;
    int target_min = 16, target_max = 1024;
};

class Estimator {
  public:
    Estimator(Buffer &filmBuffer, const EstimatorConfig &config, BufferRegistry &reg)
        : filmBuffer(filmBuffer), cfg(config), reg(reg), width(filmBuffer.width), height(filmBuffer.height) {
        K = (int)cfg.transforms.size();
        if (K < 1 || K > STATER_MAX_TRANSFORMS || cfg.transforms[0].kind != STATER_TK_IDENTITY)
            throw std::invalid_argument("Estimator: 1..8 transforms, the first the identity");
        if (cfg.n_features < 0 || cfg.n_features > STATER_MAX_FEATURES)
            throw std::invalid_argument("Estimator: bad number of feature channels");
        check(stater_setup(), "stat_denoiser::setup");
        check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        AllocateBuffers();
    }
    ~Estimator() {
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }
    Estimator(const Estimator &) = delete;
    Estimator &operator=(const Estimator &) = delete;

    // G-buffers of the range kernels (RegisterVarGBuffer / RegisterMeanGBuffer,
    // estimator.cpp:10-18): `channels` feature means starting at `first_feature`.
    void RegisterVarGBuffer(int first_feature, int channels, float filterSD) {
        add_gbuffer(varG, first_feature, channels, filterSD);
    }
    void RegisterMeanGBuffer(int first_feature, int channels, float filterSD) {
        add_gbuffer(meanG, first_feature, channels, filterSD);
    }
    // Names the feature means [first, first + channels) as the "t<type>-b0-film-mean"
    // buffer of a G-buffer statistics type, for output and replay.
    void RegisterFeatureBuffer(int type, int first_feature, int channels) {
        if (first_feature < 0 || channels < 1 || first_feature + channels > cfg.n_features)
            throw std::invalid_argument("RegisterFeatureBuffer: outside the feature channels");
        Buffer &b = new_buffer("t" + std::to_string(type) + "-b0-film-mean", channels, elem());
        b.device = (char *)gmean_.get() + (size_t)first_feature * HW() * esize();
    }

    // Stage 1 on the GPU in place of the CPU tiles: every sample of the device
    // sample planes [S][5+G][H*W] (the first count[p] for pixel p, count may be
    // NULL). With `film`, the same pass adds the samples to the film's sums
    // (Film::AddSamples in one read of the samples).
    void AddSamples(const float *samples, int n_samples, const int32_t *count, Film *film = nullptr) {
        stater_accumulate_args a;
        std::memset(&a, 0, sizeof(a));
        a.width = width;
        a.height = height;
        a.n_samples = n_samples;
        a.n_features = cfg.n_features;
        a.samples = samples;
        a.count = count;
        a.n_transforms = K;
        for (int k = 0; k < K; k++) a.transforms[k] = cfg.transforms[k];
        a.max_moment = cfg.max_moment;
        a.precision = cfg.precision;
        a.mode = cfg.acc_mode;
        a.n = n_ptr();
        a.stats = stats_.get();
        a.gmean = cfg.n_features ? gmean_.get() : nullptr;
        if (film) {
            if (film->width != width || film->height != height || film->n_features != cfg.n_features)
                throw std::invalid_argument("Estimator::AddSamples: film geometry differs");
            a.film_contrib_sum = film->contrib_sum();
            a.film_weight_sum = film->weight_sum();
            a.film_spill = film->spill();
            a.film_max_sample_luminance = film->max_sample_luminance;
        }
        check(stater_accumulate(&a, (stater_stream)stream), "Estimator::AddSamples");
    }

    // Estimator::MergeTransformTiles (estimator.cpp:301-343) from the reference's
    // own tile records: records[j] holds the StatTilePixel<Vec3> records (float
    // build, 320 bytes each) of Box-Cox index j for every tile in order, bounds the
    // int32 [n_tiles][4] tile rectangles; host memory. FP32 statistics only. The
    // sets are merged from the last index to the first: each merge writes the
    // untransformed copy into the plane the next one overwrites with its
    // transformed set, and the last writes transform 0.
    void MergeTransformTiles(const std::vector<const void *> &records, const int32_t *bounds, int n_tiles) {
        if (cfg.precision != STATER_F32) throw std::invalid_argument("MergeTransformTiles: FP32 statistics only");
        if ((int)records.size() != K - 1 || K < 2)
            throw std::invalid_argument("MergeTransformTiles: one record set per transformed set");
        const size_t rec_bytes = 320 * HW();
        auto drec = device_alloc(rec_bytes);
        auto dbounds = device_alloc((size_t)n_tiles * 4 * sizeof(int32_t));
        check_cuda(cudaMemcpyAsync(dbounds.get(), bounds, (size_t)n_tiles * 4 * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, stream),
                   "MergeTransformTiles bounds");
        for (int j = K - 2; j >= 0; j--) {
            check_cuda(cudaMemcpyAsync(drec.get(), records[j], rec_bytes, cudaMemcpyHostToDevice, stream),
                       "MergeTransformTiles records");
            float *dst = (float *)stats_.get() + (size_t)j * STATER_NQ * 3 * HW();
            check(stater_merge_tiles(width, height, n_tiles, (const int32_t *)dbounds.get(), drec.get(), 2, n_ptr(),
                                     dst, (stater_stream)stream),
                  "Estimator::MergeTransformTiles");
        }
        check_cuda(cudaStreamSynchronize(stream), "MergeTransformTiles");
    }

    // Estimator::MergeTiles (estimator.cpp:268-298) for the untransformed set:
    // records holds the plain tiles' StatTilePixel<Vec3> records (float build,
    // 320 bytes each) for every tile in order, bounds the int32 [n_tiles][4]
    // tile rectangles; host memory. Sets n and the set's mean, M2, M3 and M4, as
    // MergeTile does. FP32 statistics only.
    void MergeTiles(const void *records, const int32_t *bounds, int n_tiles) {
        if (cfg.precision != STATER_F32) throw std::invalid_argument("MergeTiles: FP32 statistics only");
        const size_t rec_bytes = 320 * HW();
        auto drec = device_alloc(rec_bytes);
        auto dbounds = device_alloc((size_t)n_tiles * 4 * sizeof(int32_t));
        check_cuda(cudaMemcpyAsync(dbounds.get(), bounds, (size_t)n_tiles * 4 * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, stream),
                   "MergeTiles bounds");
        check_cuda(cudaMemcpyAsync(drec.get(), records, rec_bytes, cudaMemcpyHostToDevice, stream),
                   "MergeTiles records");
        check(stater_merge_tiles(width, height, n_tiles, (const int32_t *)dbounds.get(), drec.get(), 1, n_ptr(),
                                 (float *)stats_.get(), (stater_stream)stream),
              "Estimator::MergeTiles");
        check_cuda(cudaStreamSynchronize(stream), "MergeTiles");
    }

    // Estimator::Upload (estimator.cpp:346-353): host copies changed since the
    // last upload (buffers read from files) and, with denoisefilm, the film.
    void Upload() {
        for (Buffer *b : reg.buffers)
            if (b->host_dirty) upload(*b, stream);
        if (filmBuffer.host_dirty) upload(filmBuffer, stream);
    }
    // Estimator::Download (estimator.cpp:355-362): filmD with denoisefilm,
    // targetspp with adaptive sampling.
    void Download() {
        if (cfg.denoise_film) download(filmFilteredBuffer, stream);
        if (cfg.enable_as) download(targetSPPBuffer, stream);
    }
    // Host copies of every buffer of an output selection, for Write.
    void Download(const OutputBufferSelection &sel) {
        for (Buffer *b : sel.buffers)
            if (b->device) download(*b, stream);
    }

    // stat_denoiser::denoiseVars (estimator.cpp:365-416).
    void DenoiseVars() {
        stater_denoise_vars_args a;
        std::memset(&a, 0, sizeof(a));
        a.n_buffers = K;
        a.width = width;
        a.height = height;
        a.filter_radius = cfg.filter_radius;
        a.ds_factor = -.5f / (cfg.filter_sd * cfg.filter_sd);
        a.var_z = cfg.var_z_value;
        a.max_moment = cfg.max_moment;
        a.precision = cfg.precision;
        a.n = n_ptr();
        for (int k = 0; k < K; k++) {
            a.m2[k] = stat(k, STATER_Q_M2);
            a.m3[k] = stat(k, STATER_Q_M3);
            a.m4[k] = stat(k, STATER_Q_M4);
            a.c2X[k] = stat(k, STATER_Q_C2X);
            a.c2Y[k] = stat(k, STATER_Q_C2Y);
            a.jb[k] = out(7, k);
            a.lnS2[k] = out(8, k);
            a.se2[k] = out(9, k);
            a.m2C[k] = out(10, k);
            a.varD[k] = out(11, k);
            a.varCD[k] = out(12, k);
        }
        a.gbuffers = gbuffers(varG);
        check(stater_denoise_vars(&a, (stater_stream)stream), "Estimator::DenoiseVars");
    }

    // stat_denoiser::denoiseFilm (estimator.cpp:419-459): the film buffer is the
    // mean of the untransformed set (the running mean when denoisefilm is off).
    void DenoiseMeans() {
        stater_denoise_film_args a;
        std::memset(&a, 0, sizeof(a));
        a.n_buffers = K;
        a.width = width;
        a.height = height;
        a.filter_radius = cfg.filter_radius;
        a.ds_factor = -.5f / (cfg.filter_sd * cfg.filter_sd);
        a.alpha = (float)cfg.alpha;
        a.mt_mode = cfg.mt_mode;
        a.use_levc = cfg.use_levc ? 1 : 0;
        a.discr_source = cfg.cascade ? STATER_DISCR_DENOISED : STATER_DISCR_SAMPLE;
        a.precision = cfg.precision;
        a.n = n_ptr();
        a.film = film_for_precision();
        for (int k = 0; k < K; k++) {
            a.mean[k] = stat(k, STATER_Q_MEAN);
            a.varD[k] = out(11, k);
            a.varCD[k] = out(12, k);
            a.jb[k] = out(7, k);
            a.discr[k] = out(13, k);
            a.m2[k] = stat(k, STATER_Q_M2);
            a.m2C[k] = out(10, k);
        }
        a.gbuffers = gbuffers(meanG);
        a.filmD = filmD_.get();
        check(stater_test_order(cfg.transforms.data(), K, a.test_order), "Estimator::DenoiseMeans");
        check(stater_denoise_film(&a, (stater_stream)stream), "Estimator::DenoiseMeans");
    }

    // Estimator::CalcMeanVars / calcMatMeanVar (estimator.cpp:462-496): meanVar of
    // the untransformed set (FP32 statistics).
    void CalcMeanVars() {
        if (cfg.precision != STATER_F32) throw std::invalid_argument("CalcMeanVars: FP32 statistics only");
        check(stater_calc_mean_var(width, height, n_ptr(), (const float *)stat(0, STATER_Q_M2),
                                   (float *)meanVar_.get(), (stater_stream)stream),
              "Estimator::CalcMeanVars");
    }

    // stat_denoiser::calcTargetSPP (estimator.cpp:498-513).
    void CalcTargetSPPs(uint64_t spp) {
        stater_target_spp_args a;
        std::memset(&a, 0, sizeof(a));
        a.width = width;
        a.height = height;
        a.spp = (int32_t)spp;
        a.precision = cfg.precision;
        a.n = n_ptr();
        a.m2 = stat(0, STATER_Q_M2);
        a.varD = out(11, 0);
        a.mean = stat(0, STATER_Q_MEAN);
        a.eps = cfg.target_eps;
        a.tmin = cfg.target_min;
        a.tmax = cfg.target_max;
        a.as_source = cfg.as_source;
        a.targetspp = (int32_t *)targetSPPBuffer.device;
        check(stater_calc_target_spp_ex(&a, (stater_stream)stream), "Estimator::CalcTargetSPPs");
    }

    void Synchronize() { check(stater_synchronize((stater_stream)stream), "Estimator::Synchronize"); }
    void PrintMacroConfiguration() { stater_print_macro_configuration(); }

    // Buffer of the untransformed (t0, "film-") or transformed (t1) set of Box-Cox
    // index j, by BUF_LIST / FILM_BUF_LIST name; nullptr if there is none.
    Buffer *t0(const std::string &name, int j, int type = Radiance) { return find("t" + std::to_string(type) + "-b" + std::to_string(j) + "-film-" + name); }
    Buffer *t1(const std::string &name, int j, int type = Radiance) { return find("t" + std::to_string(type) + "-b" + std::to_string(j) + "-" + name); }
    Buffer *find(const std::string &name) {
        for (auto &b : owned_)
            if (b->name == name) return b.get();
        return nullptr;
    }

    // Denoise-only replay input (StatPathIntegrator::Denoise, statpath.cpp:506-547):
    // "<stem>-<spp>-film.pfm" into the film buffer, every "<stem>-<spp>-t<T>-b<j>-<suffix>.pfm"
    // into the buffer of that name. Returns the number of files read.
    int ReadReplayFiles(const std::string &stem, uint64_t spp) {
        const std::string prefix = stem + "-" + std::to_string(spp) + "-";
        std::string err;
        int nread = 0;
        const std::string film = prefix + "film.pfm";
        if (std::filesystem::exists(film)) {
            if (!read_buffer(film, filmBuffer, &err, pinned_host)) throw std::runtime_error(err);
            nread++;
        }
        for (const auto &f : list_replay_files(prefix)) {
            const BufferFileId id = parse_buffer_file_id(f.second);
            if (id.t < 0 || id.b < 0 || id.suffix.empty()) continue;
            Buffer *b = find(f.second);
            if (!b) continue;
            if (!read_buffer(f.first, *b, &err, pinned_host)) throw std::runtime_error(err);
            nread++;
        }
        return nread;
    }

    Buffer &filmBuffer;
    EstimatorConfig cfg;
    BufferRegistry &reg;
    const int width, height;
    int K = 0;
    cudaStream_t stream = nullptr;
    Buffer filmFilteredBuffer;  // "filmD"
    Buffer targetSPPBuffer;     // "targetspp"

  private:
    struct GBuf {
        int first, channels;
        float dr;
    };

    size_t HW() const { return (size_t)width * height; }
    Elem elem() const { return cfg.precision == STATER_F64 ? Elem::F64 : Elem::F32; }
    size_t esize() const { return elem_size(elem()); }
    int32_t *n_ptr() const { return (int32_t *)n_.get(); }
    void *stat(int k, int q) const { return (char *)stats_.get() + ((size_t)(k * STATER_NQ + q) * 3) * HW() * esize(); }
    // Output list index i (7..13 of kBufList) of transform k.
    void *out(int i, int k) const {
        if (i == 7) return (char *)jb_.get() + (size_t)k * HW() * esize();
        return (char *)outs_.get() + ((size_t)((i - 8) * K + k) * 3) * HW() * esize();
    }

    Buffer &new_buffer(const std::string &name, int channels, Elem e) {
        owned_.push_back(std::make_unique<Buffer>());
        Buffer &b = *owned_.back();
        b.name = name;
        b.width = width;
        b.height = height;
        b.channels = channels;
        b.elem = e;
        reg.Register(b);
        return b;
    }

    void AllocateBuffers() {
        n_ = device_alloc(HW() * sizeof(int32_t));
        stats_ = device_alloc((size_t)K * STATER_NQ * 3 * HW() * esize());
        gmean_ = device_alloc((size_t)(cfg.n_features ? cfg.n_features : 1) * HW() * esize());
        jb_ = device_alloc((size_t)K * HW() * esize());
        outs_ = device_alloc((size_t)6 * K * 3 * HW() * esize());
        meanVar_ = device_alloc(3 * HW() * sizeof(float));
        filmD_ = device_alloc(3 * HW() * esize());
        target_ = device_alloc(HW() * sizeof(int32_t));
        if (cfg.precision == STATER_F64) film64_ = device_alloc(3 * HW() * sizeof(double));

        filmFilteredBuffer.name = "filmD";
        filmFilteredBuffer.width = width;
        filmFilteredBuffer.height = height;
        filmFilteredBuffer.channels = 3;
        filmFilteredBuffer.elem = elem();
        filmFilteredBuffer.device = filmD_.get();
        targetSPPBuffer.name = "targetspp";
        targetSPPBuffer.width = width;
        targetSPPBuffer.height = height;
        targetSPPBuffer.channels = 1;
        targetSPPBuffer.elem = Elem::I32;
        targetSPPBuffer.device = target_.get();
        reg.Register(filmFilteredBuffer);
        reg.Register(targetSPPBuffer);

        // Box-Cox indices j = 0 .. nb-1; with a single transform, index 0's
        // transformed set is the identity itself.
        const int nb = K > 1 ? K - 1 : 1;
        for (int j = 0; j < nb; j++) {
            const int kt = K > 1 ? j + 1 : 0;
            const std::string pre = "t" + std::to_string((int)Radiance) + "-b" + std::to_string(j) + "-";
            for (int i = 0; i < kNBufList; i++) {
                const int ch = i == 7 ? 1 : 3;
                Buffer &b1 = new_buffer(pre + kBufList[i], ch, elem());
                b1.device = i < 7 ? stat(kt, i) : out(i, kt);
            }
            for (int i = 0; i < kNBufList; i++) {
                const int ch = i == 7 ? 1 : 3;
                Buffer &b0 = new_buffer(pre + "film-" + kBufList[i], ch, elem());
                b0.device = i < 7 ? stat(0, i) : out(i, 0);
            }
            Buffer &bn = new_buffer(pre + "film-n", 1, Elem::I32);
            bn.device = n_.get();
            Buffer &bv = new_buffer(pre + "film-meanVar", 3, Elem::F32);
            bv.device = meanVar_.get();
        }
    }

    void add_gbuffer(std::vector<GBuf> &list, int first, int channels, float sd) {
        if ((channels != 1 && channels != 3) || first < 0 || first + channels > cfg.n_features)
            throw std::invalid_argument("G-buffer outside the feature channels");
        if ((int)list.size() >= STATER_MAX_GBUFFERS) throw std::invalid_argument("too many G-buffers");
        list.push_back({first, channels, -.5f / (sd * sd)});
    }

    stater_gbuffers gbuffers(const std::vector<GBuf> &list) const {
        stater_gbuffers g;
        std::memset(&g, 0, sizeof(g));
        g.count = (int32_t)list.size();
        for (size_t i = 0; i < list.size(); i++) {
            g.planes[i] = (char *)gmean_.get() + (size_t)list[i].first * HW() * esize();
            g.channels[i] = list[i].channels;
            g.dr_factor[i] = list[i].dr;
        }
        return g;
    }

    // The film in the statistics' precision: FP32 as is; for the FP64 form a
    // widened copy (host round trip; the plain FP64 form is a reference path).
    const void *film_for_precision() {
        if (!cfg.denoise_film) return stat(0, STATER_Q_MEAN);
        if (cfg.precision == STATER_F32) return filmBuffer.device;
        std::vector<float> f(3 * HW());
        std::vector<double> d(3 * HW());
        check_cuda(cudaMemcpyAsync(f.data(), filmBuffer.device, f.size() * 4, cudaMemcpyDeviceToHost, stream),
                   "film download");
        check_cuda(cudaStreamSynchronize(stream), "film download");
        for (size_t i = 0; i < f.size(); i++) d[i] = f[i];
        check_cuda(cudaMemcpyAsync(film64_.get(), d.data(), d.size() * 8, cudaMemcpyHostToDevice, stream),
                   "film upload");
        check_cuda(cudaStreamSynchronize(stream), "film upload");
        return film64_.get();
    }

    std::vector<GBuf> varG, meanG;
    std::vector<std::unique_ptr<Buffer>> owned_;
    std::shared_ptr<void> n_, stats_, gmean_, jb_, outs_, meanVar_, filmD_, target_, film64_;
};

}  // namespace host
}  // namespace stater
