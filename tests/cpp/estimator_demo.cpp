// Drives the C++ Estimator mirror (stater_gb300/host/estimator.hpp) the way
// StatPathIntegrator::Render and ::Denoise drive the reference's Estimator
// (statpath.cpp:176-441, 500-560), over libstater.
//
//   estimator_demo render <dir> <W> <H> <spp> <seed> <radius>
//       seeded samples on the device -> Estimator::AddSamples (with the film) ->
//       Film::UpdateImage -> Upload -> DenoiseVars -> DenoiseMeans ->
//       CalcTargetSPPs -> CalcMeanVars -> Download -> Synchronize, then every
//       registered buffer written as <dir>/scene-<spp>-<name>.pfm
//   estimator_demo replay <dir> <W> <H> <spp> <seed> <radius>
//       a fresh Estimator reads those files (ReadReplayFiles), runs Upload ->
//       DenoiseVars -> DenoiseMeans -> Download -> Synchronize and writes
//       <dir>/replay-<spp>-filmD.pfm
//
// Test driver: built and run by tests/test_gpu_host_cpp.py.
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <string>

#include "estimator.hpp"

using namespace stater::host;

static EstimatorConfig config(int radius) {
    EstimatorConfig c;
    const int kinds[5] = {STATER_TK_IDENTITY, STATER_TK_LOG1P, STATER_TK_SQRT, STATER_TK_CBRT, STATER_TK_ASINH};
    for (int k : kinds) c.transforms.push_back(stater_transform{k, 1.0f});
    c.n_features = 7;
    c.max_moment = 5;
    c.filter_radius = radius;
    c.enable_as = true;
    c.denoise_film = true;
    c.use_levc = false;  // the MC variant, as the Python side of the test runs it
    c.cascade = true;
    c.precision = STATER_F32;
    c.acc_mode = STATER_ACC_FAST;
    return c;
}

static void register_gbuffers(Estimator &est) {
    est.RegisterFeatureBuffer(StatAlbedo, 0, 3);
    est.RegisterFeatureBuffer(StatNormal, 3, 3);
    est.RegisterFeatureBuffer(StatDepth, 6, 1);
    est.RegisterVarGBuffer(0, 3, 0.02f);
    est.RegisterVarGBuffer(3, 3, 0.1f);
    est.RegisterMeanGBuffer(0, 3, 0.02f);
    est.RegisterMeanGBuffer(3, 3, 0.1f);
}

static int render(const std::string &dir, int W, int H, int spp, unsigned long long seed, int radius) {
    Film film(W, H, 7);
    BufferRegistry reg;
    reg.Register(film.buffer);
    Estimator est(film.buffer, config(radius), reg);
    register_gbuffers(est);

    const size_t HW = (size_t)W * H;
    auto samples = device_alloc((size_t)spp * 12 * HW * sizeof(float));
    stater_generate_args g;
    std::memset(&g, 0, sizeof(g));
    g.width = W;
    g.height = H;
    g.n_samples = spp;
    g.n_features = 7;
    g.seed = seed;
    g.region = 8;
    g.mean_mu = -1.f;
    g.mean_sigma = 1.f;
    g.noise_sigma = 0.5f;
    g.firefly_prob = 1e-3f;
    g.firefly_scale = 1e3f;
    g.samples = (float *)samples.get();
    check(stater_generate_samples(&g, (stater_stream)est.stream), "generate");

    film.Clear(est.stream);
    est.AddSamples((const float *)samples.get(), spp, nullptr, &film);  // statistics and film in one pass
    film.UpdateImage(est.stream);

    est.Upload();
    est.DenoiseVars();
    est.DenoiseMeans();
    est.CalcTargetSPPs(spp);
    est.CalcMeanVars();
    est.Download();
    est.Synchronize();

    OutputBufferSelection sel(reg, std::regex(".*"), dir + "/scene.pfm");
    est.Download(sel);
    est.Synchronize();
    std::string err;
    if (!sel.Write(std::to_string(spp), &err)) throw std::runtime_error(err);
    std::printf("render: wrote %zu buffers\n", sel.buffers.size());
    return 0;
}

static int replay(const std::string &dir, int W, int H, int spp, int radius) {
    Film film(W, H, 7);
    BufferRegistry reg;
    reg.Register(film.buffer);
    EstimatorConfig c = config(radius);
    c.enable_as = false;
    Estimator est(film.buffer, c, reg);
    register_gbuffers(est);
    const int nread = est.ReadReplayFiles(dir + "/scene", spp);
    est.Upload();
    est.DenoiseVars();
    est.DenoiseMeans();
    est.Download();
    est.Synchronize();
    OutputBufferSelection sel(reg, std::regex("filmD"), dir + "/replay.pfm");
    std::string err;
    if (!sel.Write(std::to_string(spp), &err)) throw std::runtime_error(err);
    std::printf("replay: read %d files\n", nread);
    return 0;
}

int main(int argc, char **argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s render|replay <dir> <W> <H> <spp> <seed> <radius>\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[1], dir = argv[2];
    const int W = std::atoi(argv[3]), H = std::atoi(argv[4]), spp = std::atoi(argv[5]);
    const unsigned long long seed = std::strtoull(argv[6], nullptr, 10);
    const int radius = std::atoi(argv[7]);
    try {
        if (mode == "render") return render(dir, W, H, spp, seed, radius);
        if (mode == "replay") return replay(dir, W, H, spp, radius);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 2;
}
