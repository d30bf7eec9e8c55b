// Harness that drives the reference's own StatTile arithmetic
// (src/statistics/estimator.h:143-330, compiled from the reference tree with
// the stand-in headers in ref_shim/) the way StatPathIntegrator::Render feeds it
// (src/statistics/statpath.cpp:339-379): 16x16 tiles, per pixel all samples in
// order, radiance through AddTransformSample*/AddSample*, every feature channel
// through AddSampleM1. Tile state persists across calls to ref_add, as the
// render loop keeps its tiles across iterations (statpath.cpp:133-150).
//
// TEST INFRASTRUCTURE ONLY: used to generate the golden vectors that pin the
// oracle. Built by oracle/build_ref.sh into oracle/_ref/.
#include "estimator.h"
#include <cstring>
#include <memory>

using namespace pbrt;

namespace {
typedef StatTile<Vec3> RTile;
typedef StatTile<Float> FTile;

struct RefState {
    int W, H, G, nL;
    std::vector<Bounds2i> bounds;
    std::vector<std::vector<RTile>> rad;   // [tile][lambda]
    std::vector<std::vector<FTile>> feat;  // [tile][feature channel]
};

#if FULL_MULTI_TRANSFORM == 1
#define LAMBDA_ARG , (Float)lambdas[j]
#else
#define LAMBDA_ARG
#endif
#if FULL_MULTI_TRANSFORM == 1
#define LAMBDA1_ARG , (Float)1.f
#else
#define LAMBDA1_ARG
#endif
}  // namespace

extern "C" {

int ref_float_size() { return (int)sizeof(Float); }
int ref_pixel_record_size() { return (int)sizeof(StatTilePixel<Vec3>); }
int ref_stats_offset_t0() { return (int)offsetof(StatTilePixel<Vec3>, t0); }
int ref_stats_offset_t1() { return (int)offsetof(StatTilePixel<Vec3>, t1); }

void *ref_create(int W, int H, int G, int nL) {
    RefState *st = new RefState();
    st->W = W; st->H = H; st->G = G; st->nL = nL;
    const int ts = 16;
    for (int ty = 0; ty < (H + ts - 1) / ts; ty++)
        for (int tx = 0; tx < (W + ts - 1) / ts; tx++) {
            Bounds2i b(Point2i(tx * ts, ty * ts), Point2i(std::min(tx * ts + ts, W), std::min(ty * ts + ts, H)));
            st->bounds.push_back(b);
            st->rad.emplace_back(std::vector<RTile>(nL, RTile(b)));
            st->feat.emplace_back(std::vector<FTile>(G, FTile(b)));
        }
    return st;
}

void ref_destroy(void *h) { delete (RefState *)h; }

// samples: float32 planes [S][5+G][H*W] (R,G,B,u,v,features...), count: per-pixel
// number of valid samples (NULL = S). transform: 1 = AddTransformSample* (t0 raw,
// t1 Box-Cox), 0 = AddSample*. max_moment: 1..5 as the "maxmoment" parameter
// (statpath.cpp:36-60). lambdas: nL Box-Cox lambdas (multi-transform build only).
void ref_add(void *h, int S, const float *samples, const int *count, int transform,
             int max_moment, const float *lambdas) {
    RefState *st = (RefState *)h;
    const int W = st->W, H = st->H, G = st->G, NCH = 5 + G;
    const size_t HW = (size_t)W * H;
    (void)lambdas;
    for (size_t t = 0; t < st->bounds.size(); t++) {
        const Bounds2i &b = st->bounds[t];
        for (int y = b.pMin.y; y < b.pMax.y; y++)
            for (int x = b.pMin.x; x < b.pMax.x; x++) {
                const size_t p = (size_t)y * W + x;
                const int ns = count ? count[p] : S;
                for (int s = 0; s < ns; s++) {
                    const float *sp = samples + (size_t)s * NCH * HW + p;
                    Vec3 rgb((Float)sp[0], (Float)sp[HW], (Float)sp[2 * HW]);
                    Point2f inPxP((Float)sp[3 * HW], (Float)sp[4 * HW]);
                    Point2i pix(x, y);
                    for (int j = 0; j < st->nL; j++) {
                        RTile &tile = st->rad[t][j];
                        if (transform) {
                            switch (max_moment) {
                                case 1: tile.AddTransformSampleM1(pix, inPxP, rgb LAMBDA_ARG); break;
                                case 2: tile.AddTransformSampleM2(pix, inPxP, rgb LAMBDA_ARG); break;
                                case 3: tile.AddTransformSampleM3(pix, inPxP, rgb LAMBDA_ARG); break;
                                case 4: tile.AddTransformSampleM4(pix, inPxP, rgb LAMBDA_ARG); break;
                                default: tile.AddTransformSampleM4C(pix, inPxP, rgb LAMBDA_ARG); break;
                            }
                        } else {
                            switch (max_moment) {
                                case 1: tile.AddSampleM1(pix, inPxP, rgb LAMBDA_ARG); break;
                                case 2: tile.AddSampleM2(pix, inPxP, rgb LAMBDA_ARG); break;
                                case 3: tile.AddSampleM3(pix, inPxP, rgb LAMBDA_ARG); break;
                                case 4: tile.AddSampleM4(pix, inPxP, rgb LAMBDA_ARG); break;
                                default: tile.AddSampleM4C(pix, inPxP, rgb LAMBDA_ARG); break;
                            }
                        }
                    }
                    for (int g = 0; g < G; g++)
                        st->feat[t][g].AddSampleM1(pix, inPxP, (Float)sp[(5 + g) * HW] LAMBDA1_ARG);
                }
            }
    }
}

// Reads the tile state back. n: int64 [H*W]; stats: Float [nL][2][7][3][H*W]
// (transform set t0/t1, moments mean,m2,m3,m4,c2X,c2Y,m1, channel);
// gmean: Float [G][H*W]; records: raw StatTilePixel<Vec3> bytes for every tile in
// tile order, pixels row-major inside a tile (lambda 0 only), may be NULL.
void ref_read(void *h, long long *n, Float *stats, Float *gmean, unsigned char *records) {
    RefState *st = (RefState *)h;
    const int W = st->W, G = st->G;
    const size_t HW = (size_t)W * st->H;
    size_t rec = 0;
    for (size_t t = 0; t < st->bounds.size(); t++) {
        const Bounds2i &b = st->bounds[t];
        for (int y = b.pMin.y; y < b.pMax.y; y++)
            for (int x = b.pMin.x; x < b.pMax.x; x++) {
                const size_t p = (size_t)y * W + x;
                Point2i pix(x, y);
                for (int j = 0; j < st->nL; j++) {
                    const StatTilePixel<Vec3> &px = st->rad[t][j].GetPixel(pix);
                    if (j == 0) {
                        n[p] = (long long)px.n;
                        if (records) {
                            std::memcpy(records + rec * sizeof(px), &px, sizeof(px));
                            rec++;
                        }
                    }
                    const StatTilePixelStats<Vec3> *sets[2] = {&px.t0, &px.t1};
                    for (int ts = 0; ts < 2; ts++) {
                        const StatTilePixelStats<Vec3> &s = *sets[ts];
                        const Vec3 *mom[7] = {&s.mean, &s.m2, &s.m3, &s.m4, &s.c2X, &s.c2Y, &s.m1};
                        for (int q = 0; q < 7; q++)
                            for (int c = 0; c < 3; c++)
                                stats[((((size_t)j * 2 + ts) * 7 + q) * 3 + c) * HW + p] = (*mom[q])[c];
                    }
                }
                for (int g = 0; g < G; g++) gmean[(size_t)g * HW + p] = st->feat[t][g].GetPixel(pix).t0.mean;
            }
    }
}
}
