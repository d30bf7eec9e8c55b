// Host-side checks of the TMA-fed accumulation's warp plan (acc_plan in
// acc_kernels.cuh), compiled with nvcc as host code: for every transform set
// tried, the plan puts each transform on exactly one warp, hands every feature
// channel to exactly one transform within the ceil(G/K) cap, keeps the film
// with transform 0 as costed, gives the same plan twice, and finishes quickly
// for eight transforms. Prints "ok" and exits 0, or names the failure.
#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "acc_kernels.cuh"

using namespace stater;

static int fail(const char *what, int K, int G) {
    std::printf("FAIL: %s (K=%d, G=%d)\n", what, K, G);
    return 1;
}

static int check(const int *kinds, int K, int G, bool film) {
    const AccPlan p = acc_plan(kinds, K, G, film);
    const AccPlan q = acc_plan(kinds, K, G, film);
    int seen[STATER_MAX_TRANSFORMS] = {0};
    for (int w = 0; w < K; w++) {
        if (p.wt[w] < 0 || p.wt[w] >= K) return fail("warp keeps no transform of the set", K, G);
        seen[p.wt[w]]++;
        if (p.wt[w] != q.wt[w]) return fail("plan differs between two calls", K, G);
    }
    for (int k = 0; k < K; k++)
        if (seen[k] != 1) return fail("transform not on exactly one warp", K, G);
    const int cap = (G + K - 1) / K;
    int fseen[STATER_MAX_FEATURES] = {0}, maxc = 0;
    for (int k = 0; k < STATER_MAX_TRANSFORMS; k++) {
        int c = 0;
        for (int j = 0; j < STATER_MAX_FEATURES; j++) {
            const int g = p.featmap[k][j];
            if (g < 0) continue;
            if (k >= K || g >= G) return fail("feature on a transform outside the set", K, G);
            fseen[g]++;
            c++;
        }
        if (c > cap) return fail("more features than the cap on one transform", K, G);
        if (c > maxc) maxc = c;
    }
    for (int g = 0; g < G; g++)
        if (fseen[g] != 1) return fail("feature not kept exactly once", K, G);
    if (maxc != p.maxf) return fail("maxf is not the largest feature count", K, G);
    return 0;
}

int main() {
    const int sets[][8] = {{0, 1, 2, 3, 4, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 0, 0}, {0, 4, 4, 4, 4, 0, 0, 0},
                           {0, 5, 5, 1, 2, 3, 4, 5}, {0, 2, 3, 0, 0, 0, 0, 0}, {0, 1, 0, 0, 0, 0, 0, 0}};
    int bad = 0;
    for (const auto &s : sets)
        for (int K = 1; K <= STATER_MAX_TRANSFORMS; K++)
            for (int G : {0, 1, 3, 7, 16})
                for (bool film : {false, true}) bad += check(s, K, G, film);
    // the K = 5 benchmark set: the two cheap transforms share the scheduler of
    // warps 0 and 4, and the costliest sits beside the producer warp (warp 5)
    const int mix[5] = {STATER_TK_IDENTITY, STATER_TK_LOG1P, STATER_TK_SQRT, STATER_TK_CBRT, STATER_TK_ASINH};
    const AccPlan m = acc_plan(mix, 5, 7, true);
    const int k0 = mix[m.wt[0]], k4 = mix[m.wt[4]], k1 = mix[m.wt[1]];
    if (!((k0 == STATER_TK_SQRT && k4 == STATER_TK_CBRT) || (k0 == STATER_TK_CBRT && k4 == STATER_TK_SQRT)))
        bad += fail("cheap transforms not paired on warps 0 and 4", 5, 7);
    if (k1 != STATER_TK_ASINH) bad += fail("costliest transform not beside the producer", 5, 7);
    const int k8[8] = {0, 1, 2, 3, 4, 5, 5, 5};
    const auto t0 = std::chrono::steady_clock::now();
    bad += check(k8, 8, 16, true);
    const double s8 = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (s8 > 2.0) bad += fail("planning eight transforms takes more than 2 s", 8, 16);
    if (bad) return 1;
    std::printf("ok\n");
    return 0;
}
