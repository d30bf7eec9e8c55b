"""Self-consistency of the oracle's stage-2/3 restatements (CPU only).

Stages 2-3 have no source in the reference tree, so these check the oracle
against independent restatements: scipy's Student-t quantiles, numpy least
squares, exact summation, sequential accumulation, and a pure-Python loop
version of both windowed filters.
"""
import math

import numpy as np
import pytest

import oracle
from helpers import synth_samples

scipy_stats = pytest.importorskip("scipy.stats")


@pytest.mark.parametrize("p,df", [(0.995, 1), (0.995, 2), (0.995, 7.5), (0.995, 63), (0.995, 255),
                                  (0.975, 30), (0.9975, 1000), (0.995, 1e5)])
def test_t_quantile_matches_scipy(p, df):
    assert oracle.t_quantile(p, df) == pytest.approx(scipy_stats.t.ppf(p, df), rel=1e-10)


def test_normal_quantile_matches_scipy():
    assert oracle.t_quantile(0.995, 0.0) == pytest.approx(scipy_stats.norm.ppf(0.995), rel=1e-12)


def test_tcrit_table_monotone_and_exact_at_nodes():
    t = oracle.tcrit2_table(0.01, 1024)
    assert np.all(np.diff(t) > 0)
    for m in (1, 16, 512, 1024):
        assert t[m] == pytest.approx(scipy_stats.t.ppf(0.995, 1024 / m) ** 2, rel=1e-10)


def test_tree_sum_is_accurate():
    rng = np.random.default_rng(1)
    for n in (1, 7, 1024, 1025, 300001):
        v = rng.random(n) * 10 ** rng.uniform(-3, 3, n)
        assert oracle.tree_sum(v) == pytest.approx(math.fsum(v), rel=1e-13)


def test_pebay_merge_matches_sequential():
    W, H, G = 9, 7, 0
    a = synth_samples(W, H, 40, G=G, seed=3)
    b = synth_samples(W, H, 25, G=G, seed=4)
    tr = ["identity", "log1p", "sqrt"]
    nA, sA, gA = oracle.new_state(3, G, H, W)
    oracle.accumulate(a, tr, 5, nA, sA, gA)
    nB, sB, gB = oracle.new_state(3, G, H, W)
    oracle.accumulate(b, tr, 5, nB, sB, gB)
    nS, sS, gS = oracle.new_state(3, G, H, W)
    oracle.accumulate(np.concatenate([a, b]), tr, 5, nS, sS, gS)
    oracle.merge_moments(nA, sA, nB, sB, 5)
    assert np.array_equal(nA, nS)
    for q in range(4):  # mean, m2, m3, m4
        scale = np.abs(sS[:, 1]) ** ((q + 1) / 2 if q else 0.5) + np.abs(sS[:, 0]) + 1e-12
        assert np.max(np.abs(sA[:, q] - sS[:, q]) / scale) < 1e-10


def test_lev_matches_numpy_lstsq():
    W, H, G, S = 4, 3, 7, 60
    rng = np.random.default_rng(5)
    smp = synth_samples(W, H, S, G=G, seed=6)
    smp[:, 5:] = rng.random((S, G, H, W))
    smp[:, 0:3] += 0.3 * smp[:, 5:8]
    st = np.zeros((oracle.lev_nstate(G), H, W))
    oracle.lev_accumulate(smp[:30], st)
    oracle.lev_accumulate(smp[30:], st)
    out = oracle.lev_solve(st, G, H, W, lam=0.0)
    for y in range(H):
        for x in range(W):
            X = np.concatenate([np.ones((S, 1)), smp[:, 5:, y, x].astype(np.float64)], 1)
            for c in range(3):
                yv = smp[:, c, y, x].astype(np.float64)
                beta, *_ = np.linalg.lstsq(X, yv, rcond=None)
                rss = np.sum((yv - X @ beta) ** 2)
                assert out["m2C"][c, y, x] == pytest.approx(rss, rel=1e-8)
                assert np.allclose(out["beta"][c, :, y, x], beta, rtol=1e-7, atol=1e-9)


def _py_denoise(n, stats, gmean, mm, R, ds, z, gspec, alpha, mt_mode, use_levc, lut, discr_source=0):
    """Pure-Python restatement of both filters (small images only). discr_source
    1: the Welch discriminator from the pixel's own sample variance (the
    reference's CASCADE_MODE=0) instead of the denoised one."""
    K, _, _, H, W = stats.shape
    s2 = np.zeros((K, 3, H, W)); s2c = np.zeros_like(s2); ln = np.zeros_like(s2); se = np.zeros_like(s2)
    jb = np.zeros((K, H, W))
    for k in range(K):
        for y in range(H):
            for x in range(W):
                nn = float(n[y, x])
                for c in range(3):
                    M2, M3, M4 = stats[k, 1, c, y, x], stats[k, 2, c, y, x], stats[k, 3, c, y, x]
                    s2[k, c, y, x] = M2 / (nn - 1)
                    cB = nn / (nn - z) if nn > z + 1 else 1.0
                    kurt = nn * M4 / M2 ** 2 if (mm >= 4 and M2 > 0) else 3.0
                    m2c = M2
                    if mm >= 5:
                        cx, cy = stats[k, 4, c, y, x], stats[k, 5, c, y, x]
                        m2c = max(M2 - 12 * (cx * cx + cy * cy) / nn, 0.0)
                    s2c[k, c, y, x] = m2c / (nn - 1)
                    ln[k, c, y, x] = math.log(cB * max(s2[k, c, y, x], 1e-30))
                    se[k, c, y, x] = cB * cB * (kurt - (nn - 3) / nn) / (nn - 1)
                    if M2 > 0:
                        j = nn * M3 * M3 / M2 ** 3 + ((kurt - 3) ** 2 / 4 if mm >= 4 else 0)
                        jb[k, y, x] += nn / 6 * j

    def w(y, x, yy, xx):
        a = ds * ((xx - x) ** 2 + (yy - y) ** 2)
        for f, ch, dr in gspec:
            a += dr * sum((gmean[f + q, y, x] - gmean[f + q, yy, xx]) ** 2 for q in range(ch))
        return math.exp(a)

    varD = np.zeros_like(s2); varCD = np.zeros_like(s2)
    for k in range(K):
        for y in range(H):
            for x in range(W):
                for c in range(3):
                    sw = sv = svc = 0.0
                    for yy in range(max(0, y - R), min(H, y + R + 1)):
                        for xx in range(max(0, x - R), min(W, x + R + 1)):
                            if (yy, xx) != (y, x):
                                dl = ln[k, c, y, x] - ln[k, c, yy, xx]
                                if dl * dl > z * z * (se[k, c, y, x] + se[k, c, yy, xx]):
                                    continue
                            ww = w(y, x, yy, xx)
                            sw += ww; sv += ww * s2[k, c, yy, xx]; svc += ww * s2c[k, c, yy, xx]
                    varD[k, c, y, x] = sv / sw; varCD[k, c, y, x] = svc / sw
    if discr_source == 1:
        v = s2c if use_levc else s2
    else:
        v = varCD if use_levc else varD
    d = v / n[None, None]
    e = d * d / (n[None, None] - 1)
    film = stats[0, 0]
    N = len(lut) - 1

    def t2(u):
        u = min(u, 1.0); f = u * N; m = min(int(f), N - 1)
        return lut[m] + (f - m) * (lut[m + 1] - lut[m])

    filmD = np.zeros((3, H, W))
    for y in range(H):
        for x in range(W):
            ks = range(K) if mt_mode == 2 else [int(np.argmin(jb[:, y, x]))]
            sw = 0.0; sf = np.zeros(3)
            for yy in range(max(0, y - R), min(H, y + R + 1)):
                for xx in range(max(0, x - R), min(W, x + R + 1)):
                    ok = True
                    if (yy, xx) != (y, x):
                        for k in ks:
                            mu = film if k == 0 else stats[k, 0]
                            for c in range(3):
                                s = d[k, c, y, x] + d[k, c, yy, xx]
                                diff = mu[c, y, x] - mu[c, yy, xx]
                                if not s > 0:
                                    ok = ok and diff == 0
                                    continue
                                u = (e[k, c, y, x] + e[k, c, yy, xx]) / (s * s)
                                if diff * diff > t2(u) * s:
                                    ok = False
                    if ok:
                        ww = w(y, x, yy, xx)
                        sw += ww; sf += ww * film[:, yy, xx]
            filmD[:, y, x] = sf / sw
    return dict(jb=jb, lnS2=ln, se2=se, varD=varD, varCD=varCD, filmD=filmD, discr=d)


@pytest.mark.parametrize("mm,mt_mode,use_levc,discr_source", [(3, 2, False, 0), (5, 2, True, 0), (5, 3, False, 0),
                                                               (3, 2, False, 1), (5, 2, True, 1)])
def test_filters_match_python_restatement(mm, mt_mode, use_levc, discr_source):
    W, H, G, S, R = 7, 6, 7, 24, 2
    smp = synth_samples(W, H, S, G=G, seed=21, region=3, noise_sigma=0.3)
    tr = ["identity", "log1p", "sqrt"]
    n, st, gm = oracle.new_state(3, G, H, W)
    oracle.accumulate(smp, tr, mm, n, st, gm)
    gspec = [(0, 3, 0.2), (3, 3, 0.3)]
    ds = float(np.float32(-0.5 / 4.0))
    z = float(np.float32(2.80703))
    v = oracle.denoise_vars(n, st, gm, mm, R, ds, z, gspec)
    lut = oracle.tcrit2_table(0.01)
    f = oracle.denoise_film(n, st, v["varD"], v["varCD"], v["jb"], gm, st[0, 0], R, ds, 0.01, gspec,
                            mt_mode=mt_mode, use_levc=use_levc, lut=lut, discr_source=discr_source, m2C=v["m2C"])
    gpy = [(a, b, float(np.float32(-0.5 / (s * s)))) for a, b, s in gspec]
    py = _py_denoise(n, st, gm, mm, R, ds, z, gpy, 0.01, mt_mode, use_levc, lut, discr_source)
    for key in ("jb", "lnS2", "se2", "varD", "varCD"):
        assert np.allclose(v[key], py[key], rtol=1e-12, atol=1e-300), key
    assert np.allclose(f["discr"], py["discr"], rtol=1e-12)
    assert np.allclose(f["filmD"], py["filmD"], rtol=1e-12)


def test_target_spp_budget_and_clamp():
    rng = np.random.default_rng(8)
    H, W = 37, 41
    n = rng.integers(16, 64, size=(H, W)).astype(np.int32)
    varD = rng.random((3, H, W)) ** 3
    mean = rng.random((3, H, W)) + 0.1
    t = oracle.calc_target_spp(n, varD, mean, spp=64, tmin=0, tmax=1 << 30)
    assert abs(int(t.sum()) - 64 * H * W) <= H * W  # rounding only
    t2 = oracle.calc_target_spp(n, varD, mean, spp=64, tmin=16, tmax=1024)
    assert t2.min() >= 16 and t2.max() <= 1024
    n[0, 0] = 1
    assert oracle.calc_target_spp(n, varD, mean, spp=64)[0, 0] == 1024


def test_target_spp_sample_variance_source():
    """ASN (the reference's AS_MODE=0) ranks pixels by the sample variance m2/(n-1)."""
    rng = np.random.default_rng(10)
    H, W = 23, 29
    n = rng.integers(16, 64, size=(H, W)).astype(np.int32)
    m2 = rng.random((3, H, W)) * 5
    mean = rng.random((3, H, W)) + 0.1
    asn = oracle.calc_target_spp(n, None, mean, spp=64, m2=m2, as_source=1)
    asm = oracle.calc_target_spp(n, m2 / (n[None] - 1.0), mean, spp=64)
    assert np.array_equal(asn, asm)


def test_mean_var_f32_matches_formula():
    rng = np.random.default_rng(9)
    n = rng.integers(2, 100, size=(5, 6)).astype(np.int32)
    m2 = rng.random((3, 5, 6)).astype(np.float32)
    out = oracle.calc_mean_var_f32(n, m2)
    nf = n.astype(np.float32)
    assert np.array_equal(out, m2 / ((nf - np.float32(1)) * nf))
