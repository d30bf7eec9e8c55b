"""Film path on the GPU (stater_film_add_samples / stater_film_update_image)
against the oracle: pbrt-v3 FilmTile::AddSample with the box filter of radius
0.5 and Film::UpdateImage (core/film.h:152-190, core/film.cpp:187-222).

Own-pixel sums, weights and the film RGB are bit-exact. Edge samples (u or v
exactly 0 or 1) reach the neighbour's spill planes through atomic adds, whose
order is not fixed: where a pixel receives more than one, its spill agrees to
float rounding (rtol 1e-6) and its RGB to 2e-6 of the pixel's largest channel
(the XYZ -> RGB matrix cancels), elsewhere bit for bit.
"""
import numpy as np
import pytest

import oracle
from helpers import synth_samples
from test_oracle_film import _edge_samples

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import stater_gb300 as S
    S.setup()
    return S


def _gpu_film(S, rounds, G, max_lum=float("inf"), scale=1.0):
    H, W = rounds[0][0].shape[2:]
    f = S.Film(W, H, n_features=G, max_sample_luminance=max_lum, scale=scale)
    for smp, cnt in rounds:
        f.add_samples(torch.from_numpy(smp).cuda(), None if cnt is None else torch.from_numpy(cnt).cuda())
    rgb = f.update_image()
    torch.cuda.synchronize()
    return (f.contrib_sum.cpu().numpy(), f.weight_sum.cpu().numpy(), f.spill.cpu().numpy()), rgb.cpu().numpy()


def _orc_film(rounds, max_lum=np.inf, scale=1.0):
    st = None
    for smp, cnt in rounds:
        st = oracle.film_add_samples(smp, count=cnt, max_lum=max_lum, state=st)
    return st, oracle.film_update_image(st, scale=scale)


def test_film_bitwise_two_rounds_with_counts(S):
    W, H, G = 97, 61, 3
    s1 = synth_samples(W, H, 24, G=G, seed=1)
    s2 = synth_samples(W, H, 40, G=G, seed=2)
    c2 = np.random.default_rng(3).integers(0, 41, size=(H, W)).astype(np.int32)
    rounds = [(s1, None), (s2, c2)]
    (gc, gw, gs), grgb = _gpu_film(S, rounds, G)
    (oc, ow, os_), orgb = _orc_film(rounds)
    assert np.array_equal(gc, oc) and np.array_equal(gw, ow) and np.array_equal(gs, os_)
    assert np.array_equal(grgb, orgb)


def test_film_luminance_clamp_and_scale(S):
    W, H, G = 64, 48, 1
    smp = synth_samples(W, H, 32, G=G, seed=4, firefly_prob=0.05)
    (gc, gw, _), grgb = _gpu_film(S, [(smp, None)], G, max_lum=5.0, scale=0.5)
    (oc, ow, _), orgb = _orc_film([(smp, None)], max_lum=5.0, scale=0.5)
    assert np.array_equal(gc, oc) and np.array_equal(gw, ow)
    assert np.array_equal(grgb, orgb)


def test_film_edge_samples(S):
    W, H, G = 40, 33, 1
    smp = _edge_samples(W, H, 12, seed=5)
    (gc, gw, gs), grgb = _gpu_film(S, [(smp, None)], G)
    (oc, ow, os_), orgb = _orc_film([(smp, None)])
    assert np.array_equal(gc, oc) and np.array_equal(gw, ow)
    assert np.array_equal(gs[3], os_[3])  # integer-valued weights: order-free
    assert np.allclose(gs, os_, rtol=1e-6, atol=0)
    # XYZ -> RGB cancels: compare against the pixel's largest channel
    scale = np.maximum(np.abs(orgb).max(axis=0, keepdims=True), 1e-30)
    assert np.max(np.abs(grgb - orgb) / scale) < 2e-6
    single = os_[3] <= 1
    assert np.array_equal(grgb[:, single], orgb[:, single])


def test_film_feeds_denoise_film(S):
    """FP64 pipeline with the film RGB as the untransformed mean, against the oracle."""
    W, H, G, N = 48, 40, 7, 32
    smp = synth_samples(W, H, N, G=G, seed=6)
    tr = ("identity", "log1p", "sqrt")
    b = S.StatBuffers(W, H, tr, G, 3, S.F64)
    t = torch.from_numpy(smp).cuda()
    b.accumulate(t)
    film = S.Film(W, H, n_features=G)
    film.add_samples(t)
    rgb = film.update_image()
    b.denoise_vars(radius=4)
    b.denoise_film(radius=4, film=rgb.double())
    torch.cuda.synchronize()
    st, orgb = _orc_film([(smp, None)])
    assert np.array_equal(rgb.cpu().numpy(), orgb)
    n, so, go = oracle.new_state(len(tr), G, H, W)
    oracle.accumulate(smp, tr, 3, n, so, go)
    ds = float(np.float32(-0.5 / 100.0))
    gspec = [(sp.first, sp.channels, sp.sigma) for sp in S.GBUFFERS_ALBEDO_NORMAL]
    v = oracle.denoise_vars(n, so, go, 3, 4, ds, float(np.float32(2.80703)), gspec)
    d = oracle.denoise_film(n, so, v["varD"], v["varCD"], v["jb"], go, orgb.astype(np.float64), 4, ds,
                            float(np.float32(0.01)), gspec)
    assert np.allclose(b.filmD.cpu().numpy(), d["filmD"], rtol=1e-5, atol=0)
    # the film differs from the running mean of the untransformed set
    assert not np.array_equal(orgb.astype(np.float64), so[0, 0])


@pytest.mark.parametrize("W,H,precision,mode,mm", [
    (96, 64, "F32", "ACC_FAST", 3),    # TMA-fed FP32 kernel
    (97, 61, "F32", "ACC_FAST", 5),    # W*H % 4 != 0: plain FP32 kernel
    (80, 48, "F32", "ACC_EXACT", 3),
    (80, 48, "F64", "ACC_EXACT", 5),
])
def test_film_fused_into_accumulate(S, W, H, precision, mode, mm):
    """The film sums taken inside stater_accumulate equal the standalone film pass."""
    G = 7
    s1 = synth_samples(W, H, 20, G=G, seed=11)
    s2 = _edge_samples(W, H, 9, seed=12)
    s2 = np.concatenate([s2, np.zeros((9, G - 1, H, W), np.float32)], axis=1)
    c2 = np.random.default_rng(13).integers(0, 10, size=(H, W)).astype(np.int32)
    b = S.StatBuffers(W, H, ("identity", "log1p", "sqrt"), G, mm, getattr(S, precision))
    fused = S.Film(W, H, n_features=G, max_sample_luminance=50.0)
    for smp, cnt in ((s1, None), (s2, c2)):
        b.accumulate(torch.from_numpy(smp).cuda(), None if cnt is None else torch.from_numpy(cnt).cuda(),
                     mode=getattr(S, mode), film=fused)
    rgb = fused.update_image()
    torch.cuda.synchronize()
    (oc, ow, os_), orgb = _orc_film([(s1, None), (s2, c2)], max_lum=50.0)
    assert np.array_equal(fused.contrib_sum.cpu().numpy(), oc)
    assert np.array_equal(fused.weight_sum.cpu().numpy(), ow)
    assert np.array_equal(fused.spill[3].cpu().numpy(), os_[3])
    assert np.allclose(fused.spill.cpu().numpy(), os_, rtol=1e-6, atol=0)
    single = os_[3] <= 1
    assert np.array_equal(rgb.cpu().numpy()[:, single], orgb[:, single])
    # the statistics are those of an accumulation without the film
    ref = S.StatBuffers(W, H, ("identity", "log1p", "sqrt"), G, mm, getattr(S, precision))
    for smp, cnt in ((s1, None), (s2, c2)):
        ref.accumulate(torch.from_numpy(smp).cuda(), None if cnt is None else torch.from_numpy(cnt).cuda(),
                       mode=getattr(S, mode))
    torch.cuda.synchronize()
    assert torch.equal(ref.stats, b.stats) and torch.equal(ref.n, b.n) and torch.equal(ref.gmean, b.gmean)
