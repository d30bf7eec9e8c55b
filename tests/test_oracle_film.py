"""Film path of the oracle (CPU only): pbrt-v3 FilmTile::AddSample with the box
filter of radius 0.5 and Film::UpdateImage (core/film.h:152-190,
core/film.cpp:187-222).

* the colour matrices and luminance weights equal the literals of the
  reference's core/spectrum.h (fixture extracted by
  tests/golden/make_film_constants.py);
* the pixel footprint of every sample equals a loop restatement of
  FilmTile::AddSample's raster bounds in float32 (p0 = ceil(pFilm - 0.5 - r),
  p1 = floor(pFilm - 0.5 + r) + 1, r = 0.5), including samples on pixel edges;
* UpdateImage's XYZ round trip, clamp at zero and weight normalisation.
"""
import json
from pathlib import Path

import numpy as np

import oracle
from helpers import synth_samples

GOLDEN = Path(__file__).resolve().parent / "golden" / "film_constants.json"


def test_constants_match_reference_source():
    g = json.loads(GOLDEN.read_text())
    a, b, y = oracle.film_constants()
    assert np.array_equal(a, np.array(g["rgb_to_xyz"], np.float32))
    assert np.array_equal(b, np.array(g["xyz_to_rgb"], np.float32))
    assert np.array_equal(y, np.array(g["y_weight"], np.float32))


def _edge_samples(W, H, S, seed):
    """Samples whose in-pixel positions are often exactly 0 or 1."""
    smp = synth_samples(W, H, S, G=1, seed=seed, region=1)
    rng = np.random.default_rng(seed + 100)
    pick = rng.integers(0, 4, size=(S, 2, H, W))
    uv = np.choose(pick, [smp[:, 3:5], np.zeros_like(smp[:, 3:5]), np.ones_like(smp[:, 3:5]),
                          np.full_like(smp[:, 3:5], 0.5)])
    smp[:, 3:5] = uv.astype(np.float32)
    return smp


def _footprint_restatement(smp, count=None, max_lum=np.inf):
    """Total (contribution, weight) per pixel from AddSample's raster bounds."""
    S, _, H, W = smp.shape
    f32 = np.float32
    tot = np.zeros((3, H, W), np.float64)
    wt = np.zeros((H, W), np.float64)
    yw = oracle.film_constants()[2]
    for y in range(H):
        for x in range(W):
            cnt = S if count is None else int(count[y, x])
            for s in range(cnt):
                L = smp[s, 0:3, y, x].astype(f32)
                lum = f32(f32(yw[0] * L[0]) + f32(yw[1] * L[1])) + f32(yw[2] * L[2])
                if lum > max_lum:
                    L = (L * f32(f32(max_lum) / lum)).astype(f32)
                pf = (f32(x) + smp[s, 3, y, x], f32(y) + smp[s, 4, y, x])
                pd = (f32(pf[0] - f32(0.5)), f32(pf[1] - f32(0.5)))
                x0, y0 = int(np.ceil(f32(pd[0] - f32(0.5)))), int(np.ceil(f32(pd[1] - f32(0.5))))
                x1, y1 = int(np.floor(f32(pd[0] + f32(0.5)))) + 1, int(np.floor(f32(pd[1] + f32(0.5)))) + 1
                for qy in range(max(y0, 0), min(y1, H)):
                    for qx in range(max(x0, 0), min(x1, W)):
                        tot[:, qy, qx] += L
                        wt[qy, qx] += 1.0
    return tot, wt


def test_footprint_matches_addsample_bounds():
    W, H, S = 9, 7, 6
    smp = _edge_samples(W, H, S, seed=3)
    cnt = np.random.default_rng(4).integers(0, S + 1, size=(H, W)).astype(np.int32)
    for count in (None, cnt):
        cs, ws, sp = oracle.film_add_samples(smp, count=count)
        tot, wt = _footprint_restatement(smp, count)
        assert np.array_equal(ws + sp[3], wt)
        assert np.allclose(cs + sp[:3], tot, rtol=1e-6, atol=0)
        assert sp[3].sum() > 0  # the case under test occurs


def test_luminance_clamp():
    W, H, S = 6, 5, 8
    smp = synth_samples(W, H, S, G=0, seed=5, firefly_prob=0.2)
    cs, ws, sp = oracle.film_add_samples(smp, max_lum=2.0)
    tot, wt = _footprint_restatement(smp, max_lum=2.0)
    assert np.allclose(cs + sp[:3], tot, rtol=1e-6, atol=0)
    raw, _, _ = oracle.film_add_samples(smp)
    assert np.all(cs <= raw) and np.any(cs < raw)


def test_own_sum_is_sequential_float_sum():
    W, H, S = 8, 8, 16
    smp = synth_samples(W, H, S, G=2, seed=6)
    cs, ws, _ = oracle.film_add_samples(smp)
    ref = np.zeros((3, H, W), np.float32)
    for s in range(S):
        ref = ref + smp[s, 0:3]
    assert np.array_equal(cs, ref)
    assert np.array_equal(ws, np.full((H, W), S, np.float32))


def test_update_image_round_trip_and_clamp():
    W, H, S = 8, 6, 4
    smp = synth_samples(W, H, S, G=0, seed=7)
    # pure primaries: the XYZ round trip is not exact and pushes some channels below zero
    smp[:, 0:3, 0, 0] = [1.0, 0.0, 0.0]
    smp[:, 0:3, 0, 1] = [0.0, 0.0, 1.0]
    st = oracle.film_add_samples(smp)
    rgb = oracle.film_update_image(st, scale=1.0)
    a, b, _ = oracle.film_constants()
    cs, ws, sp = st
    xyz = np.einsum("ij,jhw->ihw", a.astype(np.float64), cs.astype(np.float64))
    back = np.einsum("ij,jhw->ihw", b.astype(np.float64), xyz) / ws
    assert np.allclose(rgb, np.maximum(back, 0.0), rtol=1e-6, atol=1e-7)
    assert np.all(rgb >= 0)
    assert np.any(back[:, 0, :2] < 0) and np.all(rgb[:, 0, :2][back[:, 0, :2] < 0] == 0)
    # scale multiplies the normalised value; empty pixels stay zero
    rgb2 = oracle.film_update_image(st, scale=2.0)
    assert np.array_equal(rgb2, rgb * np.float32(2.0))
    empty = (np.zeros((3, H, W), np.float32), np.zeros((H, W), np.float32), np.zeros((4, H, W), np.float32))
    assert np.all(oracle.film_update_image(empty) == 0)
