"""GPU parity of libstater against the oracle (and, for stage 1, against the
reference's own StatTile through the golden vectors).

Tolerances (from the target): moments of the FP64 form within 1e-12 relative
(floor: the moment's natural scale n*s^q), denoised pixels of the FP64 form
within 1e-5, the FP32 form within 1e-4 of the FP64 oracle with at most 0.1% of
the Welch accept/reject decisions flipped. The FP32 bound holds at every pixel
whose window keeps the same neighbours in both forms: for filmD, every pixel
with no flipped Welch decision (accept bits of both sides); for varD, every
pixel none of whose variance-test decisions lies within 1e-4 of its threshold.
A pixel with a flipped decision averages a different set of neighbours, and
its error is that of the decision, bounded by the flip fraction instead.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from helpers import decision_flips, moment_scale, split_rel_error, synth_samples, var_test_near_boundary

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
BASE_TR = ["identity", "log1p", "sqrt", "cbrt", "asinh"]
REF_TR = ["identity", ("boxcox", 0.25)]
F32_TOL = 1e-4
F64_MOMENT_TOL = 1e-12
F64_PIXEL_TOL = 1e-5
FLIP_TOL = 1e-3


@pytest.fixture(scope="module")
def st():
    import stater_gb300 as S
    S.setup()
    return S


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def moment_err(gpu_stats, ref_stats, n, mm, resolution=0.0):
    """Largest error of the moments relative to their natural scale n*s^q.
    `resolution` > 0 widens s to s + resolution*|mean|: an FP32 form cannot
    resolve within-pixel spreads of a few ulp of the values themselves (a pixel
    with two nearly equal samples), whatever its implementation."""
    worst = 0.0
    qs = {1: [0], 2: [0, 1], 3: [0, 1, 2], 4: [0, 1, 2, 3], 5: [0, 1, 2, 3, 4, 5, 6]}[mm]
    nn = np.maximum(n, 1)[None, None]
    s = np.sqrt(np.abs(ref_stats[:, 1]) / nn) + resolution * np.abs(ref_stats[:, 0])
    for q in qs:
        # c2X, c2Y are covariances with the in-pixel offset (sd 1/sqrt(12)): scale n s / sqrt(12)
        power = {0: 1, 1: 2, 2: 3, 3: 4, 4: 1, 5: 1, 6: 1}[q]
        floor = nn * s ** power * (0.2887 if q in (4, 5) else 1.0) + 1e-300
        if q == 0:
            floor = np.abs(ref_stats[:, 0]) + s + 1e-300
        worst = max(worst, float(np.max(np.abs(gpu_stats[:, q] - ref_stats[:, q]) / floor)))
    return worst


# ---------------------------------------------------------------------------
# stage 1
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("tr,mm", [(BASE_TR, 3), (REF_TR, 5), (["identity"], 1), (BASE_TR, 4)])
def test_accumulate_f64_matches_oracle(st, tr, mm):
    W, H, G = 67, 45, 7
    s1 = synth_samples(W, H, 48, G=G, seed=1, zero_prob=0.01)
    s2 = synth_samples(W, H, 40, G=G, seed=2)
    c2 = np.random.default_rng(3).integers(0, 41, size=(H, W)).astype(np.int32)
    b = st.StatBuffers(W, H, tr, G, mm, st.F64)
    b.accumulate(dev(s1))
    b.accumulate(dev(s2), count=dev(c2))
    n, so, go = oracle.new_state(len(tr), G, H, W)
    oracle.accumulate(s1, tr, mm, n, so, go)
    oracle.accumulate(s2, tr, mm, n, so, go, count=c2)
    assert np.array_equal(host(b.n), n)
    assert moment_err(host(b.stats), so, n, mm) <= F64_MOMENT_TOL
    assert np.max(np.abs(host(b.gmean) - go)) <= 1e-14
    # the identity transform involves no libm call: bit-exact
    assert np.array_equal(host(b.stats)[0], so[0])


def test_accumulate_exact_f32_bitwise_reference_t0(st):
    """FP32 EXACT mode repeats the reference's float arithmetic: the untransformed
    set, n and the feature means equal the reference's StatTile bit for bit."""
    d = np.load(GOLD / "stattile_inputs.npz")
    W, H, G = int(d["W"]), int(d["H"]), int(d["G"])
    for prec, dt in (("f32", st.F32), ("f64", st.F64)):
        case = np.load(GOLD / f"stattile_boxcox_{prec}_mm5.npz")
        b = st.StatBuffers(W, H, REF_TR, G, 5, dt)
        b.accumulate(dev(d["s1"]))
        b.accumulate(dev(d["s2"]), count=dev(d["c2"]))
        assert np.array_equal(host(b.n), case["n"].astype(np.int32))
        assert np.array_equal(host(b.stats)[0], case["stats"][0])
        assert np.array_equal(host(b.gmean), case["gmean"])
        # Box-Cox goes through CUDA's pow: within a few ulps of the reference
        t1 = host(b.stats)[1]
        tol = 1e-12 if prec == "f64" else 1e-4
        assert moment_err(t1[None], case["stats"][1][None], case["n"], 5, resolution=0.0 if prec == "f64" else 1e-3) <= tol


def test_accumulate_fast_f32_vs_f64_oracle(st):
    W, H, G = 96, 64, 7
    s1 = synth_samples(W, H, 128, G=G, seed=5)
    b = st.StatBuffers(W, H, BASE_TR, G, 3, st.F32)
    b.accumulate(dev(s1), mode=st.ACC_FAST)
    n, so, go = oracle.new_state(5, G, H, W)
    oracle.accumulate(s1, BASE_TR, 3, n, so, go)
    assert np.array_equal(host(b.n), n)
    assert moment_err(host(b.stats).astype(np.float64), so, n, 3, resolution=1e-3) <= F32_TOL


def test_accumulate_fast_1024spp(st):
    """The FP32 form's uncompensated online update at the largest sample count of
    the serving trace: moments within 1e-4 of their scale after 1024 samples."""
    W, H, G = 32, 24, 7
    s = synth_samples(W, H, 1024, G=G, seed=15)
    b = st.StatBuffers(W, H, BASE_TR, G, 3, st.F32)
    b.accumulate(dev(s), mode=st.ACC_FAST)
    n, so, go = oracle.new_state(5, G, H, W)
    oracle.accumulate(s, BASE_TR, 3, n, so, go)
    assert np.array_equal(host(b.n), n)
    assert moment_err(host(b.stats).astype(np.float64), so, n, 3, resolution=1e-3) <= F32_TOL
    assert np.max(np.abs(host(b.gmean).astype(np.float64) - go)) <= 1e-5


@pytest.mark.parametrize("W,H", [(96, 40), (37, 23)])
def test_accumulate_fast_with_counts(st, W, H):
    """FP32 form with uneven per-pixel counts over two rounds (the TMA-fed path
    when W*H is a multiple of 4, the plain path otherwise)."""
    G = 7
    s1 = synth_samples(W, H, 40, G=G, seed=11)
    s2 = synth_samples(W, H, 33, G=G, seed=12)
    c1 = np.random.default_rng(13).integers(0, 41, size=(H, W)).astype(np.int32)
    c2 = np.random.default_rng(14).integers(0, 34, size=(H, W)).astype(np.int32)
    for tr, mm in ((BASE_TR, 3), (REF_TR, 5)):
        b = st.StatBuffers(W, H, tr, G, mm, st.F32)
        b.accumulate(dev(s1), count=dev(c1), mode=st.ACC_FAST)
        b.accumulate(dev(s2), count=dev(c2), mode=st.ACC_FAST)
        st.load().stater_synchronize(None)
        n, so, go = oracle.new_state(len(tr), G, H, W)
        oracle.accumulate(s1, tr, mm, n, so, go, count=c1)
        oracle.accumulate(s2, tr, mm, n, so, go, count=c2)
        assert np.array_equal(host(b.n), n)
        valid = n >= 2
        gs = host(b.stats).astype(np.float64)
        err = moment_err(gs[..., valid][..., None], so[..., valid][..., None], n[valid][:, None], mm,
                         resolution=1e-3)
        assert err <= F32_TOL, err
        assert np.max(np.abs(host(b.gmean).astype(np.float64) - go)) <= 1e-5


def test_rounds_equal_single_pass(st):
    """Round persistence: two calls equal one call over the concatenated samples."""
    W, H, G = 40, 24, 7
    s = synth_samples(W, H, 64, G=G, seed=7)
    a = st.StatBuffers(W, H, BASE_TR, G, 3, st.F64)
    a.accumulate(dev(s[:20]))
    a.accumulate(dev(s[20:]))
    b = st.StatBuffers(W, H, BASE_TR, G, 3, st.F64)
    b.accumulate(dev(s))
    assert torch.equal(a.stats, b.stats) and torch.equal(a.n, b.n)


def test_merge_tiles_matches_reference_records(st):
    d = np.load(GOLD / "stattile_inputs.npz")
    W, H = int(d["W"]), int(d["H"])
    case = np.load(GOLD / "stattile_boxcox_f32_mm5.npz")
    n = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    stats = torch.zeros(2, 7, 3, H, W, dtype=torch.float32, device="cuda")
    st.merge_tiles(W, H, dev(d["bounds"]), dev(case["records"]), 2, n, stats)
    assert np.array_equal(host(n), case["n"].astype(np.int32))
    assert np.array_equal(host(stats), case["stats"])


def test_merge_plain_tiles_sets_mean_to_m4(st):
    """A plain tile (n_sets = 1, Estimator::MergeTile, estimator.cpp:268-279)
    sets n and t0's mean, M2, M3 and M4, the values a transform tile writes to
    its set 0, and leaves the c2X, c2Y and m1 planes as they were."""
    d = np.load(GOLD / "stattile_inputs.npz")
    W, H = int(d["W"]), int(d["H"])
    case = np.load(GOLD / "stattile_boxcox_f32_mm5.npz")
    n = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    stats = torch.full((1, 7, 3, H, W), 7.25, dtype=torch.float32, device="cuda")
    st.merge_tiles(W, H, dev(d["bounds"]), dev(case["records"]), 1, n, stats)
    got = host(stats)
    assert np.array_equal(host(n), case["n"].astype(np.int32))
    assert np.array_equal(got[0, :4], case["stats"][0, :4])
    assert (got[0, 4:] == np.float32(7.25)).all()


def test_merge_moments_matches_oracle(st):
    W, H, G = 33, 21, 0
    a = synth_samples(W, H, 30, G=G, seed=8)
    bb = synth_samples(W, H, 50, G=G, seed=9)
    A = st.StatBuffers(W, H, BASE_TR, G, 5, st.F64)
    B = st.StatBuffers(W, H, BASE_TR, G, 5, st.F64)
    A.accumulate(dev(a))
    B.accumulate(dev(bb))
    nA, sA, gA = oracle.new_state(5, G, H, W)
    oracle.accumulate(a, BASE_TR, 5, nA, sA, gA)
    nB, sB, gB = oracle.new_state(5, G, H, W)
    oracle.accumulate(bb, BASE_TR, 5, nB, sB, gB)
    st.merge_moments(A, B)
    oracle.merge_moments(nA, sA, nB, sB, 5)
    assert np.array_equal(host(A.n), nA)
    assert moment_err(host(A.stats), sA, nA, 5) <= F64_MOMENT_TOL


def test_mean_var_bitwise(st):
    rng = np.random.default_rng(10)
    H, W = 30, 50
    n = rng.integers(2, 300, size=(H, W)).astype(np.int32)
    m2 = (rng.random((3, H, W)) * 10).astype(np.float32)
    out = torch.zeros(3, H, W, dtype=torch.float32, device="cuda")
    st.calc_mean_var(W, H, dev(n), dev(m2), out)
    assert np.array_equal(host(out), oracle.calc_mean_var_f32(n, m2))


def test_generator_is_deterministic_and_counter_based(st):
    a = st.generate_samples(64, 32, 8, seed=42)
    b = st.generate_samples(64, 32, 8, seed=42)
    assert torch.equal(a, b)
    first = torch.full((32, 64), 5, dtype=torch.int32, device="cuda")
    c = st.generate_samples(64, 32, 3, seed=42, first_index=first)
    assert torch.equal(c, a[5:8])
    x = host(a)
    assert np.all(x[:, 3:5] >= 0) and np.all(x[:, 3:5] < 1) and np.all(x[:, 0:3] > 0)


# ---------------------------------------------------------------------------
# stage 2
# ---------------------------------------------------------------------------
GSPEC = [(0, 3, 0.02), (3, 3, 0.1)]


def _oracle_pipeline(s, tr, mm, R, alpha, mt_mode=2, use_levc=False, sd=10.0, gspec=GSPEC):
    K = len(tr)
    S, nch, H, W = s.shape
    G = nch - 5
    n, so, go = oracle.new_state(K, G, H, W)
    oracle.accumulate(s, tr, mm, n, so, go)
    ds = float(np.float32(-0.5 / (sd * sd)))
    z = float(np.float32(2.80703))
    v = oracle.denoise_vars(n, so, go, mm, R, ds, z, gspec)
    f = oracle.denoise_film(n, so, v["varD"], v["varCD"], v["jb"], go, so[0, 0], R, ds, float(np.float32(alpha)),
                            gspec, mt_mode=mt_mode, use_levc=use_levc, want_bits=True)
    return n, so, go, v, f


def _gpu_pipeline(st, s, tr, mm, R, alpha, precision, mode, mt_mode=2, use_levc=False, sd=10.0):
    S, nch, H, W = s.shape
    b = st.StatBuffers(W, H, tr, nch - 5, mm, precision)
    b.accumulate(dev(s), mode=mode)
    specs = [st.GBufferSpec(a, c, sg) for a, c, sg in GSPEC]
    b.denoise_vars(radius=R, filter_sd=sd, gbuffers=specs)
    bits = torch.zeros(H * W, len(tr), st.bits_words(R), dtype=torch.int32, device="cuda")
    b.denoise_film(radius=R, filter_sd=sd, alpha=alpha, gbuffers=specs, mt_mode=mt_mode, use_levc=use_levc,
                   accept_bits=bits)
    return b, host(bits).view(np.uint32)


def _flip_fraction(bits_a, bits_b, R):
    D = 2 * R + 1
    diff = np.bitwise_xor(bits_a, bits_b)
    nflip = int(np.unpackbits(diff.view(np.uint8)).sum())
    total = bits_a.shape[0] * bits_a.shape[1] * D * D
    return nflip / total


@pytest.mark.parametrize("tr,mm,R,mt_mode,use_levc", [
    (BASE_TR, 3, 7, 2, False),
    (REF_TR, 5, 5, 2, True),
    (BASE_TR, 4, 4, 3, False),
])
def test_denoise_f64_matches_oracle(st, tr, mm, R, mt_mode, use_levc):
    W, H = 48, 40
    s = synth_samples(W, H, 64, G=7, seed=31, region=6)
    n, so, go, v, f = _oracle_pipeline(s, tr, mm, R, 0.01, mt_mode, use_levc)
    b, bits = _gpu_pipeline(st, s, tr, mm, R, 0.01, st.F64, st.ACC_EXACT, mt_mode, use_levc)
    assert np.allclose(host(b.jb), v["jb"], rtol=1e-10, atol=1e-300)
    assert np.allclose(host(b.lnS2), v["lnS2"], rtol=1e-12, atol=1e-12)
    assert np.allclose(host(b.se2), v["se2"], rtol=1e-12)
    assert np.allclose(host(b.varD), v["varD"], rtol=1e-10)
    assert np.allclose(host(b.varCD), v["varCD"], rtol=1e-10)
    assert np.allclose(host(b.discr), f["discr"], rtol=1e-10)
    assert _flip_fraction(bits, f["bits"], R) <= 1e-6
    rel = np.abs(host(b.filmD) - f["filmD"]) / np.maximum(np.abs(f["filmD"]), 1e-12)
    assert rel.max() <= F64_PIXEL_TOL


@pytest.mark.parametrize("tr,mm,R,mt_mode", [(BASE_TR, 3, 10, 2), (REF_TR, 5, 7, 2), (BASE_TR, 3, 7, 3)])
def test_denoise_f32_vs_f64_oracle(st, tr, mm, R, mt_mode):
    W, H = 80, 64
    s = synth_samples(W, H, 96, G=7, seed=41, region=8)
    n, so, go, v, f = _oracle_pipeline(s, tr, mm, R, 0.01, mt_mode)
    b, bits = _gpu_pipeline(st, s, tr, mm, R, 0.01, st.F32, st.ACC_FAST, mt_mode)
    flips = _flip_fraction(bits, f["bits"], R)
    assert flips <= FLIP_TOL, flips
    near = var_test_near_boundary(v["lnS2"], v["se2"], n, R, np.float32(2.80703), rel_margin=1e-4)
    vmax, _, _ = split_rel_error(host(b.varD), v["varD"], near, floor=1e-30)
    assert vmax <= F32_TOL, vmax
    fmax, _, ffrac = split_rel_error(host(b.filmD), f["filmD"], decision_flips(bits, f["bits"]))
    assert fmax <= F32_TOL and ffrac <= 0.05, (fmax, ffrac)


def test_denoise_max_radius_and_ragged_image(st):
    """R = 20 (the reference default) on an image smaller than the window."""
    W, H = 19, 13
    s = synth_samples(W, H, 32, G=7, seed=51, region=5)
    n, so, go, v, f = _oracle_pipeline(s, BASE_TR, 3, 20, 0.01)
    for prec, mode, tol in ((st.F64, st.ACC_EXACT, 1e-10), (st.F32, st.ACC_FAST, F32_TOL)):
        b, bits = _gpu_pipeline(st, s, BASE_TR, 3, 20, 0.01, prec, mode)
        fmax, _, _ = split_rel_error(host(b.filmD), f["filmD"], decision_flips(bits, f["bits"]))
        assert fmax <= tol, fmax
        assert _flip_fraction(bits, f["bits"], 20) <= FLIP_TOL


def test_target_spp_bitwise(st):
    rng = np.random.default_rng(61)
    H, W = 70, 90
    n = rng.integers(16, 200, size=(H, W)).astype(np.int32)
    n[3, 4] = 1
    varD = rng.random((3, H, W)) ** 3
    mean = rng.random((3, H, W)) + 0.05
    b = st.StatBuffers(W, H, ["identity"], 0, 3, st.F64)
    b.n.copy_(dev(n))
    b.varD[0].copy_(dev(varD))
    b.stats[0, 0].copy_(dev(mean))
    out = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    b.calc_target_spp(64, out, relative=True)
    assert np.array_equal(host(out), oracle.calc_target_spp(n, varD, mean, 64))
    b.calc_target_spp(64, out, relative=False)
    assert np.array_equal(host(out), oracle.calc_target_spp(n, varD, None, 64))


# ---------------------------------------------------------------------------
# stage 3
# ---------------------------------------------------------------------------
def test_lev_matches_oracle(st):
    W, H, G = 40, 30, 7
    s = host(st.generate_samples(W, H, 96, n_features=G, seed=71, lev_r2=0.6))
    stt = np.zeros((oracle.lev_nstate(G), H, W))
    oracle.lev_accumulate(s[:50], stt)
    oracle.lev_accumulate(s[50:], stt)
    ref = oracle.lev_solve(stt, G, H, W, lam=1e-6)
    for prec, tol in ((st.F64, 1e-9), (st.F32, F32_TOL)):
        lev = st.LevState(W, H, G, prec)
        lev.accumulate(dev(s[:50]))
        lev.accumulate(dev(s[50:]))
        lev.solve(1e-6)
        m2c = host(lev.m2C).astype(np.float64)
        assert np.max(np.abs(m2c - ref["m2C"]) / np.maximum(ref["m2C"], 1e-12)) <= tol
        r2 = host(lev.r2).astype(np.float64)
        assert np.max(np.abs(r2 - ref["r2"])) <= tol
    assert 0.4 < float(np.median(ref["r2"])) < 0.8


@pytest.mark.parametrize("W,H,tr,mm,R,mt_mode", [
    (160, 96, BASE_TR, 3, 10, 2),
    (97, 61, BASE_TR[:3], 5, 7, 3),
    (64, 48, BASE_TR[:1], 4, 20, 2),
])
def test_fp32_film_filter_forms_agree(st, W, H, tr, mm, R, mt_mode):
    """The row-ring film filter (all transforms per neighbour) and the
    per-transform filter that also writes the decision bits give the same filmD."""
    s = synth_samples(W, H, 48, G=7, seed=21, region=2)
    b = st.StatBuffers(W, H, tr, 7, mm, st.F32)
    b.accumulate(dev(s), mode=st.ACC_FAST)
    specs = [st.GBufferSpec(a, c, sg) for a, c, sg in GSPEC]
    b.denoise_vars(radius=R, gbuffers=specs)
    b.denoise_film(radius=R, gbuffers=specs, mt_mode=mt_mode)
    ring = b.filmD.clone()
    bits = torch.zeros(H * W, len(tr), st.bits_words(R), dtype=torch.int32, device="cuda")
    b.denoise_film(radius=R, gbuffers=specs, mt_mode=mt_mode, accept_bits=bits)
    torch.cuda.synchronize()
    assert torch.equal(ring, b.filmD)


@pytest.mark.parametrize("W,H", [(64, 40), (100, 36)])
def test_lev_tma_equals_plain_kernel(st, W, H):
    """The TMA-fed LEV accumulation (two pixels per lane in packed FP32) and the
    plain one-thread-per-pixel kernel (taken when the sample planes are not
    16-byte aligned) keep the same state bit for bit, with uneven per-pixel
    counts over two calls."""
    G = 7
    s = st.generate_samples(W, H, 37, n_features=G, seed=19, lev_r2=0.6)
    cnt = torch.from_numpy(np.random.default_rng(3).integers(0, 38, size=(H, W)).astype(np.int32)).cuda()
    # the same planes one float off 16-byte alignment: the plain kernel
    buf = torch.empty(s.numel() + 1, dtype=torch.float32, device="cuda")
    mis = buf[1:].view(s.shape)
    mis.copy_(s)
    a = st.LevState(W, H, G, st.F32)
    b = st.LevState(W, H, G, st.F32)
    for _ in range(2):
        a.accumulate(s, count=cnt)
        b.accumulate(mis, count=cnt)
    torch.cuda.synchronize()
    assert torch.equal(a.state, b.state)
