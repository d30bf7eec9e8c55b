"""Edge cases of the GPU path against the oracle: the largest transform count
(per-transform filter kernels), the largest radius with LEV-corrected
variances (row-ring kernels with 4-row tiles), images narrower than the
window down to one pixel, pixels with no or a single sample, and the largest
number of feature channels."""
import numpy as np
import pytest

import oracle
from helpers import decision_flips, split_rel_error, synth_samples, var_test_near_boundary

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TR8 = ["identity", "log1p", "sqrt", "cbrt", "asinh", ("boxcox", 0.25), ("boxcox", 0.5), ("boxcox", 2.0)]
TR5 = TR8[:5]
GSPEC = [(0, 3, 0.02), (3, 3, 0.1)]


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


def _oracle(s, tr, mm, R, count=None, use_levc=False):
    S_, nch, H, W = s.shape
    n, so, go = oracle.new_state(len(tr), nch - 5, H, W)
    oracle.accumulate(s, tr, mm, n, so, go, count=count)
    ds = float(np.float32(-0.5 / 100.0))
    v = oracle.denoise_vars(n, so, go, mm, R, ds, float(np.float32(2.80703)), GSPEC)
    f = oracle.denoise_film(n, so, v["varD"], v["varCD"], v["jb"], go, so[0, 0], R, ds, float(np.float32(0.01)),
                            GSPEC, use_levc=use_levc, want_bits=True)
    return n, so, go, v, f


def _gpu(st, s, tr, mm, R, precision, mode, count=None, use_levc=False, bits=False):
    S_, nch, H, W = s.shape
    b = st.StatBuffers(W, H, tr, nch - 5, mm, precision)
    b.accumulate(dev(s), count=None if count is None else dev(count), mode=mode)
    specs = [st.GBufferSpec(a, c, sg) for a, c, sg in GSPEC]
    b.denoise_vars(radius=R, gbuffers=specs)
    ab = torch.zeros(H * W, len(tr), st.bits_words(R), dtype=torch.int32, device="cuda") if bits else None
    b.denoise_film(radius=R, gbuffers=specs, use_levc=use_levc, accept_bits=ab)
    if bits:
        b.bits = host(ab).view(np.uint32)
    return b


def _rel(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.mark.parametrize("tr,mm,R,use_levc", [(TR8, 3, 6, False), (TR5, 5, 20, True), (TR8[:6], 4, 9, False)])
def test_f32_transform_count_and_radius(st, tr, mm, R, use_levc):
    W, H = 72, 56
    s = synth_samples(W, H, 64, G=7, seed=81, region=6)
    n, so, go, v, f = _oracle(s, tr, mm, R, use_levc=use_levc)
    b = _gpu(st, s, tr, mm, R, st.F32, st.ACC_FAST, use_levc=use_levc, bits=True)
    near = var_test_near_boundary(v["lnS2"], v["se2"], n, R, np.float32(2.80703), rel_margin=1e-4)
    vmax, _, _ = split_rel_error(host(b.varD), v["varD"], near, floor=1e-30)
    assert vmax <= 1e-4, vmax
    if use_levc:
        vcmax, _, _ = split_rel_error(host(b.varCD), v["varCD"], near, floor=1e-30)
        assert vcmax <= 1e-4, vcmax
    fmax, _, frac = split_rel_error(host(b.filmD), f["filmD"], decision_flips(b.bits, f["bits"]))
    assert fmax <= 1e-4 and frac <= 0.05, (fmax, frac)


@pytest.mark.parametrize("W,H", [(1, 1), (1, 40), (40, 1), (3, 2)])
def test_images_narrower_than_the_window(st, W, H):
    s = synth_samples(W, H, 24, G=7, seed=82, region=1)
    n, so, go, v, f = _oracle(s, TR5, 3, 10)
    b = _gpu(st, s, TR5, 3, 10, st.F64, st.ACC_EXACT)
    assert np.allclose(host(b.filmD), f["filmD"], rtol=1e-10, atol=0)
    assert np.allclose(host(b.varD), v["varD"], rtol=1e-10, atol=1e-300)
    b32 = _gpu(st, s, TR5, 3, 10, st.F32, st.ACC_FAST, bits=True)
    fd = host(b32.filmD).astype(np.float64)
    assert np.all(np.isfinite(fd))
    fmax, _, _ = split_rel_error(fd, f["filmD"], decision_flips(b32.bits, f["bits"]))
    assert fmax <= 1e-4, fmax


def test_pixels_with_no_or_one_sample(st):
    W, H = 30, 20
    s = synth_samples(W, H, 16, G=7, seed=83, region=3)
    cnt = np.random.default_rng(84).integers(0, 17, size=(H, W)).astype(np.int32)
    cnt[::4, ::3] = 0
    cnt[1::5, ::2] = 1
    n, so, go, v, f = _oracle(s, TR5, 3, 5, count=cnt)
    b = _gpu(st, s, TR5, 3, 5, st.F64, st.ACC_EXACT, count=cnt)
    assert np.array_equal(host(b.n), n)
    assert np.allclose(host(b.filmD), f["filmD"], rtol=1e-10, atol=1e-300)
    assert np.allclose(host(b.varD), v["varD"], rtol=1e-10, atol=1e-300)
    b32 = _gpu(st, s, TR5, 3, 5, st.F32, st.ACC_FAST, count=cnt)
    fd = host(b32.filmD).astype(np.float64)
    assert np.all(np.isfinite(fd))
    few = n < 2
    # pixels without a usable variance keep their own film value and get no variance
    assert np.allclose(fd[:, few], f["filmD"][:, few], rtol=1e-6, atol=0)
    assert np.all(host(b32.varD)[:, :, few] == 0)


def test_sixteen_feature_channels(st):
    W, H, G = 44, 28, 16
    s = synth_samples(W, H, 40, G=G, seed=85, region=4)
    n, so, go = oracle.new_state(3, G, H, W)
    oracle.accumulate(s, TR5[:3], 3, n, so, go)
    for prec, mode, tol in ((st.F64, st.ACC_EXACT, 1e-12), (st.F32, st.ACC_FAST, 1e-5)):
        b = st.StatBuffers(W, H, TR5[:3], G, 3, prec)
        b.accumulate(dev(s), mode=mode)
        gm = host(b.gmean).astype(np.float64)
        assert np.max(_rel(gm, go, 1e-6)) <= tol


@pytest.mark.parametrize("W,H", [(64, 32), (37, 23)])  # TMA-fed and plain FP32 kernels
def test_fast_first_sample_is_exact(st, W, H):
    """FAST form, a pixel's first sample: the update runs with n = 1 and the
    hardware reciprocal of 1, and must leave every central moment exactly 0
    and the identity mean equal to the sample (no special case in the code)."""
    s = synth_samples(W, H, 1, G=7, seed=86, region=2)
    b = st.StatBuffers(W, H, TR5, 7, 5, st.F32)
    b.accumulate(dev(s), mode=st.ACC_FAST)
    stats = host(b.stats)  # [K][7][3][H][W]
    assert np.array_equal(stats[0, 0], s[0, 0:3])
    assert not np.any(stats[:, 1:])
    assert np.array_equal(host(b.n), np.ones((H, W), np.int32))
