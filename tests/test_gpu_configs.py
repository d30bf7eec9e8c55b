"""Parity at the sizes of the stated workloads, against the FP64 oracle.

* The plain method, exactly as configured: 256x256, 64 spp, per-pixel
  lognormal(-1, 1) means x lognormal(0, 0.5) noise with 0.1% fireflies x1e3,
  the identity transform only, moments M1-M3, variance denoise and a single-
  transform Welch filter with a 15x15 window (R = 7), alpha = 0.01, in FP64.
  The film buffer (Film::UpdateImage of the same samples) is the filter's mean,
  as the reference passes it. The untransformed moments, the counts and the
  feature means equal the oracle bit for bit (the identity involves no libm
  call); denoised pixels agree within 1e-5. The FP32 form of the same job is
  checked as every FP32 form is (1e-4 at pixels without a flipped decision).
* The plain FP64 form of the five-transform workload at 256x256 (same
  transforms, 21x21 window, M1-M3), which pins the FP64 form that the 1080p
  test compares the FP32 form with.
* LEV at 256x256 and 512 spp (7 features + intercept, ridge 1e-6), accumulated
  in 64-sample chunks, against the oracle's FP64 accumulation and solve.
"""
import numpy as np
import pytest

import oracle
from helpers import decision_flips, split_rel_error

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TR5 = ["identity", "log1p", "sqrt", "cbrt", "asinh"]
Z = float(np.float32(2.80703))
ALPHA = float(np.float32(0.01))


@pytest.fixture(scope="module")
def st():
    import stater_gb300 as S
    S.setup()
    return S


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def _specs(G):
    return [(0, 3, 0.02), (3, 3, 0.1), (6, 1, 0.1)] if G >= 7 else []


def _oracle_job(s, tr, R, G, want_bits=True):
    S_, nch, H, W = s.shape
    n, so, go = oracle.new_state(len(tr), G, H, W)
    oracle.accumulate(s, tr, 3, n, so, go)
    film = oracle.film_update_image(oracle.film_add_samples(s)).astype(np.float64)
    ds = float(np.float32(-0.5 / 100.0))
    gs = _specs(G)
    v = oracle.denoise_vars(n, so, go, 3, R, ds, Z, gs)
    f = oracle.denoise_film(n, so, v["varD"], v["varCD"], v["jb"], go, film, R, ds, ALPHA, gs,
                            want_bits=want_bits)
    return n, so, go, v, f


def _gpu_job(st, smp, tr, R, G, precision, mode):
    S_, nch, H, W = smp.shape
    b = st.StatBuffers(W, H, tr, G, 3, precision)
    film = st.Film(W, H, n_features=G)
    b.accumulate(smp, mode=mode, film=film)
    rgb = film.update_image()
    if precision == st.F64:
        rgb = rgb.double()
    specs = [st.GBufferSpec(a, c, sg) for a, c, sg in _specs(G)]
    b.denoise_vars(radius=R, gbuffers=specs)
    bits = torch.zeros(H * W, len(tr), st.bits_words(R), dtype=torch.int32, device="cuda")
    b.denoise_film(radius=R, gbuffers=specs, film=rgb, alpha=0.01, accept_bits=bits)
    return b, host(bits).view(np.uint32)


@pytest.mark.parametrize("G", [7, 0])
def test_plain_method_configuration(st, G):
    W, H, SPP, R = 256, 256, 64, 7
    smp = st.generate_samples(W, H, SPP, n_features=G, seed=2024, region=1)
    s = host(smp)
    n, so, go, v, f = _oracle_job(s, ["identity"], R, G)
    b, bits = _gpu_job(st, smp, ["identity"], R, G, st.F64, st.ACC_EXACT)
    assert np.array_equal(host(b.n), n) and int(n.min()) == SPP
    assert np.array_equal(host(b.stats)[0, :3], so[0, :3])
    if G:
        assert np.array_equal(host(b.gmean), go)
    assert np.allclose(host(b.varD), v["varD"], rtol=1e-10, atol=0)
    assert np.allclose(host(b.discr), f["discr"], rtol=1e-10, atol=0)
    assert np.array_equal(bits, f["bits"])
    rel = np.abs(host(b.filmD) - f["filmD"]) / np.maximum(np.abs(f["filmD"]), 1e-12)
    assert rel.max() <= 1e-5, rel.max()
    # the FP32 form of the same job
    b32, bits32 = _gpu_job(st, smp, ["identity"], R, G, st.F32, st.ACC_FAST)
    flips = decision_flips(bits32, f["bits"])
    fmax, _, frac = split_rel_error(host(b32.filmD), f["filmD"], flips)
    assert fmax <= 1e-4 and frac <= 0.01, (fmax, frac)


def test_plain_fp64_five_transforms_256(st):
    W, H, SPP, R, G = 256, 256, 64, 10, 7
    smp = st.generate_samples(W, H, SPP, n_features=G, seed=2025)
    s = host(smp)
    n, so, go, v, f = _oracle_job(s, TR5, R, G)
    b, bits = _gpu_job(st, smp, TR5, R, G, st.F64, st.ACC_EXACT)
    assert np.array_equal(host(b.n), n)
    gs = host(b.stats)
    assert np.array_equal(gs[0, :3], so[0, :3])
    # transformed sets: CUDA's libm against glibc's, relative to each moment's scale
    nn = np.maximum(n, 1)[None, None]
    sd = np.sqrt(np.abs(so[:, 1]) / nn)
    for q, power in ((0, 1), (1, 2), (2, 3)):
        floor = (np.abs(so[:, 0]) + sd) if q == 0 else nn * sd ** power
        assert np.max(np.abs(gs[:, q] - so[:, q]) / (floor + 1e-300)) <= 1e-12
    assert np.allclose(host(b.varD), v["varD"], rtol=1e-10, atol=0)
    flips = int(np.unpackbits(np.bitwise_xor(bits, f["bits"]).view(np.uint8)).sum())
    assert flips <= 1e-6 * H * W * len(TR5) * (2 * R + 1) ** 2
    rel = np.abs(host(b.filmD) - f["filmD"]) / np.maximum(np.abs(f["filmD"]), 1e-12)
    assert rel.max() <= 1e-5, rel.max()


def test_lev_256_512spp(st):
    W, H, SPP, G, CH = 256, 256, 512, 7, 64
    nst = oracle.lev_nstate(G)
    ref_state = np.zeros((nst, H, W))
    levs = {p: st.LevState(W, H, G, p) for p in (st.F64, st.F32)}
    first = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    for c0 in range(0, SPP, CH):
        first.fill_(c0)
        smp = st.generate_samples(W, H, CH, n_features=G, seed=71, lev_r2=0.6, first_index=first)
        for lev in levs.values():
            lev.accumulate(smp)
        oracle.lev_accumulate(host(smp), ref_state)
    ref = oracle.lev_solve(ref_state, G, H, W, lam=1e-6)
    assert 0.45 < float(np.median(ref["r2"])) < 0.75
    for prec, tol in ((st.F64, 1e-9), (st.F32, 1e-4)):
        lev = levs[prec]
        lev.solve(1e-6)
        m2c = host(lev.m2C).astype(np.float64)
        assert np.max(np.abs(m2c - ref["m2C"]) / np.maximum(ref["m2C"], 1e-12)) <= tol
        assert np.max(np.abs(host(lev.r2).astype(np.float64) - ref["r2"])) <= tol
        if prec == st.F64:
            beta = host(lev.beta)
            scale = np.abs(ref["beta"]).max(axis=1, keepdims=True) + 1e-12
            assert np.max(np.abs(beta - ref["beta"]) / scale) <= 1e-9
