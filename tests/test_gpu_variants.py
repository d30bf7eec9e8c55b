"""The reference's build variants as runtime switches, against the oracle.

scripts/alternate-builds/*.sh of the reference select, at compile time:
CASCADE_MODE (0 in "M": the Welch discriminator from each pixel's own sample
variance instead of the denoised one), USE_LEVC (0 in "M" and "MC": varD
instead of the LEV-corrected varCD), AS_MODE (0 in "ASN": the adaptive-sampling
error from the sample variance instead of varD) and FILM_MULTI_TRANSFORM_MODE
(3 in "MT-JB"). Here they are the discr_source, use_levc, as_source and mt_mode
arguments. Each variant: the plain FP64 form equals the oracle (1e-10, same
Welch decisions), the FP32 form is within 1e-4 at every pixel without a flipped
decision, the two FP32 film-filter forms agree bit for bit, and the target
sample counts of ASN equal the oracle's.
"""
import numpy as np
import pytest

import oracle
from helpers import decision_flips, split_rel_error, synth_samples

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TR = ["identity", "log1p", "sqrt", "cbrt", "asinh"]
GSPEC = [(0, 3, 0.02), (3, 3, 0.1)]
Z = float(np.float32(2.80703))
DS = float(np.float32(-0.5 / 100.0))

VARIANTS = {  # name: (cascade, use_levc, mt_mode)
    "M": (False, False, 2),
    "MC": (True, False, 2),
    "MCL": (True, True, 2),
    "ML": (False, True, 2),
    "M-JB": (False, False, 3),
}


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


@pytest.fixture(scope="module")
def case():
    W, H, R = 64, 48, 6
    s = synth_samples(W, H, 64, G=7, seed=91, region=6)
    n, so, go = oracle.new_state(len(TR), 7, H, W)
    oracle.accumulate(s, TR, 5, n, so, go)
    v = oracle.denoise_vars(n, so, go, 5, R, DS, Z, GSPEC)
    return dict(W=W, H=H, R=R, s=s, n=n, so=so, go=go, v=v)


def _gpu(st, c, precision, mode, cascade, use_levc, mt_mode, bits=True, ring_too=False):
    W, H, R = c["W"], c["H"], c["R"]
    b = st.StatBuffers(W, H, TR, 7, 5, precision)
    b.accumulate(dev(c["s"]), mode=mode)
    specs = [st.GBufferSpec(a, ch, sg) for a, ch, sg in GSPEC]
    b.denoise_vars(radius=R, gbuffers=specs)
    ring = None
    if ring_too:
        b.denoise_film(radius=R, gbuffers=specs, mt_mode=mt_mode, use_levc=use_levc, cascade=cascade)
        ring = b.filmD.clone()
    ab = torch.zeros(H * W, len(TR), st.bits_words(R), dtype=torch.int32, device="cuda")
    b.denoise_film(radius=R, gbuffers=specs, mt_mode=mt_mode, use_levc=use_levc, cascade=cascade, accept_bits=ab)
    return b, host(ab).view(np.uint32), ring


@pytest.mark.parametrize("name", list(VARIANTS))
def test_variant_matches_oracle(st, case, name):
    cascade, use_levc, mt_mode = VARIANTS[name]
    c = case
    v = c["v"]
    f = oracle.denoise_film(c["n"], c["so"], v["varD"], v["varCD"], v["jb"], c["go"], c["so"][0, 0], c["R"], DS,
                            float(np.float32(0.01)), GSPEC, mt_mode=mt_mode, use_levc=use_levc, want_bits=True,
                            discr_source=0 if cascade else 1, m2C=v["m2C"])
    b, bits, _ = _gpu(st, c, st.F64, st.ACC_EXACT, cascade, use_levc, mt_mode)
    assert np.allclose(host(b.discr), f["discr"], rtol=1e-10, atol=0)
    assert np.array_equal(bits, f["bits"])
    rel = np.abs(host(b.filmD) - f["filmD"]) / np.maximum(np.abs(f["filmD"]), 1e-12)
    assert rel.max() <= 1e-10
    b32, bits32, ring = _gpu(st, c, st.F32, st.ACC_FAST, cascade, use_levc, mt_mode, ring_too=True)
    assert torch.equal(ring, b32.filmD)
    nflip = int(np.unpackbits(np.bitwise_xor(bits32, f["bits"]).view(np.uint8)).sum())
    assert nflip <= 1e-3 * bits32.shape[0] * len(TR) * (2 * c["R"] + 1) ** 2
    fmax, _, _ = split_rel_error(host(b32.filmD), f["filmD"], decision_flips(bits32, f["bits"]))
    assert fmax <= 1e-4, fmax


def test_cascade_changes_the_discriminator(st, case):
    """M and MC differ (the switch is live), and M's discriminator is s^2 / n."""
    bm, _, _ = _gpu(st, case, st.F64, st.ACC_EXACT, False, False, 2, bits=False)
    bc, _, _ = _gpu(st, case, st.F64, st.ACC_EXACT, True, False, 2, bits=False)
    n = case["n"].astype(np.float64)
    s2 = case["so"][:, 1] / (n - 1.0)
    assert np.allclose(host(bm.discr), s2 / n, rtol=1e-12)
    assert not np.allclose(host(bm.discr), host(bc.discr))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_asn_target_spp_matches_oracle(st, precision):
    rng = np.random.default_rng(93)
    H, W = 70, 90
    n = rng.integers(16, 200, size=(H, W)).astype(np.int32)
    n[3, 4] = 1
    m2 = rng.random((3, H, W)) * 3
    mean = rng.random((3, H, W)) + 0.05
    prec = st.F64 if precision == "f64" else st.F32
    dt = np.float64 if precision == "f64" else np.float32
    m2 = m2.astype(dt)
    mean = mean.astype(dt)
    b = st.StatBuffers(W, H, ["identity"], 0, 3, prec)
    b.n.copy_(dev(n))
    b.stats[0, 1].copy_(dev(m2))
    b.stats[0, 0].copy_(dev(mean))
    out = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    for relative in (True, False):
        b.calc_target_spp(64, out, relative=relative, as_source=st.AS_SAMPLE)
        ref = oracle.calc_target_spp(n, None, mean.astype(np.float64) if relative else None, 64,
                                     m2=m2.astype(np.float64), as_source=1)
        assert np.array_equal(host(out), ref)
