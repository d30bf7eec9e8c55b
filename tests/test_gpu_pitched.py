"""denoiseVars / denoiseFilm over the reference's own buffer layout.

The reference's Estimator keeps pitched GpuMat images: an RGB statistics buffer
is one image of interleaved float3 (CV_32FC3, or double3 in a
PBRT_FLOAT_AS_DOUBLE build) whose rows are padded to a pitch, and n, jb and
one-channel G-buffers are one-channel images (estimator.cpp:26-81). The
pitched entry points take such buffers unchanged; their outputs must equal the
planar entry points' bit for bit, and the row padding must stay untouched.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import synth_samples

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TR5 = ["identity", "log1p", "sqrt", "cbrt", "asinh"]
REF_TR = ["identity", ("boxcox", 0.25)]
GSPEC = [(0, 3, 0.02), (3, 3, 0.1), (6, 1, 0.1)]


@pytest.fixture(scope="module")
def st():
    import stater_gb300 as S
    S.setup()
    return S


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class Pitched:
    """Pitched images with poisoned padding: rows of `pitch` elements, the first
    C*W of which hold the pixels (channels interleaved)."""

    def __init__(self, H, W, dtype, pad):
        self.H, self.W, self.dtype = H, W, dtype
        self.rgb_p = 3 * W + pad
        self.one_p = W + pad + 1
        self.n_p = W + pad + 3
        self.poison = float("nan") if dtype.is_floating_point else -12345

    def rgb(self, planar=None):
        t = torch.full((self.H, self.rgb_p), self.poison, dtype=self.dtype, device="cuda")
        if planar is not None:
            t[:, :3 * self.W] = planar.permute(1, 2, 0).reshape(self.H, 3 * self.W).to(self.dtype)
        return t

    def one(self, planar=None, dtype=None, pitch=None):
        dt = dtype or self.dtype
        t = torch.full((self.H, pitch or self.one_p), -12345 if not dt.is_floating_point else float("nan"), dtype=dt,
                       device="cuda")
        if planar is not None:
            t[:, :self.W] = planar.to(dt)
        return t

    def rgb_planar(self, t):
        return t[:, :3 * self.W].reshape(self.H, self.W, 3).permute(2, 0, 1)

    def layout(self, S):
        L = S._lib.PitchedLayout()
        es = torch.empty(0, dtype=self.dtype).element_size()
        L.rgb_step, L.scalar_step, L.n_step = self.rgb_p * es, self.one_p * es, self.n_p * 4
        return L


def _padding_intact(P, t, width):
    pad = t[:, width:]
    if pad.numel() == 0:
        return True
    if pad.dtype.is_floating_point:
        return bool(torch.isnan(pad).all())
    return bool((pad == -12345).all())


@pytest.mark.parametrize("prec,tr,mm,mt_mode,use_levc,cascade", [
    ("f32", TR5, 3, 2, False, True),
    ("f32", REF_TR, 5, 2, True, True),
    ("f32", TR5, 4, 3, False, False),
    ("f64", TR5, 3, 2, False, True),
    ("f64", REF_TR, 5, 3, True, False),
])
def test_pitched_equals_planar(st, prec, tr, mm, mt_mode, use_levc, cascade):
    L_ = st._lib
    W, H, R, G = 83, 47, 6, 7
    precision = st.F32 if prec == "f32" else st.F64
    mode = st.ACC_FAST if prec == "f32" else st.ACC_EXACT
    dtype = torch.float32 if prec == "f32" else torch.float64
    s = torch.from_numpy(synth_samples(W, H, 48, G=G, seed=17, region=5)).cuda()
    b = st.StatBuffers(W, H, tr, G, mm, precision)
    b.accumulate(s, mode=mode)
    specs = [st.GBufferSpec(a, c, sg) for a, c, sg in GSPEC]
    b.denoise_vars(radius=R, gbuffers=specs)
    b.denoise_film(radius=R, gbuffers=specs, mt_mode=mt_mode, use_levc=use_levc, cascade=cascade)
    torch.cuda.synchronize()
    K = b.K
    P = Pitched(H, W, dtype, pad=13)
    # inputs in the reference's layout
    n_p = P.one(b.n, dtype=torch.int32, pitch=P.n_p)
    mom = {q: [P.rgb(b.stats[k, q]) for k in range(K)] for q in range(1, 6)}
    gb = [P.rgb(b.gmean[0:3]), P.rgb(b.gmean[3:6]), P.one(b.gmean[6])]
    # outputs
    jb = [P.one() for _ in range(K)]
    outs = {name: [P.rgb() for _ in range(K)] for name in ("lnS2", "se2", "m2C", "varD", "varCD", "discr")}
    filmD = P.rgb()
    film = P.rgb(b.stats[0, 0])

    def gbufs():
        g = L_.GBuffers()
        g.count = 3
        for i, ((first, ch, sg), t) in enumerate(zip(GSPEC, gb)):
            g.planes[i] = t.data_ptr()
            g.channels[i] = ch
            g.dr_factor[i] = -0.5 / (sg * sg)
        return g

    va = L_.DenoiseVarsArgs()
    va.n_buffers, va.width, va.height, va.filter_radius = K, W, H, R
    va.ds_factor, va.var_z, va.max_moment, va.precision = -0.5 / 100.0, 2.80703, mm, precision
    va.n = n_p.data_ptr()
    for k in range(K):
        va.m2[k], va.m3[k] = mom[1][k].data_ptr(), mom[2][k].data_ptr()
        va.m4[k], va.c2X[k], va.c2Y[k] = mom[3][k].data_ptr(), mom[4][k].data_ptr(), mom[5][k].data_ptr()
        va.jb[k] = jb[k].data_ptr()
        for name in ("lnS2", "se2", "m2C", "varD", "varCD"):
            getattr(va, name)[k] = outs[name][k].data_ptr()
    va.gbuffers = gbufs()
    layout = P.layout(st)
    assert L_.load().stater_denoise_vars_pitched(C.byref(va), C.byref(layout), None) == 0

    fa = L_.DenoiseFilmArgs()
    fa.n_buffers, fa.width, fa.height, fa.filter_radius = K, W, H, R
    fa.ds_factor, fa.alpha, fa.mt_mode, fa.use_levc, fa.precision = -0.5 / 100.0, 0.01, mt_mode, int(use_levc), precision
    fa.n, fa.film, fa.filmD = n_p.data_ptr(), film.data_ptr(), filmD.data_ptr()
    means = [P.rgb(b.stats[k, 0]) for k in range(K)]
    for k in range(K):
        fa.mean[k] = means[k].data_ptr()
        fa.varD[k], fa.varCD[k] = outs["varD"][k].data_ptr(), outs["varCD"][k].data_ptr()
        fa.jb[k], fa.discr[k] = jb[k].data_ptr(), outs["discr"][k].data_ptr()
        fa.m2[k], fa.m2C[k] = mom[1][k].data_ptr(), outs["m2C"][k].data_ptr()
    fa.discr_source = 0 if cascade else 1
    fa.gbuffers = gbufs()
    tr_arr = (L_.Transform * L_.MAX_TRANSFORMS)()
    for k, (kind, lam) in enumerate(b.transforms):
        tr_arr[k].kind, tr_arr[k].lambda_ = kind, lam
    assert L_.load().stater_test_order(tr_arr, K, C.cast(fa.test_order, C.c_void_p)) == 0
    assert L_.load().stater_denoise_film_pitched(C.byref(fa), C.byref(layout), None) == 0
    torch.cuda.synchronize()

    for k in range(K):
        assert torch.equal(jb[k][:, :W], b.jb[k]), ("jb", k)
        assert _padding_intact(P, jb[k], W)
        for name in ("lnS2", "se2", "m2C", "varD", "varCD", "discr"):
            got = P.rgb_planar(outs[name][k])
            assert torch.equal(got, getattr(b, name)[k]), (name, k)
            assert _padding_intact(P, outs[name][k], 3 * W), name
    assert torch.equal(P.rgb_planar(filmD), b.filmD)
    assert _padding_intact(P, filmD, 3 * W)


def test_pitched_rejects_short_steps(st):
    L_ = st._lib
    va = L_.DenoiseVarsArgs()
    va.n_buffers, va.width, va.height, va.max_moment, va.precision = 1, 64, 8, 3, st.F32
    layout = L_.PitchedLayout()
    layout.rgb_step, layout.scalar_step, layout.n_step = 3 * 64 * 4 - 4, 64 * 4, 64 * 4
    assert L_.load().stater_denoise_vars_pitched(C.byref(va), C.byref(layout), None) == 1
    assert b"rgb_step" in L_.load().stater_last_error()


@pytest.mark.parametrize("as_source", [0, 1])
def test_pitched_target_spp_equals_planar(st, as_source):
    L_ = st._lib
    W, H = 91, 53
    rng = np.random.default_rng(5)
    n = torch.from_numpy(rng.integers(1, 200, size=(H, W)).astype(np.int32)).cuda()
    m2 = torch.from_numpy(rng.random((3, H, W)).astype(np.float32) * 3).cuda()
    varD = torch.from_numpy(rng.random((3, H, W)).astype(np.float32)).cuda()
    mean = torch.from_numpy(rng.random((3, H, W)).astype(np.float32) + 0.05).cuda()
    ref = torch.zeros(H, W, dtype=torch.int32, device="cuda")

    def args(nn, mm2, vd, mu, out):
        a = L_.TargetSppArgs()
        a.width, a.height, a.spp, a.precision = W, H, 64, st.F32
        a.n, a.m2, a.varD, a.mean = nn.data_ptr(), mm2.data_ptr(), vd.data_ptr(), mu.data_ptr()
        a.eps, a.tmin, a.tmax, a.as_source, a.targetspp = 1e-4, 16, 1024, as_source, out.data_ptr()
        return a

    a = args(n, m2, varD, mean, ref)
    assert L_.load().stater_calc_target_spp_ex(C.byref(a), None) == 0
    P = Pitched(H, W, torch.float32, pad=7)
    n_p = P.one(n, dtype=torch.int32, pitch=P.n_p)
    out_p = P.one(None, dtype=torch.int32, pitch=P.n_p)
    a = args(n_p, P.rgb(m2), P.rgb(varD), P.rgb(mean), out_p)
    layout = P.layout(st)
    assert L_.load().stater_calc_target_spp_pitched(C.byref(a), C.byref(layout), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(out_p[:, :W], ref)
    assert bool((out_p[:, W:] == -12345).all())
