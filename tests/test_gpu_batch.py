"""Batches: several images through one launch per denoise stage.

A batch takes per image the arguments of accumulate (with the film sums), the
film image, denoise_vars and denoise_film, and runs each denoise stage once for
all images of the same kernel form. Every image's outputs must equal its own
calls bit for bit, on the first run (eager, tile heights tuned) and on later
runs (replayed CUDA graph), with and without resetting the state per run. The
tile-height autotuner must not change any result.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TR = ["identity", "log1p", "sqrt", "cbrt", "asinh"]
REF = ["identity", ("boxcox", 0.25)]
SPECS = None

# (W, H, spp, transforms, max_moment, R, mt_mode, use_levc, cascade)
JOBS = [
    (64, 48, 24, TR[:1], 3, 6, 2, False, True),
    (100, 70, 32, TR[:3], 3, 10, 2, False, True),
    (256, 256, 16, TR, 3, 10, 2, False, True),
    (97, 61, 24, TR, 4, 10, 3, False, True),
    (130, 90, 20, REF, 5, 10, 2, True, True),
    (40, 30, 16, TR, 3, 6, 2, False, False),
    (256, 128, 16, TR, 3, 10, 2, False, True),
]
NAMES = ("n", "stats", "gmean", "jb", "lnS2", "se2", "m2C", "varD", "varCD", "discr", "filmD")


@pytest.fixture(scope="module")
def st():
    import stater_gb300 as S
    S.setup()
    return S


def _make(st, seed0=300):
    jobs = []
    for i, (W, H, spp, tr, mm, R, mt, levc, casc) in enumerate(JOBS):
        smp = st.generate_samples(W, H, spp, n_features=7, seed=seed0 + i, region=4)
        b = st.StatBuffers(W, H, tr, 7, mm, st.F32)
        film = st.Film(W, H, n_features=7)
        jobs.append(dict(buffers=b, film=film, samples=smp, radius=R, mt_mode=mt, use_levc=levc, cascade=casc,
                         gbuffers=st.GBUFFERS_ALBEDO_NORMAL))
    return jobs


def _alone(st, j, rounds=1):
    b, film = j["buffers"], j["film"]
    for _ in range(rounds):
        b.accumulate(j["samples"], mode=st.ACC_FAST, film=film)
    rgb = film.update_image()
    b.denoise_vars(radius=j["radius"], gbuffers=j["gbuffers"])
    b.denoise_film(radius=j["radius"], gbuffers=j["gbuffers"], mt_mode=j["mt_mode"], use_levc=j["use_levc"],
                   cascade=j["cascade"], film=rgb)


def _snapshot(j):
    b = j["buffers"]
    out = {k: getattr(b, k).clone() for k in NAMES}
    out["rgb"] = j["film"].rgb.clone()
    return out


@pytest.mark.parametrize("autotune", [1, 0])
def test_batch_equals_single_image_calls(st, autotune):
    lib = st.load()
    assert lib.stater_set_autotune(autotune) == 0
    try:
        ref_jobs = _make(st)
        for j in ref_jobs:
            _alone(st, j)
        torch.cuda.synchronize()
        ref = [_snapshot(j) for j in ref_jobs]
        jobs = _make(st)
        batch = st.Batch(jobs, reset=True)
        for run in range(3):  # eager + tuned, then graph replays
            batch.run()
            torch.cuda.synchronize()
            for i, j in enumerate(jobs):
                got = _snapshot(j)
                for k, v in got.items():
                    assert torch.equal(v, ref[i][k]), (run, i, k)
        batch.close()
    finally:
        assert lib.stater_set_autotune(1) == 0


def test_batch_without_reset_keeps_adding(st):
    ref_jobs = _make(st, seed0=400)
    for j in ref_jobs:
        _alone(st, j, rounds=2)
    torch.cuda.synchronize()
    ref = [_snapshot(j) for j in ref_jobs]
    jobs = _make(st, seed0=400)
    batch = st.Batch(jobs, reset=False)
    batch.run()
    batch.run()
    torch.cuda.synchronize()
    for i, j in enumerate(jobs):
        got = _snapshot(j)
        for k, v in got.items():
            assert torch.equal(v, ref[i][k]), (i, k)
    batch.close()


def test_single_image_tuning_is_recorded_and_harmless(st):
    lib = st.load()
    W, H, R = 256, 256, 10
    smp = st.generate_samples(W, H, 32, n_features=7, seed=9)
    outs = []
    for autotune in (0, 1):
        assert lib.stater_set_autotune(autotune) == 0
        b = st.StatBuffers(W, H, TR, 7, 3, st.F32)
        b.accumulate(smp, mode=st.ACC_FAST)
        b.denoise_vars(radius=R)
        b.denoise_film(radius=R)
        torch.cuda.synchronize()
        outs.append((b.varD.clone(), b.filmD.clone()))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
    assert lib.stater_tuned_tile_height(1, 5, W, H, R) in (4, 8, 16)
    assert lib.stater_tuned_tile_height(0, 5, W, H, R) in (4, 8, 16)


def test_batch_rejects_fp64_and_capture_of_first_run(st):
    W, H = 32, 16
    b = st.StatBuffers(W, H, TR[:1], 7, 3, st.F64)
    film = st.Film(W, H, n_features=7)
    smp = st.generate_samples(W, H, 4, n_features=7, seed=1)
    with pytest.raises((ValueError, st.StaterError)):
        st.Batch([dict(buffers=b, film=film, samples=smp, radius=4)])


@pytest.mark.parametrize("W,H,tr,G,R", [
    (160, 96, TR, 7, 10),
    (97, 61, TR[:3], 7, 7),     # partial tiles
    (64, 37, TR[:1], 7, 4),
])
def test_vars_ring_forms_give_the_same_bits(st, W, H, tr, G, R):
    """The FP32 variance ring gives the same varD and varCD bits at every tile
    height (4, 8, 16, and the tuner's) as the per-transform kernel, with
    uneven counts (pixels below two samples included), partial tiles, and
    neighbours of range weight 0 (other feature regions), whose records both
    forms skip."""
    lib = st.load()
    smp = st.generate_samples(W, H, 24, n_features=G, seed=41)
    cnt = torch.from_numpy(np.random.default_rng(42).integers(0, 25, size=(H, W)).astype(np.int32)).cuda()
    res = []
    try:
        for th in (-1, 0, 4, 8, 16):
            assert lib.stater_debug_set_vars_ring_form(th) == 0
            b = st.StatBuffers(W, H, tr, G, 3, st.F32)
            b.accumulate(smp, count=cnt, mode=st.ACC_FAST)
            b.denoise_vars(radius=R)
            torch.cuda.synchronize()
            res.append((b.varD.clone(), b.varCD.clone()))
    finally:
        assert lib.stater_debug_set_vars_ring_form(0) == 0
    for vd, vcd in res[1:]:
        assert torch.equal(vd, res[0][0]) and torch.equal(vcd, res[0][1])
    assert torch.isfinite(res[0][0]).any()
