"""Serving engine: continuous batching of denoise jobs (stater_server_*).

* a job's result is the same alone and in a mix of concurrently running jobs
  of other sizes, sample counts, transform counts and adaptive rounds;
* the server's pipeline equals the same steps driven by hand through the
  public API (one pass and adaptive rounds with resident moment buffers);
* admission keeps the running jobs' footprint under the memory budget.
"""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BASE_TR = ("identity", "log1p", "sqrt", "cbrt", "asinh")


@pytest.fixture(scope="module")
def S():
    import stater_gb300 as S
    S.setup()
    return S


def _out(w, h):
    return np.zeros((3, h, w), np.float32)


def _run_alone(srv_mod, desc_kw):
    out = _out(desc_kw["width"], desc_kw["height"])
    with srv_mod.Server(max_slots=1) as srv:
        jid = srv.submit(srv_mod.job_desc(**desc_kw, out=out), keepalive=out)
        srv.wait(jid)
    return out


def test_same_result_alone_and_in_mix(S):
    from stater_gb300 import serving
    A = dict(width=160, height=96, spp=48, transforms=BASE_TR, radius=5, seed=7)
    D = dict(width=120, height=72, spp=32, rounds=3, transforms=BASE_TR, radius=4, seed=9)
    alone_a = _run_alone(serving, A)
    alone_d = _run_alone(serving, D)
    mix = [dict(width=320, height=180, spp=64, transforms=("identity", "log1p", "sqrt"), radius=6, seed=1),
           dict(width=64, height=64, spp=16, transforms=("identity",), radius=3, seed=2),
           A,
           dict(width=256, height=256, spp=128, transforms=BASE_TR, radius=10, seed=3),
           D,
           dict(width=200, height=120, spp=40, transforms=("identity", ("boxcox", 0.25)), max_moment=5, radius=7,
                seed=4),
           dict(width=96, height=80, spp=24, rounds=2, transforms=BASE_TR, radius=5, seed=5)]
    outs = [_out(m["width"], m["height"]) for m in mix]
    rng = np.random.default_rng(0)
    with serving.Server(max_slots=4) as srv:
        ids = []
        for m, o in zip(mix, outs):
            ids.append(srv.submit(serving.job_desc(**m, out=o), keepalive=o))
            time.sleep(float(rng.uniform(0, 0.01)))
        srv.drain()
        st = srv.stats()
    assert st["completed"] == len(mix) and st["failed"] == 0
    assert st["latency_p99_ms"] >= st["latency_p50_ms"] > 0
    assert np.array_equal(outs[2], alone_a)
    assert np.array_equal(outs[4], alone_d)
    for o in outs:
        assert np.all(np.isfinite(o)) and o.max() > 0


def _manual(S, width, height, spp, rounds=1, round_spp=0, transforms=BASE_TR, radius=10, seed=0, chunk=32):
    b = S.StatBuffers(width, height, transforms, 7, 3, S.F32)
    film = S.Film(width, height, 7)
    specs = list(S.GBUFFERS_ALL7)
    target = torch.zeros(height, width, dtype=torch.int32, device="cuda")

    def accumulate(samples, counts):
        for done in range(0, samples, chunk):
            n_s = min(chunk, samples - done)
            smp = S.generate_samples(width, height, n_s, n_features=7, seed=seed, region=8, first_index=b.n)
            cnt = None if counts is None else torch.clamp(counts - done, 0, n_s).to(torch.int32).contiguous()
            b.accumulate(smp, count=cnt, mode=S.ACC_FAST, film=film)

    accumulate(spp, None)
    for r in range(1, rounds):
        b.denoise_vars(radius=radius, gbuffers=specs)
        b.calc_target_spp(round_spp or spp, target, relative=True, eps=1e-4, tmin=16, tmax=1024)
        accumulate(int(target.max().item()), target)
    b.denoise_vars(radius=radius, gbuffers=specs)
    b.denoise_film(radius=radius, gbuffers=specs, film=film.update_image())
    torch.cuda.synchronize()
    return b.filmD.cpu().numpy()


@pytest.mark.parametrize("rounds,round_spp", [(1, 0), (3, 0), (4, 64)])
def test_server_equals_manual_pipeline(S, rounds, round_spp):
    from stater_gb300 import serving
    kw = dict(width=144, height=88, spp=16 if round_spp else 40, rounds=rounds, round_spp=round_spp, radius=6,
              seed=11)
    out = _run_alone(serving, kw)
    ref = _manual(S, **kw)
    assert np.array_equal(out, ref)


def test_admission_respects_memory_budget(S):
    from stater_gb300 import serving
    desc_kw = dict(width=256, height=192, spp=32, radius=5, seed=21)
    fp = serving.footprint(serving.job_desc(**desc_kw))
    budget = 1.5 * fp
    outs = [_out(256, 192) for _ in range(6)]
    with serving.Server(max_slots=4, hbm_budget_bytes=budget) as srv:
        for i, o in enumerate(outs):
            srv.submit(serving.job_desc(**dict(desc_kw, seed=21 + i), out=o), keepalive=o)
        srv.drain()
        st = srv.stats()
    assert st["completed"] == 6
    assert st["peak_footprint_bytes"] <= budget


def test_submit_rejects_bad_jobs(S):
    from stater_gb300 import serving
    from stater_gb300._lib import StaterError
    with serving.Server(max_slots=1, hbm_budget_bytes=1e6) as srv:
        with pytest.raises(StaterError):
            srv.submit(serving.job_desc(width=0, height=10, spp=4))
        with pytest.raises(StaterError):  # larger than the whole budget
            srv.submit(serving.job_desc(width=512, height=512, spp=4))
        dev = torch.zeros((3, 8, 8), dtype=torch.float32, device="cuda")
        d = serving.job_desc(width=8, height=8, spp=4, radius=2)
        d.out_host = dev.data_ptr()
        with pytest.raises(StaterError, match="device memory"):  # the result goes to host memory
            srv.submit(d)


def test_fused_small_jobs_equal_alone(S):
    """Small single-round jobs that wait together run as one fused group (one
    launch per denoise stage for the group); each job's film must equal the same
    job run alone, and a larger or adaptive job in the mix is unaffected."""
    from stater_gb300 import serving
    small = [dict(width=128, height=96, spp=24, transforms=BASE_TR, radius=10, seed=11),
             dict(width=256, height=256, spp=16, transforms=("identity", "log1p", "sqrt"), radius=10, seed=12),
             dict(width=64, height=48, spp=32, transforms=("identity",), radius=6, seed=13),
             dict(width=200, height=120, spp=20, transforms=("identity", ("boxcox", 0.25)), max_moment=5, radius=7,
                  seed=14),
             dict(width=512, height=512, spp=8, transforms=BASE_TR, radius=10, seed=15)]
    other = [dict(width=640, height=360, spp=16, transforms=BASE_TR, radius=10, seed=16),
             dict(width=96, height=80, spp=24, rounds=2, transforms=BASE_TR, radius=5, seed=17)]
    alone = [_run_alone(serving, m) for m in small + other]
    jobs = small + other
    outs = [_out(m["width"], m["height"]) for m in jobs]
    with serving.Server(max_slots=2, fuse_small_jobs=True) as srv:
        for m, o in zip(jobs, outs):
            srv.submit(serving.job_desc(**m, out=o), keepalive=o)
        srv.drain()
        st = srv.stats()
    assert st["completed"] == len(jobs) and st["failed"] == 0
    for i, (o, a) in enumerate(zip(outs, alone)):
        assert np.array_equal(o, a), i


@pytest.mark.parametrize("fuse", [False, True])
def test_pinned_and_pageable_results_agree(S, fuse):
    """A result bound for page-locked memory is written by the device copy, one
    bound for pageable memory from the engine's page-locked staging: the same
    bits either way, alone and in a fused group, with the engine reused."""
    from stater_gb300 import serving
    A = dict(width=128, height=96, spp=32, transforms=BASE_TR, radius=5, seed=31)
    B = dict(width=96, height=64, spp=16, transforms=BASE_TR, radius=4, seed=32)
    with serving.Server(max_slots=2, fuse_small_jobs=fuse) as srv:
        res = {}
        for kind in ("pageable", "pinned", "pageable"):
            outs = []
            for m in (A, B, A):
                if kind == "pinned":
                    o = torch.zeros((3, m["height"], m["width"]), dtype=torch.float32, pin_memory=True).numpy()
                else:
                    o = _out(m["width"], m["height"])
                outs.append(o)
            ids = [srv.submit(serving.job_desc(**m, out=o), keepalive=o) for m, o in zip((A, B, A), outs)]
            for jid in ids:
                srv.wait(jid)
            res.setdefault(kind, []).append(outs)
    for outs in res["pageable"] + res["pinned"]:
        assert np.array_equal(outs[0], res["pinned"][0][0])
        assert np.array_equal(outs[2], res["pinned"][0][0])
        assert np.array_equal(outs[1], res["pinned"][0][1])
        assert np.isfinite(outs[1]).all() and outs[1].any()
