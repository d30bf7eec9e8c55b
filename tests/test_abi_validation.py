"""Error behaviour of the C ABI, on the CPU: arguments the library rejects
before touching the device come back as STATER_ERR_INVALID with a message
(never an abort), and the host-only helpers (test order, job footprint) give
their documented results."""
import ctypes as C
import math

import pytest

from stater_gb300 import _lib as L
from stater_gb300 import api, serving

INVALID = 1


@pytest.fixture(scope="module")
def lib():
    from stater_gb300 import build as b
    b.build()
    return L.load()


def _acc_args(**kw):
    a = L.AccumulateArgs()
    a.width, a.height, a.n_samples, a.n_features = 8, 4, 2, 0
    a.samples = 16  # never dereferenced: validation fails first
    a.n_transforms, a.max_moment, a.precision, a.mode = 1, 3, L.F32, L.ACC_EXACT
    a.n, a.stats = 16, 16
    for k, v in kw.items():
        setattr(a, k, v)
    return a


@pytest.mark.parametrize("field,value,needle", [
    ("width", 0, b"geometry"),
    ("n_transforms", 9, b"n_transforms"),
    ("max_moment", 6, b"max_moment"),
    ("precision", 7, b"precision"),
    ("n", None, b"null buffer"),
])
def test_accumulate_rejects(lib, field, value, needle):
    a = _acc_args(**{field: value})
    assert lib.stater_accumulate(C.byref(a), None) == INVALID
    assert needle in lib.stater_last_error()


def test_accumulate_rejects_transform_and_mode(lib):
    a = _acc_args()
    a.transforms[0].kind = 2  # transform 0 must be the identity
    assert lib.stater_accumulate(C.byref(a), None) == INVALID
    assert b"identity" in lib.stater_last_error()
    a = _acc_args(precision=L.F64, mode=L.ACC_FAST)
    assert lib.stater_accumulate(C.byref(a), None) == INVALID
    assert b"FP32" in lib.stater_last_error()
    a = _acc_args(film_contrib_sum=16)  # film sums without weight and spill planes
    assert lib.stater_accumulate(C.byref(a), None) == INVALID
    assert b"film" in lib.stater_last_error()
    assert lib.stater_accumulate(None, None) == INVALID


def test_film_entry_points_reject(lib):
    f = L.FilmArgs()
    f.width, f.height, f.n_samples, f.n_features = 4, 4, 1, 0
    f.samples, f.contrib_sum, f.weight_sum, f.spill = 16, 16, 16, 16
    f.max_sample_luminance = 0.0
    assert lib.stater_film_add_samples(C.byref(f), None) == INVALID
    assert b"luminance" in lib.stater_last_error()
    f.max_sample_luminance = math.inf
    f.spill = None
    assert lib.stater_film_add_samples(C.byref(f), None) == INVALID
    assert lib.stater_film_update_image(0, 4, 16, 16, None, C.c_float(1.0), 16, None) == INVALID


def test_test_order(lib):
    def order(trs):
        codes = api.transform_codes(trs)
        tr = (L.Transform * L.MAX_TRANSFORMS)()
        for k, (kind, lam) in enumerate(codes):
            tr[k].kind, tr[k].lambda_ = kind, lam
        out = (C.c_int32 * L.MAX_TRANSFORMS)()
        assert lib.stater_test_order(tr, len(codes), out) == 0
        return list(out)[:len(codes)]

    assert order(["identity", "log1p", "sqrt", "cbrt", "asinh"]) == [4, 3, 2, 1, 0]
    assert order(["identity"]) == [0]
    got = order(["identity", ("boxcox", 0.25), ("boxcox", 3.0), "sqrt", ("boxcox", 0.75)])
    assert sorted(got) == list(range(5)) and got[-1] == 0 and got[0] == 1
    tr = (L.Transform * L.MAX_TRANSFORMS)()
    out = (C.c_int32 * L.MAX_TRANSFORMS)()
    assert lib.stater_test_order(tr, 9, out) == INVALID


def test_job_footprint_grows_with_the_job(lib):
    small = serving.footprint(serving.job_desc(256, 256, 16))
    large = serving.footprint(serving.job_desc(1920, 1080, 256))
    more_tr = serving.footprint(serving.job_desc(256, 256, 16, transforms=("identity",) * 5))
    fewer_tr = serving.footprint(serving.job_desc(256, 256, 16, transforms=("identity",)))
    f64 = serving.footprint(serving.job_desc(256, 256, 16), precision=L.F64)
    assert 0 < small < large
    assert fewer_tr < more_tr
    assert f64 > small
    # 1080p, K=5, one round, the automatic 32-spp step: about 1 GB of
    # statistics/outputs plus a 3.2 GB sample chunk; 128-spp steps: 12.7 GB
    assert 3e9 < large < 6e9
    assert 12e9 < serving.footprint(serving.job_desc(1920, 1080, 256), chunk_spp=128) < 16e9
    # a step holds no more samples than a round takes: 16 spp in one round
    assert small == serving.footprint(serving.job_desc(256, 256, 16), chunk_spp=16)
    # adaptive jobs take 128-spp steps automatically
    adaptive = serving.job_desc(256, 256, 16, rounds=3, round_spp=64)
    assert serving.footprint(adaptive) == serving.footprint(adaptive, chunk_spp=128) > small


def test_pipeline_wait_hook_rejects(lib):
    """The wait hook refuses limits above the default and stalls with long waits."""
    assert lib.stater_debug_set_pipeline_waits((1 << 22) + 1, 0) == INVALID
    assert lib.stater_debug_set_pipeline_waits(1 << 20, 1) == INVALID
    assert b"65536" in lib.stater_last_error()
    assert lib.stater_debug_set_pipeline_waits(100, 2) == INVALID
    assert lib.stater_debug_set_pipeline_waits(256, 0) == 0
    assert lib.stater_debug_set_pipeline_waits(0, 0) == 0


def test_warp_order_hook_rejects(lib):
    """The warp-order hook takes only permutations of 0 .. n-1 (n <= 8)."""
    import numpy as np
    bad = [np.array([0, 1, 1], np.int32), np.array([0, 3, 1], np.int32), np.array([-1, 0, 1], np.int32)]
    for o in bad:
        assert lib.stater_debug_set_warp_order(o.ctypes.data, 3) == INVALID
    assert lib.stater_debug_set_warp_order(None, 2) == INVALID
    assert lib.stater_debug_set_warp_order(np.zeros(9, np.int32).ctypes.data, 9) == INVALID
    ok = np.array([2, 0, 1], np.int32)
    assert lib.stater_debug_set_warp_order(ok.ctypes.data, 3) == 0
    assert lib.stater_debug_set_warp_order(None, 0) == 0


def test_vars_ring_form_hook_rejects(lib):
    """The variance-ring form hook takes tile heights 0, 4, 8 and 16, and -1
    (the per-transform kernel), only."""
    for th in (5, -8, -2, 32, 1):
        assert lib.stater_debug_set_vars_ring_form(th) == INVALID, th
    for th in (8, 16, 4, -1, 0):
        assert lib.stater_debug_set_vars_ring_form(th) == 0, th


def test_pitched_entry_points_reject_bad_layouts(lib):
    va = L.DenoiseVarsArgs()
    va.n_buffers, va.width, va.height, va.max_moment, va.precision = 1, 64, 8, 3, L.F32
    lay = L.PitchedLayout()
    lay.rgb_step, lay.scalar_step, lay.n_step = 3 * 64 * 4 - 4, 64 * 4, 64 * 4
    assert lib.stater_denoise_vars_pitched(C.byref(va), C.byref(lay), None) == INVALID
    assert b"rgb_step" in lib.stater_last_error()
    lay.rgb_step, lay.n_step = 3 * 64 * 4, 64 * 4 - 4
    assert lib.stater_denoise_vars_pitched(C.byref(va), C.byref(lay), None) == INVALID
    assert b"n_step" in lib.stater_last_error()
    fa = L.DenoiseFilmArgs()
    fa.n_buffers, fa.width, fa.height, fa.precision = 1, 64, 8, L.F64
    lay.rgb_step, lay.scalar_step, lay.n_step = 3 * 64 * 4, 64 * 8, 64 * 4  # rgb_step too short for doubles
    assert lib.stater_denoise_film_pitched(C.byref(fa), C.byref(lay), None) == INVALID
    assert lib.stater_denoise_film_pitched(C.byref(fa), None, None) == INVALID


def test_target_spp_ex_rejects(lib):
    a = L.TargetSppArgs()
    a.width, a.height, a.spp, a.precision, a.tmin, a.tmax = 8, 8, 16, L.F32, 16, 1024
    a.n, a.targetspp = 16, 16  # never dereferenced
    a.as_source = 2
    assert lib.stater_calc_target_spp_ex(C.byref(a), None) == INVALID
    a.as_source = L.AS_SAMPLE  # needs m2
    assert lib.stater_calc_target_spp_ex(C.byref(a), None) == INVALID
    assert b"bad arguments" in lib.stater_last_error()


def test_denoise_film_rejects_bad_discr_source(lib):
    fa = L.DenoiseFilmArgs()
    fa.n_buffers, fa.width, fa.height, fa.filter_radius, fa.alpha, fa.mt_mode = 1, 8, 8, 2, 0.01, 2
    fa.n, fa.film, fa.filmD = 16, 16, 16
    fa.discr[0], fa.varD[0] = 16, 16
    fa.discr_source = 3
    assert lib.stater_denoise_film(C.byref(fa), None) == INVALID
    assert b"discr_source" in lib.stater_last_error()
    fa.discr_source = L.DISCR_SAMPLE  # needs m2
    assert lib.stater_denoise_film(C.byref(fa), None) == INVALID
