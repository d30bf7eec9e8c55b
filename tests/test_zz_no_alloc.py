"""The allocation-free calcTargetSPP entry point (stater_calc_target_spp_noalloc).

Callers that cannot allocate device memory (a pool allocator owns the device,
or the host forbids the device-wide synchronisation of cudaMalloc/cudaFree)
use this variant, whose scratch is a fixed array inside libstater. It must give
exactly the integers of the allocating entry point, on consecutive calls that
reuse the array, and must refuse images larger than its fixed scratch.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_PIXELS = 1 << 21


def _inputs(H, W, seed):
    rng = np.random.default_rng(seed)
    n = rng.integers(16, 300, size=(H, W)).astype(np.int32)
    n[0, 0] = 1
    varD = (rng.random((3, H, W)) ** 3).astype(np.float64)
    mean = (rng.random((3, H, W)) + 0.05).astype(np.float64)
    return [torch.from_numpy(a).cuda() for a in (n, varD, mean)]


def _call(lib, name, W, H, n, varD, mean, out, precision=1):
    return getattr(lib, name)(W, H, 64, precision, n.data_ptr(), varD.data_ptr(),
                              None if mean is None else mean.data_ptr(), C.c_double(1e-4), 16, 1024,
                              out.data_ptr(), None)


@pytest.fixture(scope="module")
def lib():
    import stater_gb300 as S
    S.setup()
    return S.load()


def _compare(lib, H, W, n, varD, mean):
    ref = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    got = torch.full((H, W), -7, dtype=torch.int32, device="cuda")
    assert _call(lib, "stater_calc_target_spp", W, H, n, varD, mean, ref) == 0
    assert _call(lib, "stater_calc_target_spp_noalloc", W, H, n, varD, mean, got) == 0
    torch.cuda.synchronize()
    assert torch.equal(got, ref), (H, W)


def test_noalloc_matches_allocating_entry_point_twice_in_a_row(lib):
    # 1080p, a ragged size, exactly the limit (2048 x 1024 = 2^21 pixels: the
    # errors fill the whole array and the deepest reduction runs) and a single
    # pixel (no reduction level, the one-value copy)
    for (H, W, seed, relative) in ((1080, 1920, 1, True), (301, 517, 2, False), (1024, 2048, 5, True),
                                   (1, 1, 6, True), (1, 1, 7, False)):
        n, varD, mean = _inputs(H, W, seed)
        if H * W == 1:
            n.fill_(40)
        _compare(lib, H, W, n, varD, mean if relative else None)


def test_noalloc_pixels_without_statistics(lib):
    # no pixel has two samples: every target is the maximum, the sum of errors is 0
    n, varD, mean = _inputs(37, 53, 8)
    n.fill_(1)
    n[5, 5] = 0
    _compare(lib, 37, 53, n, varD, mean)
    # a mix in which every valid pixel has zero variance: total 0, targets = spp
    n, varD, mean = _inputs(37, 53, 9)
    varD.zero_()
    _compare(lib, 37, 53, n, varD, None)


def test_noalloc_after_release_cache(lib):
    # stater_release_cache forgets the array's address; the next call looks it up again
    n, varD, mean = _inputs(64, 96, 10)
    _compare(lib, 64, 96, n, varD, mean)
    assert lib.stater_release_cache() == 0
    _compare(lib, 64, 96, n, varD, mean)


def test_noalloc_f32_inputs(lib):
    n, varD, mean = _inputs(200, 300, 3)
    v32, m32 = varD.float(), mean.float()
    ref = torch.zeros(200, 300, dtype=torch.int32, device="cuda")
    got = torch.zeros_like(ref)
    assert _call(lib, "stater_calc_target_spp", 300, 200, n, v32, m32, ref, precision=0) == 0
    assert _call(lib, "stater_calc_target_spp_noalloc", 300, 200, n, v32, m32, got, precision=0) == 0
    torch.cuda.synchronize()
    assert torch.equal(got, ref)


def test_noalloc_rejects_images_above_its_scratch(lib):
    n, varD, mean = _inputs(4, 4, 4)
    out = torch.zeros(4, 4, dtype=torch.int32, device="cuda")
    # the size check happens on the host before any device work
    rc = _call(lib, "stater_calc_target_spp_noalloc", 2049, 1024, n, varD, mean, out)
    assert rc == 1
    assert b"exceeds the fixed scratch" in lib.stater_last_error()
