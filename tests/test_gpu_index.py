"""Accumulation over a pixel index (sample column i belongs to pixel
pixel_index[i]), as the serving engine uses it for adaptive rounds: the same
pixels, samples and counts give the same bits as the dense layout, in any
column order, with padding columns (count 0) skipped; the generator in index
mode writes the same samples as the dense one."""
import numpy as np
import pytest

from helpers import synth_samples

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TR = ("identity", "log1p", "sqrt", "cbrt", "asinh")


@pytest.fixture(scope="module")
def S():
    import stater_gb300 as S
    S.setup()
    return S


TR_BC = ("identity", ("boxcox", 0.3), "asinh")


@pytest.mark.parametrize("W,H,precision,mode,pad,mm,G,tr", [
    (64, 40, "F32", "ACC_FAST", 0, 5, 7, TR),     # 2560 columns: TMA-fed path (dense and index)
    (64, 40, "F32", "ACC_FAST", 3, 5, 7, TR),     # 2563 columns: plain path against the TMA-fed dense call
    (64, 40, "F32", "ACC_FAST", 3, 1, 7, TR),
    (64, 40, "F32", "ACC_FAST", 3, 2, 7, TR),
    (64, 40, "F32", "ACC_FAST", 3, 3, 7, TR),
    (64, 40, "F32", "ACC_FAST", 3, 4, 7, TR),
    (64, 40, "F32", "ACC_FAST", 3, 3, 16, TR_BC),  # more feature channels per warp, Box-Cox
    (50, 30, "F64", "ACC_EXACT", 2, 5, 7, TR),
])
def test_index_mode_equals_dense(S, W, H, precision, mode, pad, mm, G, tr):
    """The TMA-fed FP32 kernel (two columns per lane, packed arithmetic) and the
    plain FP32 kernel give the same bits: the dense call takes the TMA-fed path
    when W*H is a multiple of 4, the index call with padding the plain one."""
    N = 24
    rng = np.random.default_rng(91)
    s1 = synth_samples(W, H, N, G=G, seed=92)
    cnt = rng.integers(0, N + 1, size=(H, W)).astype(np.int32)
    # first round: uneven counts with some pixels left empty, so that the second
    # round mixes first samples and continuing pixels within a column pair
    cnt1 = rng.integers(0, N + 1, size=(H, W)).astype(np.int32)
    cnt1[:, ::5] = 0
    c1 = torch.from_numpy(cnt1).cuda()
    prec, md = getattr(S, precision), getattr(S, mode)
    # dense reference: a round with uneven counts, then a second one
    dense = S.StatBuffers(W, H, tr, G, mm, prec)
    fd = S.Film(W, H, G)
    dense.accumulate(torch.from_numpy(s1).cuda(), count=c1, mode=md, film=fd)
    s2 = synth_samples(W, H, N, G=G, seed=93)
    dense.accumulate(torch.from_numpy(s2).cuda(), count=torch.from_numpy(cnt).cuda(), mode=md, film=fd)
    # index mode: the same first round dense, the second over a shuffled index with padding
    idx = S.StatBuffers(W, H, tr, G, mm, prec)
    fi = S.Film(W, H, G)
    idx.accumulate(torch.from_numpy(s1).cuda(), count=c1, mode=md, film=fi)
    perm = rng.permutation(W * H).astype(np.int32)
    order = np.concatenate([perm, np.zeros(pad, np.int32)])
    ccol = np.concatenate([cnt.reshape(-1)[perm], np.zeros(pad, np.int32)])
    planes = s2.reshape(N, 5 + G, W * H)[:, :, order].copy()
    idx.accumulate(torch.from_numpy(planes).cuda(), count=torch.from_numpy(ccol).cuda(), mode=md, film=fi,
                   pixel_index=torch.from_numpy(order).cuda())
    torch.cuda.synchronize()
    assert torch.equal(dense.n, idx.n)
    assert torch.equal(dense.stats, idx.stats)
    assert torch.equal(dense.gmean, idx.gmean)
    assert torch.equal(fd.contrib_sum, fi.contrib_sum) and torch.equal(fd.weight_sum, fi.weight_sum)


def test_generator_index_mode(S):
    W, H, N, G = 48, 20, 12, 7
    first = torch.arange(W * H, dtype=torch.int32, device="cuda").remainder(5).reshape(H, W).contiguous()
    dense = S.generate_samples(W, H, N, G, seed=4, first_index=first)
    perm = torch.from_numpy(np.random.default_rng(95).permutation(W * H).astype(np.int32)).cuda()
    firstc = first.reshape(-1)[perm.long()].contiguous()
    cnt = torch.full((W * H,), N, dtype=torch.int32, device="cuda")
    cnt[::3] = 4
    packed = S.generate_samples(W, H, N, G, seed=4, first_index=firstc, count=cnt, pixel_index=perm)
    torch.cuda.synchronize()
    d = dense.reshape(N, 5 + G, W * H)[:, :, perm.long()]
    for i in (0, 1, 2, 3, 100, W * H - 1):
        c = int(cnt[i])
        assert torch.equal(packed[:c, :, i], d[:c, :, i])


def _acc_with_order(S, lib, order, W, H, G, mm, s, cnt):
    """One FP32 accumulation (TMA-fed: W*H a multiple of 4) with the warp order
    `order` set for the call (None: the library's plan)."""
    if order is not None:
        a = np.array(order, np.int32)
        assert lib.stater_debug_set_warp_order(a.ctypes.data, len(order)) == 0
    try:
        b = S.StatBuffers(W, H, TR, G, mm, S.F32)
        f = S.Film(W, H, G)
        b.accumulate(torch.from_numpy(s).cuda(), count=torch.from_numpy(cnt).cuda(), mode=S.ACC_FAST, film=f)
        torch.cuda.synchronize()
        return b, f
    finally:
        assert lib.stater_debug_set_warp_order(None, 0) == 0


@pytest.mark.parametrize("mm,G", [(3, 7), (5, 7), (3, 16)])
def test_warp_order_gives_the_same_bits(S, mm, G):
    """The TMA-fed kernel's placement of transforms on warps (the library's
    plan, or any order set with stater_debug_set_warp_order) changes no bit of
    the moments, feature means, counts or film sums, with uneven counts. An
    order for another number of transforms leaves the plan in place."""
    from stater_gb300 import _lib as L
    lib = L.load()
    W, H, N = 64, 40, 30
    s = synth_samples(W, H, N, G=G, seed=95)
    cnt = np.random.default_rng(96).integers(0, N + 1, size=(H, W)).astype(np.int32)
    ref_b, ref_f = _acc_with_order(S, lib, [0, 1, 2, 3, 4], W, H, G, mm, s, cnt)
    for order in (None, [4, 3, 2, 1, 0], [2, 4, 0, 1, 3], [1, 0]):
        b, f = _acc_with_order(S, lib, order, W, H, G, mm, s, cnt)
        assert torch.equal(b.stats, ref_b.stats), order
        assert torch.equal(b.gmean, ref_b.gmean) and torch.equal(b.n, ref_b.n), order
        assert torch.equal(f.contrib_sum, ref_f.contrib_sum) and torch.equal(f.weight_sum, ref_f.weight_sum), order
