"""Bounded device waits of the TMA-fed pipelines: a stall ends in an error
status, not a hang, and the context stays usable.

The test hook makes the producers of the FP32 accumulation and of the LEV
accumulation issue no copies, so their consumers wait on stages that nothing
fills; with a short wait limit those waits give up, the kernels end early and
stater_synchronize reports STATER_ERR_TIMEOUT once. No copy is in flight in
that case, nothing faults and nothing waits without a limit. The next calls on
the same context must give the bits of a clean run.
"""
import numpy as np
import pytest

from helpers import synth_samples

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TIMEOUT = 5
TR = ["identity", "log1p", "sqrt", "cbrt", "asinh"]


@pytest.fixture(scope="module")
def st():
    import stater_gb300 as S
    S.setup()
    return S


def _stalled(lib, fn):
    """Runs fn with stalled producers; returns the two stater_synchronize codes."""
    assert lib.stater_debug_set_pipeline_waits(256, 1) == 0
    try:
        fn()
        first = lib.stater_synchronize(None)
        msg = lib.stater_last_error()
        second = lib.stater_synchronize(None)
    finally:
        assert lib.stater_debug_set_pipeline_waits(0, 0) == 0
    return first, msg, second


def test_accumulate_stall_times_out_and_recovers(st):
    lib = st.load()
    W, H, G = 64, 32, 7  # W*H a multiple of 4: the TMA-fed kernel
    s = torch.from_numpy(synth_samples(W, H, 40, G=G, seed=3)).cuda()

    def run():
        b = st.StatBuffers(W, H, TR, G, 3, st.F32)
        b.accumulate(s, mode=st.ACC_FAST)
        return b

    assert lib.stater_synchronize(None) == 0
    clean = run()
    assert lib.stater_synchronize(None) == 0
    first, msg, second = _stalled(lib, run)
    assert first == TIMEOUT and b"gave up" in msg and b"lost" not in msg
    assert second == 0
    again = run()
    assert lib.stater_synchronize(None) == 0
    assert torch.equal(again.n, clean.n) and torch.equal(again.stats, clean.stats)
    assert torch.equal(again.gmean, clean.gmean)


def test_lev_stall_times_out_and_recovers(st):
    lib = st.load()
    W, H, G = 64, 24, 7
    s = st.generate_samples(W, H, 48, n_features=G, seed=5, lev_r2=0.6)

    def run():
        lev = st.LevState(W, H, G, st.F32)
        lev.accumulate(s)
        return lev

    clean = run()
    assert lib.stater_synchronize(None) == 0
    first, msg, second = _stalled(lib, run)
    assert first == TIMEOUT and b"gave up" in msg
    assert second == 0
    again = run()
    assert lib.stater_synchronize(None) == 0
    assert torch.equal(again.state, clean.state)


def test_default_limit_restored_after_the_hook(st):
    """After the hook is switched off, full-size waits run normally again."""
    lib = st.load()
    W, H, G = 128, 64, 7
    s = torch.from_numpy(synth_samples(W, H, 30, G=G, seed=9)).cuda()
    a = st.StatBuffers(W, H, TR, G, 3, st.F32)
    a.accumulate(s, mode=st.ACC_FAST)
    assert lib.stater_synchronize(None) == 0
    assert int(a.n.min().item()) == 30
