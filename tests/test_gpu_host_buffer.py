"""Page-locked host memory on huge pages (stater_host_alloc / HostBuffer):
the buffer is zeroed, page-locked (non-blocking copies to and from the device
carry its data) and freed without error."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_host_buffer_round_trip():
    import stater_gb300 as S
    S.setup()
    hb = S.HostBuffer((4, 1024, 4096))
    t = hb.tensor
    assert t.shape == (4, 1024, 4096) and not bool(t.any())
    t.copy_(torch.arange(t.numel(), dtype=torch.float32).reshape(t.shape))
    dev = torch.empty(t.shape, dtype=torch.float32, device="cuda")
    dev.copy_(t, non_blocking=True)
    back = torch.empty_like(t)
    back.copy_(dev, non_blocking=True)
    torch.cuda.synchronize()
    assert torch.equal(back, t)
    hb.close()
    hb.close()  # idempotent
