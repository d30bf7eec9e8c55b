"""bench.py's count of the variance filter's loaded records on CPU: the share of
(pixel, neighbour) positions whose range exponent is at least -127 equals a
brute-force count, and the quarter-warp and warp shares are at least the lane
share and ordered."""
import math
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parents[1]
GB = [(0, 3, 0.02), (3, 3, 0.1), (6, 1, 0.1)]


def _features(H, W, G, region, seed):
    rng = np.random.default_rng(seed)
    ry, rx = np.arange(H) // region, np.arange(W) // region
    base = rng.random((G, (H + region - 1) // region, (W + region - 1) // region))
    return base[:, ry][:, :, rx] + rng.normal(0, 3.6e-4, (G, H, W))


def _brute_lanes(gm, ok, R, sd):
    mul = np.array([math.sqrt(0.5 / s ** 2 * 1.4426950408889634) for _, c, s in GB for _ in range(c)])
    F = gm.astype(np.float32).astype(np.float64) * mul[:, None, None]
    ds2 = -0.5 / (sd * sd) * 1.4426950408889634
    G, H, W = gm.shape
    need = tot = 0
    for y in range(H):
        for x in range(W):
            if not ok[y, x]:
                continue
            for dy in range(-R, R + 1):
                for dx in range(-R, R + 1):
                    tot += 1
                    yy, xx = y + dy, x + dx
                    if 0 <= yy < H and 0 <= xx < W and ok[yy, xx]:
                        e = ds2 * (dy * dy + dx * dx) - ((F[:, y, x] - F[:, yy, xx]) ** 2).sum()
                        need += e >= -127
    return need / tot


@pytest.mark.parametrize("H,W,region,R", [(16, 64, 8, 4), (12, 45, 5, 3)])
def test_records_loaded_shares(H, W, region, R):
    sys.path.insert(0, str(ROOT))
    import bench
    gm = _features(H, W, 7, region, seed=H + W)
    ok = np.ones((H, W), bool)
    ok[3, 7] = False
    n = torch.from_numpy(np.where(ok, 64, 1).astype(np.int32))
    got = bench.vars_records_loaded(torch.from_numpy(gm.astype(np.float32)), n, GB, R, 10.0)
    assert got["lanes"] == pytest.approx(_brute_lanes(gm, ok, R, 10.0), abs=1e-12)
    assert 0.0 < got["lanes"] <= got["quarter_warps"] <= got["warps"] <= 1.0


def test_one_region_loads_everything():
    sys.path.insert(0, str(ROOT))
    import bench
    H, W, R = 8, 32, 3
    gm = torch.full((7, H, W), 0.5)
    n = torch.full((H, W), 16, dtype=torch.int32)
    got = bench.vars_records_loaded(gm, n, GB, R, 10.0)
    # only the neighbours beyond the image border are skipped
    inside = sum(max(0, min(H, y + R + 1) - max(0, y - R)) * max(0, min(W, x + R + 1) - max(0, x - R))
                 for y in range(H) for x in range(W))
    assert got["lanes"] == pytest.approx(inside / (H * W * (2 * R + 1) ** 2))
    # a warp (one 32-pixel row) skips only the neighbour rows outside the image
    rows_in = sum(min(H, y + R + 1) - max(0, y - R) for y in range(H))
    assert got["warps"] == pytest.approx(rows_in / (H * (2 * R + 1)))
