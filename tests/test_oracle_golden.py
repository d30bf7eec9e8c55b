"""Pins the oracle's stage-1 restatement against the reference's own StatTile.

tests/golden/*.npz come from the reference's src/statistics/estimator.h compiled
in place (tests/golden/make_golden.py). Bit-exact equality is required: the
oracle repeats the reference's operations in the same order in both the float
build and the PBRT_FLOAT_AS_DOUBLE build.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem.replace("stattile_", "") for p in GOLD.glob("stattile_*_mm*.npz"))


def _inputs():
    d = np.load(GOLD / "stattile_inputs.npz")
    return d["s1"], d["s2"], d["c2"], d["bounds"], int(d["W"]), int(d["H"]), int(d["G"])


def _transforms(case):
    lams = case["lambdas"]
    if int(case["transform"]) == 0:
        return ["identity"]
    return ["identity"] + [("boxcox", float(l)) for l in lams]


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_stattile(name):
    s1, s2, c2, _, W, H, G = _inputs()
    case = np.load(GOLD / f"stattile_{name}.npz")
    prec = "f64" if "_f64_" in name else "f32"
    dt = np.float64 if prec == "f64" else np.float32
    tr = _transforms(case)
    if name.startswith("boxcox"):
        tr = ["identity", ("boxcox", 0.25)]
    K = len(tr)
    mm = int(case["max_moment"])
    n, stats, gmean = oracle.new_state(K, G, H, W, dt)
    oracle.accumulate(s1, tr, mm, n, stats, gmean, precision=prec)
    oracle.accumulate(s2, tr, mm, n, stats, gmean, count=c2, precision=prec)
    ref_stats = case["stats"]
    assert np.array_equal(n, case["n"].astype(np.int32))
    assert np.array_equal(gmean[:G], case["gmean"])
    if ref_stats.ndim == 5:  # single lambda: [set][7][3][H][W]
        assert np.array_equal(stats[0], ref_stats[0])
        if K > 1:
            assert np.array_equal(stats[1], ref_stats[1])
    else:  # multi-transform build: [lambda][set][7][3][H][W]
        for j in range(ref_stats.shape[0]):
            assert np.array_equal(stats[0], ref_stats[j, 0])
            assert np.array_equal(stats[1 + j], ref_stats[j, 1])


def test_merge_transform_tiles_matches_reference_records():
    _, _, _, bounds, W, H, _ = _inputs()
    case = np.load(GOLD / "stattile_boxcox_f32_mm5.npz")
    n, stats = oracle.merge_transform_tiles_f32(W, H, bounds, case["records"])
    assert np.array_equal(n, case["n"].astype(np.int32))
    assert np.array_equal(stats, case["stats"])


def test_reference_boxcox_lambda_one_is_identity():
    case = np.load(GOLD / "stattile_mt_f32_mm5.npz")
    lams = list(case["lambdas"])
    j = lams.index(1.0)
    assert np.array_equal(case["stats"][j, 1], case["stats"][j, 0])
