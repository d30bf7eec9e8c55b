"""Shared helpers for the test suite (host-side synthetic inputs, comparisons)."""
from __future__ import annotations

import numpy as np


def synth_samples(W, H, S, G=7, seed=0, region=4, mean_mu=-1.0, mean_sigma=1.0, noise_sigma=0.5,
                  firefly_prob=1e-3, firefly_scale=1e3, zero_prob=0.0):
    """Seeded sample planes [S, 5+G, H, W] float32: per-region lognormal radiance
    means times per-sample lognormal(0, noise_sigma) noise with fireflies, uniform
    in-pixel offsets, features piecewise constant per region plus a small jitter."""
    rng = np.random.default_rng(seed)
    ry, rx = (H + region - 1) // region, (W + region - 1) // region
    mu_r = np.exp(mean_mu + mean_sigma * rng.standard_normal((3, ry, rx)))
    f_r = rng.random((G, ry, rx))
    yy, xx = np.meshgrid(np.arange(H) // region, np.arange(W) // region, indexing="ij")
    mu = mu_r[:, yy, xx]
    fb = f_r[:, yy, xx]
    out = np.empty((S, 5 + G, H, W), np.float32)
    noise = np.exp(noise_sigma * rng.standard_normal((S, 3, H, W)))
    ff = np.where(rng.random((S, 1, H, W)) < firefly_prob, firefly_scale, 1.0)
    rad = mu[None] * noise * ff
    if zero_prob > 0:
        rad = np.where(rng.random((S, 1, H, W)) < zero_prob, 0.0, rad)
    out[:, 0:3] = rad
    out[:, 3:5] = rng.random((S, 2, H, W))
    out[:, 5:] = np.clip(fb[None] + 0.02 * (rng.random((S, G, H, W)) - 0.5), 0.0, 1.0)
    return out


def rel_err(a, b, floor):
    """max |a-b| / max(|b|, floor) with a per-element floor array or scalar."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def moment_scale(stats, n, q):
    """Natural magnitude of moment q (1-based power) per element: n * s^q with s
    the per-pixel standard deviation, used as the absolute floor of relative
    errors (central moments near zero would otherwise divide by ~0)."""
    m2 = np.abs(stats[:, 1])
    nn = np.maximum(n, 1)[None, None]
    s = np.sqrt(m2 / nn)
    return nn * s ** q + 1e-300


def decision_flips(bits_a, bits_b):
    """Per-pixel flag: any Welch accept/reject decision (neighbour x transform)
    differs between two accept-bit arrays [HW, K, words]."""
    d = np.bitwise_xor(np.asarray(bits_a).view(np.uint32), np.asarray(bits_b).view(np.uint32))
    return np.any(d != 0, axis=tuple(range(1, d.ndim)))


def var_test_near_boundary(lnS2, se2, n, R, var_z, rel_margin=1e-3):
    """Per-pixel flag [H, W]: some variance-test decision of the pixel (any
    in-window neighbour with n >= 2, transform, channel) lies within rel_margin of
    its threshold, (lnS2_i - lnS2_j)^2 vs z^2 (se2_i + se2_j), in the FP64
    values given. Only there can a form whose inputs differ by ~1e-6 relative
    decide otherwise; everywhere else both forms keep the same neighbours."""
    lnS2 = np.asarray(lnS2, np.float64)
    se2 = np.asarray(se2, np.float64)
    K, C, H, W = lnS2.shape
    z2 = float(var_z) ** 2
    valid = np.asarray(n) >= 2
    near = np.zeros((H, W), bool)
    for dy in range(-R, R + 1):
        yi = slice(max(0, -dy), min(H, H - dy))
        yj = slice(max(0, dy), min(H, H + dy))
        for dx in range(-R, R + 1):
            if dx == 0 and dy == 0:
                continue
            xi = slice(max(0, -dx), min(W, W - dx))
            xj = slice(max(0, dx), min(W, W + dx))
            if yi.start >= yi.stop or xi.start >= xi.stop:
                continue
            dl = lnS2[..., yi, xi] - lnS2[..., yj, xj]
            thr = z2 * (se2[..., yi, xi] + se2[..., yj, xj])
            m = np.abs(dl * dl - thr) <= rel_margin * np.abs(thr)
            m = np.any(m, axis=(0, 1)) & valid[yi, xi] & valid[yj, xj]
            near[yi, xi] |= m
    return near


def split_rel_error(got, ref, flagged, floor=1e-12):
    """Relative error |got - ref| / max(|ref|, floor) of [..., H, W] arrays split
    by a per-pixel flag [H, W] (or [HW]): (max over unflagged pixels, max over
    flagged pixels, fraction of pixels flagged)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), floor)
    rel = rel.reshape(-1, rel.shape[-2] * rel.shape[-1]).max(axis=0)
    flagged = np.asarray(flagged).reshape(-1)
    clean = rel[~flagged]
    dirty = rel[flagged]
    return (float(clean.max()) if clean.size else 0.0, float(dirty.max()) if dirty.size else 0.0,
            float(flagged.mean()))
