"""Benchmark of the StatER statistics hot path on GB300.

Workload (default): 1920x1080 image, 256 samples per pixel, five monotone
transforms (identity, log1p, sqrt, cbrt, asinh) of RGB radiance, 7 feature
channels (albedo RGB, normal xyz, depth), moments M1-M3, 21x21 window (R=10),
Welch alpha = 0.01, range kernels on albedo (sigma 0.02), normal (0.1), depth
(0.1). One step = accumulate all samples into fresh moment buffers, the
variance-denoise pass, and the Welch-discriminated film filter, in the FP32
form. Samples are seeded synthetic planes (25.5 GB, larger than L2), resident in
HBM for `value`; `e2e` streams them from pinned host memory every step through
the same public API (chunked host-to-device copies overlapping the
accumulation) and reads the denoised image back.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl stater|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpix/s denoised (1080p, 5 transforms)"
UNIT = "Mpix/s"
WORKLOAD = dict(width=1920, height=1080, spp=256, transforms=["identity", "log1p", "sqrt", "cbrt", "asinh"],
                features=7, max_moment=3, radius=10, filter_sd=10.0, alpha=0.01, var_z=2.80703,
                gbuffers=[(0, 3, 0.02), (3, 3, 0.1), (6, 1, 0.1)])
LAUNCHES_PER_STEP = 6  # accumulate (+ film sums) 1, film image 1, denoise_vars 2, denoise_film 2


def _config(extra=None):
    w = WORKLOAD
    c = {"workload": f"multi-transform denoise {w['width']}x{w['height']} {w['spp']}spp K=5 G=7 M1-M3 "
                     f"{2 * w['radius'] + 1}x{2 * w['radius'] + 1} alpha={w['alpha']}",
         "width": w["width"], "height": w["height"], "spp": w["spp"], "transforms": w["transforms"],
         "features": w["features"], "window": 2 * w["radius"] + 1, "alpha": w["alpha"],
         "l2": "inputs larger than L2 (25.5 GB sample planes per image)", "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    # Sampling period: a 10-step timed region of the 1080p job lasts about
    # 150 ms, so the period is well below that. 200 ms is the fallback where
    # nvidia-smi refuses the shorter period.
    PERIODS_MS = (50, 200)

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []  # (time.perf_counter() when read, line)
        self.period_ms = None
        self.t_start = self.t_end = None

    def _spawn(self, period_ms):
        self.lines = []
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits", "-lms", str(period_ms)],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.thread = threading.Thread(target=self._read, args=(self.proc, self.lines), daemon=True)
        self.thread.start()
        self.period_ms = period_ms

    def __enter__(self):
        # The timed region starts once the sampler has printed its first line,
        # so that it is live for the whole region; samples read before the
        # region (an idle GPU) are left out of the summary.
        try:
            for period in self.PERIODS_MS:
                self._spawn(period)
                deadline = time.perf_counter() + 3.0
                while not self.lines and self.proc.poll() is None and time.perf_counter() < deadline:
                    time.sleep(0.005)
                if self.lines or self.proc.poll() is None:
                    break
        except OSError:
            self.proc = None
        self.t_start = time.perf_counter()
        return self

    @staticmethod
    def _read(proc, lines):
        for line in proc.stdout:
            lines.append((time.perf_counter(), line.strip()))

    def __exit__(self, *exc):
        self.t_end = time.perf_counter()
        if self.proc is not None:
            # one more sample after the region: the one that covers its last period
            deadline = self.t_end + 2.0 * self.period_ms / 1e3 + 0.1
            while (self.proc.poll() is None and time.perf_counter() < deadline
                   and not any(t > self.t_end for t, _ in self.lines)):
                time.sleep(0.005)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def _region_lines(self):
        """Lines read inside the timed region plus the first one after it. If
        the output came in one block (no time stamps to go by), all lines."""
        if self.t_start is None or self.t_end is None:
            return [ln for _, ln in self.lines]
        inside = [ln for t, ln in self.lines if self.t_start < t <= self.t_end]
        after = [ln for t, ln in self.lines if t > self.t_end][:1]
        picked = inside + after
        return picked if picked else [ln for _, ln in self.lines]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self._region_lines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "period_ms": self.period_ms}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "period_ms": self.period_ms}


# ---------------------------------------------------------------------------
# CPU pipeline (the reference's CPU path for stage 1, the oracle for 2-3)
# ---------------------------------------------------------------------------
def cpu_pipeline_mpix(samples_host, threads):
    """Times the CPU restatement on a strip: FP32 StatTile port (the reference's
    CPU accumulation) + FP64 denoise restatement. Returns (Mpix/s, seconds)."""
    import numpy as np

    import oracle
    w = WORKLOAD
    S, nch, H, W = samples_host.shape
    K = len(w["transforms"])
    n = np.zeros((H, W), np.int32)
    st32 = np.zeros((K, 7, 3, H, W), np.float32)
    g32 = np.zeros((w["features"], H, W), np.float32)
    ds = float(np.float32(-0.5 / (w["filter_sd"] ** 2)))
    t0 = time.perf_counter()
    oracle.accumulate(samples_host, w["transforms"], w["max_moment"], n, st32, g32, precision="f32",
                      nthreads=threads)
    film = oracle.film_update_image(oracle.film_add_samples(samples_host)).astype(np.float64)
    st = st32.astype(np.float64)
    gm = g32.astype(np.float64)
    v = oracle.denoise_vars(n, st, gm, w["max_moment"], w["radius"], ds, float(np.float32(w["var_z"])),
                            w["gbuffers"], nthreads=threads)
    oracle.denoise_film(n, st, v["varD"], v["varCD"], v["jb"], gm, film, w["radius"], ds,
                        float(np.float32(w["alpha"])), w["gbuffers"], nthreads=threads)
    dt = time.perf_counter() - t0
    return H * W / dt / 1e6, dt


def strip_samples(rows, seed=0):
    """Samples of a 1920 x rows strip of the workload (host float32)."""
    import numpy as np
    import torch

    import stater_gb300 as S
    w = WORKLOAD
    if torch.cuda.is_available():
        return S.generate_samples(w["width"], rows, w["spp"], n_features=w["features"], seed=seed).cpu().numpy()
    sys.path.insert(0, str(ROOT / "tests"))
    from helpers import synth_samples
    return synth_samples(w["width"], rows, w["spp"], G=w["features"], seed=seed, region=8).astype(np.float32)


def run_reference(args, rank):
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    rows = args.cpu_rows
    smp = strip_samples(rows, seed=1)
    for _ in range(args.warmup):
        cpu_pipeline_mpix(smp[:, :, : max(2, rows // 4)], threads)
    vals = []
    for _ in range(args.steps):
        v, _ = cpu_pipeline_mpix(smp, threads)
        vals.append(v)
    value = statistics.median(vals)
    sample = f"1920x{rows} strip of the workload per step ({args.spp_note})"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1920 * rows / value / 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
            "config": _config(),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _specs(S):
    return [S.GBufferSpec(a, c, sg) for a, c, sg in WORKLOAD["gbuffers"]]


def _denoise(S, b, film, stream=None):
    """Film::UpdateImage, then denoiseVars and denoiseFilm of the film image."""
    w = WORKLOAD
    rgb = film.update_image(stream=stream)
    if b.precision == S.F64:
        rgb = rgb.double()
    b.denoise_vars(radius=w["radius"], filter_sd=w["filter_sd"], var_z=w["var_z"], gbuffers=_specs(S), stream=stream)
    b.denoise_film(radius=w["radius"], filter_sd=w["filter_sd"], alpha=w["alpha"], gbuffers=_specs(S), film=rgb,
                   stream=stream)


def _reset(b, film):
    b.n.zero_()
    b.stats.zero_()
    b.gmean.zero_()
    film.clear()


def hbm_peak_gbs():
    """The measured STREAM-style copy bandwidth of this GPU model, else the fallback figure."""
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(peaks["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured)"
    except Exception:
        return 6800.0, "fallback"


def fp32_peak_tflops(S, reps=5):
    """FP32 rate of this GPU with its own FMA instructions (stater_fp32_peak_probe:
    8 independent chains per thread, scalar fma.rn.f32 and packed fma.rn.f32x2),
    timed with CUDA events; the larger of the two medians, in TFLOP/s."""
    import ctypes as C

    import torch
    lib = S.load()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    blocks = props.multi_processor_count * 8
    sink = torch.zeros(blocks, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    out = {}
    for packed in (0, 1):
        flops = C.c_double(0.0)
        ms = []
        for i in range(reps + 2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rc = lib.stater_fp32_peak_probe(blocks, 2048, packed, C.c_void_p(sink.data_ptr()), C.byref(flops),
                                            C.c_void_p(stream.cuda_stream))
            e1.record(stream)
            torch.cuda.synchronize()
            if rc != 0:
                raise RuntimeError("stater_fp32_peak_probe failed")
            if i >= 2:
                ms.append(e0.elapsed_time(e1))
        out["packed" if packed else "scalar"] = flops.value / (statistics.median(ms) / 1e3) / 1e12
    return max(out.values()), out


# Algorithmic FP32 operations per (pixel, in-window neighbour) of the two
# window filters at the benchmark's configuration (an FMA counts 2, a compare
# or exp2 1). Range weight: spatial term 2 + 3 per feature channel (difference,
# FMA) + exp2 1. Variance filter, per transform and channel: log-variance
# difference 1, threshold FMA 2, compare 1, weight sum 1, weighted variance FMA
# 2. Film filter, per transform and channel: mean difference 1, summed variance
# 1, square 1, the two df-bound products 2, two compares 2; plus the film sums,
# 4 FMAs. The film filter's count is the formula's (every transform tested for
# every neighbour); the kernel stops at the first rejecting transform, so it
# executes fewer.
def filter_flops_per_pair(K, G):
    weight = 2 + 3 * G + 1
    return {"vars": weight + K * 3 * 7, "film": weight + K * 3 * 7 + 8}


def vars_records_loaded(gmean, n, gbuffers, R, filter_sd):
    """Shares of the variance filter's (pixel, neighbour) positions whose
    transform records the ring kernel loads: a lane skips them where the range
    exponent is below -127 (weight 0), a quarter-warp (8 neighbouring pixels of
    a row, one phase of a 16-byte shared load) where all its lanes do, a warp (32)
    where all 32 do. Computed in FP32 with torch from the feature means, with
    the kernel's formula (near the threshold its rounding may differ). Returns
    {"lanes", "quarter_warps", "warps"}."""
    import math

    import torch
    G, H, W = gmean.shape
    chans, muls = [], []
    for first, count, sigma in gbuffers:
        for c in range(count):
            chans.append(first + c)
            muls.append(math.sqrt(0.5 / (sigma * sigma) * 1.4426950408889634))
    f = gmean[chans].float() * torch.tensor(muls, device=gmean.device).view(-1, 1, 1)
    ok = n >= 2
    ds2 = -0.5 / (filter_sd * filter_sd) * 1.4426950408889634
    Wp = (W + 31) // 32 * 32
    fp = torch.zeros((len(chans), H + 2 * R, Wp + 2 * R), device=gmean.device)
    fp[:, R:R + H, R:R + W] = f
    okp = torch.zeros((H + 2 * R, Wp + 2 * R), dtype=torch.bool, device=gmean.device)
    okp[R:R + H, R:R + W] = ok
    centre = torch.zeros((H, Wp), dtype=torch.bool, device=gmean.device)
    centre[:, :W] = ok
    fc = fp[:, R:R + H, R:R + Wp]
    groups = (("lanes", 1), ("quarter_warps", 8), ("warps", 32))
    counts = {key: 0 for key, _ in groups}
    # groups with a lane that runs the filter, times the neighbour positions
    totals = {key: int(centre.view(H, Wp // g, g).any(-1).sum().item()) * (2 * R + 1) ** 2 for key, g in groups}
    for dy in range(-R, R + 1):
        for dx in range(-R, R + 1):
            fj = fp[:, R + dy:R + dy + H, R + dx:R + dx + Wp]
            e = ds2 * (dy * dy + dx * dx) - ((fc - fj) ** 2).sum(0)
            need = (e >= -127.0) & okp[R + dy:R + dy + H, R + dx:R + dx + Wp] & centre
            for key, g in groups:
                counts[key] += int(need.view(H, Wp // g, g).any(-1).sum().item())
    return {k: counts[k] / max(totals[k], 1) for k in counts}


def max_over_ranks(ms, world, dist, device="cuda"):
    """The largest of the ranks' timings: the job is as slow as its slowest replica."""
    import torch
    if world <= 1 or dist is None:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def accuracy_vs_plain(S, b, film, pb, pfilm):
    """Error of the FP32 form against the plain FP64 form on the same samples:
    the fraction of Welch accept/reject decisions (pixel x neighbour x transform)
    that differ; the relative error of filmD (per channel) at its maximum over
    the pixels whose window has no flipped decision in any transform (both forms
    average the same neighbours there), the fraction of pixels with a flip and
    the maximum over them; and, for reference, the error relative to each
    pixel's largest channel over all pixels."""
    import torch
    w = WORKLOAD
    R = w["radius"]
    words = S.bits_words(R)
    K = b.K
    bits = []
    for bb, ff in ((b, film), (pb, pfilm)):
        rgb = ff.update_image()
        if bb.precision == S.F64:
            rgb = rgb.double()
        t = torch.zeros(bb.H * bb.W, K, words, dtype=torch.int32, device="cuda")
        bb.denoise_film(radius=R, filter_sd=w["filter_sd"], alpha=w["alpha"], gbuffers=_specs(S), film=rgb,
                        accept_bits=t)
        bits.append(t)
    torch.cuda.synchronize()
    v = bits[0] ^ bits[1]  # popcount of the differing decision bits, per int32 word
    v = v - ((v >> 1) & 0x55555555)
    v = (v & 0x33333333) + ((v >> 2) & 0x33333333)
    v = (v + (v >> 4)) & 0x0F0F0F0F
    v = (v & 0xFF) + ((v >> 8) & 0xFF) + ((v >> 16) & 0xFF) + ((v >> 24) & 0xFF)
    flips = int(v.sum(dtype=torch.int64).item())
    flipped = ((bits[0] ^ bits[1]) != 0).any(dim=2).any(dim=1)  # [HW]: some decision of the pixel differs
    total = b.H * b.W * K * (2 * R + 1) ** 2
    a = b.filmD.double()
    r = pb.filmD.double()
    rel_ch = ((a - r).abs() / r.abs().clamp_min(1e-12)).amax(dim=0).flatten()
    clean = rel_ch[~flipped]
    dirty = rel_ch[flipped]
    scale = r.abs().amax(dim=0, keepdim=True).clamp_min(1e-30)
    rel = ((a - r).abs() / scale).flatten()
    q = float(torch.quantile(rel[torch.randperm(rel.numel(), device=rel.device)[:1 << 20]], 0.999).item())
    del bits, v
    return {"filmD_rel_max_unflipped": float(clean.max().item()) if clean.numel() else 0.0,
            "pixels_with_flip_frac": float(flipped.double().mean().item()),
            "filmD_rel_max_flipped": float(dirty.max().item()) if dirty.numel() else 0.0,
            "filmD_rel_max": float(rel.max().item()), "filmD_rel_p999": q,
            "flipped_decisions": flips / total, "decisions": total,
            "comparator": "plain FP64 GPU form (pinned to the FP64 oracle at 256x256, same transforms and window)"}


def run_gpu(args, rank, world, dist):
    import numpy as np
    import torch

    import stater_gb300 as S
    from __graft_entry__ import build
    if rank == 0 or not (ROOT / "stater_gb300" / "libstater.so").exists():
        build()
    if world > 1:
        dist.barrier()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    S.setup()
    w = WORKLOAD
    W, H, SPP, G, K = w["width"], w["height"], w["spp"], w["features"], len(w["transforms"])
    HW = W * H
    stream = torch.cuda.current_stream()

    samples = S.generate_samples(W, H, SPP, n_features=G, seed=1234 + rank)
    b = S.StatBuffers(W, H, w["transforms"], G, w["max_moment"], S.F32)
    film = S.Film(W, H, n_features=G)

    def step():
        _reset(b, film)
        b.accumulate(samples, mode=S.ACC_FAST, film=film)
        _denoise(S, b, film)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # per-stage kernel timings (CUDA events on the launching stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    stage_ms = {"accumulate": [], "film_image": [], "denoise_vars": [], "denoise_film": []}
    for _ in range(3):
        _reset(b, film)
        ev[0].record(stream)
        b.accumulate(samples, mode=S.ACC_FAST, film=film)
        ev[1].record(stream)
        rgb = film.update_image()
        ev[2].record(stream)
        b.denoise_vars(radius=w["radius"], filter_sd=w["filter_sd"], var_z=w["var_z"], gbuffers=_specs(S))
        ev[3].record(stream)
        b.denoise_film(radius=w["radius"], filter_sd=w["filter_sd"], alpha=w["alpha"], gbuffers=_specs(S), film=rgb)
        ev[4].record(stream)
        torch.cuda.synchronize()
        stage_ms["accumulate"].append(ev[0].elapsed_time(ev[1]))
        stage_ms["film_image"].append(ev[1].elapsed_time(ev[2]))
        stage_ms["denoise_vars"].append(ev[2].elapsed_time(ev[3]))
        stage_ms["denoise_film"].append(ev[3].elapsed_time(ev[4]))

    # timed region
    steps = args.steps
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        evs[0].record(stream)
        for i in range(steps):
            step()
            evs[i + 1].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    per_step = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    total_ms = max_over_ranks(evs[0].elapsed_time(evs[steps]), world, dist)
    value = world * HW * steps / (total_ms / 1e3) / 1e6
    filmD_check = float(b.filmD.double().mean().item())

    # roofline of the accumulation kernel (HBM-bound): algorithmic bytes per launch
    acc_bytes = HW * (SPP * (5 + G) * 4 + 2 * (K * 3 * w["max_moment"] * 4 + G * 4 + 4 + 4 * 4))
    acc_ms = statistics.median(stage_ms["accumulate"])
    hbm_peak, peak_source = hbm_peak_gbs()
    # DRAM bytes per launch from one ncu capture of acc_tma_kernel at 480x272, 64 spp,
    # K=5, G=7, M1-M3: 433.16 MB read + 28.01 MB written, film sums included.
    # The per-pixel state (228 B each way) is scaled by pixels, the rest of the
    # reads (the sample planes) by pixel-samples.
    cap_px = 480 * 272
    state_rd = cap_px * (K * 3 * w["max_moment"] * 4 + G * 4 + 4 + 4 * 4)
    samp_rd = 433.160448e6 - state_rd
    traffic = (samp_rd * (HW * SPP) / (cap_px * 64) + (state_rd + 28.007680e6) * HW / cap_px) / 1e9
    roofline = {"kernel": "acc_tma_kernel (stage-1 accumulation)", "bound": "hbm",
                "achieved": acc_bytes / (acc_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": acc_bytes / (acc_ms / 1e3) / 1e9 / hbm_peak, "traffic": traffic,
                "algorithmic_gb": acc_bytes / 1e9,
                "peak_source": peak_source}

    # roofline of the two window filters: FP32 ALU work against the FP32 rate
    # measured here with the library's FMA probe
    fp32_peak, fp32_forms = fp32_peak_tflops(S)
    R = w["radius"]
    pairs = HW * (2 * R + 1) ** 2  # interior count; border pixels have fewer neighbours
    fpp = filter_flops_per_pair(K, G)
    roofline_filters = {"bound": "fp32", "unit": "TFLOP/s", "peak": fp32_peak,
                        "peak_source": "stater_fp32_peak_probe in this run (FMA chains; scalar "
                                       f"{fp32_forms['scalar']:.1f}, packed {fp32_forms['packed']:.1f} TFLOP/s)"}
    for name, stage, kern in (("vars", "denoise_vars", "vars_stats_f32 + vars_ring_f32"),
                              ("film", "denoise_film", "film_discr_f32 + film_ring_f32")):
        ms_ = statistics.median(stage_ms[stage])
        ach = pairs * fpp[name] / (ms_ / 1e3) / 1e12
        roofline_filters[name] = {"kernel": kern, "flops_per_pixel": fpp[name] * (2 * R + 1) ** 2, "ms": ms_,
                                  "achieved": ach, "frac": ach / fp32_peak}
    # the variance filter's shared-memory traffic: per neighbour, the feature
    # records (2 x 16 B) and, where the range weight is not 0, the packed
    # records of the transforms (one z per pixel, no LEVC sums:
    # ceil((6 K + 1) / 4) x 16 B, 8 for K = 5), counted per quarter-warp phase,
    # over the SMs' 128 B/clock at the sampled SM clock. The flop counts above
    # are those of every neighbour (the records of zero-weight neighbours
    # included).
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    sm_mhz = clk.summary().get("sm_mhz") or 2070.0
    loaded = vars_records_loaded(b.gmean, b.n, w["gbuffers"], R, w["filter_sd"])
    smem_bytes = pairs * (2 + loaded["quarter_warps"] * ((6 * K + 4) // 4)) * 16
    roofline_filters["vars"]["smem_frac"] = smem_bytes / (statistics.median(stage_ms["denoise_vars"]) / 1e3) / (
        props.multi_processor_count * 128 * sm_mhz * 1e6)
    roofline_filters["vars"]["records_loaded"] = loaded

    del samples
    torch.cuda.empty_cache()

    extra = {"roofline_filters": roofline_filters}
    # plain FP64 form (one image per launch), same workload
    if not args.no_plain:
        pb = S.StatBuffers(W, H, w["transforms"], G, w["max_moment"], S.F64)
        pfilm = S.Film(W, H, n_features=G)
        chunk = 32
        samples_c = torch.empty(chunk, 5 + G, H, W, dtype=torch.float32, device="cuda")
        first = torch.zeros(H, W, dtype=torch.int32, device="cuda")

        def plain_step(timed_events=None):
            _reset(pb, pfilm)
            for c0 in range(0, SPP, chunk):
                first.fill_(c0)
                S.generate_samples(W, H, chunk, n_features=G, seed=1234 + rank, first_index=first, out=samples_c)
                if timed_events is not None:
                    timed_events[0].record(stream)
                pb.accumulate(samples_c, mode=S.ACC_EXACT, film=pfilm)
                if timed_events is not None:
                    timed_events[1].record(stream)
                    torch.cuda.synchronize()
                    timed_events[2] += timed_events[0].elapsed_time(timed_events[1])
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _denoise(S, pb, pfilm)
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)

        plain_step()
        accs, dens = [], []
        for _ in range(args.plain_steps):
            te = [torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True), 0.0]
            dms = plain_step(te)
            accs.append(te[2])
            dens.append(dms)
        plain_ms = statistics.median([a + d for a, d in zip(accs, dens)])
        extra["plain_f64"] = {"value": HW / (plain_ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": plain_ms,
                              "accumulate_ms": statistics.median(accs), "denoise_ms": statistics.median(dens),
                              "note": "FP64, one image per launch, sample generation excluded"}
        extra["speedup_vs_plain_f64"] = value / world / extra["plain_f64"]["value"]
        extra["fp32_vs_fp64"] = accuracy_vs_plain(S, b, film, pb, pfilm)
        del pb, pfilm, samples_c
        torch.cuda.empty_cache()

    # end to end through the public API with pinned host samples
    e2e = None
    if not args.no_e2e:
        # 32-spp chunks (3.2 GB) keep the copy engine saturated (about 211 GB/s
        # from pinned host memory on this host link) while the accumulation of
        # the previous chunk runs; 16-spp chunks left gaps between the copies
        chunk = 32
        # page-locked host memory on huge pages (stater_host_alloc): with base
        # pages, copies of this 25.5 GB buffer varied between 65 and 210 GB/s
        # from run to run; on huge pages they hold the link's 210 GB/s
        host_buf = S.HostBuffer((SPP, 5 + G, H, W))
        host = host_buf.tensor
        first = torch.zeros(H, W, dtype=torch.int32, device="cuda")
        tmp = torch.empty(chunk, 5 + G, H, W, dtype=torch.float32, device="cuda")
        for c0 in range(0, SPP, chunk):
            first.fill_(c0)
            S.generate_samples(W, H, chunk, n_features=G, seed=1234 + rank, first_index=first, out=tmp)
            host[c0:c0 + chunk].copy_(tmp)
        del tmp
        out_host = torch.empty(3, H, W, dtype=torch.float32, pin_memory=True)
        stage = [torch.empty(chunk, 5 + G, H, W, dtype=torch.float32, device="cuda") for _ in range(2)]
        copy_stream = torch.cuda.Stream()
        free = [torch.cuda.Event(), torch.cuda.Event()]
        ready = [torch.cuda.Event(), torch.cuda.Event()]
        for e in free:
            e.record(stream)

        def e2e_step():
            _reset(b, film)
            for ci, c0 in enumerate(range(0, SPP, chunk)):
                s = ci % 2
                copy_stream.wait_event(free[s])
                with torch.cuda.stream(copy_stream):
                    stage[s].copy_(host[c0:c0 + chunk], non_blocking=True)
                ready[s].record(copy_stream)
                stream.wait_event(ready[s])
                b.accumulate(stage[s], mode=S.ACC_FAST, film=film)
                free[s].record(stream)
            _denoise(S, b, film)
            out_host.copy_(b.filmD, non_blocking=True)

        for _ in range(args.warmup):
            e2e_step()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.e2e_steps):
            e2e_step()
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1) / args.e2e_steps
        e2e_val = world * HW / (max_over_ranks(e2e_ms, world, dist) / 1e3) / 1e6
        h2d = SPP * (5 + G) * HW * 4
        # the host link alone: the same chunk copies, nothing else on the GPU
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        l0.record(copy_stream)
        for ci, c0 in enumerate(range(0, SPP, chunk)):
            with torch.cuda.stream(copy_stream):
                stage[ci % 2].copy_(host[c0:c0 + chunk], non_blocking=True)
        l1.record(copy_stream)
        torch.cuda.synchronize()
        link_gbs = h2d / (l0.elapsed_time(l1) / 1e3) / 1e9
        e2e = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 3 * HW * 4, "ms_per_step": e2e_ms,
               "h2d_gbs": h2d / (e2e_ms / 1e3) / 1e9, "link_gbs_copies_alone": link_gbs,
               "path": "page-locked huge-page host samples (stater_host_alloc) -> 32-spp chunks (copy stream) -> "
                       "accumulate + film sums -> film image -> denoise -> filmD to host"}
        del host, stage
        host_buf.close()
        torch.cuda.empty_cache()

    # the other configurations, compact: LEV at 1080p/512 spp, adaptive rounds,
    # one serving rate (each with its own clock record)
    if not args.no_configs:
        extra["lev"] = measure_lev(S, 1920, 1080, 512, steps=3, warmup=1)
        extra["adaptive"] = measure_adaptive(S, steps=3, warmup=1, chunk=0)
        extra["serving"] = measure_serving(S, njobs=args.serve_jobs, rate=200.0, slots=4, chunk=0)
        extra["batch"] = measure_batch(S)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        smp = strip_samples(args.cpu_rows, seed=1)
        # repeat the strip until about 10 s of CPU work have been timed
        secs, reps = 0.0, 0
        while secs < 10.0 and reps < 64:
            _, dt = cpu_pipeline_mpix(smp, threads)
            secs += dt
            reps += 1
        v = reps * 1920 * args.cpu_rows / secs / 1e6
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{reps} x a 1920x{args.cpu_rows} strip of the workload, {secs:.1f} s (FP32 StatTile "
                         f"port + film + FP64 denoise restatement)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
                "warmup": args.warmup, "ms_per_step": total_ms / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Philox planes)",
                "config": _config(), "latency_ms": {"p50": float(np.percentile(per_step, 50)),
                                                     "p99": float(np.percentile(per_step, 99))},
                "stage_ms": {k: statistics.median(v) for k, v in stage_ms.items()},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": LAUNCHES_PER_STEP * steps, "clocks": clk.summary(), "checksum_filmD_mean": filmD_check}
        line.update(extra)
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Other configurations: serving (mixed jobs, Poisson arrivals), adaptive rounds, LEV
# ---------------------------------------------------------------------------
SERVE_RES = [(256, 256), (512, 512), (1280, 720), (1920, 1080), (3840, 2160)]
SERVE_SPP = [16, 64, 256, 1024]
SERVE_K = [1, 3, 5]


def serving_trace(njobs, seed=0):
    import numpy as np
    rng = np.random.default_rng(seed)
    tr = WORKLOAD["transforms"]
    jobs = []
    for i in range(njobs):
        w, h = SERVE_RES[rng.integers(len(SERVE_RES))]
        spp = int(SERVE_SPP[rng.integers(len(SERVE_SPP))])
        k = int(SERVE_K[rng.integers(len(SERVE_K))])
        jobs.append(dict(width=w, height=h, spp=spp, transforms=tuple(tr[:k]), radius=WORKLOAD["radius"], seed=100 + i))
    return jobs


def run_serving_trace(S, jobs, rate, slots, precision, with_output=True, seed=1, chunk=0, fuse=False):
    """Submits `jobs` at Poisson arrival times (rate jobs/s; rate <= 0: all at once)
    and returns the server statistics."""
    import numpy as np
    from stater_gb300 import serving
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, len(jobs)) if rate > 0 else np.zeros(len(jobs))
    arrivals = np.cumsum(gaps)
    outs = [np.zeros((3, j["height"], j["width"]), np.float32) if with_output else None for j in jobs]
    with serving.Server(max_slots=slots, precision=precision, chunk_spp=chunk, fuse_small_jobs=fuse) as srv:
        t0 = time.perf_counter()
        for j, o, at in zip(jobs, outs, arrivals):
            delay = at - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            srv.submit(serving.job_desc(**j, out=o), keepalive=o)
        srv.drain(3600)
        st = srv.stats()
    st["pixels"] = float(sum(j["width"] * j["height"] for j in jobs))
    return st


def measure_adaptive(S, steps, warmup, chunk, with_plain=False):
    """Adaptive sampling at 1080p through the serving engine: 16 spp, then 3
    rounds of 64 extra spp on average (targets from calcTargetSPP, clamped to
    [16, 1024]), K = 5, R = 10, moment buffers resident between rounds. One job
    at a time; the job's latency is the step."""
    import numpy as np

    from stater_gb300 import serving
    W, H = 1920, 1080
    job = dict(width=W, height=H, spp=16, rounds=4, round_spp=64, transforms=tuple(WORKLOAD["transforms"]),
               radius=WORKLOAD["radius"], seed=5)
    res = {}
    precs = ((S.F32, "f32"), (S.F64, "f64")) if with_plain else ((S.F32, "f32"),)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        for prec, name in precs:
            lat = []
            with serving.Server(max_slots=1, precision=prec, chunk_spp=chunk) as srv:
                for it in range(warmup + steps if prec == S.F32 else 2):
                    out = np.zeros((3, H, W), np.float32) if prec == S.F32 else None
                    jid = srv.submit(serving.job_desc(**job, out=out), keepalive=out)
                    srv.wait(jid, 3600)
                    lat.append(srv.poll(jid)[1])
            res[name] = lat[-steps:] if prec == S.F32 else lat[-1:]
    ms = statistics.median(res["f32"])
    r = {"value": W * H / ms / 1e3, "unit": UNIT, "ms": ms,
         "workload": "1920x1080, 16 spp then 3 rounds of 64 extra spp on average, clamped to [16, 1024] per pixel "
                     "by relative variance; K=5, R=10; moment buffers resident between rounds",
         "latency_ms": {"p50": ms, "p99": float(np.percentile(res["f32"], 99))}, "clocks": clk.summary()}
    if with_plain:
        r["plain_f64"] = {"ms_per_job": res["f64"][0], "value": W * H / res["f64"][0] / 1e3}
        r["speedup_vs_plain_f64"] = res["f64"][0] / ms
    return r


def measure_lev(S, W, H, SPP, steps, warmup, with_plain=False):
    """LEV: per-pixel ridge regression of RGB on 7 features + intercept, all SPP
    samples resident in HBM and accumulated in one call, then the FP64 solve."""
    import torch
    G = 7
    smp = S.generate_samples(W, H, SPP, n_features=G, seed=9, lev_r2=0.6)
    res = {}
    stream = torch.cuda.current_stream()
    precs = ((S.F32, "f32"), (S.F64, "f64")) if with_plain else ((S.F32, "f32"),)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        for prec, name in precs:
            lev = S.LevState(W, H, G, prec)
            times, acc_times = [], []
            em = torch.cuda.Event(enable_timing=True)
            for it in range(warmup + steps if prec == S.F32 else 2):
                lev.state.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                lev.accumulate(smp)
                em.record(stream)
                lev.solve(1e-6)
                e1.record(stream)
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
                acc_times.append(e0.elapsed_time(em))
            res[name] = statistics.median(times[-steps:]) if prec == S.F32 else times[-1]
            res[name + "_acc"] = statistics.median(acc_times[-steps:]) if prec == S.F32 else acc_times[-1]
            res[name + "_r2"] = float(lev.r2.double().median().item())
            del lev
    del smp
    torch.cuda.empty_cache()
    acc_bytes = W * H * SPP * (G + 3) * 4
    acc_gbs = acc_bytes / (res["f32_acc"] / 1e3) / 1e9
    hbm_peak, peak_source = hbm_peak_gbs()
    # DRAM bytes per launch from one ncu capture of lev_tma_f32 at 480x272, 64 spp:
    # 406.1 MB read + 58.7 MB written, of which the per-pixel state is 58.7 MB each
    # way (scaled by pixels) and the rest sample planes (scaled by pixel-samples).
    state_b, samp_b = 58.726656e6, 406.123520e6 - 58.726656e6
    traffic = (2 * state_b * (W * H) / (480 * 272) + samp_b * (W * H * SPP) / (480 * 272 * 64)) / 1e9
    r = {"value": W * H / res["f32"] / 1e3, "unit": UNIT, "ms": res["f32"],
         "workload": f"{W}x{H}, {SPP} spp, 7 features + intercept, ridge lambda 1e-6, samples resident in HBM "
                     f"({W * H * SPP * (5 + G) * 4 / 1e9:.1f} GB of planes, {acc_bytes / 1e9:.1f} GB read by the "
                     "regression)",
         "stage_ms": {"accumulate": res["f32_acc"], "solve": res["f32"] - res["f32_acc"]},
         "roofline": {"kernel": "lev_tma_f32", "bound": "hbm", "achieved": acc_gbs, "peak": hbm_peak, "unit": "GB/s",
                      "frac": acc_gbs / hbm_peak, "traffic": traffic, "algorithmic_gb": acc_bytes / 1e9,
                      "peak_source": peak_source},
         "median_r2": res["f32_r2"], "clocks": clk.summary()}
    if with_plain:
        r["plain_f64"] = {"ms_per_step": res["f64"], "median_r2": res["f64_r2"]}
        r["speedup_vs_plain_f64"] = res["f64"] / res["f32"]
    return r


def measure_batch(S, njobs=32, steps=5, seed=11):
    """Many small images (256x256 and 512x512; 16 or 64 spp; K = 1, 3 or 5;
    21x21 window), samples resident in HBM: one step denoises all of them from
    zeroed statistics, either as the per-image call sequence on one stream
    (accumulate + film sums, film image, denoiseVars, denoiseFilm) or as one
    batch (one launch per denoise stage for all images, replayed as a CUDA
    graph). Same bits either way."""
    import numpy as np
    import torch
    rng = np.random.default_rng(seed)
    tr = WORKLOAD["transforms"]
    jobs = []
    for i in range(njobs):
        side = int(rng.choice([256, 512]))
        spp = int(rng.choice([16, 64]))
        k = int(rng.choice([1, 3, 5]))
        smp = S.generate_samples(side, side, spp, n_features=7, seed=500 + i)
        b = S.StatBuffers(side, side, tr[:k], 7, 3, S.F32)
        film = S.Film(side, side, n_features=7)
        jobs.append(dict(buffers=b, film=film, samples=smp, radius=WORKLOAD["radius"], gbuffers=_specs(S)))
    pixels = sum(j["buffers"].HW for j in jobs)
    stream = torch.cuda.current_stream()

    def sequential():
        for j in jobs:
            b, film = j["buffers"], j["film"]
            _reset(b, film)
            b.accumulate(j["samples"], mode=S.ACC_FAST, film=film)
            rgb = film.update_image()
            b.denoise_vars(radius=j["radius"], gbuffers=j["gbuffers"])
            b.denoise_film(radius=j["radius"], gbuffers=j["gbuffers"], film=rgb)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for i in range(steps):
            fn()
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        return [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]

    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        seq = timed(sequential)
        batch = S.Batch(jobs, reset=True)
        bat = timed(batch.run)
    batch.close()
    seq_ms, bat_ms = statistics.median(seq), statistics.median(bat)
    out = {"value": pixels / bat_ms / 1e3, "unit": UNIT, "ms_per_step": bat_ms, "jobs": njobs,
           "pixels": pixels, "per_image_calls": {"value": pixels / seq_ms / 1e3, "ms_per_step": seq_ms},
           "speedup_vs_per_image_calls": seq_ms / bat_ms,
           "latency_ms": {"p50": float(np.percentile(bat, 50)), "p99": float(np.percentile(bat, 99))},
           "workload": f"{njobs} images of 256x256 or 512x512, 16 or 64 spp, K 1/3/5, R 10, samples resident",
           "clocks": clk.summary()}
    del jobs
    torch.cuda.empty_cache()
    return out


def small_trace(njobs, seed=0):
    """Small single-round jobs only: 256x256 or 512x512, 16 or 64 spp, K 1/3/5."""
    import numpy as np
    rng = np.random.default_rng(seed)
    tr = WORKLOAD["transforms"]
    return [dict(width=int(side), height=int(side), spp=int(rng.choice([16, 64])),
                 transforms=tuple(tr[:int(rng.choice([1, 3, 5]))]), radius=WORKLOAD["radius"], seed=700 + i)
            for i, side in enumerate(rng.choice([256, 512], size=njobs))]


def measure_serving(S, njobs, rate, slots, chunk, seed=0):
    """One Poisson arrival rate of the mixed-job trace through the serving engine."""
    jobs = serving_trace(njobs, seed=seed)
    for fuse in (False, True):  # warm-up: scratch, tables, tuned tile heights
        run_serving_trace(S, serving_trace(6, seed=99), 0, slots, S.F32, fuse=fuse)
    res = {}
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        for fuse in (True, False):
            res[fuse] = run_serving_trace(S, jobs, rate, slots, S.F32, chunk=chunk, fuse=fuse)
        # a stream of small jobs only, where fusion has work to fuse
        sjobs = small_trace(48, seed=seed)
        for fuse in (True, False):
            res[("small", fuse)] = run_serving_trace(S, sjobs, 2000.0, slots, S.F32, chunk=chunk, fuse=fuse)
    st = res[False]
    small = sum(1 for j in jobs if j["width"] * j["height"] <= 512 * 512)
    small_only = {}
    for fuse in (True, False):
        r = res[("small", fuse)]
        small_only["fused" if fuse else "not_fused"] = {
            "value": r["mpix_per_s"], "latency_ms": {"p50": r["latency_p50_ms"], "p99": r["latency_p99_ms"]}}
    return {"value": st["mpix_per_s"], "unit": UNIT, "rate_jobs_per_s": rate, "jobs": njobs, "slots": slots,
            "latency_ms": {"p50": st["latency_p50_ms"], "p99": st["latency_p99_ms"], "mean": st["latency_mean_ms"]},
            "completed": st["completed"], "failed": st["failed"], "peak_footprint_gb": st["peak_footprint_bytes"] / 1e9,
            "fused_small_jobs": False, "small_jobs": small,
            "small_jobs_only": dict(small_only, workload="48 jobs of 256x256 or 512x512, 16 or 64 spp, K 1/3/5, "
                                                          "Poisson arrivals at 2000 jobs/s"),
            "with_fusion": {"value": res[True]["mpix_per_s"],
                            "latency_ms": {"p50": res[True]["latency_p50_ms"], "p99": res[True]["latency_p99_ms"],
                                           "mean": res[True]["latency_mean_ms"]}},
            "workload": f"{njobs} jobs, resolutions {SERVE_RES}, spp {SERVE_SPP}, K {SERVE_K}, Poisson arrivals "
                        "(headline: the default engine; with_fusion: small single-round jobs waiting together fused "
                        "into groups)",
            "clocks": clk.summary()}


def measure_vars_scenes(S, steps, warmup):
    """The variance stage (statistics + ring filter) of the 1080p job on two
    scenes of the same sizes: features constant over 8x8 regions (the
    benchmark's scene) and one region over the whole image, where no range
    weight is 0 and no neighbour's records are skipped. Per tile height (the
    tuner's, then 4, 8 and 16 forced), CUDA events on the launching stream,
    median of `steps` after `warmup`; with the share of positions whose
    records are loaded and a checksum of the varD bits."""
    import torch
    w = WORKLOAD
    W, H, SPP, G = w["width"], w["height"], w["spp"], w["features"]
    lib = S.load()
    stream = torch.cuda.current_stream()
    out = {}
    for name, region in (("regions_8px", 8), ("one_region", max(W, H))):
        smp = S.generate_samples(W, H, SPP, n_features=G, seed=1234, region=region)
        b = S.StatBuffers(W, H, w["transforms"], G, w["max_moment"], S.F32)
        film = S.Film(W, H, n_features=G)
        b.accumulate(smp, mode=S.ACC_FAST, film=film)
        torch.cuda.synchronize()
        del smp
        torch.cuda.empty_cache()
        res = {}
        try:
            for th in (0, 4, 8, 16):
                if lib.stater_debug_set_vars_ring_form(th) != 0:
                    raise RuntimeError(f"variance ring form {th} refused")
                ts = []
                for i in range(warmup + steps):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    b.denoise_vars(radius=w["radius"], filter_sd=w["filter_sd"], var_z=w["var_z"], gbuffers=_specs(S))
                    e1.record(stream)
                    torch.cuda.synchronize()
                    if i >= warmup:
                        ts.append(e0.elapsed_time(e1))
                res["tuned_ms" if th == 0 else f"rows{th}_ms"] = statistics.median(ts)
        finally:
            lib.stater_debug_set_vars_ring_form(0)
        res["records_loaded"] = vars_records_loaded(b.gmean, b.n, w["gbuffers"], w["radius"], w["filter_sd"])
        res["varD_bits_sum"] = int(b.varD.contiguous().view(torch.int32).to(torch.int64).sum().item())
        out[name] = res
        del b, film
        torch.cuda.empty_cache()
    return out


def run_config(args, rank, world, dist):
    import numpy as np
    import torch

    import stater_gb300 as S
    from __graft_entry__ import build
    if rank == 0 or not (ROOT / "stater_gb300" / "libstater.so").exists():
        build()
    if world > 1:
        dist.barrier()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    S.setup()
    line = None
    if args.config == "serving":
        jobs = serving_trace(args.jobs, seed=rank)
        # warm-up: one small job per slot (scratch buffers, tables)
        run_serving_trace(S, serving_trace(4, seed=99)[:4], 0, args.slots, S.F32)
        rates = [float(r) for r in args.rates.split(",")] if args.rates else [args.rate]
        sweep = []
        with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
            for rate in rates:
                st = run_serving_trace(S, jobs, rate, args.slots, S.F32, chunk=args.chunk)
                sweep.append({"rate_jobs_per_s": rate, "mpix_per_s": st["mpix_per_s"],
                              "latency_p50_ms": st["latency_p50_ms"], "latency_p99_ms": st["latency_p99_ms"],
                              "peak_footprint_gb": st["peak_footprint_bytes"] / 1e9})
        # the headline is the highest rate of the sweep (arrivals faster than the GPU: its capacity)
        # one job at a time, plain FP64 form, on the part of the trace small enough to finish quickly
        small = [j for j in jobs if j["width"] * j["height"] * j["spp"] <= 1280 * 720 * 256][:args.f64_jobs]
        f32_small = run_serving_trace(S, small, 0, args.slots, S.F32)
        f64_small = run_serving_trace(S, small, 0, 1, S.F64, with_output=False)
        line = {"metric": "Mpix/s served (mixed jobs, Poisson arrivals)", "value": sweep[-1]["mpix_per_s"], "unit": UNIT,
                "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded on-device generation)",
                "config": {"workload": f"{len(jobs)} jobs, resolutions {SERVE_RES}, spp {SERVE_SPP}, K {SERVE_K}",
                           "rate_jobs_per_s": rates[-1], "slots": args.slots},
                "rate_sweep": sweep,
                "latency_ms": {"p50": st["latency_p50_ms"], "p99": st["latency_p99_ms"], "mean": st["latency_mean_ms"]},
                "completed": st["completed"], "failed": st["failed"], "peak_footprint_gb": st["peak_footprint_bytes"] / 1e9,
                "subset_vs_plain_f64": {"jobs": len(small), "f32_batched_mpix_s": f32_small["mpix_per_s"],
                                         "f64_one_job_per_launch_mpix_s": f64_small["mpix_per_s"],
                                         "speedup": f32_small["mpix_per_s"] / max(f64_small["mpix_per_s"], 1e-12),
                                         "f64_latency_ms": {"p50": f64_small["latency_p50_ms"],
                                                            "p99": f64_small["latency_p99_ms"]}},
                "clocks": clk.summary()}
    elif args.config == "adaptive":
        r = measure_adaptive(S, args.steps, args.warmup, args.chunk, with_plain=True)
        line = {"metric": "Mpix/s denoised, adaptive sampling 1080p 4 rounds", "value": r["value"], "unit": UNIT,
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded on-device generation)", "config": {"workload": r["workload"]},
                "latency_ms": r["latency_ms"], "plain_f64": r["plain_f64"],
                "speedup_vs_plain_f64": r["speedup_vs_plain_f64"], "clocks": r["clocks"]}
    elif args.config == "lev":
        W, H, SPP = args.width or 1920, args.height or 1080, args.spp or 512
        r = measure_lev(S, W, H, SPP, args.steps, args.warmup, with_plain=True)
        line = {"metric": "Mpix/s LEV regression (1080p, 512 spp, 7 features)", "value": r["value"],
                "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (compensated) + f64 solve",
                "data": "synthetic (seeded, radiance linear in the features, target R^2 0.6)",
                "config": {"workload": r["workload"]}, "stage_ms": r["stage_ms"], "roofline": r["roofline"],
                "median_r2": r["median_r2"], "plain_f64": r["plain_f64"],
                "speedup_vs_plain_f64": r["speedup_vs_plain_f64"], "clocks": r["clocks"]}
    elif args.config == "vars_scenes":
        with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
            scenes = measure_vars_scenes(S, args.steps, args.warmup)
        w = WORKLOAD
        line = {"metric": "ms per variance stage (stats + ring filter), 1080p K=5 R=10, benchmark scene",
                "value": scenes["regions_8px"]["tuned_ms"], "unit": "ms", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded on-device generation)",
                "config": {"workload": f"variance stage of the {w['width']}x{w['height']} {w['spp']}spp K=5 job, "
                                       "features constant over 8x8 regions (the benchmark) or over the whole image"},
                "scenes": scenes, "clocks": clk.summary()}
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="stater", choices=["stater", "reference"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-rows", type=int, default=32)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the compact LEV / adaptive / serving legs")
    ap.add_argument("--serve-jobs", type=int, default=24, help="jobs of the compact serving leg")
    ap.add_argument("--config", default="denoise", choices=["denoise", "serving", "adaptive", "lev", "vars_scenes"])
    ap.add_argument("--rate", type=float, default=10.0, help="serving: job arrivals per second")
    ap.add_argument("--rates", default="10,50,200,500", help="serving: comma-separated arrival rates to sweep")
    ap.add_argument("--jobs", type=int, default=40, help="serving: jobs in the trace")
    ap.add_argument("--slots", type=int, default=4, help="serving: concurrent jobs")
    ap.add_argument("--chunk", type=int, default=0,
                    help="serving / adaptive: samples generated and accumulated per step (0: the engine's automatic "
                         "choice, 128 for adaptive jobs, 32 for one-round jobs)")
    ap.add_argument("--f64-jobs", type=int, default=6, help="serving: jobs timed in the plain FP64 form")
    ap.add_argument("--width", type=int, default=None, help="smaller image for profiling captures")
    ap.add_argument("--height", type=int, default=None)
    ap.add_argument("--spp", type=int, default=None)
    args = ap.parse_args()
    for key in ("width", "height", "spp"):
        if getattr(args, key) is not None:
            WORKLOAD[key] = getattr(args, key)
    args.warmup = max(args.warmup, 3)
    args.spp_note = f"{WORKLOAD['spp']} spp"
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "stater" else "gloo"
        dist.init_process_group(backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank)
        elif args.config != "denoise":
            run_config(args, rank, world, dist)
        else:
            run_gpu(args, rank, world, dist)
    finally:
        if dist is not None and dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
