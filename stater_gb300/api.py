"""Python front end of libstater over device-resident torch tensors.

`StatBuffers` holds the statistics buffers of one image the way the reference's
Estimator does (estimator.h:459-519, estimator.cpp:83-245): per transform b and
per BUF_LIST name one RGB buffer, plus the per-pixel sample count n. Here every
buffer is a planar [3, H, W] slice of one contiguous tensor, so pointer tables
for the C ABI are plain offsets.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import torch

from . import _lib as L

TRANSFORM_NAMES = {"identity": L.TK_IDENTITY, "log1p": L.TK_LOG1P, "sqrt": L.TK_SQRT,
                   "cbrt": L.TK_CBRT, "asinh": L.TK_ASINH, "boxcox": L.TK_BOXCOX}

# The five monotone transforms of the multi-transform configuration.
MULTI_TRANSFORMS = (("identity", 1.0), ("log1p", 1.0), ("sqrt", 1.0), ("cbrt", 1.0), ("asinh", 1.0))
# The reference's default single Box-Cox build: t0 raw + t1 Box-Cox(0.25) (estimator.h:48-56).
REFERENCE_TRANSFORMS = (("identity", 1.0), ("boxcox", 0.25))


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    if t is None:
        return None
    return t.data_ptr()


def _stream_ptr(stream: Optional[torch.cuda.Stream]) -> Optional[int]:
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream or None


def _dtype(precision: int) -> torch.dtype:
    return torch.float64 if precision == L.F64 else torch.float32


def transform_codes(transforms: Sequence) -> list[tuple[int, float]]:
    out = []
    for t in transforms:
        if isinstance(t, str):
            out.append((TRANSFORM_NAMES[t], 1.0))
        else:
            name, lam = t
            out.append((TRANSFORM_NAMES[name] if isinstance(name, str) else int(name), float(lam)))
    return out


@dataclass
class GBufferSpec:
    """A G-buffer for a range kernel: `channels` feature channels starting at
    `first` in the feature-mean planes, with range standard deviation `sigma`
    (dr factor -0.5/sigma^2, estimator.cpp:10-18)."""
    first: int
    channels: int
    sigma: float


# albedo RGB, normal xyz, depth (feature channel order of the synthetic scenes)
GBUFFERS_ALBEDO_NORMAL = (GBufferSpec(0, 3, 0.02), GBufferSpec(3, 3, 0.1))
GBUFFERS_ALL7 = (GBufferSpec(0, 3, 0.02), GBufferSpec(3, 3, 0.1), GBufferSpec(6, 1, 0.1))


class StatBuffers:
    """Device buffers of one image: moments, feature means and denoiser outputs."""

    def __init__(self, width: int, height: int, transforms=MULTI_TRANSFORMS, n_features: int = 7,
                 max_moment: int = 3, precision: int = L.F32, device="cuda"):
        self.W, self.H = int(width), int(height)
        self.HW = self.W * self.H
        self.transforms = transform_codes(transforms)
        self.K = len(self.transforms)
        self.G = int(n_features)
        self.max_moment = int(max_moment)
        self.precision = int(precision)
        dt = _dtype(precision)
        dev = torch.device(device)
        H, W, K = self.H, self.W, self.K
        self.n = torch.zeros(H, W, dtype=torch.int32, device=dev)
        self.stats = torch.zeros(K, L.NQ, 3, H, W, dtype=dt, device=dev)
        self.gmean = torch.zeros(max(self.G, 1), H, W, dtype=dt, device=dev)
        self.jb = torch.zeros(K, H, W, dtype=dt, device=dev)
        self.lnS2 = torch.zeros(K, 3, H, W, dtype=dt, device=dev)
        self.se2 = torch.zeros_like(self.lnS2)
        self.m2C = torch.zeros_like(self.lnS2)
        self.varD = torch.zeros_like(self.lnS2)
        self.varCD = torch.zeros_like(self.lnS2)
        self.discr = torch.zeros_like(self.lnS2)
        self.filmD = torch.zeros(3, H, W, dtype=dt, device=dev)

    # -- helpers ---------------------------------------------------------------
    def moment(self, k: int, q: int) -> torch.Tensor:
        return self.stats[k, q]

    def reset(self) -> None:
        self.n.zero_()
        self.stats.zero_()
        self.gmean.zero_()

    def _gbuffers(self, specs: Sequence[GBufferSpec]) -> L.GBuffers:
        g = L.GBuffers()
        g.count = len(specs)
        for i, s in enumerate(specs):
            if s.first + s.channels > self.G:
                raise ValueError("G-buffer spec outside the feature channels")
            g.planes[i] = _ptr(self.gmean[s.first])
            g.channels[i] = s.channels
            g.dr_factor[i] = -0.5 / (s.sigma * s.sigma)
        return g

    # -- stage 1 -----------------------------------------------------------------
    def accumulate(self, samples: torch.Tensor, count: Optional[torch.Tensor] = None, mode: int = L.ACC_EXACT,
                   film: Optional["Film"] = None, pixel_index: Optional[torch.Tensor] = None,
                   stream=None) -> None:
        """StatTile::AddTransformSample* over sample planes [S, 5+G, H, W] (float32);
        with `film`, also FilmTile::AddSample of the same samples in the same pass.
        With `pixel_index` (int32 [N]), the planes are [S, 5+G, N] and column i
        belongs to pixel pixel_index[i] (count, if given, is per column)."""
        if samples.dtype != torch.float32 or not samples.is_contiguous():
            raise ValueError("samples must be contiguous float32 [S, 5+G, H, W]")
        S = samples.shape[0]
        if pixel_index is not None:
            if samples.dim() != 3 or samples.shape[1:] != (5 + self.G, pixel_index.numel()):
                raise ValueError("with pixel_index the samples are [S, 5+G, N]")
        elif samples.shape[1:] != (5 + self.G, self.H, self.W):
            raise ValueError(f"samples shape {tuple(samples.shape)} does not match the buffers")
        a = self._acc_args(samples, count, mode, film, pixel_index)
        L.call("stater_accumulate", C.byref(a), _stream_ptr(stream))

    def _acc_args(self, samples, count, mode, film, pixel_index=None) -> L.AccumulateArgs:
        S = samples.shape[0]
        a = L.AccumulateArgs()
        a.width, a.height, a.n_samples, a.n_features = self.W, self.H, S, self.G
        a.samples, a.count = _ptr(samples), _ptr(count)
        a.n_transforms = self.K
        for k, (kind, lam) in enumerate(self.transforms):
            a.transforms[k].kind = kind
            a.transforms[k].lambda_ = lam
        a.max_moment, a.precision, a.mode = self.max_moment, self.precision, int(mode)
        a.n, a.stats, a.gmean = _ptr(self.n), _ptr(self.stats), _ptr(self.gmean)
        if pixel_index is not None:
            a.pixel_index, a.n_active = _ptr(pixel_index), int(pixel_index.numel())
        if film is not None:
            if (film.W, film.H, film.G) != (self.W, self.H, self.G):
                raise ValueError("film geometry does not match the buffers")
            a.film_contrib_sum, a.film_weight_sum = _ptr(film.contrib_sum), _ptr(film.weight_sum)
            a.film_spill, a.film_max_sample_luminance = _ptr(film.spill), film.max_sample_luminance
        return a

    # -- stage 2 -----------------------------------------------------------------
    def denoise_vars(self, radius: int = 10, filter_sd: float = 10.0, var_z: float = 2.80703,
                     gbuffers: Sequence[GBufferSpec] = GBUFFERS_ALBEDO_NORMAL,
                     m2c_in: Optional[torch.Tensor] = None, stream=None) -> None:
        a = self._vars_args(radius, filter_sd, var_z, gbuffers, m2c_in)
        L.call("stater_denoise_vars", C.byref(a), _stream_ptr(stream))

    def _vars_args(self, radius=10, filter_sd=10.0, var_z=2.80703, gbuffers=GBUFFERS_ALBEDO_NORMAL,
                   m2c_in=None) -> L.DenoiseVarsArgs:
        a = L.DenoiseVarsArgs()
        a.n_buffers, a.width, a.height = self.K, self.W, self.H
        a.filter_radius, a.ds_factor, a.var_z = int(radius), -0.5 / (filter_sd * filter_sd), float(var_z)
        a.max_moment, a.precision, a.n = self.max_moment, self.precision, _ptr(self.n)
        for k in range(self.K):
            a.m2[k] = _ptr(self.stats[k, L.Q_M2])
            a.m3[k] = _ptr(self.stats[k, L.Q_M3])
            a.m4[k] = _ptr(self.stats[k, L.Q_M4])
            a.c2X[k] = _ptr(self.stats[k, L.Q_C2X])
            a.c2Y[k] = _ptr(self.stats[k, L.Q_C2Y])
            a.jb[k] = _ptr(self.jb[k])
            a.lnS2[k] = _ptr(self.lnS2[k])
            a.se2[k] = _ptr(self.se2[k])
            a.m2C[k] = _ptr(self.m2C[k])
            a.varD[k] = _ptr(self.varD[k])
            a.varCD[k] = _ptr(self.varCD[k])
        a.m2C_in = _ptr(m2c_in)
        a.gbuffers = self._gbuffers(gbuffers)
        return a

    def denoise_film(self, radius: int = 10, filter_sd: float = 10.0, alpha: float = 0.01,
                     gbuffers: Sequence[GBufferSpec] = GBUFFERS_ALBEDO_NORMAL, mt_mode: int = L.MT_ALL,
                     use_levc: bool = False, film: Optional[torch.Tensor] = None,
                     accept_bits: Optional[torch.Tensor] = None, cascade: bool = True, stream=None) -> None:
        """denoiseFilm. cascade=False is the reference's CASCADE_MODE=0 build (the
        "M" variant): the Welch discriminator uses each pixel's own sample
        variance (m2, or the LEV-corrected m2C with use_levc) instead of the
        denoised variance of denoise_vars."""
        a = self._film_args(radius, filter_sd, alpha, gbuffers, mt_mode, use_levc, film, accept_bits, cascade)
        L.call("stater_denoise_film", C.byref(a), _stream_ptr(stream))

    def _film_args(self, radius=10, filter_sd=10.0, alpha=0.01, gbuffers=GBUFFERS_ALBEDO_NORMAL, mt_mode=L.MT_ALL,
                   use_levc=False, film=None, accept_bits=None, cascade=True) -> L.DenoiseFilmArgs:
        a = L.DenoiseFilmArgs()
        a.n_buffers, a.width, a.height = self.K, self.W, self.H
        a.filter_radius, a.ds_factor, a.alpha = int(radius), -0.5 / (filter_sd * filter_sd), float(alpha)
        a.mt_mode, a.use_levc, a.precision = int(mt_mode), int(bool(use_levc)), self.precision
        a.n = _ptr(self.n)
        a.film = _ptr(film if film is not None else self.stats[0, L.Q_MEAN])
        for k in range(self.K):
            a.mean[k] = _ptr(self.stats[k, L.Q_MEAN])
            a.varD[k] = _ptr(self.varD[k])
            a.varCD[k] = _ptr(self.varCD[k])
            a.jb[k] = _ptr(self.jb[k])
            a.discr[k] = _ptr(self.discr[k])
            a.m2[k] = _ptr(self.stats[k, L.Q_M2])
            a.m2C[k] = _ptr(self.m2C[k])
        a.discr_source = L.DISCR_DENOISED if cascade else L.DISCR_SAMPLE
        a.filmD = _ptr(self.filmD)
        a.accept_bits = _ptr(accept_bits)
        a.gbuffers = self._gbuffers(gbuffers)
        tr = (L.Transform * L.MAX_TRANSFORMS)()
        for k, (kind, lam) in enumerate(self.transforms):
            tr[k].kind, tr[k].lambda_ = kind, lam
        L.call("stater_test_order", tr, self.K, C.cast(a.test_order, C.c_void_p))
        return a

    def calc_target_spp(self, spp: int, out: torch.Tensor, relative: bool = True, eps: float = 1e-4,
                        tmin: int = 16, tmax: int = 1024, as_source: int = L.AS_DENOISED, stream=None) -> None:
        """calcTargetSPP. as_source=AS_SAMPLE is the reference's AS_MODE=0 build
        ("ASN": the sample variance m2 / (n - 1) instead of the denoised varD)."""
        mean = self.stats[0, L.Q_MEAN] if relative else None
        if as_source == L.AS_DENOISED:
            L.call("stater_calc_target_spp", self.W, self.H, int(spp), self.precision, _ptr(self.n),
                   _ptr(self.varD[0]), _ptr(mean), float(eps), int(tmin), int(tmax), _ptr(out),
                   _stream_ptr(stream))
            return
        a = L.TargetSppArgs()
        a.width, a.height, a.spp, a.precision = self.W, self.H, int(spp), self.precision
        a.n, a.m2, a.varD, a.mean = _ptr(self.n), _ptr(self.stats[0, L.Q_M2]), _ptr(self.varD[0]), _ptr(mean)
        a.eps, a.tmin, a.tmax, a.as_source, a.targetspp = float(eps), int(tmin), int(tmax), int(as_source), _ptr(out)
        L.call("stater_calc_target_spp_ex", C.byref(a), _stream_ptr(stream))


def bits_words(radius: int) -> int:
    d = 2 * radius + 1
    return (d * d + 31) // 32


def generate_samples(width: int, height: int, n_samples: int, n_features: int = 7, seed: int = 0,
                     region: int = 8, mean_mu: float = -1.0, mean_sigma: float = 1.0, noise_sigma: float = 0.5,
                     firefly_prob: float = 1e-3, firefly_scale: float = 1e3, lev_r2: float = 0.0,
                     first_index: Optional[torch.Tensor] = None, count: Optional[torch.Tensor] = None,
                     out: Optional[torch.Tensor] = None, pixel_index: Optional[torch.Tensor] = None,
                     device="cuda", stream=None) -> torch.Tensor:
    """Seeded synthetic sample planes [S, 5+G, H, W] generated on the device
    ([S, 5+G, N] for the pixels of `pixel_index`)."""
    if out is None:
        shape = (n_samples, 5 + n_features, pixel_index.numel()) if pixel_index is not None else \
            (n_samples, 5 + n_features, height, width)
        out = torch.empty(*shape, dtype=torch.float32, device=device)
    g = L.GenerateArgs()
    g.width, g.height, g.n_samples, g.n_features = width, height, n_samples, n_features
    g.seed, g.region = int(seed), int(region)
    g.mean_mu, g.mean_sigma, g.noise_sigma = mean_mu, mean_sigma, noise_sigma
    g.firefly_prob, g.firefly_scale, g.lev_r2 = firefly_prob, firefly_scale, lev_r2
    g.first_index, g.count, g.samples = _ptr(first_index), _ptr(count), _ptr(out)
    if pixel_index is not None:
        g.pixel_index, g.n_active = _ptr(pixel_index), int(pixel_index.numel())
    L.call("stater_generate_samples", C.byref(g), _stream_ptr(stream))
    return out


def merge_tiles(width: int, height: int, bounds: torch.Tensor, records: torch.Tensor, n_sets: int,
                n: torch.Tensor, stats: torch.Tensor, stream=None) -> None:
    L.call("stater_merge_tiles", width, height, int(bounds.shape[0]), _ptr(bounds), _ptr(records), int(n_sets),
           _ptr(n), _ptr(stats), _stream_ptr(stream))


def merge_moments(a: StatBuffers, b: StatBuffers, stream=None) -> None:
    L.call("stater_merge_moments", a.W, a.H, a.K, a.max_moment, a.precision, _ptr(a.n), _ptr(a.stats),
           _ptr(b.n), _ptr(b.stats), _stream_ptr(stream))


def calc_mean_var(width: int, height: int, n: torch.Tensor, m2: torch.Tensor, out: torch.Tensor,
                  stream=None) -> None:
    L.call("stater_calc_mean_var", width, height, _ptr(n), _ptr(m2), _ptr(out), _stream_ptr(stream))


class Film:
    """The renderer's film (pbrt-v3 Film + FilmTiles with the box filter of radius
    0.5): per-pixel radiance sums that persist across rounds, and the RGB image
    Film::UpdateImage makes of them, which denoise_film takes as `film`."""

    def __init__(self, width: int, height: int, n_features: int = 7, max_sample_luminance: float = float("inf"),
                 scale: float = 1.0, device="cuda"):
        self.W, self.H, self.G = int(width), int(height), int(n_features)
        self.max_sample_luminance, self.scale = float(max_sample_luminance), float(scale)
        dev = torch.device(device)
        self.contrib_sum = torch.zeros(3, self.H, self.W, dtype=torch.float32, device=dev)
        self.weight_sum = torch.zeros(self.H, self.W, dtype=torch.float32, device=dev)
        self.spill = torch.zeros(4, self.H, self.W, dtype=torch.float32, device=dev)
        self.rgb = torch.zeros(3, self.H, self.W, dtype=torch.float32, device=dev)

    def clear(self) -> None:
        self.contrib_sum.zero_()
        self.weight_sum.zero_()
        self.spill.zero_()

    def add_samples(self, samples: torch.Tensor, count: Optional[torch.Tensor] = None, stream=None) -> None:
        """FilmTile::AddSample for sample planes [S, 5+G, H, W] (float32)."""
        if samples.dtype != torch.float32 or not samples.is_contiguous() or \
                samples.shape[1:] != (5 + self.G, self.H, self.W):
            raise ValueError("samples must be contiguous float32 [S, 5+G, H, W] of the film's size")
        a = L.FilmArgs()
        a.width, a.height, a.n_samples, a.n_features = self.W, self.H, samples.shape[0], self.G
        a.samples, a.count = _ptr(samples), _ptr(count)
        a.max_sample_luminance = self.max_sample_luminance
        a.contrib_sum, a.weight_sum, a.spill = _ptr(self.contrib_sum), _ptr(self.weight_sum), _ptr(self.spill)
        L.call("stater_film_add_samples", C.byref(a), _stream_ptr(stream))

    def update_image(self, stream=None) -> torch.Tensor:
        """Film::UpdateImage: writes and returns the film RGB planes [3, H, W]."""
        L.call("stater_film_update_image", self.W, self.H, _ptr(self.contrib_sum), _ptr(self.weight_sum),
               _ptr(self.spill), self.scale, _ptr(self.rgb), _stream_ptr(stream))
        return self.rgb


class LevState:
    """Per-pixel LEV accumulation state and the regression outputs."""

    def __init__(self, width: int, height: int, n_features: int = 7, precision: int = L.F64, device="cuda"):
        self.W, self.H, self.G, self.precision = width, height, n_features, precision
        lib = L.load()
        ns = lib.stater_lev_state_size(n_features, precision)
        if ns <= 0:
            raise ValueError("unsupported number of features for LEV")
        dt = _dtype(precision)
        self.state = torch.zeros(ns, height, width, dtype=dt, device=device)
        self.beta = torch.zeros(3, n_features + 1, height, width, dtype=dt, device=device)
        self.m2C = torch.zeros(3, height, width, dtype=dt, device=device)
        self.r2 = torch.zeros(3, height, width, dtype=dt, device=device)

    def accumulate(self, samples: torch.Tensor, count: Optional[torch.Tensor] = None, stream=None) -> None:
        L.call("stater_lev_accumulate", self.W, self.H, self.G, int(samples.shape[0]), _ptr(samples),
               _ptr(count), self.precision, _ptr(self.state), _stream_ptr(stream))

    def solve(self, lam: float = 1e-6, stream=None) -> None:
        L.call("stater_lev_solve", self.W, self.H, self.G, self.precision, _ptr(self.state), float(lam),
               _ptr(self.beta), _ptr(self.m2C), _ptr(self.r2), _stream_ptr(stream))


class Batch:
    """Several images through one launch per denoise stage (stater_batch_*).

    Each job is a dict with `buffers` (an FP32 StatBuffers), `film` (its Film),
    `samples` (planes [S, 5+G, H, W]) and optionally `count`, `radius`,
    `filter_sd`, `alpha`, `var_z`, `gbuffers` (both filters), `mt_mode`,
    `use_levc`, `cascade`. One run accumulates every job's samples (with the film
    sums), makes its film image and runs denoise_vars and denoise_film, each
    image giving the same bits as those calls made one by one. With reset=True
    every run starts from zeroed statistics and film sums. The first run tunes
    and records a CUDA graph; later runs replay it. The buffers must outlive the
    batch."""

    def __init__(self, jobs, reset: bool = True):
        arr = (L.BatchJob * len(jobs))()
        for i, j in enumerate(jobs):
            b, film = j["buffers"], j["film"]
            if b.precision != L.F32:
                raise ValueError("a batch runs the FP32 form")
            g = j.get("gbuffers", GBUFFERS_ALBEDO_NORMAL)
            R, sd = j.get("radius", 10), j.get("filter_sd", 10.0)
            arr[i].acc = b._acc_args(j["samples"], j.get("count"), L.ACC_FAST, film)
            arr[i].film_rgb, arr[i].film_scale = _ptr(film.rgb), film.scale
            arr[i].vars = b._vars_args(R, sd, j.get("var_z", 2.80703), g)
            arr[i].film = b._film_args(R, sd, j.get("alpha", 0.01), g, j.get("mt_mode", L.MT_ALL),
                                       j.get("use_levc", False), film.rgb, None, j.get("cascade", True))
        self._jobs = list(jobs)
        self._h = C.c_void_p()
        L.call("stater_batch_create", arr, len(jobs), int(bool(reset)), C.byref(self._h))

    def run(self, stream=None) -> None:
        L.call("stater_batch_run", self._h, _stream_ptr(stream))

    def close(self) -> None:
        if self._h:
            L.call("stater_batch_destroy", self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HostBuffer:
    """Page-locked host memory on huge pages (stater_host_alloc), viewed as a
    float32 torch tensor of `shape` on the CPU: the source of host-to-device
    sample copies that run at the link's rate every time."""

    def __init__(self, shape, dtype=torch.float32):
        import numpy as np
        n = 1
        for d in shape:
            n *= int(d)
        self.bytes = n * torch.empty(0, dtype=dtype).element_size()
        self._ptr = C.c_void_p()
        L.call("stater_host_alloc", self.bytes, C.byref(self._ptr))
        np_dtype = {torch.float32: np.float32, torch.int32: np.int32, torch.float64: np.float64}[dtype]
        buf = (C.c_char * self.bytes).from_address(self._ptr.value)
        self.tensor = torch.from_numpy(np.frombuffer(buf, dtype=np_dtype).reshape(shape))

    def close(self) -> None:
        if self._ptr:
            self.tensor = None
            L.call("stater_host_free", self._ptr, self.bytes)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def setup() -> None:
    L.call("stater_setup")


def tcrit2_table(alpha: float):
    import numpy as np
    lib = L.load()
    n = lib.stater_tcrit_lut_intervals()
    out = np.zeros(n + 1, dtype=np.float64)
    L.call("stater_tcrit2_table", float(alpha), out.ctypes.data)
    return out
