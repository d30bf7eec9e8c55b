"""Python front end of the serving engine (stater_server_* in include/stater.h)."""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib as L
from .api import transform_codes


class ServerConfig(C.Structure):
    _fields_ = [("max_slots", C.c_int32), ("hbm_budget_bytes", C.c_double), ("precision", C.c_int32),
                ("chunk_spp", C.c_int32), ("fuse_small_jobs", C.c_int32)]


class JobDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("rounds", C.c_int32),
                ("round_spp", C.c_int32), ("n_transforms", C.c_int32), ("transforms", L.Transform * L.MAX_TRANSFORMS),
                ("n_features", C.c_int32), ("max_moment", C.c_int32), ("filter_radius", C.c_int32),
                ("filter_sd", C.c_float), ("alpha", C.c_float), ("var_z", C.c_float), ("seed", C.c_uint64),
                ("out_host", C.c_void_p)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("running", C.c_int64), ("queued", C.c_int64), ("latency_p50_ms", C.c_double),
                ("latency_p99_ms", C.c_double), ("latency_mean_ms", C.c_double), ("mpix_per_s", C.c_double),
                ("peak_footprint_bytes", C.c_double)]


_bound = False


def _bind():
    global _bound
    lib = L.load()
    if _bound:
        return lib
    st = C.c_int
    sig = {
        "stater_server_create": (st, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
        "stater_server_submit": (st, [C.c_void_p, C.POINTER(JobDesc), C.POINTER(C.c_int64)]),
        "stater_server_poll": (st, [C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
        "stater_server_wait": (st, [C.c_void_p, C.c_int64, C.c_double]),
        "stater_server_drain": (st, [C.c_void_p, C.c_double]),
        "stater_server_stats_get": (st, [C.c_void_p, C.POINTER(ServerStats)]),
        "stater_job_footprint": (C.c_double, [C.POINTER(JobDesc), C.c_int32, C.c_int32]),
        "stater_server_destroy": (st, [C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _bound = True
    return lib


def job_desc(width: int, height: int, spp: int, transforms: Sequence = ("identity", "log1p", "sqrt", "cbrt", "asinh"),
             rounds: int = 1, round_spp: int = 0, n_features: int = 7, max_moment: int = 3, radius: int = 10, filter_sd: float = 10.0,
             alpha: float = 0.01, var_z: float = 2.80703, seed: int = 0,
             out: Optional[np.ndarray] = None) -> JobDesc:
    d = JobDesc()
    d.width, d.height, d.spp, d.rounds, d.round_spp = width, height, spp, rounds, round_spp
    codes = transform_codes(transforms)
    d.n_transforms = len(codes)
    for k, (kind, lam) in enumerate(codes):
        d.transforms[k].kind = kind
        d.transforms[k].lambda_ = lam
    d.n_features, d.max_moment, d.filter_radius = n_features, max_moment, radius
    d.filter_sd, d.alpha, d.var_z, d.seed = filter_sd, alpha, var_z, seed
    if out is not None:
        if out.dtype != np.float32 or out.shape != (3, height, width) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float32 array [3, H, W]")
        d.out_host = out.ctypes.data
    return d


class Server:
    """Continuous-batching denoise server on the current CUDA device."""

    def __init__(self, max_slots: int = 4, hbm_budget_bytes: float = 0.0, precision: int = L.F32,
                 chunk_spp: int = 0, fuse_small_jobs: bool = False):
        self.lib = _bind()
        cfg = ServerConfig(max_slots, hbm_budget_bytes, precision, chunk_spp, int(bool(fuse_small_jobs)))
        h = C.c_void_p()
        L.call("stater_server_create", C.byref(cfg), C.byref(h))
        self.h = h
        self._keep = {}

    def submit(self, desc: JobDesc, keepalive=None) -> int:
        jid = C.c_int64()
        L.call("stater_server_submit", self.h, C.byref(desc), C.byref(jid))
        if keepalive is not None:
            self._keep[jid.value] = keepalive
        return jid.value

    def poll(self, jid: int):
        state = C.c_int32()
        lat = C.c_double()
        L.call("stater_server_poll", self.h, jid, C.byref(state), C.byref(lat))
        return state.value, lat.value

    def wait(self, jid: int, timeout_s: float = 600.0) -> None:
        L.call("stater_server_wait", self.h, jid, timeout_s)
        self._keep.pop(jid, None)

    def drain(self, timeout_s: float = 600.0) -> None:
        L.call("stater_server_drain", self.h, timeout_s)
        self._keep.clear()

    def stats(self) -> dict:
        s = ServerStats()
        L.call("stater_server_stats_get", self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if self.h:
            L.call("stater_server_destroy", self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def footprint(desc: JobDesc, precision: int = L.F32, chunk_spp: int = 0) -> float:
    return _bind().stater_job_footprint(C.byref(desc), precision, chunk_spp)
