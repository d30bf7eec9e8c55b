"""Python binding of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py as the checker. The product (stater_gb300) never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

TK = {"identity": 0, "log1p": 1, "sqrt": 2, "cbrt": 3, "asinh": 4, "boxcox": 5}
NQ = 7
MT_ALL, MT_JB = 2, 3

_lib = None


def build(force: bool = False) -> Path:
    """Compiles liboracle.so with the Makefile next to this file."""
    src = [HERE / "oracle.c", HERE / "oracle_acc.inc", HERE / "oracle.h"]
    if not force and LIB_PATH.exists() and all(p.stat().st_mtime <= LIB_PATH.stat().st_mtime for p in src):
        return LIB_PATH
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB_PATH


class GBuf(C.Structure):
    _fields_ = [("first_channel", C.c_int), ("channels", C.c_int), ("dr_factor", C.c_double)]


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB_PATH))
        _lib.orc_t_quantile.restype = C.c_double
        _lib.orc_t_quantile.argtypes = [C.c_double, C.c_double]
        _lib.orc_tree_sum.restype = C.c_double
        _lib.orc_tree_sum.argtypes = [C.c_void_p, C.c_int64]
        _lib.orc_lev_nstate.restype = C.c_int
        _lib.orc_transform_f64.restype = C.c_double
        _lib.orc_transform_f64.argtypes = [C.c_int, C.c_double, C.c_double]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def threads() -> int:
    return max(1, os.cpu_count() or 1)


def transform_arrays(transforms):
    kinds, lams = [], []
    for t in transforms:
        name, lam = (t, 1.0) if isinstance(t, str) else t
        kinds.append(TK[name] if isinstance(name, str) else int(name))
        lams.append(float(lam))
    return np.array(kinds, dtype=np.int32), lams


def accumulate(samples, K_transforms, max_moment, n, stats, gmean, count=None, precision="f64", nthreads=None):
    """In-place stage-1 update. samples float32 [S, 5+G, H, W]; n int32 [H, W];
    stats [K, 7, 3, H, W]; gmean [G, H, W] (f64 or f32 arrays)."""
    lib = load()
    S, nch, H, W = samples.shape
    G = nch - 5
    kinds, lams = transform_arrays(K_transforms)
    samples = _c(samples, np.float32)
    cnt = None if count is None else _c(count, np.int32)
    nthreads = nthreads or threads()
    if precision == "f64":
        lam = np.array(lams, dtype=np.float64)
        lib.orc_accumulate_f64(W, H, G, S, _p(samples), _p(cnt), len(kinds), _p(kinds), _p(lam), max_moment,
                               _p(n), _p(stats), _p(gmean), nthreads)
    else:
        lam = np.array(lams, dtype=np.float32)
        lib.orc_accumulate_f32(W, H, G, S, _p(samples), _p(cnt), len(kinds), _p(kinds), _p(lam), max_moment,
                               _p(n), _p(stats), _p(gmean), nthreads)


def new_state(K, G, H, W, dtype=np.float64):
    return (np.zeros((H, W), np.int32), np.zeros((K, NQ, 3, H, W), dtype), np.zeros((max(G, 1), H, W), dtype))


def gbufs(specs):
    """specs: iterable of (first_channel, channels, sigma)."""
    arr = (GBuf * max(1, len(specs)))()
    for i, (f, ch, sig) in enumerate(specs):
        arr[i].first_channel = f
        arr[i].channels = ch
        arr[i].dr_factor = float(np.float32(-0.5 / (sig * sig)))
    return arr, len(specs)


def denoise_vars(n, stats, gmean, max_moment, R, ds_factor, var_z, gspecs, m2c_ext=None, nthreads=None):
    lib = load()
    K, _, _, H, W = stats.shape
    out = {k: np.zeros((K, 3, H, W)) for k in ("lnS2", "se2", "m2C", "varD", "varCD")}
    out["jb"] = np.zeros((K, H, W))
    g, ng = gbufs(gspecs)
    stats = _c(stats, np.float64)
    gmean = _c(gmean, np.float64)
    lib.orc_denoise_vars_f64(W, H, K, max_moment, _p(_c(n, np.int32)), _p(stats), R, C.c_double(ds_factor),
                             C.c_double(var_z), ng, g, _p(gmean), _p(None if m2c_ext is None else _c(m2c_ext, np.float64)),
                             _p(out["jb"]), _p(out["lnS2"]), _p(out["se2"]), _p(out["m2C"]), _p(out["varD"]),
                             _p(out["varCD"]), nthreads or threads())
    return out


def tcrit2_table(alpha, N=1024):
    lib = load()
    t = np.zeros(N + 1)
    lib.orc_tcrit2_table(C.c_double(alpha), N, _p(t))
    return t


def denoise_film(n, stats, varD, varCD, jb, gmean, film, R, ds_factor, alpha, gspecs, mt_mode=MT_ALL,
                 use_levc=False, want_bits=False, lut=None, nthreads=None, discr_source=0, m2C=None):
    """discr_source 0: Welch discriminator from varCD (use_levc) or varD; 1 (the
    reference's CASCADE_MODE=0): from m2C (use_levc; denoise_vars' output) or the
    m2 moments, divided by n - 1."""
    lib = load()
    K, _, _, H, W = stats.shape
    if lut is None:
        lut = tcrit2_table(alpha)
    discr = np.zeros((K, 3, H, W))
    filmD = np.zeros((3, H, W))
    D = 2 * R + 1
    words = (D * D + 31) // 32
    bits = np.zeros((H * W, K, words), np.uint32) if want_bits else None
    g, ng = gbufs(gspecs)
    lib.orc_denoise_film_f64(W, H, K, _p(_c(n, np.int32)), _p(_c(stats, np.float64)), _p(_c(varD, np.float64)),
                             _p(_c(varCD, np.float64)), _p(_c(jb, np.float64)), int(use_levc), int(discr_source),
                             _p(None if m2C is None else _c(m2C, np.float64)), int(mt_mode), R,
                             C.c_double(ds_factor), len(lut) - 1, _p(_c(lut, np.float64)), ng, g,
                             _p(_c(gmean, np.float64)), _p(_c(film, np.float64)), _p(discr), _p(filmD), _p(bits),
                             nthreads or threads())
    return {"discr": discr, "filmD": filmD, "bits": bits}


def calc_target_spp(n, varD, mean, spp, eps=1e-4, tmin=16, tmax=1024, m2=None, as_source=0):
    """as_source 0 ("ASM"): from varD; 1 ("ASN"): from the sample variance m2 / (n - 1)."""
    lib = load()
    H, W = n.shape
    out = np.zeros((H, W), np.int32)
    lib.orc_calc_target_spp_src(W, H, int(spp), _p(_c(n, np.int32)),
                                _p(None if varD is None else _c(varD, np.float64)),
                                _p(None if m2 is None else _c(m2, np.float64)), int(as_source),
                                _p(None if mean is None else _c(mean, np.float64)), C.c_double(eps), tmin, tmax,
                                _p(out))
    return out


def tree_sum(v):
    v = _c(v, np.float64)
    return load().orc_tree_sum(_p(v), v.size)


def t_quantile(p, nu):
    return load().orc_t_quantile(p, nu)


def calc_mean_var_f32(n, m2):
    lib = load()
    H, W = n.shape
    out = np.zeros((3, H, W), np.float32)
    lib.orc_calc_mean_var_f32(H * W, _p(_c(n, np.int32)), _p(_c(m2, np.float32)), _p(out))
    return out


def merge_transform_tiles_f32(W, H, bounds, records):
    lib = load()
    n = np.zeros((H, W), np.int32)
    stats = np.zeros((2, NQ, 3, H, W), np.float32)
    b = _c(bounds, np.int32)
    lib.orc_merge_transform_tiles_f32(W, H, b.shape[0], _p(b), _p(_c(records, np.uint8)), _p(n), _p(stats))
    return n, stats


def merge_moments(nA, statsA, nB, statsB, max_moment):
    lib = load()
    K = statsA.shape[0]
    HW = nA.size
    lib.orc_merge_moments_f64(HW, K, max_moment, _p(nA), _p(statsA), _p(_c(nB, np.int32)), _p(_c(statsB, np.float64)))


def lev_nstate(G):
    return load().orc_lev_nstate(G)


def lev_accumulate(samples, state, count=None, nthreads=None):
    lib = load()
    S, nch, H, W = samples.shape
    lib.orc_lev_accumulate_f64(W, H, nch - 5, S, _p(_c(samples, np.float32)),
                               _p(None if count is None else _c(count, np.int32)), _p(state), nthreads or threads())


def lev_solve(state, G, H, W, lam=1e-6, nthreads=None):
    lib = load()
    beta = np.zeros((3, G + 1, H, W))
    m2C = np.zeros((3, H, W))
    r2 = np.zeros((3, H, W))
    lib.orc_lev_solve_f64(W, H, G, _p(_c(state, np.float64)), C.c_double(lam), _p(beta), _p(m2C), _p(r2),
                          nthreads or threads())
    return {"beta": beta, "m2C": m2C, "r2": r2}


def film_constants():
    """(RGB->XYZ 3x3, XYZ->RGB 3x3, luminance weights 3) as the oracle uses them."""
    lib = load()
    a = np.zeros((3, 3), np.float32)
    b = np.zeros((3, 3), np.float32)
    y = np.zeros(3, np.float32)
    lib.orc_film_constants(_p(a), _p(b), _p(y))
    return a, b, y


def film_add_samples(samples, count=None, max_lum=np.inf, state=None):
    """FilmTile::AddSample over sample planes [S][5+G][H][W]. state = (contrib_sum
    [3,H,W], weight_sum [H,W], spill [4,H,W]) continued in place; new if None."""
    lib = load()
    samples = _c(samples, np.float32)
    S, NCH, H, W = samples.shape
    if state is None:
        state = (np.zeros((3, H, W), np.float32), np.zeros((H, W), np.float32), np.zeros((4, H, W), np.float32))
    cs, ws, sp = state
    cnt = None if count is None else _c(count, np.int32)
    lib.orc_film_add_samples(W, H, NCH - 5, S, _p(samples), _p(cnt), C.c_float(max_lum), _p(cs), _p(ws), _p(sp))
    return state


def film_update_image(state, scale=1.0):
    """Film::UpdateImage: film RGB [3,H,W] from film_add_samples' state."""
    lib = load()
    cs, ws, sp = state
    H, W = ws.shape
    rgb = np.zeros((3, H, W), np.float32)
    lib.orc_film_update_image(W, H, _p(cs), _p(ws), _p(sp), C.c_float(scale), _p(rgb))
    return rgb
