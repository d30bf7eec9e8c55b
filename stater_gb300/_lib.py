"""ctypes binding of libstater.so (include/stater.h).

The library is loaded from this package directory. There is no fallback: if the
shared object is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libstater.so"

MAX_TRANSFORMS = 8
MAX_GBUFFERS = 8
MAX_FEATURES = 16
MAX_RADIUS = 20

F32, F64 = 0, 1
TK_IDENTITY, TK_LOG1P, TK_SQRT, TK_CBRT, TK_ASINH, TK_BOXCOX = range(6)
Q_MEAN, Q_M2, Q_M3, Q_M4, Q_C2X, Q_C2Y, Q_M1 = range(7)
NQ = 7
MT_ALL, MT_JB = 2, 3
DISCR_DENOISED, DISCR_SAMPLE = 0, 1  # the reference's CASCADE_MODE 1 / 0
AS_DENOISED, AS_SAMPLE = 0, 1        # the reference's AS_MODE 1 ("ASM") / 0 ("ASN")
ACC_EXACT, ACC_FAST = 0, 1

STATUS = {0: "STATER_OK", 1: "STATER_ERR_INVALID", 2: "STATER_ERR_CUDA", 3: "STATER_ERR_NOMEM",
          4: "STATER_ERR_UNSUPPORTED", 5: "STATER_ERR_TIMEOUT"}

VP = C.c_void_p
P8 = VP * MAX_TRANSFORMS


class Transform(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lambda_", C.c_float)]


class GBuffers(C.Structure):
    _fields_ = [("count", C.c_int32), ("planes", VP * MAX_GBUFFERS),
                ("channels", C.c_int32 * MAX_GBUFFERS), ("dr_factor", C.c_float * MAX_GBUFFERS)]


class AccumulateArgs(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("n_samples", C.c_int32),
                ("n_features", C.c_int32), ("samples", VP), ("count", VP),
                ("n_transforms", C.c_int32), ("transforms", Transform * MAX_TRANSFORMS),
                ("max_moment", C.c_int32), ("precision", C.c_int32), ("mode", C.c_int32),
                ("n", VP), ("stats", VP), ("gmean", VP),
                ("film_contrib_sum", VP), ("film_weight_sum", VP), ("film_spill", VP),
                ("film_max_sample_luminance", C.c_float), ("pixel_index", VP), ("n_active", C.c_int32)]


class GenerateArgs(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("n_samples", C.c_int32),
                ("n_features", C.c_int32), ("seed", C.c_uint64), ("region", C.c_int32),
                ("mean_mu", C.c_float), ("mean_sigma", C.c_float), ("noise_sigma", C.c_float),
                ("firefly_prob", C.c_float), ("firefly_scale", C.c_float), ("lev_r2", C.c_float),
                ("first_index", VP), ("count", VP), ("samples", VP), ("pixel_index", VP), ("n_active", C.c_int32)]


class DenoiseVarsArgs(C.Structure):
    _fields_ = [("n_buffers", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("filter_radius", C.c_int32), ("ds_factor", C.c_float), ("var_z", C.c_float),
                ("max_moment", C.c_int32), ("precision", C.c_int32), ("n", VP),
                ("m2", P8), ("m3", P8), ("m4", P8), ("c2X", P8), ("c2Y", P8), ("m2C_in", VP),
                ("gbuffers", GBuffers),
                ("jb", P8), ("lnS2", P8), ("se2", P8), ("m2C", P8), ("varD", P8), ("varCD", P8)]


class DenoiseFilmArgs(C.Structure):
    _fields_ = [("n_buffers", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("filter_radius", C.c_int32), ("ds_factor", C.c_float), ("alpha", C.c_float),
                ("mt_mode", C.c_int32), ("use_levc", C.c_int32), ("precision", C.c_int32),
                ("n", VP), ("film", VP), ("mean", P8), ("varD", P8), ("varCD", P8), ("jb", P8),
                ("gbuffers", GBuffers), ("discr", P8), ("filmD", VP), ("accept_bits", VP),
                ("test_order", C.c_int32 * MAX_TRANSFORMS), ("discr_source", C.c_int32), ("m2", P8), ("m2C", P8)]


class TargetSppArgs(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("precision", C.c_int32),
                ("n", VP), ("m2", VP), ("varD", VP), ("mean", VP), ("eps", C.c_double), ("tmin", C.c_int32),
                ("tmax", C.c_int32), ("as_source", C.c_int32), ("targetspp", VP)]


class BatchJob(C.Structure):
    _fields_ = [("acc", AccumulateArgs), ("film_rgb", VP), ("film_scale", C.c_float), ("vars", DenoiseVarsArgs),
                ("film", DenoiseFilmArgs)]


class PitchedLayout(C.Structure):
    _fields_ = [("rgb_step", C.c_int64), ("scalar_step", C.c_int64), ("n_step", C.c_int64)]


class StaterError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed with {STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


class FilmArgs(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("n_samples", C.c_int32),
                ("n_features", C.c_int32), ("samples", VP), ("count", VP),
                ("max_sample_luminance", C.c_float), ("contrib_sum", VP), ("weight_sum", VP), ("spill", VP)]


def load() -> C.CDLL:
    """Loads libstater.so from the package directory (raises if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m stater_gb300.build` "
                           "or __graft_entry__.build()")
    lib = C.CDLL(str(LIB_PATH), mode=os.RTLD_GLOBAL if hasattr(os, "RTLD_GLOBAL") else 0)
    st = C.c_int
    sig = {
        "stater_setup": (st, []),
        "stater_synchronize": (st, [VP]),
        "stater_print_macro_configuration": (None, []),
        "stater_last_error": (C.c_char_p, []),
        "stater_abi_version": (C.c_int32, []),
        "stater_release_cache": (st, []),
        "stater_host_alloc": (st, [C.c_size_t, C.POINTER(VP)]),
        "stater_host_free": (st, [VP, C.c_size_t]),
        "stater_debug_set_pipeline_waits": (st, [C.c_uint32, C.c_int32]),
        "stater_debug_set_warp_order": (st, [VP, C.c_int32]),
        "stater_debug_set_vars_ring_form": (st, [C.c_int32]),
        "stater_fp32_peak_probe": (st, [C.c_int32, C.c_int32, C.c_int32, VP, C.POINTER(C.c_double), VP]),
        "stater_accumulate": (st, [C.POINTER(AccumulateArgs), VP]),
        "stater_generate_samples": (st, [C.POINTER(GenerateArgs), VP]),
        "stater_merge_tiles": (st, [C.c_int32, C.c_int32, C.c_int32, VP, VP, C.c_int32, VP, VP, VP]),
        "stater_merge_moments": (st, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, VP, VP, VP, VP, VP]),
        "stater_denoise_vars": (st, [C.POINTER(DenoiseVarsArgs), VP]),
        "stater_denoise_film": (st, [C.POINTER(DenoiseFilmArgs), VP]),
        "stater_denoise_vars_pitched": (st, [C.POINTER(DenoiseVarsArgs), C.POINTER(PitchedLayout), VP]),
        "stater_denoise_film_pitched": (st, [C.POINTER(DenoiseFilmArgs), C.POINTER(PitchedLayout), VP]),
        "stater_calc_target_spp_pitched": (st, [C.POINTER(TargetSppArgs), C.POINTER(PitchedLayout), VP]),
        "stater_tcrit_lut_intervals": (C.c_int32, []),
        "stater_tcrit2_table": (st, [C.c_double, VP]),
        "stater_t_quantile": (C.c_double, [C.c_double, C.c_double]),
        "stater_calc_target_spp": (st, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, VP, VP, VP, C.c_double,
                                        C.c_int32, C.c_int32, VP, VP]),
        "stater_calc_target_spp_ex": (st, [C.POINTER(TargetSppArgs), VP]),
        "stater_calc_target_spp_noalloc": (st, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, VP, VP, VP,
                                                C.c_double, C.c_int32, C.c_int32, VP, VP]),
        "stater_calc_mean_var": (st, [C.c_int32, C.c_int32, VP, VP, VP, VP]),
        "stater_film_add_samples": (st, [C.POINTER(FilmArgs), VP]),
        "stater_test_order": (st, [C.POINTER(Transform), C.c_int32, VP]),
        "stater_set_autotune": (st, [C.c_int32]),
        "stater_batch_create": (st, [C.POINTER(BatchJob), C.c_int32, C.c_int32, C.POINTER(VP)]),
        "stater_batch_run": (st, [VP, VP]),
        "stater_batch_destroy": (st, [VP]),
        "stater_tuned_tile_height": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
        "stater_film_update_image": (st, [C.c_int32, C.c_int32, VP, VP, VP, C.c_float, VP, VP]),
        "stater_lev_state_size": (C.c_int32, [C.c_int32, C.c_int32]),
        "stater_lev_accumulate": (st, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, VP, VP, C.c_int32, VP, VP]),
        "stater_lev_solve": (st, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, VP, C.c_double, VP, VP, VP, VP]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def call(name: str, *args) -> None:
    """Calls a status-returning entry point; raises StaterError on failure."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.stater_last_error().decode(errors="replace")
        raise StaterError(name, rc, msg)
