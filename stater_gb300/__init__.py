"""stater_gb300: GB300-native (sm_103a) statistics hot path of StatER.

Stage 1: per-pixel online moments of radiance under K monotone transforms
(StatTile, src/statistics/estimator.h:226-324) with tile and round merges.
Stage 2: variance denoising and the Welch-t-test neighbourhood filter
(stat_denoiser::denoiseVars / denoiseFilm call sites, estimator.cpp:365-459).
Stage 3: linear explained-variance regression; target SPP for adaptive rounds.
Film: the renderer's box-filtered film and its XYZ round trip (core/film.cpp:187-222),
the input of the Welch filter for the untransformed set.

All compute runs in libstater.so (stater_gb300/csrc, C ABI in include/stater.h).
"""
from ._lib import (ACC_EXACT, ACC_FAST, AS_DENOISED, AS_SAMPLE, DISCR_DENOISED, DISCR_SAMPLE, F32, F64, MT_ALL,
                   MT_JB, NQ, Q_C2X, Q_C2Y, Q_M1, Q_M2, Q_M3, Q_M4, Q_MEAN, StaterError, load)
from .api import (MULTI_TRANSFORMS, GBUFFERS_ALBEDO_NORMAL, GBUFFERS_ALL7, REFERENCE_TRANSFORMS, Batch, Film, HostBuffer,
                  GBufferSpec, LevState, StatBuffers, bits_words, calc_mean_var, generate_samples, merge_moments, merge_tiles,
                  setup, tcrit2_table)

__all__ = [
    "ACC_EXACT", "ACC_FAST", "AS_DENOISED", "AS_SAMPLE", "DISCR_DENOISED", "DISCR_SAMPLE", "F32", "F64", "MT_ALL", "MT_JB", "NQ", "Q_C2X", "Q_C2Y", "Q_M1", "Q_M2", "Q_M3",
    "Q_M4", "Q_MEAN", "StaterError", "load", "MULTI_TRANSFORMS", "GBUFFERS_ALBEDO_NORMAL", "GBUFFERS_ALL7",
    "REFERENCE_TRANSFORMS", "Batch", "Film", "HostBuffer", "GBufferSpec", "LevState", "StatBuffers", "bits_words", "calc_mean_var",
    "generate_samples", "merge_moments", "merge_tiles", "setup", "tcrit2_table",
]
