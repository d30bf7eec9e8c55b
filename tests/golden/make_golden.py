"""Generates the golden vectors that pin the oracle's stage-1 restatement.

Runs the reference's own StatTile arithmetic (src/statistics/estimator.h of the
StatER tree, compiled in place by oracle/build_ref.sh into oracle/_ref/) on seeded
synthetic samples, the way StatPathIntegrator feeds it (16x16 tiles, two render
iterations with persistent tile state, the second with uneven per-pixel sample
counts), and stores inputs and outputs as .npz fixtures next to this script.

Needs oracle/_ref, which oracle/build_ref.sh compiles from the reference tree
named by STATER_REFERENCE; run from the repository root:
    STATER_REFERENCE=<StatER tree> bash oracle/build_ref.sh
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))
from helpers import synth_samples  # noqa: E402

OUT = Path(__file__).resolve().parent
REF = ROOT / "oracle" / "_ref"


def run_ref(lib_name, samples_rounds, counts_rounds, W, H, G, transform, max_moment, lambdas):
    lib = C.CDLL(str(REF / lib_name))
    fsize = lib.ref_float_size()
    ftype = np.float64 if fsize == 8 else np.float32
    lib.ref_create.restype = C.c_void_p
    lib.ref_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
    lib.ref_add.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lib.ref_read.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ref_destroy.argtypes = [C.c_void_p]
    nL = len(lambdas)
    h = lib.ref_create(W, H, G, nL)
    lam = np.array(lambdas, np.float32)
    for smp, cnt in zip(samples_rounds, counts_rounds):
        smp = np.ascontiguousarray(smp, np.float32)
        cptr = None if cnt is None else np.ascontiguousarray(cnt, np.int32).ctypes.data_as(C.c_void_p)
        lib.ref_add(h, smp.shape[0], smp.ctypes.data_as(C.c_void_p), cptr, transform, max_moment,
                    lam.ctypes.data_as(C.c_void_p))
    n = np.zeros(H * W, np.int64)
    stats = np.zeros((nL, 2, 7, 3, H * W), ftype)
    gmean = np.zeros((G, H * W), ftype)
    rec = np.zeros(H * W * lib.ref_pixel_record_size(), np.uint8)
    lib.ref_read(h, n.ctypes.data_as(C.c_void_p), stats.ctypes.data_as(C.c_void_p),
                 gmean.ctypes.data_as(C.c_void_p), rec.ctypes.data_as(C.c_void_p))
    lib.ref_destroy(h)
    return n.reshape(H, W), stats.reshape(nL, 2, 7, 3, H, W), gmean.reshape(G, H, W), rec


def tile_bounds(W, H, ts=16):
    b = []
    for ty in range((H + ts - 1) // ts):
        for tx in range((W + ts - 1) // ts):
            b.append((tx * ts, ty * ts, min(tx * ts + ts, W), min(ty * ts + ts, H)))
    return np.array(b, np.int32)


def main():
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)
    W, H, G = 20, 18, 7
    s1 = synth_samples(W, H, 24, G=G, seed=11, region=4, zero_prob=0.02)
    s2 = synth_samples(W, H, 16, G=G, seed=12, region=4)
    c2 = np.random.default_rng(13).integers(0, 17, size=(H, W)).astype(np.int32)
    rounds, counts = [s1, s2], [None, c2]
    cases = {}
    for prec in ("f32", "f64"):
        for mm in (1, 2, 3, 4, 5):
            n, st, gm, rec = run_ref(f"libref_{prec}.so", rounds, counts, W, H, G, 1, mm, [1.0])
            cases[f"boxcox_{prec}_mm{mm}"] = dict(n=n, stats=st[0], gmean=gm, transform=1, max_moment=mm,
                                                  lambdas=np.array([0.25], np.float32), records=rec)
        n, st, gm, rec = run_ref(f"libref_{prec}.so", rounds, counts, W, H, G, 0, 5, [1.0])
        cases[f"plain_{prec}_mm5"] = dict(n=n, stats=st[0], gmean=gm, transform=0, max_moment=5,
                                          lambdas=np.array([], np.float32), records=rec)
        lams = [0.01, 0.5, 1.0, 3.0]
        n, st, gm, rec = run_ref(f"libref_mt_{prec}.so", rounds, counts, W, H, G, 1, 5, lams)
        cases[f"mt_{prec}_mm5"] = dict(n=n, stats=st, gmean=gm, transform=1, max_moment=5,
                                       lambdas=np.array(lams, np.float32), records=rec)
    np.savez_compressed(OUT / "stattile_inputs.npz", s1=s1, s2=s2, c2=c2, bounds=tile_bounds(W, H),
                        W=W, H=H, G=G)
    for name, d in cases.items():
        keep = {k: v for k, v in d.items() if not (k == "records" and not name.startswith("boxcox_f32_mm5"))}
        np.savez_compressed(OUT / f"stattile_{name}.npz", **keep)
    print("wrote", len(cases), "cases to", OUT)


if __name__ == "__main__":
    main()
