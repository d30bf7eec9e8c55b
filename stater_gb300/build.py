"""Builds libstater.so (sm_103a) in-tree with nvcc, translation units in parallel.

Translation units that must round every operation like the CPU restatement
(the plain FP64 form, the reference-exact FP32 accumulation, target-SPP, the
FP64 LEV) are compiled with -fmad=false; the FP32 forms keep FMA contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libstater.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EXACT_UNITS = ["accumulate.cu", "denoise.cu", "target_spp.cu", "lev.cu", "film.cu"]
FAST_UNITS = ["accumulate_fast.cu", "accumulate_tma.cu", "denoise_fast.cu", "lev_fast.cu", "runtime.cu",
              "server.cu", "probe.cu", "pitched.cu"]
HOST_UNITS = ["tquantile.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*")) + [INCLUDE / "stater.h", Path(__file__)]


def _up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources() if p.is_file())


def _run(cmd: list[str]) -> tuple[list[str], int, str]:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return cmd, proc.returncode, proc.stdout


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compiles every CUDA unit for sm_103a and links libstater.so. Returns its path."""
    if not force and _up_to_date():
        return LIB
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    common = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
              f"-I{INCLUDE}", f"-I{CSRC}", "-c"]
    if ptxas_info:
        common.append("-Xptxas=-v")
    jobs = []
    for u in EXACT_UNITS:
        jobs.append(common + ["-fmad=false", str(CSRC / u), "-o", str(BUILD / (u + ".o"))])
    for u in FAST_UNITS:
        jobs.append(common + [str(CSRC / u), "-o", str(BUILD / (u + ".o"))])
    gxx = shutil.which("g++") or "g++"
    for u in HOST_UNITS:
        jobs.append([gxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}", "-c",
                     str(CSRC / u), "-o", str(BUILD / (u + ".o"))])
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=workers) as ex:
        results = list(ex.map(_run, jobs))
    failed = [(c, out) for c, rc, out in results if rc != 0]
    for c, rc, out in results:
        if verbose or rc != 0 or ptxas_info:
            if out.strip():
                sys.stderr.write(out)
    if failed:
        raise RuntimeError("libstater build failed:\n" + "\n".join(" ".join(c) for c, _ in failed))
    objs = [str(BUILD / (u + ".o")) for u in EXACT_UNITS + FAST_UNITS + HOST_UNITS]
    tmp = LIB.with_suffix(".so.tmp")
    cmd, rc, out = _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs])
    if rc != 0:
        raise RuntimeError("libstater link failed:\n" + out)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(force=force, verbose=True, ptxas_info="--ptxas" in sys.argv))
