"""The TMA-fed accumulation's warp plan (host code in acc_kernels.cuh): every
transform on exactly one warp, every feature channel kept exactly once within
its cap, deterministic, quick for eight transforms, and the measured placement
of the five-transform benchmark set (tests/cpp/acc_plan_check.cu, built with
nvcc as host code)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CPP = Path(__file__).resolve().parent / "cpp"


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    pytest.skip("nvcc not available")


def test_acc_plan(tmp_path):
    exe = tmp_path / "acc_plan_check"
    subprocess.run([_nvcc(), "-std=c++17", "-O2", f"-I{ROOT / 'include'}", f"-I{ROOT / 'stater_gb300' / 'csrc'}",
                    str(CPP / "acc_plan_check.cu"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"
