"""Host-side buffer surface on the CPU: the C++ headers (stater_gb300/host/)
compile and pass their checks, and the Python PFM module agrees with them
(file naming of buffer.cpp:48-63, replay ids of statpath.cpp:520-531)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from stater_gb300 import pfm

ROOT = Path(__file__).resolve().parents[1]
HOST = ROOT / "stater_gb300" / "host"
CPP = Path(__file__).resolve().parent / "cpp"


def _gxx():
    g = shutil.which("g++")
    if g is None:
        pytest.skip("g++ not available")
    return g


def test_cpp_buffer_io(tmp_path):
    exe = tmp_path / "test_host_io"
    subprocess.run([_gxx(), "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{ROOT / 'include'}", f"-I{HOST}",
                    str(CPP / "test_host_io.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "OK"
    # files written by the C++ side read back in Python
    a = pfm.read_pfm(tmp_path / "scene-64-t0-b0-film-mean.pfm")
    assert a.shape == (3, 3, 5) and np.array_equal(a.ravel(), np.arange(45, dtype=np.float32))
    n = pfm.read_pfm(tmp_path / "scene-64-t0-b0-film-n.pfm")
    assert n.shape == (1, 3, 5) and np.array_equal(n.ravel(), 1000 + np.arange(15, dtype=np.float32))


def test_estimator_header_compiles():
    cuda_inc = Path("/usr/local/cuda/include")
    if not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("CUDA headers not available")
    subprocess.run([_gxx(), "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", f"-I{ROOT / 'include'}",
                    f"-I{HOST}", f"-I{cuda_inc}", str(CPP / "estimator_demo.cpp")], check=True)


def test_python_pfm_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    rgb = rng.standard_normal((3, 7, 11)).astype(np.float32)
    one = rng.standard_normal((7, 11)).astype(np.float32)
    pfm.write_pfm(tmp_path / "a.pfm", rgb)
    pfm.write_pfm(tmp_path / "b.pfm", one)
    assert np.array_equal(pfm.read_pfm(tmp_path / "a.pfm"), rgb)
    assert np.array_equal(pfm.read_pfm(tmp_path / "b.pfm")[0], one)
    # first stored row is the bottom image row, channels interleaved
    raw = (tmp_path / "a.pfm").read_bytes()
    body = np.frombuffer(raw[raw.index(b"-1.0\n") + 5:], "<f4")
    assert np.array_equal(body[:3], rgb[:, -1, 0])


def test_python_names_match_reference():
    assert pfm.buffer_name("mean", 0, True) == "t0-b0-film-mean"
    assert pfm.buffer_name("varD", 3) == "t0-b3-varD"
    assert str(pfm.output_path("out/scene", "256", "t0-b0-film-n")) == "out/scene-256-t0-b0-film-n.pfm"
    assert str(pfm.output_path("scene", "", "filmD")) == "scene-filmD.pfm"
    assert pfm.parse_file_id("t0-b2-film-m2") == (0, 2, "film-m2")
    assert pfm.parse_file_id("t6-b0-film-mean") == (6, 0, "film-mean")
    assert pfm.parse_file_id("filmD") == (-1, -1, "")
