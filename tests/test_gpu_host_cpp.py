"""The C++ Estimator mirror (stater_gb300/host/estimator.hpp) on the GPU.

tests/cpp/estimator_demo.cpp runs the reference's per-round call sequence
(Film -> Upload -> DenoiseVars -> DenoiseMeans -> CalcTargetSPPs -> Download ->
Synchronize, statpath.cpp:176-441) through the C++ host mirror and writes every
registered buffer with the reference's file names; its replay mode reads them
back as the reference's denoise-only run does (statpath.cpp:500-560). Checks:
the C++ path equals the same pipeline through the Python API bit for bit, the
buffer names map onto the right transforms, and the replay of the written files
reproduces filmD exactly.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from stater_gb300 import pfm

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
BASE_TR = ("identity", "log1p", "sqrt", "cbrt", "asinh")


@pytest.fixture(scope="module")
def demo(tmp_path_factory):
    import stater_gb300 as S
    S.setup()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path_factory.mktemp("bin") / "estimator_demo"
    lib_dir = ROOT / "stater_gb300"
    subprocess.run([nvcc, "-std=c++17", "-O2", f"-I{ROOT / 'include'}", f"-I{lib_dir / 'host'}",
                    str(ROOT / "tests" / "cpp" / "estimator_demo.cpp"), f"-L{lib_dir}", "-lstater",
                    "-Xlinker", "-rpath", "-Xlinker", str(lib_dir), "-o", str(exe)], check=True)
    return exe


def _python_pipeline(W, H, spp, seed, R):
    import stater_gb300 as S
    b = S.StatBuffers(W, H, BASE_TR, 7, 5, S.F32)
    smp = S.generate_samples(W, H, spp, 7, seed=seed, region=8)
    film = S.Film(W, H, 7)
    film.add_samples(smp)
    rgb = film.update_image()
    b.accumulate(smp, mode=S.ACC_FAST)
    b.denoise_vars(radius=R, gbuffers=S.GBUFFERS_ALBEDO_NORMAL)
    b.denoise_film(radius=R, gbuffers=S.GBUFFERS_ALBEDO_NORMAL, film=rgb)
    target = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    b.calc_target_spp(spp, target, relative=True, eps=1e-4, tmin=16, tmax=1024)
    torch.cuda.synchronize()
    return b, rgb.cpu().numpy(), target.cpu().numpy()


def test_cpp_estimator_matches_python_and_replays(demo, tmp_path):
    W, H, spp, seed, R = 120, 72, 24, 5, 6
    run = subprocess.run([str(demo), "render", str(tmp_path), str(W), str(H), str(spp), str(seed), str(R)],
                         capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    b, rgb, target = _python_pipeline(W, H, spp, seed, R)

    def rd(name):
        return pfm.read_pfm(pfm.output_path(tmp_path / "scene", str(spp), name))

    assert np.array_equal(rd("film"), rgb)
    assert np.array_equal(rd("filmD"), b.filmD.cpu().numpy())
    assert np.array_equal(rd("targetspp")[0], target.astype(np.float32))
    stats = b.stats.cpu().numpy()
    n = b.n.cpu().numpy()
    assert np.array_equal(rd("t0-b0-film-n")[0], n.astype(np.float32))
    assert np.array_equal(rd("t0-b0-film-mean"), stats[0, 0])
    assert np.array_equal(rd("t0-b3-film-m2"), stats[0, 1])  # untransformed set repeated for every j
    for j in range(4):  # transformed set j is transform j + 1
        assert np.array_equal(rd(f"t0-b{j}-m3"), stats[j + 1, 2])
        assert np.array_equal(rd(f"t0-b{j}-varD"), b.varD[j + 1].cpu().numpy())
        assert np.array_equal(rd(f"t0-b{j}-jb")[0], b.jb[j + 1].cpu().numpy())
    assert np.array_equal(rd("t0-b0-film-discr"), b.discr[0].cpu().numpy())
    gm = b.gmean.cpu().numpy()
    assert np.array_equal(rd("t6-b0-film-mean"), gm[0:3])
    assert np.array_equal(rd("t5-b0-film-mean"), gm[3:6])
    assert np.array_equal(rd("t4-b0-film-mean")[0], gm[6])
    mv = rd("t0-b0-film-meanVar")
    m2 = stats[0, 1].astype(np.float32)
    nn = n.astype(np.float32)[None]
    with np.errstate(divide="ignore", invalid="ignore"):
        assert np.array_equal(mv, (m2 / ((nn - np.float32(1)) * nn)).astype(np.float32))

    run = subprocess.run([str(demo), "replay", str(tmp_path), str(W), str(H), str(spp), str(seed), str(R)],
                         capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    assert "read" in run.stdout and int(run.stdout.split("read ")[1].split()[0]) > 100
    replay = pfm.read_pfm(pfm.output_path(tmp_path / "replay", str(spp), "filmD"))
    assert np.array_equal(replay, rd("filmD"))
