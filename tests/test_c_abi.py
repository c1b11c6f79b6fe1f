"""The drop-in boundary from C: tests/c_abi/drop_in.c (an MPM life cycle through include/si_cuda.h
only) compiles as C99 with warnings as errors and links against libsi_cuda.so (CPU); it runs on the
GPU and exits 0 (GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from shaderintel_gb300 import build as B
    lib = B.build()
    exe = str(tmp_path / "drop_in")
    cmd = ["gcc", "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi", "drop_in.c"), "-o", exe, "-L", os.path.dirname(lib), "-lsi_cuda",
           "-lm", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_host_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_c_host_runs(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "stepCount 13" in r.stdout
