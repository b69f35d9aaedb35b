"""The C++ drop-in: a program written against the reference's header
(gpuShareLib/GpuClauseSharer.h) compiles and links against this library
(CPU), and passes two of the reference's known-answer tests (GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp")
LIBDIR = os.path.join(ROOT, "gpusharesat_gb300")


def _build(tmp_path):
    exe = str(tmp_path / "dropin_test")
    subprocess.run(["g++", "-std=c++11", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                    "-L", LIBDIR, "-lgpusharesat", "-Wl,-rpath," + LIBDIR], check=True)
    return exe


def test_dropin_compiles_and_links(lib, tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_dropin_runs_reference_known_answers(lib, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "passed" in r.stdout
