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


# ---- the reference's own solvers, built unchanged against this library ----
#
# The consumer Makefiles compile every .cc of the solver's gpu directory and
# of its DEPDIR directories except their Main.cc (mtl/template.mk:14-17,
# glucose-syrup/gpu/Makefile:9, rel-newtech/gpu/Makefile:9). gpuShareLib is
# dropped from DEPDIR: its headers come from include/ (first on the include
# path) and its code from libgpusharesat.so. The sources are read where they
# lie in the reference tree, named by the GPUSHARESAT_REFERENCE environment
# variable (the tests skip without it; the outputs go to pytest's temporary
# directory).
REFERENCE = os.environ.get("GPUSHARESAT_REFERENCE")
SOLVERS = {
    "glucose-syrup": ["glucose-syrup/mtl", "glucose-syrup/utils", "glucose-syrup/core", "glucose-syrup/simp",
                      "glucose-syrup/satUtils"],
    "rel-newtech": ["rel-newtech/mtl", "rel-newtech/utils", "rel-newtech/core", "rel-newtech/simp",
                    "rel-newtech/satUtils"],
}


def _solver_sources(name):
    import glob
    srcs = sorted(glob.glob(os.path.join(REFERENCE, name, "gpu", "*.cc")))
    for d in SOLVERS[name]:
        srcs += [f for f in sorted(glob.glob(os.path.join(REFERENCE, d, "*.cc"))) if os.path.basename(f) != "Main.cc"]
    return srcs


@pytest.mark.parametrize("name", sorted(SOLVERS))
def test_reference_solver_builds_unchanged(lib, tmp_path, name):
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, name, "gpu")):
        pytest.skip("GPUSHARESAT_REFERENCE does not name a checkout of the reference's solver sources")
    from concurrent.futures import ThreadPoolExecutor
    srcs = _solver_sources(name)
    assert len(srcs) >= 10

    def compile_one(src):
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        r = subprocess.run(["g++", "-std=c++11", "-O0", "-w", "-I", os.path.join(ROOT, "include"), "-I", REFERENCE,
                            "-D", "__STDC_LIMIT_MACROS", "-D", "__STDC_FORMAT_MACROS", "-c", src, "-o", obj],
                           capture_output=True, text=True)
        assert r.returncode == 0, src + "\n" + r.stderr
        return obj

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    exe = str(tmp_path / (name + "-gpu"))
    r = subprocess.run(["g++", "-o", exe, *objs, "-L", LIBDIR, "-lgpusharesat", "-lz", "-lpthread",
                        "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # it loads, resolves every symbol of the library and parses its options
    r = subprocess.run([exe, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "USAGE" in (r.stdout + r.stderr)
