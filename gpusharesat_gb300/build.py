"""Builds libgpusharesat.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel into gpusharesat_gb300/_build/,
then nvcc links the shared library next to this file. No cmake; the same
recipe runs on x86_64 and aarch64 hosts.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgpusharesat.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _cuda_include():
    return os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def compile_commands(ptxas_verbose=False):
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    cmds = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
               "--expt-relaxed-constexpr", *inc, "-c", src, "-o", obj]
        if ptxas_verbose:
            cmd.insert(1, "-Xptxas=-v")
        cmds.append((src, obj, cmd))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-Wall", *inc,
               "-I", _cuda_include(), "-c", src, "-o", obj]
        cmds.append((src, obj, cmd))
    return cmds


def build(force=False, ptxas_verbose=False, quiet=True):
    """Compiles every source that changed and links libgpusharesat.so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    newest_header = max([os.path.getmtime(h) for h in headers] + [0])
    todo = []
    objs = []
    for src, obj, cmd in compile_commands(ptxas_verbose):
        objs.append(obj)
        if force or ptxas_verbose or not os.path.exists(obj) or \
                os.path.getmtime(obj) < max(os.path.getmtime(src), newest_header):
            todo.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, todo))
    if not quiet:
        for o in outs:
            if o.strip():
                sys.stdout.write(o)
    if todo or not os.path.exists(LIB):
        _run([_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv, quiet=False)
    print(LIB)
