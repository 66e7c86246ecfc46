"""Build the CUDA library in-tree: ``powerfit_gb300/libpowerfit_gb300.so``.

nvcc for sm_103a only.  The C ABI and the runtime-planned kernels live in
``csrc/pf_api.cu``; each compile-time-specialised grid size has its own
translation unit (``csrc/pf_fast_<n>.cu``).  The units compile in parallel and
link into one shared library; the exported C ABI is declared in
``include/powerfit_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libpowerfit_gb300.so")
OBJ_DIR = os.path.join(PKG, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC"]


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def deps():
    return sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + \
        [os.path.join(ROOT, "include", "powerfit_gb300.h")]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


STAMP = os.path.join(OBJ_DIR, "flags.txt")


def extra_flags():
    """Build-variant knob (e.g. ``-DPF_PACKED_F32X2=0``)."""
    return os.environ.get("POWERFIT_NVCC_FLAGS", "").split()


def up_to_date():
    if not os.path.exists(LIB):
        return False
    try:
        if open(STAMP).read() != " ".join(extra_flags()):
            return False          # built with other variant flags
    except OSError:
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in deps())


def _compile(src, verbose):
    obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + extra_flags() + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s" % (src, res.stdout))
    return obj, res.stdout


def build(force=False, verbose=False, jobs=None):
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, out in results:
            print(out, file=sys.stderr)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lcudart"]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stdout)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(" ".join(extra_flags()))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
