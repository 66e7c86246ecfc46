"""Build the CUDA library in-tree: ``powerfit_gb300/libpowerfit_gb300.so``.

One translation unit, compiled by nvcc for sm_103a only.  The C ABI it exports
is declared in ``include/powerfit_gb300.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB = os.path.join(PKG, "libpowerfit_gb300.so")
SOURCES = [os.path.join(PKG, "csrc", "pf_api.cu")]
DEPS = SOURCES + [os.path.join(PKG, "csrc", f) for f in ("pf_fft.cuh", "pf_kernels.cuh")] + \
    [os.path.join(ROOT, "include", "powerfit_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in DEPS)


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                             "-Xcompiler", "-fPIC", "-shared", "-o", tmp] + SOURCES + ["-lcudart"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + res.stdout)
    if verbose:
        print(res.stdout, file=sys.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
