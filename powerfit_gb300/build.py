"""Build the CUDA library in-tree: ``powerfit_gb300/libpowerfit_gb300.so``.

nvcc for sm_103a only.  The C ABI and the runtime-planned kernels live in
``csrc/pf_api.cu``; each compile-time-specialised grid size has its own
translation unit (``csrc/pf_fast_<n>.cu``).  The units compile in parallel and
link into one shared library; the exported C ABI is declared in
``include/powerfit_gb300.h``.

Two variants: the library itself, and ``libpowerfit_gb300_checked.so``, the
same sources built with ``-DPF_BOUNDS_CHECK`` (every index of the search
kernels checked against its array's extent; a debugging build, loaded when
``POWERFIT_GB300_VARIANT=checked``).
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
# variant -> (defines, library, object folder)
VARIANTS = {
    "": ([], LIB, OBJ_DIR),
    "checked": (["-DPF_BOUNDS_CHECK"], os.path.join(PKG, "libpowerfit_gb300_checked.so"),
                os.path.join(PKG, "_build", "checked")),
}
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


def extra_flags():
    """Build-variant knob (e.g. ``-DPF_PACKED_F32X2=0``)."""
    return os.environ.get("POWERFIT_NVCC_FLAGS", "").split()


def _stamp(variant):
    return os.path.join(VARIANTS[variant][2], "flags.txt")


def up_to_date(variant=""):
    lib = VARIANTS[variant][1]
    if not os.path.exists(lib):
        return False
    try:
        with open(_stamp(variant)) as f:
            stamp = f.read()
        if stamp != " ".join(extra_flags()):
            return False          # built with other variant flags
    except OSError:
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in deps())


def _compile(src, variant, verbose):
    defines, _, obj_dir = VARIANTS[variant]
    obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + defines + extra_flags() + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s" % (src, res.stdout))
    return obj, res.stdout


def _link(variant, objs):
    lib = VARIANTS[variant][1]
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stdout)
    os.replace(tmp, lib)
    with open(_stamp(variant), "w") as f:
        f.write(" ".join(extra_flags()))
    return lib


def build_variants(variants=("",), force=False, verbose=False, jobs=None):
    """Build the given variants ("" and/or "checked"); the translation units
    of all of them compile in one pool.  Returns the library paths."""
    todo = [v for v in variants if force or not up_to_date(v)]
    if todo:
        srcs = sources()
        for v in todo:
            os.makedirs(VARIANTS[v][2], exist_ok=True)
        units = [(s, v) for v in todo for s in srcs]
        jobs = jobs or min(len(units), os.cpu_count() or 1)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            results = list(ex.map(lambda u: (u[1],) + _compile(u[0], u[1], verbose), units))
        if verbose:
            for _, _, out in results:
                print(out, file=sys.stderr)
        for v in todo:
            _link(v, [o for rv, o, _ in results if rv == v])
    return [VARIANTS[v][1] for v in variants]


def build(force=False, verbose=False, jobs=None, variant=""):
    return build_variants((variant,), force, verbose, jobs)[0]


if __name__ == "__main__":
    variant = "checked" if "--checked" in sys.argv else ""
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, variant=variant))
