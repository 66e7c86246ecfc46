"""Build recipe for the oracle (test infrastructure only).

``build_oracle()`` compiles the C restatement ``rotate_grid3d.c`` into
``oracle/liboracle_rotate.so`` (plain gcc, works on x86-64 and aarch64).

``build_ref()`` compiles the reference's own native sources where they lie
(``src/powerfit_em/_extensions.c`` and ``_powerfit.pyx`` of the reference
checkout named by ``$POWERFIT_REFERENCE_ROOT``, by default the build
container's checkout) into ``oracle/_ref/``, with the flags of the
reference's ``setup.py:11-25`` (``-ffast-math`` for ``_extensions.c``).  It
runs only where the reference tree and Cython are present; nothing is copied
out of the reference tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("POWERFIT_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src", "powerfit_em")
REF_OUT = os.path.join(HERE, "_ref")


def _run(cmd):
    subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)


def build_oracle():
    src = os.path.join(HERE, "rotate_grid3d.c")
    out = os.path.join(HERE, "liboracle_rotate.so")
    tmp = out + ".tmp%d" % os.getpid()
    _run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, src, "-lm"])
    os.replace(tmp, out)
    return out


def reference_present():
    return os.path.isfile(os.path.join(REF_SRC, "_extensions.c"))


def build_ref():
    """Compile the reference's native helpers into oracle/_ref (returns False if
    the reference tree or Cython is absent, e.g. on the GPU host)."""
    if not reference_present() or shutil.which("cython") is None:
        return False
    import numpy
    os.makedirs(REF_OUT, exist_ok=True)
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    inc = ["-I" + numpy.get_include(), "-I" + sysconfig.get_paths()["include"]]
    cflags = ["-O2", "-fPIC", "-shared", "-Wno-unused-function", "-Wno-cpp"]
    pyx_c = os.path.join(REF_OUT, "_powerfit.c")
    _run(["cython", "-3", os.path.join(REF_SRC, "_powerfit.pyx"), "-o", pyx_c])
    _run(["gcc"] + cflags + inc + [pyx_c, "-o", os.path.join(REF_OUT, "_powerfit" + suffix), "-lm"])
    _run(["gcc"] + cflags + ["-ffast-math"] + inc +
         [os.path.join(REF_SRC, "_extensions.c"), "-o", os.path.join(REF_OUT, "_extensions" + suffix), "-lm"])
    return True


if __name__ == "__main__":
    print(build_oracle())
    print("reference built:", build_ref(), file=sys.stderr)
