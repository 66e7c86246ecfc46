"""Import the real reference package on top of ``oracle/_ref`` (test infrastructure).

The reference's Python modules are imported from where they lie; its two
native modules come from ``oracle/_ref`` (built by ``oracle/build.py``).  The
package object is assembled by hand so that nothing is copied out of the
reference tree and its ``__init__`` (which pulls in structure/volume I/O) is
not needed.  Available only where the reference tree exists.
"""
from __future__ import annotations

import importlib
import os
import sys
import types
import warnings

from . import build as _build

_PKG = "powerfit_em"


def load():
    """Return the reference ``powerfit_em`` package, or None if unavailable."""
    if _PKG in sys.modules and getattr(sys.modules[_PKG], "_oracle_ref", False):
        return sys.modules[_PKG]
    if not _build.reference_present():
        return None
    if not os.path.isdir(_build.REF_OUT) or not any(
            f.startswith("_extensions") for f in os.listdir(_build.REF_OUT)):
        if not _build.build_ref():
            return None
    pkg = types.ModuleType(_PKG)
    pkg.__path__ = [_build.REF_OUT, _build.REF_SRC]
    pkg._oracle_ref = True
    sys.modules[_PKG] = pkg
    return pkg


def module(name):
    pkg = load()
    if pkg is None:
        return None
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return importlib.import_module(_PKG + "." + name)
