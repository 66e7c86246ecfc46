"""Scans for the bounds-checked build (run as a script by test_gpu_bounds.py).

    POWERFIT_GB300_VARIANT=checked python tests/bounds_cases.py OUT.npz

loads ``libpowerfit_gb300_checked.so`` (the search kernels built with
-DPF_BOUNDS_CHECK), runs every case of CASES through the C ABI, and after each
one reads the violations the checks recorded.  Two more runs shrink the extent
of the intermediate buffer the kernels are told (the accesses beyond it stay
inside the allocation) to show that the checks see them, then restore it.
Results and violation counts go to OUT.npz; the test compares them with the
unchecked library and with the oracle.

The cases cover every kernel family of the search: the runtime-planned
kernels on tiny and odd grids (4x5x6, 5x6x7, 8^3, 10x12x14, 15x16x21,
40x48x36), the compile-time kernels of every specialised size (32 .. 160),
the clustered plane pass (192^3), the three-step plane pass (192x192x12),
pruning on and off, the per-rotation maxima, float64 normalisation, the
tensor-core DFT stages of the precision study (mma.sync, and tcgen05 in the
plane pass), and batch and tile shapes other than the defaults.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

FP64, NO_PRUNE, GENERIC, ROT_MAX, TENSOR_DFT, TENSOR_TC05 = 1, 2, 8, 16, 32, 64

# name, shape, inputs ("rand": uniform noise, "synth": seeded map), rotations,
# flags, tuning (pairs per batch, pass-1 rows, pass-3 rows; 0: default) or None
CASES = [
    ("tiny_4x5x6", (4, 5, 6), "rand", 12, 0, None),
    ("tiny_5x6x7", (5, 6, 7), "rand", 12, ROT_MAX, None),
    ("tiny_8", (8, 8, 8), "rand", 12, NO_PRUNE, (2, 3, 4)),
    ("odd_10x12x14_fp64", (10, 12, 14), "rand", 9, FP64, (3, 5, 4)),
    ("odd_15x16x21", (15, 16, 21), "rand", 10, 0, None),
    ("generic_40x48x36", (40, 48, 36), "synth", 16, ROT_MAX, None),
    ("fast32", (32, 32, 32), "synth", 24, 0, None),
    ("fast32_generic", (32, 32, 32), "synth", 24, GENERIC, None),
    ("fast48_noprune", (48, 48, 48), "synth", 20, NO_PRUNE | ROT_MAX, (3, 7, 2)),
    ("fast64_pairs", (64, 64, 64), "synth", 30, ROT_MAX, (8, 0, 0)),
    ("fast96_pairs", (96, 96, 96), "synth", 34, 0, (16, 0, 0)),
    ("fast128", (128, 128, 128), "synth", 12, ROT_MAX, (4, 0, 0)),
    ("fast160", (160, 160, 160), "synth", 8, 0, None),
    ("cluster192", (192, 192, 192), "synth", 6, 0, None),
    ("split_192x192x12", (192, 192, 12), "synth", 6, 0, None),
    ("tensor_dft_48", (48, 48, 48), "synth", 10, TENSOR_DFT, None),
    ("tensor_dft_split", (192, 192, 12), "synth", 6, TENSOR_DFT, None),
    ("tensor_tc05_48", (48, 48, 48), "synth", 10, TENSOR_DFT | TENSOR_TC05, None),
    ("tensor_tc05_40x36x30", (40, 36, 30), "synth", 10, TENSOR_DFT | TENSOR_TC05, None),
]

# cases re-run with a shrunk buffer extent (the checks must report accesses)
SHRINK = ("tiny_8", "fast64_pairs")


def build_case(shape, kind, nrot, seed):
    """Inputs of one case: (target, template, mask, rotation matrices)."""
    from powerfit_gb300 import synth
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    if kind == "rand":
        rng = np.random.default_rng(seed)
        target = rng.random(shape).astype(np.float32).astype(np.float64)
        template = rng.random(shape).astype(np.float32).astype(np.float64)
        mask = (rng.random(shape) > 0.4).astype(np.float64)
    else:
        vs = 2.0 if min(shape) >= 32 else 1.5
        c = synth.make_case(shape, vs, 600, 2, 8.0, 5.0, seed)
        target, template, mask = c.target.astype(np.float64), c.template, c.mask
    rot = quat_to_rotmat(super_fibonacci(7 * nrot + 1))[::7][:nrot]
    return target, template, mask, rot


def prepared(shape, kind, nrot, seed):
    """The correlator's host preprocessing of a case (the product's, not the oracle's)."""
    from powerfit_gb300.correlator import BaseCorrelator
    target, template, mask, rot = build_case(shape, kind, nrot, seed)
    b = BaseCorrelator(target)
    b.template = template
    b.mask = mask
    return b, rot


def run_case(lib, i, extent=None):
    """Scan case i with the loaded library: (lcc, rot, per-rotation max or None)."""
    name, shape, kind, nrot, flags, tuning = CASES[i]
    b, rot = prepared(shape, kind, nrot, 100 + i)
    ctx = lib.Context(shape)
    try:
        ctx.set_target(b._target, b._lcc_mask)
        ctx.set_template_mask(b._template, b._mask, float(b._norm_factor), b._rmax)
        if tuning:
            ctx.set_tuning(*tuning)
        if extent is not None:
            pairs = ctx.get_tuning()[0]
            n = int(np.prod(shape))
            ctx.debug_buffer_extent(3 * n * (pairs - 1) + n)   # part of the last pair's first field
        lcc, r = ctx.scan(rot, flags=flags)
        rmax = ctx.rotation_max() if flags & ROT_MAX else None
        return lcc, r, rmax
    finally:
        ctx.close()


def main(out):
    from powerfit_gb300 import _lib
    assert _lib.bounds_checked(), "the bounds-checked library is not the one loaded"
    _lib.debug_bounds()                       # start clean
    arrays, summary = {}, {}
    for i, (name, *_rest) in enumerate(CASES):
        lcc, r, rmax = run_case(_lib, i)
        count, site, index = _lib.debug_bounds()
        summary[name] = dict(violations=count, site=site, index=index)
        arrays[name + "_lcc"] = lcc
        arrays[name + "_rot"] = r
        if rmax is not None:
            arrays[name + "_rotmax"] = rmax
        print(name, summary[name], flush=True)
    for name in SHRINK:
        i = [c[0] for c in CASES].index(name)
        run_case(_lib, i, extent=True)
        count, site, index = _lib.debug_bounds()
        summary[name + "_shrunk"] = dict(violations=count, site=site, index=index)
        lcc, r, _ = run_case(_lib, i)           # full extent again
        count, site, index = _lib.debug_bounds()
        summary[name + "_restored"] = dict(violations=count, site=site, index=index,
                                           same=bool(np.array_equal(lcc, arrays[name + "_lcc"]) and
                                                     np.array_equal(r, arrays[name + "_rot"])))
        print(name, summary[name + "_shrunk"], summary[name + "_restored"], flush=True)
    np.savez_compressed(out, summary=json.dumps(summary), **arrays)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1]))
