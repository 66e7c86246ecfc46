"""Checkpoint and resume of a long search.

The running best (lcc, rot) after the first k rotations is all the state a
search has, and partial maxima merge with ``_combine`` semantics
(``powerfitter.py:146-163``).  A search in chunks saves it after every chunk;
a search started again from the same checkpoint file loads it
(``pf_set_results``) and continues with the next rotation, accumulating.
"""
from __future__ import annotations

import os

import numpy as np

from . import _lib


def save(path, lcc, rot, next_rotation, nrot):
    tmp = path + ".tmp.npz"
    np.savez(tmp, lcc=lcc, rot=rot, next_rotation=int(next_rotation), nrot=int(nrot))
    os.replace(tmp, path)


def load(path):
    d = np.load(path)
    return d["lcc"], d["rot"], int(d["next_rotation"]), int(d["nrot"])


def scan_resumable(ctx, rotmats, path, chunk=4096, rot_offset=0, flags=0, stop_after=None):
    """Scan `rotmats` on `ctx` (target and template set) in chunks, saving the
    running best to `path` after each; resumes from `path` if it exists.
    `stop_after`: stop after that many chunks (to test an interrupted search).
    Returns (lcc, rot, done)."""
    nrot = ctx.set_rotations(rotmats)
    start = 0
    if os.path.exists(path):
        lcc, rot, start, saved = load(path)
        if saved != nrot:
            raise ValueError("checkpoint is for %d rotations, not %d" % (saved, nrot))
        ctx.set_results(lcc, rot)
    else:
        ctx.reset_results()
    chunks = 0
    while start < nrot:
        count = min(chunk, nrot - start)
        ctx.scan_resident(start, count, rot_offset, flags | _lib.PF_FLAG_ACCUMULATE)
        start += count
        lcc, rot = ctx.get_results()
        save(path, lcc, rot, start, nrot)
        chunks += 1
        if stop_after is not None and chunks >= stop_after and start < nrot:
            return lcc, rot, False
    lcc, rot = ctx.get_results()
    return lcc, rot, True
