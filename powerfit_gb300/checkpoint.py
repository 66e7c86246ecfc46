"""Checkpoint and resume of a long search.

The running best (lcc, rot) after the first k rotations is all the state a
search has, and partial maxima merge with ``_combine`` semantics
(``powerfitter.py:146-163``).  A search in chunks saves it after every chunk;
a search started again from the same checkpoint file loads it
(``pf_set_results``) and continues with the next rotation, accumulating.

The file also records which search it belongs to: a SHA-256 digest of the
rotation matrices and the rotation offset added to the stored indices.  A
resume with a different rotation set (even one of the same size) or another
offset is refused instead of being merged into the wrong search.
"""
from __future__ import annotations

import hashlib
import os

import numpy as np

from . import _lib


def rotation_digest(rotmats):
    """SHA-256 of the rotation matrices (float64, row-major) of a search."""
    r = np.ascontiguousarray(rotmats, dtype=np.float64).reshape(-1, 9)
    return hashlib.sha256(r.tobytes()).hexdigest()


def save(path, lcc, rot, next_rotation, nrot, digest="", rot_offset=0):
    tmp = path + ".tmp.npz"
    np.savez(tmp, lcc=lcc, rot=rot, next_rotation=int(next_rotation), nrot=int(nrot),
             digest=np.array(digest), rot_offset=int(rot_offset))
    os.replace(tmp, path)


def load(path):
    with np.load(path) as d:
        return d["lcc"], d["rot"], int(d["next_rotation"]), int(d["nrot"])


def load_identity(path):
    """(rotation digest, rotation offset) recorded with a checkpoint."""
    with np.load(path) as d:
        digest = str(d["digest"]) if "digest" in d.files else ""
        off = int(d["rot_offset"]) if "rot_offset" in d.files else 0
    return digest, off


def scan_resumable(ctx, rotmats, path, chunk=4096, rot_offset=0, flags=0, stop_after=None):
    """Scan `rotmats` on `ctx` (target and template set) in chunks, saving the
    running best to `path` after each; resumes from `path` if it exists.
    `stop_after`: stop after that many chunks (to test an interrupted search).
    Returns (lcc, rot, done).  Raises ValueError, before any device work, if
    `path` holds a checkpoint of another search (rotation count, rotation
    matrices or offset differ)."""
    nrot = int(np.asarray(rotmats).size // 9)
    digest = rotation_digest(rotmats)
    resume = None
    if os.path.exists(path):
        lcc, rot, start, saved = load(path)
        saved_digest, saved_off = load_identity(path)
        if saved != nrot:
            raise ValueError("checkpoint is for %d rotations, not %d" % (saved, nrot))
        if saved_digest != digest:
            raise ValueError("checkpoint is for another rotation set (digest %s..., not %s...)"
                             % (saved_digest[:12], digest[:12]))
        if saved_off != int(rot_offset):
            raise ValueError("checkpoint is for rotation offset %d, not %d" % (saved_off, rot_offset))
        resume = (lcc, rot, start)
    ctx.set_rotations(rotmats)
    start = 0
    if resume is not None:
        lcc, rot, start = resume
        ctx.set_results(lcc, rot)
    else:
        ctx.reset_results()
    chunks = 0
    while start < nrot:
        count = min(chunk, nrot - start)
        ctx.scan_resident(start, count, rot_offset, flags | _lib.PF_FLAG_ACCUMULATE)
        start += count
        lcc, rot = ctx.get_results()
        save(path, lcc, rot, start, nrot, digest, rot_offset)
        chunks += 1
        if stop_after is not None and chunks >= stop_after and start < nrot:
            return lcc, rot, False
    lcc, rot = ctx.get_results()
    return lcc, rot, True
