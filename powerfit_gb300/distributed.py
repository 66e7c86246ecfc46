"""Rotation sharding across ranks (one process per GPU) and the final merge.

Rotations are independent, so a search shards into contiguous rotation slices
with no data-path communication; the only exchange is one gather of the
per-voxel (lcc, rot) volumes at the end, merged with the semantics of the
reference's ``PowerFitter._combine`` (``powerfitter.py:146-163``): strict
``>``, so on ties the shard holding the lower rotation indices keeps the voxel.
"""
from __future__ import annotations

import numpy as np


def rotation_shard(nrot, rank, world):
    """[start, stop) of rank's contiguous slice, as ``_cpu_scan`` splits
    (``powerfitter.py:95-108``: equal slices, the last one takes the rest)."""
    per = nrot // world
    start = rank * per
    stop = nrot if rank == world - 1 else start + per
    return start, stop


def weak_scaling_shard(rotations_for, nset, rank, world):
    """Rotations of `rank` when every rank scans `nset` rotations of its own
    (weak scaling): one set of ``world * nset`` rotations (``rotations_for(count)``
    builds a set of that size) split into contiguous shards, so that no two
    ranks scan the same rotation and every stored index is a global index of
    that set.  Returns (the rank's (nset, 3, 3) rotations, the global index of
    its first rotation); scanning with that index as the rotation offset makes
    the merged indices lie in [0, world * nset)."""
    if world <= 1:
        return rotations_for(nset), 0
    full = rotations_for(world * nset)
    start, stop = rotation_shard(world * nset, rank, world)
    return full[start:stop], start


def merge_parts(parts, offsets, merge_one=None):
    """Merge [(lcc, rot), ...] in shard order; shard n's indices get offsets[n].

    ``merge_one(lcc, rot, part_lcc, part_rot, offset)`` merges one shard in
    place; the default runs the library's GPU merge (``pf_combine``)."""
    if merge_one is None:
        from ._lib import combine_into as merge_one
    shape = np.asarray(parts[0][0]).shape
    lcc = np.zeros(int(np.prod(shape)), dtype=np.float32)
    rot = np.zeros(int(np.prod(shape)), dtype=np.int32)
    for (plcc, prot), off in zip(parts, offsets):
        merge_one(lcc, rot, np.asarray(plcc, np.float32).reshape(-1), np.asarray(prot, np.int32).reshape(-1),
                  int(off))
    return lcc.reshape(shape), rot.reshape(shape)


def gather_and_merge(lcc, rot, rank_offset, group=None, merge_one=None, dst=0):
    """Gather every rank's (lcc, rot, offset) on ``dst`` and merge there.

    Uses ``torch.distributed`` (gloo or nccl); returns the merged volumes on
    ``dst`` and None elsewhere."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    tl = torch.from_numpy(np.ascontiguousarray(lcc, np.float32).reshape(-1)).to(dev)
    tr = torch.from_numpy(np.ascontiguousarray(rot, np.int32).reshape(-1)).to(dev)
    to = torch.tensor([int(rank_offset)], dtype=torch.int64, device=dev)
    gl = [torch.empty_like(tl) for _ in range(world)]
    gr = [torch.empty_like(tr) for _ in range(world)]
    go = [torch.empty_like(to) for _ in range(world)]
    dist.all_gather(gl, tl, group=group)
    dist.all_gather(gr, tr, group=group)
    dist.all_gather(go, to, group=group)
    if rank != dst:
        return None
    shape = np.asarray(lcc).shape
    parts = [(a.cpu().numpy().reshape(shape), b.cpu().numpy().reshape(shape)) for a, b in zip(gl, gr)]
    offsets = [int(o.item()) for o in go]
    order = np.argsort(offsets, kind="stable")
    return merge_parts([parts[i] for i in order], [offsets[i] for i in order], merge_one)
