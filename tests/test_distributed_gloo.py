"""Multi-rank sharding and merge on CPU ranks (gloo, world size 2).

Each rank scans its contiguous rotation slice with the oracle (standing in for
its GPU), the per-voxel results are gathered with torch.distributed and merged
with the product's merge logic; the result must equal one scan over all
rotations (``PowerFitter._combine`` semantics)."""
import os
import socket

import numpy as np
import pytest

from powerfit_gb300.distributed import merge_parts, rotation_shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _oracle_merge_one(lcc, rot, plcc, prot, off):
    ind = plcc > lcc
    lcc[ind] = plcc[ind]
    rot[ind] = prot[ind] + off


def _case():
    from oracle import oracle as O
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    rng = np.random.default_rng(8)
    shape = (12, 12, 12)
    target = rng.random(shape)
    template = rng.random(shape)
    mask = (rng.random(shape) > 0.5).astype(float)
    rot = quat_to_rotmat(super_fibonacci(11))
    p = O.prepare(target, template, mask, False)
    return p, rot


def _weak_set(count):
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    return quat_to_rotmat(super_fibonacci(count))


def _rank_main(rank, world, port, q, weak=False):
    import torch.distributed as dist
    from oracle import oracle as O
    from powerfit_gb300.distributed import gather_and_merge, weak_scaling_shard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p, rot = _case()
        if weak:
            # the bench's multi-rank form: every rank scans 5 rotations of its
            # own, stored with global indices (the rotation offset), merged
            # without a rank offset
            mine, first = weak_scaling_shard(_weak_set, 5, rank, world)
            lcc, r = O.scan(p, mine)
            out = gather_and_merge(lcc.astype(np.float32), (r + first).astype(np.int32), 0,
                                   merge_one=_oracle_merge_one)
        else:
            a, b = rotation_shard(rot.shape[0], rank, world)
            lcc, r = O.scan(p, rot[a:b])
            out = gather_and_merge(lcc.astype(np.float32), r.astype(np.int32), a, merge_one=_oracle_merge_one)
        if rank == 0:
            q.put((out[0], out[1]))
        else:
            q.put(None if out is None else "unexpected")
    finally:
        dist.destroy_process_group()


def test_rotation_shard_covers_set():
    for n, w in [(11, 2), (7416, 8), (3, 4), (70728, 3)]:
        spans = [rotation_shard(n, r, w) for r in range(w)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        assert all(spans[i][1] == spans[i + 1][0] for i in range(w - 1))


def test_merge_ties_keep_lower_shard():
    a = (np.array([0.5, 0.2], np.float32), np.array([1, 2], np.int32))
    b = (np.array([0.5, 0.3], np.float32), np.array([0, 1], np.int32))
    lcc, rot = merge_parts([a, b], [0, 10], merge_one=_oracle_merge_one)
    assert np.array_equal(rot, [1, 11]) and np.array_equal(lcc, np.array([0.5, 0.3], np.float32))


def _run_ranks(weak):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q, weak)) for r in range(2)]
    for pr in procs:
        pr.start()
    results = [q.get(timeout=120) for _ in procs]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    merged = [r for r in results if r is not None]
    assert len(merged) == 1
    return merged[0]


def test_two_gloo_ranks_equal_single_scan():
    pytest.importorskip("torch")
    from oracle import oracle as O
    lcc, rot = _run_ranks(False)
    p, rots = _case()
    rl, rr = O.scan(p, rots)
    assert np.allclose(lcc, rl.astype(np.float32))
    upd = rl > 0
    assert np.array_equal(rot[upd], rr[upd].astype(np.int32))


def test_weak_scaling_shards_merge_to_global_indices():
    """Two ranks, each scanning a shard of its own (the bench's torchrun
    form): the merged volumes equal one scan over the two ranks' whole set,
    and every merged index lies inside that set."""
    pytest.importorskip("torch")
    from oracle import oracle as O
    from powerfit_gb300.distributed import weak_scaling_shard
    a, fa = weak_scaling_shard(_weak_set, 5, 0, 2)
    b, fb = weak_scaling_shard(_weak_set, 5, 1, 2)
    assert (fa, fb) == (0, 5) and np.array_equal(np.concatenate([a, b]), _weak_set(10))
    lcc, rot = _run_ranks(True)
    p, _ = _case()
    rl, rr = O.scan(p, _weak_set(10))
    assert np.allclose(lcc, rl.astype(np.float32))
    upd = rl > 0
    assert np.array_equal(rot[upd], rr[upd].astype(np.int32))
    assert rot.min() >= 0 and rot.max() < 10
