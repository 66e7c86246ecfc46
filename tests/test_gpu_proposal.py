"""Learned rotation proposal on the GPU: the network's CUDA kernels against
the float64 oracle (oracle/mlp.py), the per-rotation best LCC against the
oracle correlator, and the proposal search's exhaustive fallback."""
import numpy as np
import pytest

from oracle import mlp
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    torch.cuda.set_device(0)
    return torch


@pytest.mark.parametrize("nin,nh,n", [(15, 32, 1000), (5, 16, 130), (20, 64, 257)])
def test_network_kernels_match_oracle(torch, nin, nh, n):
    from powerfit_gb300 import _lib
    rng = np.random.default_rng(nin * 100 + nh)
    count = _lib.mlp_param_count(nin, nh)
    assert count == nh * nin + nh + nh * nh + nh + nh + 1
    p32 = (rng.normal(size=count) * 0.4).astype(np.float32)
    pbf = mlp.bf16_round(p32)                       # the values the kernels compute with
    x = rng.normal(size=(n, nin)).astype(np.float32)
    t = rng.normal(size=n).astype(np.float32)
    w = (rng.random(n) + 0.5).astype(np.float32)
    dev = "cuda:0"
    pb = torch.tensor(p32, device=dev).to(torch.bfloat16)
    assert np.array_equal(pb.float().cpu().numpy(), pbf)   # torch's rounding = the oracle's (nearest even)
    X, T, W = (torch.tensor(a, device=dev) for a in (x, t, w))
    y = torch.empty(n, device=dev)
    _lib.mlp_forward(X, nin, nh, pb, y)
    ref = mlp.forward(pbf, x, nin, nh)
    assert np.max(np.abs(y.cpu().numpy() - ref)) <= 1e-4 * max(1.0, np.max(np.abs(ref)))
    for weights in (W, None):
        grad = torch.zeros(count, device=dev)
        loss = torch.zeros(1, device=dev)
        _lib.mlp_grad(X, T, weights, nin, nh, pb, 0.01, grad, loss)
        L, g = mlp.loss_grad(pbf, x, t, None if weights is None else w, 0.01, nin, nh)
        assert abs(float(loss.item()) - L) <= 1e-4 * abs(L)
        err = np.max(np.abs(grad.cpu().numpy() - g))
        assert err <= 1e-4 * np.max(np.abs(g)), "gradient error %g of max %g" % (err, np.max(np.abs(g)))


def test_adam_step_matches_formula(torch):
    from powerfit_gb300 import _lib
    rng = np.random.default_rng(7)
    n = 1601
    p = rng.normal(size=n).astype(np.float32)
    g = rng.normal(size=n).astype(np.float32)
    m = (rng.normal(size=n) * 0.1).astype(np.float32)
    v = (rng.random(n) * 0.1).astype(np.float32)
    dev = "cuda:0"
    P, G, M, V = (torch.tensor(a, device=dev) for a in (p, g, m, v))
    PB = P.to(torch.bfloat16)
    lr, b1, b2, eps, step = 1e-3, 0.9, 0.999, 1e-8, 3
    _lib.mlp_adam(P, PB, G, M, V, lr, step, b1, b2, eps)
    m1 = b1 * m.astype(np.float64) + (1 - b1) * g
    v1 = b2 * v.astype(np.float64) + (1 - b2) * g.astype(np.float64) ** 2
    p1 = p - lr * (m1 / (1 - b1 ** step)) / (np.sqrt(v1 / (1 - b2 ** step)) + eps)
    assert np.max(np.abs(P.cpu().numpy() - p1)) < 1e-6
    assert np.array_equal(PB.float().cpu().numpy(), mlp.bf16_round(P.cpu().numpy()))


@pytest.mark.parametrize("n,flags", [(32, 0), (24, 0), (32, 8)])
def test_rotation_max_matches_oracle(n, flags):
    from powerfit_gb300 import _lib, synth
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    c = synth.make_case((n, n, n), 2.0, 300, 1, 6.0, 4.0, 21)
    p = O.prepare(c.target.astype(np.float64), c.template, c.mask, False)
    rot = quat_to_rotmat(super_fibonacci(13))
    ctx = _lib.Context(p.target.shape)
    ctx.set_target(p.target, p.lcc_mask)
    ctx.set_template_mask(p.template, p.mask, float(p.norm_factor), p.rmax)
    ctx.scan(rot, flags=flags | _lib.PF_FLAG_ROT_MAX)
    got = ctx.rotation_max()
    val, vox = ctx.rotation_best()
    assert np.array_equal(got, val)
    sel = p.lcc_mask.astype(bool)
    for i, r in enumerate(rot):
        lcc = O.lcc_one_rotation(p, r)
        ref = np.nanmax(lcc[sel])
        assert abs(got[i] - ref) < 1e-4, (i, got[i], ref)
        assert sel.ravel()[vox[i]] and abs(lcc.ravel()[vox[i]] - ref) < 1e-4   # the voxel holding it
    ctx.close()


def test_proposal_full_fraction_equals_exhaustive(torch):
    from powerfit_gb300 import proposal as PR, synth
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    c = synth.make_case((64, 64, 64), 2.0, 1200, 2, 7.0, 4.0, 5)
    rot = quat_to_rotmat(super_fibonacci(300))
    pair = PR.SearchPair(c.target, c.template, c.mask, c.voxelspacing, c.resolution, rot)
    nbr = PR.rotation_neighbours(rot)
    lcc_x, rot_x = pair.fine_exhaustive()
    lcc_p, rot_p, sel = PR.proposal_search(pair, None, nbr, fraction=1.0)
    assert sel.size == rot.shape[0]
    assert np.array_equal(lcc_p, lcc_x) and np.array_equal(rot_p, rot_x)
    # a proper subset keeps the set's rotation indices
    lcc_s, rot_s, sel = PR.proposal_search(pair, None, nbr, fraction=0.2)
    hit = lcc_s > 0
    assert np.isin(rot_s[hit], sel).all()
    assert np.all(lcc_s <= lcc_x + 1e-6)
    pair.close()


def test_trained_network_ranks_best_fits_higher_than_coarse_score(torch):
    """What the trained network gains over the method without it: on eight
    seeded 96^3 maps of the validation seeds (the 207,576-rotation set) it
    ranks the exhaustive best fit higher than the coarse score alone does,
    and always inside the top 5% of the set (TOP_FRACTION, the default
    fraction of a proposal without a trained operating point)."""
    import math
    from powerfit_gb300 import proposal as PR, proposal_train as T
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    rot = quat_to_rotmat(super_fibonacci(T.SET_SIZE))
    nbr = PR.rotation_neighbours(rot)
    net = PR.ProposalNet.load(PR.default_weights())
    maps = T.search_data([T.VALID_SEED0 + i for i in range(8)], 96, rot, log=lambda m: None)
    q_net, _ = T.rank_quality(net, maps, nbr)
    q_coarse, _ = T.rank_quality(None, maps, nbr)
    assert q_net < q_coarse - 0.1, (q_net, q_coarse)
    for m in maps:
        score = PR.rank_scores(net, m["coarse"], nbr, m["shape"]).float().cpu().numpy()
        assert T.best_rank(score, m["fine"], T.FOUND_TOL) < math.ceil(PR.TOP_FRACTION * rot.shape[0])


def test_queue_graph_equals_stream_queue(torch):
    """The uneven-map queue captured into one CUDA graph gives the results of
    the queue on concurrent streams, replay after replay."""
    from powerfit_gb300 import synth
    from powerfit_gb300.queue import MapJob, QueueGraph, scan_queue
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    rot = quat_to_rotmat(super_fibonacci(300))
    cases = [synth.make_case((n, n, n), 2.0, 600, 1, 7.0, 4.0, 40 + n) for n in (48, 64, 96)]
    mk = lambda: [MapJob(c.target.astype(np.float64), c.template, c.mask, rot, pairs=16) for c in cases]
    ref = scan_queue(mk(), autotune_trial=0)
    qg = QueueGraph(mk(), autotune_trial=0)
    for _ in range(2):
        qg.replay()
        got = qg.results()
        for a, b in zip(got, ref):
            assert np.array_equal(a.lcc, b.lcc) and np.array_equal(a.rot, b.rot)
    qg.close()


def test_checkpoint_resume_equals_uninterrupted_scan(tmp_path):
    """A search stopped after its first chunks and resumed in a new context
    from the checkpoint gives the uninterrupted search's results."""
    from powerfit_gb300 import _lib, checkpoint, synth
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    c = synth.make_case((64, 64, 64), 2.0, 900, 2, 7.0, 4.0, 77)
    p = O.prepare(c.target.astype(np.float64), c.template, c.mask, False)
    rot = quat_to_rotmat(super_fibonacci(350))

    def context():
        ctx = _lib.Context(p.target.shape)
        ctx.set_target(p.target, p.lcc_mask)
        ctx.set_template_mask(p.template, p.mask, float(p.norm_factor), p.rmax)
        return ctx

    ref_lcc, ref_rot = context().scan(rot)
    path = str(tmp_path / "search.npz")
    lcc, r, done = checkpoint.scan_resumable(context(), rot, path, chunk=100, stop_after=2)
    assert not done and checkpoint.load(path)[2] == 200
    lcc, r, done = checkpoint.scan_resumable(context(), rot, path, chunk=100)
    assert done
    assert np.array_equal(lcc, ref_lcc) and np.array_equal(r, ref_rot)


def test_allocation_failure_is_reported_and_recovered():
    """An injected device-allocation failure comes back as PF_E_NOMEM with a
    message, and the next context is unaffected."""
    from powerfit_gb300 import _lib
    _lib.debug_fail_alloc(2)
    with pytest.raises(_lib.PowerFitError) as e:
        _lib.Context((32, 32, 32))
    assert e.value.code == -3 and "injected" in str(e.value)
    _lib.debug_fail_alloc(-1)
    ctx = _lib.Context((32, 32, 32))
    ctx.close()
