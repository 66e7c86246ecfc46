"""Host side of the learned proposal (no GPU): the float64 network oracle
against finite differences, rotation-set geometry, coarse maps."""
import numpy as np
import pytest

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    nin, nh = 6, 16
    count = nh * nin + nh + nh * nh + nh + nh + 1
    p = rng.normal(size=count) * 0.3
    x = rng.normal(size=(9, nin))
    t = rng.normal(size=9)
    w = rng.random(9)
    L, g = mlp.loss_grad(p, x, t, w, 0.5, nin, nh)
    assert np.isclose(L, np.sum(0.5 * w * (mlp.forward(p, x, nin, nh) - t) ** 2))
    eps = 1e-6
    num = np.empty(count)
    for i in range(count):
        d = np.zeros(count)
        d[i] = eps
        num[i] = (mlp.loss_grad(p + d, x, t, w, 0.5, nin, nh)[0] - mlp.loss_grad(p - d, x, t, w, 0.5, nin, nh)[0]) / (2 * eps)
    assert np.max(np.abs(num - g)) < 1e-6 * max(1.0, np.max(np.abs(g)))


def test_bf16_rounding_is_nearest_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7 + 2 ** -9, -2.5], dtype=np.float32)
    got = mlp.bf16_round(vals)
    assert np.array_equal(got, np.array([1.0, 1.0, 1.0 + 2 ** -6, 1.0 + 2 ** -7, -2.5], dtype=np.float32))


def test_quaternions_and_neighbours():
    from powerfit_gb300 import proposal as PR
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    R = quat_to_rotmat(super_fibonacci(2000))
    q = PR.rotmat_to_quat(R)
    assert np.max(np.abs(quat_to_rotmat(q) - R)) < 1e-7
    nb = PR.rotation_neighbours(R, k=8)
    assert nb.shape == (2000, 8)
    assert not (nb == np.arange(2000)[:, None]).any()
    # the nearest neighbour is no farther than the 8th, and every rotation's
    # nearest neighbour lies within a few set spacings
    ang = lambda a, b: np.degrees(np.arccos(np.clip((np.einsum("nij,nij->n", a, b) - 1) / 2, -1, 1)))
    d1, d8 = ang(R[nb[:, 0]], R), ang(R[nb[:, 7]], R)
    assert np.all(d1 <= d8 + 1e-9)
    assert np.median(d1) < 25.0


def test_coarse_maps_keep_the_rotation_centre():
    from powerfit_gb300 import proposal as PR
    n = 96
    t = np.zeros((n, n, n))
    t[0, 0, 0] = 1.0
    t[3, 0, 0] = 0.5
    m = np.zeros((n, n, n))
    m[0, 0, 1] = 1
    ct, ctm, cm, cs, res = PR.coarsen(t, t, m, 1.5, 6.0)
    assert ct.shape == (32, 32, 32) and cs == 4.5 and res == 9.0
    assert np.argmax(ct) == 0                  # fine voxel 0 stays coarse voxel 0
    assert cm[0, 0, 0] == 1 and cm.sum() == 1
    assert PR.coarse_factor(128) == 4 and PR.coarse_factor(48) == 2 and PR.coarse_factor(160) == 5


def test_checkpoint_file_round_trip(tmp_path):
    from powerfit_gb300 import checkpoint
    rng = np.random.default_rng(3)
    lcc = rng.random((4, 5, 6)).astype(np.float32)
    rot = rng.integers(0, 100, size=(4, 5, 6)).astype(np.int32)
    path = str(tmp_path / "c.npz")
    checkpoint.save(path, lcc, rot, 40, 100)
    l2, r2, nxt, nrot = checkpoint.load(path)
    assert np.array_equal(l2, lcc) and np.array_equal(r2, rot) and (nxt, nrot) == (40, 100)
    checkpoint.save(path, lcc * 2, rot, 60, 100)          # replaced atomically
    assert checkpoint.load(path)[2] == 60


def test_checkpoint_refuses_another_search(tmp_path):
    """A checkpoint records its rotation set's digest and the rotation offset;
    resuming with the same count but other rotations, or another offset, is
    refused before any device call."""
    from powerfit_gb300 import checkpoint
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci

    class NoDevice:
        def __getattr__(self, name):
            raise AssertionError("device call %s before the checkpoint was checked" % name)

    rot = quat_to_rotmat(super_fibonacci(30))
    path = str(tmp_path / "c.npz")
    lcc = np.zeros((4, 5, 6), np.float32)
    checkpoint.save(path, lcc, lcc.astype(np.int32), 10, 30, checkpoint.rotation_digest(rot), 7)
    assert checkpoint.load_identity(path) == (checkpoint.rotation_digest(rot), 7)
    other = rot.copy()
    other[3] = other[4]
    with pytest.raises(ValueError, match="another rotation set"):
        checkpoint.scan_resumable(NoDevice(), other, path, rot_offset=7)
    with pytest.raises(ValueError, match="offset"):
        checkpoint.scan_resumable(NoDevice(), rot, path, rot_offset=0)
    with pytest.raises(ValueError, match="rotations"):
        checkpoint.scan_resumable(NoDevice(), rot[:29], path, rot_offset=7)


def test_best_rank_counts_rotations_scored_above_the_best_fit():
    from powerfit_gb300 import proposal_train as T
    fine = np.array([0.10, 0.50, 0.499995, np.nan, 0.30])   # rotation 1 is the best fit; 2 is within 1e-5
    score = np.array([5.0, 1.0, 4.0, 9.0, 2.0])
    # rotation 2 counts as the best fit too; 2 rotations (0 and 3) score above it
    assert T.best_rank(score, fine, 1e-5) == 2
    assert T.best_rank(score, fine, 1e-7) == 4                 # only rotation 1: 0, 2, 3 and 4 above it


def test_summary_of_held_out_rows():
    from powerfit_gb300 import proposal_train as T
    rows = []
    for i, (found, rank) in enumerate([(True, 0), (True, 3), (False, 50)]):
        row = dict(exhaustive_s=2.0)
        for name in ("network", "coarse_only"):
            row[name] = dict(found=found, rank=rank, rank_fraction=rank / 1000.0, time_s=0.5,
                             found_at={str(f): rank < f * 1000 for f in T.FRACTIONS})
        rows.append(row)
    s = T.summarise(rows)
    assert s["network"]["recall"] == 2 / 3 and s["network"]["time_vs_exhaustive"] == 0.25
    assert s["network"]["median_rank_fraction"] == 0.003 and s["network"]["worst_rank_fraction"] == 0.05
    assert s["network"]["recall_at"]["0.005"] == 2 / 3 and s["exhaustive_s"] == 2.0


def test_case_parameters_are_seeded_and_in_range():
    from powerfit_gb300 import proposal_train as T
    a, b = T.case_params(1234, 96), T.case_params(1234, 96)
    assert a == b
    for seed in range(50):
        p = T.case_params(seed, 96)
        assert 1000 <= p["natoms"] <= 8000 and 5.0 <= p["resolution"] <= 9.0 and 1.0 <= p["snr"] <= 6.0
        assert 1 <= p["ncopies"] <= 3 and 1.2 <= p["voxelspacing"] <= 3.0


def test_operating_fraction_is_the_smallest_that_keeps_validation_recall():
    from powerfit_gb300 import proposal_train as T
    # every map must rank its best fit inside half of the fraction
    assert T.choose_fraction([0, 1, 2], 1000) == 0.005          # 2 < 0.005 * 1000 / 2
    assert T.choose_fraction([0, 1, 9], 1000) == 0.02           # 9 < 10
    assert T.choose_fraction([0, 300], 1000) == 1.0             # no candidate: the exhaustive search


def test_peak_votes_count_the_top_rotations_peaking_nearby():
    torch = pytest.importorskip("torch")
    from powerfit_gb300 import proposal as PR
    shape = (8, 8, 8)
    n = 1000
    g = torch.Generator().manual_seed(0)
    z = torch.randn(n, generator=g)
    v = torch.randint(0, 512, (n,), generator=g)
    top = torch.argsort(z, descending=True)[:20]                # the top 2% cast votes
    v[top] = 7 * 64 + 3 * 8 + 5                                 # all peak at voxel (7, 3, 5)
    v[0] = 0 * 64 + 3 * 8 + 5                                   # one voxel away across the periodic z edge
    v[1] = 3 * 64 + 3 * 8 + 1                                   # far away
    cnt, wsum = PR.peak_votes(z, v, shape)
    hits = int((v[top] == 7 * 64 + 3 * 8 + 5).sum())
    assert abs(float(cnt[top[0]]) - np.log1p(hits)) < 1e-5 and float(cnt[0]) >= float(np.log1p(hits - 2))
    assert float(cnt[1]) < 1.0 and float(wsum[top[0]]) > float(wsum[1])


def test_zscore_of_a_constant_feature_is_zero():
    """A vote feature that is the same for every rotation (every peak at one
    voxel) must not turn its rounding residue into inputs of 1e5."""
    torch = pytest.importorskip("torch")
    from powerfit_gb300 import proposal as PR
    a = torch.full((207576,), float(np.log1p(4151.0)), dtype=torch.float32)
    assert torch.count_nonzero(PR.zscore(a)) == 0
    z = torch.randn(1000, generator=torch.Generator().manual_seed(1))
    v = torch.full((1000,), 77, dtype=torch.int64)           # every rotation peaks at one voxel
    cnt, wsum = PR.peak_votes(z, v, (8, 8, 8))
    assert torch.count_nonzero(PR.zscore(cnt)) == 0
    b = PR.zscore(z)
    assert abs(float(b.mean())) < 1e-5 and abs(float(b.std()) - 1.0) < 1e-4


def test_shipped_network_report_meets_the_recall_and_time_targets():
    """The committed held-out evaluation of the shipped weights: at the
    operating fraction stored with them, the network finds at least 99% of
    the exhaustive best fits in at most 0.25x the exhaustive time, and finds
    at least as many as the coarse score alone at the same fraction."""
    import json
    from powerfit_gb300 import proposal as PR, proposal_train as T
    fr = T.operating_fractions(PR.default_weights())
    report = PR.default_weights().replace("proposal_net.npz", "proposal_net_report.json")
    with open(report) as f:
        rep = json.load(f)
    s, rows = rep["summary"], rep["rows"]
    assert len(rows) >= 100 and s["fractions"] == fr
    assert all(r["network"]["fraction"] == fr["network"] for r in rows)
    assert s["network"]["recall"] >= 0.99 and s["network"]["time_vs_exhaustive"] <= 0.25
    assert s["network"]["recall"] >= s["coarse_only"]["recall"]
    assert s == {**s, **T.summarise(rows)}
