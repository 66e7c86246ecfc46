"""Host side of the learned proposal (no GPU): the float64 network oracle
against finite differences, rotation-set geometry, coarse maps."""
import numpy as np

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
