"""Pin the oracle restatement against the reference's own outputs (CPU only).

The fixtures in tests/golden were produced by running the real reference
(``_extensions.rotate_grid3d``, ``_powerfit.conj_multiply`` / ``calc_lcc`` and
``CPUCorrelator.scan``) on seeded inputs; see tests/golden/make_golden.py.
Where the reference tree is present (the build container), the oracle is also
compared with it live.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_rotate_grid3d_matches_reference_outputs():
    d = np.load(os.path.join(GOLD, "rotate_grid3d.npz"))
    assert len(d["names"]) >= 20
    for name in d["names"]:
        grid = d[name + "_grid"].astype(np.float64)
        out = np.zeros_like(grid)
        O.rotate_grid3d(grid, d[name + "_rotmat"], int(d[name + "_radius"]), out, int(d[name + "_nearest"]))
        ref = d[name + "_out"]
        if int(d[name + "_nearest"]):
            assert np.array_equal(out, ref), name
        else:
            assert np.max(np.abs(out - ref)) < 1e-12, name


def test_rotate_known_answer_90deg_z():
    # the reference test's known answer: 90 degree z rotation of a 4x5x6 grid, radius 2
    grid = np.zeros((4, 5, 6))
    for idx in [(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 0, 2), (0, 0, -1), (-1, 0, 0)]:
        grid[idx] = 1
    out = np.zeros_like(grid)
    O.rotate_grid3d(grid, np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], float), 2, out, False)
    answer = np.zeros_like(out)
    for idx in [(0, 0, 0), (0, 1, 0), (0, 1, -1), (0, 2, 0), (0, -1, 0), (-1, 0, 0)]:
        answer[idx] = 1
    assert np.allclose(answer, out)


def test_helpers_match_reference_outputs():
    d = np.load(os.path.join(GOLD, "lcc_helpers.npz"))
    out = np.empty_like(d["a"])
    O.conj_multiply(d["a"], d["b"], out)
    assert np.allclose(out, d["conj"], rtol=1e-15, atol=0)
    lcc = np.full(d["gcc"].shape, -7.0)
    O.calc_lcc(d["gcc"], d["ave"], d["ave2"], d["mask"], lcc)
    assert np.array_equal(lcc, d["lcc"], equal_nan=True)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "scan_*.npz"))))
def test_scan_matches_reference_outputs(path):
    d = np.load(path)
    t = d["target"].astype(np.float64)
    p = O.prepare(t, d["template"].astype(np.float64), d["mask"].astype(np.float64), bool(d["laplace"]))
    lcc, rot, second = O.scan(p, d["rotmats"], track_second=True)
    assert np.nanmax(np.abs(lcc - d["lcc"])) < 1e-9
    clear = (lcc - second) > 1e-9
    assert np.array_equal(rot[clear], d["rot"][clear])
    assert np.allclose(second, d["second"], atol=1e-9, equal_nan=True)


def test_perfect_fit_peaks_at_origin():
    d = np.load(os.path.join(GOLD, "scan_perfect_10x12x14.npz"))
    assert np.argmax(d["lcc"]) == 0 and d["rot"].flat[0] == 0


def test_combine_semantics():
    a = (np.array([0.5, 0.2, 0.0, 0.3]), np.array([1.0, 2.0, 0.0, 3.0]))
    b = (np.array([0.5, 0.4, -0.1, 0.3]), np.array([4.0, 5.0, 6.0, 7.0]))
    lcc, rot = O.combine([a, b], 10)
    assert np.array_equal(lcc, [0.5, 0.4, 0.0, 0.3])
    assert np.array_equal(rot, [1.0, 15.0, 0.0, 3.0])    # ties keep the earlier shard


def test_oracle_matches_live_reference():
    from oracle import refimport
    if refimport.load() is None:
        pytest.skip("reference tree not available")
    pf = refimport.module("powerfitter")
    rng = np.random.default_rng(5)
    shape = (10, 11, 12)
    target = rng.random(shape)
    template = rng.random(shape)
    mask = (rng.random(shape) > 0.6).astype(np.float64)
    from powerfit_gb300.rotations import quat_to_rotmat
    rot = quat_to_rotmat(rng.normal(size=(5, 4)))
    for laplace in (False, True):
        corr = pf.CPUCorrelator(target, laplace=laplace)
        corr.template = template
        corr.mask = mask
        corr.rotations = rot
        corr.scan()
        p = O.prepare(target, template, mask, laplace)
        lcc, r = O.scan(p, rot)
        assert np.max(np.abs(lcc - corr.lcc)) < 1e-12
        assert np.array_equal(r, corr.rot)


def test_reference_rotation_slice_matches_quat_to_rotmat():
    """The 4.71 degree set slice (the reference's quaternions and its own
    quat_to_rotmat of them): this package's quat_to_rotmat gives the same
    matrices, element for element."""
    from powerfit_gb300.rotations import quat_to_rotmat
    d = np.load(os.path.join(GOLD, "rotset_471.npz"))
    assert int(d["set_size"]) == 70728 and d["rows"].shape[0] == 2048
    assert np.array_equal(quat_to_rotmat(d["quat"]), d["rotmats"])


def test_top2_slices_merge_like_one_scan():
    """Contiguous rotation slices merged with merge_top2 give the serial
    scan's best LCC, best rotation and runner-up exactly."""
    from powerfit_gb300 import synth
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    c = synth.make_case((16, 18, 20), 2.0, 150, 2, 8.0, 5.0, 5)
    rot = quat_to_rotmat(super_fibonacci(11))
    rot[4] = rot[3]                      # an exact tie across the slice boundary below
    t = c.target.astype(np.float64)
    p = O.prepare(t, c.template, c.mask, False)
    ref = O.scan(p, rot, track_second=True)
    offsets = [0, 4, 7]
    parts = [O.scan(p, rot[o:e], track_second=True) for o, e in zip(offsets, offsets[1:] + [rot.shape[0]])]
    got = O.merge_top2(parts, offsets)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
