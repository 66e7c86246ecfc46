"""Generate the golden fixtures from the real reference (run where the reference
checkout is present, ``$POWERFIT_REFERENCE_ROOT`` as in ``oracle/build.py``; the
fixtures are committed).

    python tests/golden/make_golden.py [prep|rotset]
        (``prep``: only prep.npz, ref_map.mrc, analyzer.npz; ``rotset``: those and rotset_471.npz)

Each fixture records reference outputs for seeded inputs:

* ``rotate_grid3d.npz``: ``_extensions.rotate_grid3d`` on the 4x5x6 known-answer
  grid of the reference's ``tests/test_extensions.py`` recipe plus random grids,
  random rotations, both interpolation modes and several radii.
* ``lcc_helpers.npz``: ``_powerfit.conj_multiply`` and ``_powerfit.calc_lcc``.
* ``prep.npz``: ``_powerfit.blur_points`` / ``dilate_points`` (template and
  mask builders), ``BaseCorrelator._laplace_filter`` and
  ``helpers.determine_core_indices`` on seeded inputs.
* ``ref_map.mrc``: a map written by the reference's ``volume.to_mrc``;
  ``analyzer.npz``: the reference ``Analyzer``'s solutions on seeded peaks.
* ``rotset_471.npz``: a strided 2,048-row slice of the reference's 4.71 degree
  orientation set (``c48u2947.npy`` through ``rotations.proportional_orientations``),
  its quaternions, weights and the reference's ``quat_to_rotmat`` of them: the
  128^3 parity tests scan the reference's own rotations.
* ``scan_<name>.npz``: ``CPUCorrelator`` (numpy.fft path) full scans:
  inputs (float32-exact), rotations, best LCC, best rotation and, from the
  oracle restatement (checked equal to the reference first), the per-voxel
  second-best LCC used by the argmax-gap criterion.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import refimport  # noqa: E402
from powerfit_gb300 import synth  # noqa: E402
from powerfit_gb300.rotations import quat_to_rotmat, euler  # noqa: E402


def f32(a):
    """Round to float32 and back so fixtures replay exactly."""
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def gen_rotate(ext, rot):
    rng = np.random.default_rng(11)
    cases = {}
    # known-answer grid of the reference's rotate_grid3d test recipe
    grid = np.zeros((4, 5, 6))
    for idx in [(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 0, 2), (0, 0, -1), (-1, 0, 0)]:
        grid[idx] = 1
    mats = [np.eye(3), euler(np.pi / 2, "z")]
    k = 0
    for R in mats:
        for nearest in (1, 0):
            out = np.zeros_like(grid)
            ext.rotate_grid3d(grid, np.ascontiguousarray(R), 2, out, nearest)
            cases["c%d" % k] = dict(grid=grid, rotmat=R, radius=2, nearest=nearest, out=out.copy())
            k += 1
    for shape, radius in [((12, 14, 16), 6), ((9, 10, 11), 4), ((16, 16, 16), 8), ((7, 12, 9), 3)]:
        g = f32(rng.random(shape))
        for _ in range(2):
            q = rng.normal(size=(1, 4))
            R = quat_to_rotmat(q / np.linalg.norm(q))[0]
            for nearest in (1, 0):
                out = np.zeros(shape)
                ext.rotate_grid3d(g, R, radius, out, nearest)
                cases["c%d" % k] = dict(grid=g, rotmat=R, radius=radius, nearest=nearest, out=out.copy())
                k += 1
    flat = {}
    for name, c in cases.items():
        for key, val in c.items():
            val = np.asarray(val)
            if key == "grid":
                val = val.astype(np.float32)     # float32-exact inputs
            flat["%s_%s" % (name, key)] = val
    flat["names"] = np.array(sorted(cases))
    np.savez_compressed(os.path.join(HERE, "rotate_grid3d.npz"), **flat)


def gen_helpers(pf):
    rng = np.random.default_rng(12)
    n = 257
    a = rng.random(n) + 1j * rng.random(n)
    b = rng.random(n) + 1j * rng.random(n)
    out = np.empty(n, dtype=np.complex128)
    pf.conj_multiply(a, b, out)
    gcc = rng.random(n) - 0.3
    ave = rng.random(n)
    ave2 = 2 * ave ** 2
    ave2[::17] = ave[::17] ** 2 * 0.5      # negative variance -> NaN
    ave2[5] = ave[5] ** 2                  # zero variance -> inf
    mask = (rng.random(n) > 0.2).astype(np.uint8)
    lcc = np.full(n, -7.0)
    pf.calc_lcc(gcc, ave, ave2, mask, lcc)
    np.savez_compressed(os.path.join(HERE, "lcc_helpers.npz"), a=a, b=b, conj=out,
                        gcc=gcc, ave=ave, ave2=ave2, mask=mask, lcc=lcc)


def gen_prep(pfx, powerfitter, helpers):
    rng = np.random.default_rng(31)
    out = {}
    shape = (20, 22, 24)
    pts = rng.random((3, 60)) * np.array([[24.0], [22.0], [20.0]]) - 4.0
    w = rng.random(60) + 0.5
    for wrap in (True, False):
        a = np.zeros(shape)
        pfx.blur_points(pts.copy(), w.copy(), 1.3, a, wrap)
        out["blur_%d" % wrap] = a
        b = np.zeros(shape)
        radii = 1.0 + 2.0 * rng.random(60)
        pfx.dilate_points(pts.copy(), radii.copy(), b, wrap)
        out["dilate_%d" % wrap] = b
        out["radii_%d" % wrap] = radii
    out["points"] = pts
    out["weights"] = w
    grid = rng.random((9, 10, 11))
    out["lap_in"] = grid
    out["lap_out"] = powerfitter.BaseCorrelator._laplace_filter(grid)
    blob = np.zeros((16, 18, 20))
    blob[2:14, 3:15, 1:19] = 1
    blob[5:9, 0:18, 8:12] = 1
    blob[0, 0, 0] = 1
    out["core_in"] = blob
    out["core_out"] = helpers.determine_core_indices(blob)
    np.savez_compressed(os.path.join(HERE, "prep.npz"), **out)


def gen_io(volume_mod, analyzer_mod):
    rng = np.random.default_rng(41)
    arr = rng.random((10, 12, 14)).astype(np.float32).astype(np.float64)
    vol = volume_mod.Volume(arr, 1.5, np.array([3.0, -2.0, 5.0]))
    volume_mod.to_mrc(os.path.join(HERE, "ref_map.mrc"), vol)
    # analyzer: a few smooth peaks on a 24^3 grid
    shape = (24, 24, 24)
    lcc = np.zeros(shape)
    zz, yy, xx = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    for c, h in zip(rng.random((5, 3)) * 20 + 2, rng.random(5) * 0.5 + 0.3):
        lcc = np.maximum(lcc, h * np.exp(-((zz - c[0]) ** 2 + (yy - c[1]) ** 2 + (xx - c[2]) ** 2) / 6.0))
    rot_ind = rng.integers(0, 7, shape).astype(np.float64)
    rotmats = quat_to_rotmat(rng.normal(size=(7, 4)))
    an = analyzer_mod.Analyzer(lcc, rotmats, rot_ind, voxelspacing=1.7, origin=(1.0, 2.0, 3.0), z_sigma=0.12)
    sols = np.array(an.solutions)
    np.savez_compressed(os.path.join(HERE, "analyzer.npz"), lcc=lcc, rot_ind=rot_ind, rotmats=rotmats,
                        solutions=sols)


def random_case(shape, seed):
    rng = np.random.default_rng(seed)
    target = f32(rng.random(shape))
    pts = rng.random((3, 12)) * np.array(shape[::-1])[:, None] * 0.3 - 1.5
    template = np.zeros(shape)
    synth.blur_points(pts, rng.random(12) + 0.5, 1.2, template, True)
    template = f32(template)
    mask = np.zeros(shape)
    synth.dilate_points(pts, 2.5, mask, True)
    return target, template, mask


def synth_case(shape, seed, natoms, vs, res):
    c = synth.make_case(shape, vs, natoms, 2, res, 5.0, seed)
    return f32(c.target), f32(c.template), c.mask


def run_scan(powerfitter, target, template, mask, rotmats, laplace):
    corr = powerfitter.CPUCorrelator(target, laplace=laplace)
    corr.template = template
    corr.mask = mask
    corr.rotations = rotmats
    corr.scan()
    return corr.lcc.copy(), corr.rot.copy()


def gen_scan(powerfitter, helpers, name, target, template, mask, rotmats, laplace, core_weighted):
    if core_weighted:
        mask = helpers.determine_core_indices(mask)
    lcc, rot = run_scan(powerfitter, target, template, mask, rotmats, laplace)
    p = O.prepare(target, template, mask, laplace)
    olcc, orot, second = O.scan(p, rotmats, track_second=True)
    err = np.nanmax(np.abs(olcc - lcc))
    assert err < 1e-9, (name, err)
    assert np.array_equal(orot, rot) or np.all((orot == rot) | (np.abs(olcc - second) < 1e-9)), name
    np.savez_compressed(
        os.path.join(HERE, "scan_%s.npz" % name),
        target=target.astype(np.float32), template=template.astype(np.float32),
        mask=mask.astype(np.float32), rotmats=rotmats, laplace=laplace,
        core_weighted=core_weighted, lcc=lcc, rot=rot.astype(np.int32), second=second)
    print(name, "max lcc %.4f" % np.nanmax(lcc), "oracle err %.2e" % err)


def gen_rotset(rot):
    """A strided slice (every 34th row, 2,048 rows) of the 4.71 degree set."""
    q, w, degree = rot.proportional_orientations(4.71)
    rows = np.arange(0, q.shape[0], 34)[:2048]
    np.savez_compressed(os.path.join(HERE, "rotset_471.npz"), rows=rows, quat=q[rows], weights=w[rows],
                        rotmats=rot.quat_to_rotmat(q[rows]), degree=degree, set_size=q.shape[0])
    print("rotset_471", rows.shape[0], "rows of", q.shape[0], degree)


def main():
    if refimport.load() is None:
        raise SystemExit("reference tree not available")
    ext = refimport.module("_extensions")
    pfx = refimport.module("_powerfit")
    powerfitter = refimport.module("powerfitter")
    helpers = refimport.module("helpers")
    rot = refimport.module("rotations")
    gen_prep(pfx, powerfitter, helpers)
    gen_io(refimport.module("volume"), refimport.module("analyzer"))
    if len(sys.argv) > 1 and sys.argv[1] == "prep":
        return
    gen_rotset(rot)
    if len(sys.argv) > 1 and sys.argv[1] == "rotset":
        return
    gen_rotate(ext, rot)
    gen_helpers(pfx)

    rng = np.random.default_rng(21)
    rand_rots = quat_to_rotmat(rng.normal(size=(16, 4)))
    karney, _, _ = rot.proportional_orientations(10.0)      # 9.72 deg set, 7416 rotations
    kar_rots = rot.quat_to_rotmat(karney[:48])

    t, m_, k = random_case((14, 16, 18), 1)
    gen_scan(powerfitter, helpers, "rand_14x16x18", t, m_, k, rand_rots, False, False)
    gen_scan(powerfitter, helpers, "rand_lapcw_14x16x18", t, m_, k, rand_rots, True, True)
    t, m_, k = random_case((15, 16, 21), 2)
    gen_scan(powerfitter, helpers, "rand_odd_15x16x21", t, m_, k, rand_rots[:8], False, False)
    t, m_, k = synth_case((24, 24, 24), 3, 150, 3.0, 8.0)
    gen_scan(powerfitter, helpers, "synth_24", t, m_, k, kar_rots, False, False)
    gen_scan(powerfitter, helpers, "synth_lapcw_24", t, m_, k, kar_rots, True, True)
    # perfect fit: template = target, mask = ones, identity first (test_get_lcc recipe)
    t = f32(np.random.default_rng(4).random((10, 12, 14)))
    ident = np.concatenate([np.eye(3)[None], rand_rots[:3]])
    gen_scan(powerfitter, helpers, "perfect_10x12x14", t, t.copy(), np.ones_like(t), ident, False, False)


if __name__ == "__main__":
    main()
