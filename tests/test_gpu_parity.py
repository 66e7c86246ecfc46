"""GPU parity tests: the CUDA path through the C ABI against the reference's
golden outputs (tests/golden, produced by the real reference) and against the
oracle restatement run live on the same seeded inputs.

Tolerances (from the search's correctness criterion): best LCC within 1e-4
absolute; best rotation identical wherever the reference's top-two LCC gap at
that voxel exceeds 1e-4.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LCC_TOL = 1e-4
GAP_TOL = 1e-4
# precision-study variant (split-bf16x3 tensor-core DFT stages): held to the
# parity tolerance (measured on a GB300: 1.1e-5 to 1.8e-5, float32 stages 3e-7 to 6e-7)
TENSOR_DFT_LCC_BOUND = LCC_TOL


@pytest.fixture(scope="module")
def lib():
    from powerfit_gb300 import _lib
    return _lib


def check_parity(lcc, rot, ref_lcc, ref_rot, ref_second, label=""):
    ref_lcc = np.asarray(ref_lcc, dtype=np.float64)
    finite = np.isfinite(ref_lcc)
    assert np.array_equal(np.isfinite(lcc), finite), label + ": non-finite pattern differs"
    err = float(np.max(np.abs(lcc[finite] - ref_lcc[finite]))) if finite.any() else 0.0
    assert err < LCC_TOL, "%s: max |dLCC| = %g" % (label, err)
    clear = finite & ((ref_lcc - ref_second) > GAP_TOL)
    bad = int(np.sum(rot[clear] != ref_rot[clear]))
    assert bad == 0, "%s: %d of %d clear voxels pick a different rotation" % (label, bad, int(clear.sum()))
    return err


def correlator(target, template, mask, rotmats, laplace, flags=0, **tuning):
    from powerfit_gb300 import CUDACorrelator
    corr = CUDACorrelator(np.asarray(target, np.float64), laplace=laplace, flags=flags)
    if tuning:
        corr.context.set_tuning(**tuning)
    corr.template = np.asarray(template, np.float64)
    corr.mask = np.asarray(mask, np.float64)
    corr.rotations = rotmats
    corr.scan()
    return corr


# --------------------------------------------------------------------------
# unit-level mirrors against the reference's own outputs
# --------------------------------------------------------------------------

def test_rotate_grid3d_golden(lib):
    d = np.load(os.path.join(GOLD, "rotate_grid3d.npz"))
    for name in d["names"]:
        grid = d[name + "_grid"].astype(np.float64)
        out = np.zeros_like(grid)
        lib.rotate_grid3d(grid, d[name + "_rotmat"], int(d[name + "_radius"]), out, int(d[name + "_nearest"]))
        ref = d[name + "_out"]
        if int(d[name + "_nearest"]):
            assert np.array_equal(out, ref), name
        else:
            assert np.max(np.abs(out - ref)) < 1e-5, (name, np.max(np.abs(out - ref)))


def test_rotate_grid3d_preserves_outside(lib):
    grid = np.random.default_rng(0).random((8, 9, 10))
    out = np.full_like(grid, 7.0)
    lib.rotate_grid3d(grid, np.eye(3), 2, out, 1)
    zz, yy, xx = np.meshgrid(*[np.where(np.arange(n) * 2 <= n, np.arange(n), np.arange(n) - n) for n in grid.shape],
                             indexing="ij")
    inside = zz ** 2 + yy ** 2 + xx ** 2 <= 4
    assert np.all(out[~inside] == 7.0)
    assert np.allclose(out[inside], grid[inside].astype(np.float32))


def test_conj_multiply_and_calc_lcc_golden(lib):
    d = np.load(os.path.join(GOLD, "lcc_helpers.npz"))
    out = np.empty_like(d["a"])
    lib.conj_multiply(d["a"], d["b"], out)
    assert np.allclose(out, d["conj"], rtol=1e-14, atol=0)
    lcc = np.full(d["gcc"].shape, -7.0)
    lib.calc_lcc(d["gcc"], d["ave"], d["ave2"], d["mask"], lcc)
    ref = d["lcc"]
    assert np.array_equal(np.isnan(lcc), np.isnan(ref))
    fin = np.isfinite(ref)
    assert np.array_equal(np.isinf(lcc), np.isinf(ref))
    assert np.allclose(lcc[fin], ref[fin], rtol=1e-14)


def test_combine_matches_reference_merge(lib):
    rng = np.random.default_rng(3)
    parts = [(rng.random(1000).astype(np.float32), rng.integers(0, 50, 1000).astype(np.int32)) for _ in range(3)]
    parts[1][0][:10] = parts[0][0][:10]        # ties: the earlier shard keeps the voxel
    from powerfit_gb300 import combine_shards
    lcc, rot = combine_shards(parts, 50)
    rlcc, rrot = O.combine([(p[0].astype(np.float64), p[1].astype(np.float64)) for p in parts], 50)
    assert np.array_equal(lcc, rlcc.astype(np.float32))
    assert np.array_equal(rot, rrot.astype(np.int32))


# --------------------------------------------------------------------------
# FFT engine
# --------------------------------------------------------------------------

@pytest.mark.parametrize("shape", [(8, 8, 8), (10, 12, 14), (15, 16, 21), (24, 20, 18), (48, 48, 48),
                                   (64, 64, 64), (7, 9, 25), (96, 80, 36), (1, 4, 6)])
def test_fft3d_matches_numpy(lib, shape):
    a = np.random.default_rng(sum(shape)).standard_normal(shape).astype(np.float32)
    ctx = lib.Context(shape)
    out = ctx.fft3d(a)
    ref = np.fft.fftn(a.astype(np.float64))
    rel = np.max(np.abs(out - ref)) / np.max(np.abs(ref))
    assert rel < 2e-6, (shape, rel)


# --------------------------------------------------------------------------
# full scans against the reference's golden outputs
# --------------------------------------------------------------------------

SCANS = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLD, "scan_*.npz")))


@pytest.mark.parametrize("name", SCANS)
def test_scan_golden(name):
    d = np.load(os.path.join(GOLD, "scan_%s.npz" % name))
    corr = correlator(d["target"], d["template"], d["mask"], d["rotmats"], bool(d["laplace"]))
    assert corr.lcc.dtype == np.float32 and corr.rot.dtype == np.int32
    check_parity(corr.lcc, corr.rot, d["lcc"], d["rot"], d["second"], name)


@pytest.mark.parametrize("name", SCANS)
def test_scan_golden_fp64_normalisation(name):
    from powerfit_gb300._lib import PF_FLAG_FP64_NORM
    d = np.load(os.path.join(GOLD, "scan_%s.npz" % name))
    corr = correlator(d["target"], d["template"], d["mask"], d["rotmats"], bool(d["laplace"]),
                      flags=PF_FLAG_FP64_NORM)
    check_parity(corr.lcc, corr.rot, d["lcc"], d["rot"], d["second"], name)


# --------------------------------------------------------------------------
# live oracle comparisons on synthetic maps
# --------------------------------------------------------------------------

def _synthetic(shape, vs, natoms, res, seed, core_weighted):
    from powerfit_gb300 import synth
    c = synth.make_case(shape, vs, natoms, 3, res, 4.0, seed)
    mask = O.determine_core_indices(c.mask) if core_weighted else c.mask
    return c.target.astype(np.float64), c.template, mask


@pytest.mark.parametrize("laplace,cw", [(False, False), (True, True)])
def test_scan_oracle_64(laplace, cw):
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    target, template, mask = _synthetic((64, 64, 64), 2.0, 1500, 8.0, 11, cw)
    rot = quat_to_rotmat(super_fibonacci(300))[::10]   # 30 rotations spread over SO(3)
    corr = correlator(target, template, mask, rot, laplace)
    p = O.prepare(target, template, mask, laplace)
    lcc, rrot, second = O.scan(p, rot, track_second=True)
    err = check_parity(corr.lcc, corr.rot, lcc, rrot, second, "64^3")
    print("64^3 laplace=%s cw=%s max|dLCC|=%.2e" % (laplace, cw, err))


def test_scan_oracle_128_subset():
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    target, template, mask = _synthetic((128, 128, 128), 1.5, 4000, 6.0, 5, True)
    rot = quat_to_rotmat(super_fibonacci(4000))[::800]  # 5 rotations
    corr = correlator(target, template, mask, rot, True)
    p = O.prepare(target, template, mask, True)
    lcc, rrot, second = O.scan(p, rot, track_second=True)
    err = check_parity(corr.lcc, corr.rot, lcc, rrot, second, "128^3")
    print("128^3 laplace+cw max|dLCC|=%.2e" % err)


# --------------------------------------------------------------------------
# invariances of the batched / pruned implementation (bitwise)
# --------------------------------------------------------------------------

def test_batching_pruning_and_accumulate_are_exact(lib):
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    from powerfit_gb300._lib import PF_FLAG_ACCUMULATE, PF_FLAG_NO_PRUNE
    target, template, mask = _synthetic((48, 48, 48), 2.5, 800, 8.0, 3, False)
    rot = quat_to_rotmat(super_fibonacci(37))            # odd count: last pair half-empty
    base = correlator(target, template, mask, rot, False)
    geo = base.context.get_geometry()
    assert geo["valid_planes"] <= 48
    ctx = base.context
    for pairs in (1, 3, 8):
        ctx.set_tuning(pairs=pairs, rows1=4, rows3=8)
        lcc, r = ctx.scan(rot)
        assert np.array_equal(lcc, base.lcc) and np.array_equal(r, base.rot), pairs
    lcc, r = ctx.scan(rot, flags=PF_FLAG_NO_PRUNE)
    assert np.array_equal(lcc, base.lcc) and np.array_equal(r, base.rot)
    # two slices accumulated == one scan
    ctx.set_rotations(rot)
    ctx.scan_resident(0, 20)
    ctx.scan_resident(20, 17, flags=PF_FLAG_ACCUMULATE)
    lcc, r = ctx.get_results()
    assert np.array_equal(lcc, base.lcc) and np.array_equal(r, base.rot)
    # rotation offset is added to the stored index
    lcc, r = ctx.scan(rot, rot_offset=1000)
    upd = base.lcc > 0
    assert np.array_equal(r[upd], base.rot[upd] + 1000)


def test_pass3_pair_parts_are_exact(lib):
    """At 32^3 a pass-3 grid of 32 z planes x 2 tiles leaves most of the GPU
    idle, so the batch's pairs are split over up to four blocks per tile and
    merged in part order.  Every split (2, 3 and 4 parts, a last part left
    empty, partial batches without a split) gives the unsplit result bit for
    bit, and that result meets the oracle's parity criterion."""
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    target, template, mask = _synthetic((32, 32, 32), 3.0, 300, 8.0, 5, False)
    rot = quat_to_rotmat(super_fibonacci(75))            # 38 pairs, the last half-empty
    base = correlator(target, template, mask, rot, False, pairs=1, rows1=8, rows3=16)
    ctx = base.context
    for pairs in (4, 6, 9, 16, 38):
        ctx.set_tuning(pairs=pairs, rows1=8, rows3=16)
        lcc, r = ctx.scan(rot)
        assert np.array_equal(lcc, base.lcc) and np.array_equal(r, base.rot), pairs
    p = O.prepare(target, template, mask, False)
    ref_lcc, ref_rot, ref_second = O.scan(p, rot, track_second=True)
    check_parity(base.lcc, base.rot, ref_lcc, ref_rot, ref_second, "32^3 parts")


def test_translation_equivariance(lib):
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    target, template, mask = _synthetic((48, 48, 48), 2.5, 800, 8.0, 4, False)
    rot = quat_to_rotmat(super_fibonacci(8))
    a = correlator(target, template, mask, rot, False)
    shift = (5, -7, 11)
    b = correlator(np.roll(target, shift, axis=(0, 1, 2)), template, mask, rot, False)
    assert np.max(np.abs(np.roll(a.lcc, shift, axis=(0, 1, 2)) - b.lcc)) < 1e-5


# --------------------------------------------------------------------------
# error contract of the C ABI
# --------------------------------------------------------------------------

def test_error_contract(lib):
    with pytest.raises(lib.PowerFitError):
        lib.Context((11, 16, 16))          # prime factor 11
    ctx = lib.Context((16, 16, 16))
    with pytest.raises(lib.PowerFitError):
        ctx.scan(np.eye(3))                # target/template not set
    with pytest.raises(lib.PowerFitError):
        ctx.set_template_mask(np.zeros((16, 16, 16)), np.ones((16, 16, 16)), 0.0, 8)
    with pytest.raises(lib.PowerFitError):
        ctx.set_tuning(rows1=100000)


@pytest.mark.parametrize("n", [32, 48, 64, 96, 128, 160, 192])
def test_fast_path_equals_generic(lib, n):
    """The compile-time-specialised kernels (cubic grids) give the same result
    as the runtime-planned ones."""
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    from powerfit_gb300._lib import PF_FLAG_GENERIC
    from powerfit_gb300 import synth
    c = synth.make_case((n, n, n), 192.0 / n, 1200, 2, 6.0, 4.0, 13)
    rot = quat_to_rotmat(super_fibonacci(9))
    corr = correlator(c.target.astype(np.float64), c.template, O.determine_core_indices(c.mask), rot, True)
    lg, rg = corr.context.scan(rot, flags=PF_FLAG_GENERIC)
    assert np.max(np.abs(corr.lcc - lg)) <= 1e-6
    upd = np.abs(corr.lcc - lg) == 0
    assert np.mean(corr.rot[upd] == rg[upd]) == 1.0


def test_autotune_keeps_results(lib):
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    target, template, mask = _synthetic((64, 64, 64), 2.0, 1000, 8.0, 6, False)
    rot = quat_to_rotmat(super_fibonacci(41))
    base = correlator(target, template, mask, rot, False)
    ctx = base.context
    ctx.set_rotations(rot)
    cfg = ctx.autotune(40)
    assert cfg["pairs"] >= 1 and cfg["rows1"] >= 1 and cfg["rows3"] >= 1
    assert cfg["rows3"] & (cfg["rows3"] - 1) == 0
    lcc, r = ctx.scan(rot)
    assert np.array_equal(lcc, base.lcc) and np.array_equal(r, base.rot)


@pytest.mark.parametrize("shape", [(48, 48, 48), (40, 36, 30), (192, 192, 12)])
def test_tensor_dft_variant_against_oracle(lib, shape):
    """The precision-study variant with the DFT stages on the tensor cores in
    split-bf16x3 (PF_FLAG_TENSOR_DFT): a correct search (the LCC against the
    oracle within the bound below, the argmax where the oracle's top-two gap
    exceeds 1e-4), less precise than the float32 stages it replaces."""
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    from powerfit_gb300._lib import PF_FLAG_GENERIC, PF_FLAG_TENSOR_DFT
    from powerfit_gb300 import synth
    c = synth.make_case(shape, 2.0, 500, 2, 8.0, 5.0, 31)
    rot = quat_to_rotmat(super_fibonacci(96))[::8]
    target = c.target.astype(np.float64)
    p = O.prepare(target, c.template, c.mask, False)
    ref, ref_rot, second = O.scan(p, rot, track_second=True)
    corr = correlator(target, c.template, c.mask, rot, False, flags=PF_FLAG_TENSOR_DFT)
    fin = np.isfinite(ref)
    err_tc = float(np.max(np.abs(corr.lcc[fin] - ref[fin])))
    clear = fin & ((ref - second) > 1e-4) & (ref > 0)
    agree = float(np.mean(corr.rot[clear] == ref_rot[clear]))
    lg, _ = corr.context.scan(rot, flags=PF_FLAG_GENERIC)
    err_fp32 = float(np.max(np.abs(lg[fin] - ref[fin])))
    print("%s tensor-core split-bf16x3 max|dLCC| %.2e, argmax %.5f of %d clear voxels; float32 %.2e"
          % (shape, err_tc, agree, int(clear.sum()), err_fp32))
    assert err_tc < TENSOR_DFT_LCC_BOUND and agree >= 0.999
    assert err_fp32 <= err_tc


@pytest.mark.parametrize("shape", [(48, 48, 48), (40, 36, 30), (128, 128, 128)])
def test_tensor_dft_tcgen05_against_oracle(lib, shape):
    """The precision-study variant with the plane pass's DFT stages on the
    fifth-generation tensor cores (tcgen05.mma, operands by shared-memory
    descriptors, accumulators in tensor memory; PF_FLAG_TENSOR_DFT |
    PF_FLAG_TENSOR_TC05): the same split-bf16x3 products as the mma.sync form,
    so the same bound against the oracle."""
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    from powerfit_gb300._lib import PF_FLAG_TENSOR_DFT, PF_FLAG_TENSOR_TC05
    from powerfit_gb300 import synth
    vs = 2.0 if shape[0] < 100 else 1.5
    c = synth.make_case(shape, vs, 500 if shape[0] < 100 else 2000, 2, 8.0, 5.0, 31)
    rot = quat_to_rotmat(super_fibonacci(96))[::8]
    target = c.target.astype(np.float64)
    ref, ref_rot, second = O.scan_top2_parallel(target, c.template, c.mask, rot, False)
    corr = correlator(target, c.template, c.mask, rot, False, flags=PF_FLAG_TENSOR_DFT | PF_FLAG_TENSOR_TC05)
    fin = np.isfinite(ref)
    err = float(np.max(np.abs(corr.lcc[fin] - ref[fin])))
    clear = fin & ((ref - second) > 1e-4) & (ref > 0)
    agree = float(np.mean(corr.rot[clear] == ref_rot[clear]))
    print("%s tcgen05 split-bf16x3 max|dLCC| %.2e, argmax %.5f of %d clear voxels" % (shape, err, agree,
                                                                                  int(clear.sum())))
    assert err < TENSOR_DFT_LCC_BOUND and agree >= 0.999


def test_split_plane_path_vs_oracle(lib):
    """(z, y) planes larger than shared memory take the three-step pass 2."""
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    from powerfit_gb300 import synth
    shape = (192, 192, 12)
    c = synth.make_case(shape, 2.0, 300, 2, 8.0, 5.0, 21)
    rot = quat_to_rotmat(super_fibonacci(60))[::12]
    target = c.target.astype(np.float64)
    corr = correlator(target, c.template, c.mask, rot, False)
    p = O.prepare(target, c.template, c.mask, False)
    lcc, rrot, second = O.scan(p, rot, track_second=True)
    check_parity(corr.lcc, corr.rot, lcc, rrot, second, "split 192x192x12")
    a = np.random.default_rng(2).standard_normal((192, 160, 8)).astype(np.float32)
    out = lib.Context(a.shape).fft3d(a)
    ref = np.fft.fftn(a.astype(np.float64))
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 2e-6


def test_map_queue_equals_single_scans():
    from powerfit_gb300 import synth
    from powerfit_gb300.queue import MapJob, scan_queue
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    rot = quat_to_rotmat(super_fibonacci(21))
    jobs = []
    for i, (n, lap) in enumerate(((48, False), (64, True), (40, False))):
        c = synth.make_case((n, n, n), 2.0, 500, 2, 8.0, 5.0, 30 + i)
        jobs.append(MapJob(c.target.astype(np.float64), c.template, c.mask, rot, laplace=lap, pairs=4))
    scan_queue(jobs)
    for job in jobs:
        ref = correlator(job.target, job.template, job.mask, rot, job.laplace)
        assert np.array_equal(job.lcc, ref.lcc) and np.array_equal(job.rot, ref.rot)


def test_queue16_autotuned_equals_single_scans():
    """The uneven-map queue of the benchmark (16 seeded maps, 48^3-160^3),
    every map's scan on its own stream with autotuned batch and tile shapes
    (tuned once per grid size), equals a single scan of each map, bit for bit;
    so does one replay of the same queue captured as a CUDA graph."""
    from powerfit_gb300.queue import MapJob, QueueGraph, make_queue, scan_queue
    from powerfit_gb300.rotations import rotation_set
    rot, _ = rotation_set(10.0, data_dir="/nonexistent")
    rot = rot[::100]                                       # 75 rotations of the 9.72 degree set's size
    cases = make_queue(16, seed=0)
    mk = lambda: [MapJob(c.target.astype(np.float64), c.template, c.mask, rot) for c in cases]
    tuning = {}
    jobs = scan_queue(mk(), autotune_trial=64, tuning=tuning)
    assert sorted(tuning) == sorted({tuple(c.target.shape) for c in cases})
    qg = QueueGraph(mk(), tuning=tuning)
    qg.replay()
    gjobs = qg.results()
    for job, gjob in zip(jobs, gjobs):
        ref = correlator(job.target, job.template, job.mask, rot, job.laplace)
        assert np.array_equal(job.lcc, ref.lcc) and np.array_equal(job.rot, ref.rot), job.target.shape
        assert np.array_equal(gjob.lcc, ref.lcc) and np.array_equal(gjob.rot, ref.rot), job.target.shape
    qg.close()


def test_progress_counter_and_concurrent_devices():
    """The progress counter advances while the scan runs, one slice of whole
    batches at a time (the reference increments it per rotation and polls
    it, powerfitter.py:120-128, 332-333), with results equal to one call; and
    PowerFitter over two device slots (both device 0 here) launches every
    slot's slice before waiting on any and merges them to the single scan."""
    from powerfit_gb300 import CUDACorrelator
    from powerfit_gb300.correlator import PowerFitter
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    target, template, mask = _synthetic((48, 48, 48), 2.5, 800, 8.0, 9, False)
    rot = quat_to_rotmat(super_fibonacci(40))    # 20 per device slot: the same rotation pairs as one scan
    base = correlator(target, template, mask, rot, False)

    class Counter:
        n = 0

        def increment(self):
            self.n += 1

    corr = CUDACorrelator(target)
    corr.context.set_tuning(pairs=2)             # batches of 4 rotations: 10 slices
    corr.template = template
    corr.mask = mask
    corr.rotations = rot
    corr._counter = Counter()
    seen = []
    sync = corr.context.synchronize
    corr.context.synchronize = lambda: (seen.append(corr._counter.n), sync())
    corr.scan()
    assert corr._counter.n == 40 and seen == list(range(0, 40, 4))
    assert np.array_equal(corr.lcc, base.lcc) and np.array_equal(corr.rot, base.rot)

    pf = PowerFitter(target)
    pf._template, pf._mask, pf._rotations, pf._devices = template, mask, rot, [0, 0]
    pf.scan()
    assert np.array_equal(pf._lcc, base.lcc) and np.array_equal(pf._rot, base.rot)
