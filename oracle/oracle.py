"""numpy FP64 restatement of the reference correlator (test infrastructure only).

Every function cites the reference file:line it restates.  The FFTs use
numpy.fft (pocketfft), which is exactly the path the reference takes when
pyFFTW is not installed (``powerfitter.py:19-20, 311-315``).

Only tests, ``smoke()`` and ``bench.py``'s CPU baseline use this module.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np
from numpy.fft import irfftn, rfftn
from scipy.ndimage import binary_erosion, laplace

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def _lib():
    """Load the C restatement of rotate_grid3d (built by oracle/build.py)."""
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle_rotate.so")
        if not os.path.exists(path):
            from . import build as _build
            _build.build_oracle()
        lib = ctypes.CDLL(path)
        lib.oracle_rotate_grid3d.restype = ctypes.c_int
        lib.oracle_rotate_grid3d.argtypes = [
            ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        _LIB = lib
    return _LIB


def rotate_grid3d(grid, rotmat, radius, out, nearest):
    """Restates ``_extensions.c:7-196`` (writes only inside the sphere)."""
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    rotmat = np.ascontiguousarray(rotmat, dtype=np.float64).reshape(9)
    if out.dtype != np.float64 or not out.flags.c_contiguous or out.shape != grid.shape:
        raise ValueError("out must be a C-contiguous float64 array of the grid's shape")
    nz, ny, nx = grid.shape
    rc = _lib().oracle_rotate_grid3d(grid.ctypes.data, nz, ny, nx, rotmat.ctypes.data,
                                     int(radius), out.ctypes.data, int(bool(nearest)))
    if rc != 0:
        raise ValueError("bad rotate_grid3d arguments")
    return out


def conj_multiply(in1, in2, out):
    """Restates ``_powerfit.pyx:45-53``: out = conj(in1) * in2."""
    np.multiply(np.conj(in1), in2, out=out)
    return out


def calc_lcc(gcc, ave, ave2, mask, lcc):
    """Restates ``_powerfit.pyx:56-72``: lcc = gcc / sqrt(ave2 - ave^2) where mask.

    Voxels outside ``mask`` are left untouched, as in the reference.
    """
    m = mask != 0
    with np.errstate(divide="ignore", invalid="ignore"):
        lcc[m] = gcc[m] / np.sqrt(ave2[m] - ave[m] ** 2)
    return lcc


def determine_core_indices(mask):
    """Restates ``helpers.py:26-34``: number of binary erosions each voxel survives."""
    core = np.zeros(mask.shape)
    eroded = mask > 0
    while eroded.sum() > 0:
        core += eroded
        eroded = binary_erosion(eroded)
    return core


@dataclass
class Prepared:
    """State that ``BaseCorrelator``/``CPUCorrelator`` hold before scanning."""
    target: np.ndarray          # target / max (unfiltered), powerfitter.py:170
    lcc_mask: np.ndarray        # uint8, powerfitter.py:178-180
    rmax: int                   # powerfitter.py:176
    template: np.ndarray        # filtered, masked, normalised, masked again (:190-220)
    mask: np.ndarray            # copy of the mask (:204)
    norm_factor: int            # count of mask != 0 (:197-199)
    ft_target: np.ndarray       # rfftn(target'), powerfitter.py:268-277
    ft_target2: np.ndarray      # rfftn(target'^2)
    filtered_target: np.ndarray  # target' = laplace(target) if laplace else target


def prepare(target, template, mask, laplace_filter=False):
    """Restates ``BaseCorrelator.__init__`` + setters and ``CPUCorrelator.__init__``.

    ``powerfitter.py:169-176`` (normalise, lcc mask, rmax), ``:190-220`` (mask
    setter: Laplace, mask, normalise over the mask, mask again), ``:262-277``
    (target spectra).
    """
    target = np.asarray(target, dtype=np.float64)
    tnorm = target / target.max()
    lcc_mask = (tnorm > tnorm.max() * 0.05).astype(np.uint8)
    rmax = min(target.shape) // 2
    if template.shape != tnorm.shape:
        raise ValueError("Shape of template does not match the target.")
    if mask.shape != tnorm.shape:
        raise ValueError("Shape of the mask is different from target.")
    ind = mask != 0
    norm_factor = int(ind.sum())
    if norm_factor == 0:
        raise ValueError("Zero-filled mask is not allowed.")
    mask = np.array(mask, dtype=np.float64, copy=True)
    tmpl = np.array(template, dtype=np.float64, copy=True)
    if laplace_filter:
        tmpl = laplace(tmpl, mode="wrap")
    tmpl *= mask
    tmpl[ind] -= tmpl[ind].mean()
    tmpl[ind] /= tmpl[ind].std()
    tmpl *= mask
    ftarget = laplace(tnorm, mode="wrap") if laplace_filter else tnorm
    return Prepared(tnorm, lcc_mask, rmax, tmpl, mask, norm_factor,
                    rfftn(ftarget), rfftn(ftarget ** 2), ftarget)


def lcc_one_rotation(p: Prepared, rotmat, lcc_scan=None):
    """Restates ``CPUCorrelator._translational_scan`` (``powerfitter.py:335-373``).

    Returns the per-voxel LCC for one rotation (zero outside the lcc mask).
    """
    shape = p.target.shape
    rot_t = np.zeros(shape)
    rot_m = np.zeros(shape)
    rotate_grid3d(p.template, rotmat, p.rmax, rot_t, False)
    rotate_grid3d(p.mask, rotmat, p.rmax, rot_m, True)
    rot_m2 = rot_m * rot_m
    gcc = irfftn(np.conj(rfftn(rot_t)) * p.ft_target, s=shape, axes=(0, 1, 2))
    ave = irfftn(np.conj(rfftn(rot_m)) * p.ft_target, s=shape, axes=(0, 1, 2))
    ave2 = irfftn(np.conj(rfftn(rot_m2)) * p.ft_target2, s=shape, axes=(0, 1, 2))
    ave2 *= p.norm_factor
    if lcc_scan is None:
        lcc_scan = np.zeros(shape)
    calc_lcc(gcc.ravel(), ave.ravel(), ave2.ravel(), p.lcc_mask.ravel(), lcc_scan.ravel())
    return lcc_scan


def scan(p: Prepared, rotations, track_second=False, progress=None):
    """Restates ``CPUCorrelator.scan`` (``powerfitter.py:317-333``).

    Strict ``>`` against a running best initialised to 0, so the lowest
    rotation index wins ties and NaN never wins.  With ``track_second`` the
    per-voxel second-best LCC is also returned (the parity checker needs the
    top-two gap to decide where the argmax is well defined).
    """
    rotations = np.asarray(rotations, dtype=np.float64).reshape(-1, 3, 3)
    shape = p.target.shape
    lcc = np.zeros(shape)
    rot = np.zeros(shape)
    second = np.zeros(shape) if track_second else None
    lcc_scan = np.zeros(shape)
    for n in range(rotations.shape[0]):
        lcc_one_rotation(p, rotations[n], lcc_scan)
        ind = lcc_scan > lcc
        if track_second:
            # a value that does not beat the best may still beat the runner-up
            with np.errstate(invalid="ignore"):
                sec = (~ind) & (lcc_scan > second)
            second[sec] = lcc_scan[sec]
            second[ind] = lcc[ind]
        lcc[ind] = lcc_scan[ind]
        rot[ind] = n
        if progress is not None:
            progress(n)
    if track_second:
        return lcc, rot, second
    return lcc, rot


def combine(parts, nrot_per_job):
    """Restates ``PowerFitter._combine`` (``powerfitter.py:146-163``).

    ``parts`` is a list of (lcc, rot) per contiguous rotation shard; shard n's
    indices are offset by ``n * nrot_per_job``; strict ``>`` merge.
    """
    lcc = np.zeros(parts[0][0].shape)
    rot = np.zeros(parts[0][0].shape)
    for n, (plcc, prot) in enumerate(parts):
        ind = plcc > lcc
        lcc[ind] = plcc[ind]
        rot[ind] = prot[ind] + nrot_per_job * n
    return lcc, rot


# ---------------------------------------------------------------------------
# Multi-process CPU scan: restates PowerFitter._cpu_scan (powerfitter.py:94-132)
# with a spawn-started pool (fork after CUDA initialisation would hang).
# ---------------------------------------------------------------------------

def _worker(args):
    target, template, mask, laplace_filter, rotations = args
    p = prepare(target, template, mask, laplace_filter)
    return scan(p, rotations)


def _timed_worker(args):
    """``_worker`` with its two phases timed: the correlator's set-up
    (``prepare``: Laplace filter and target spectra) and the rotation loop."""
    import time
    target, template, mask, laplace_filter, rotations = args
    t0 = time.perf_counter()
    p = prepare(target, template, mask, laplace_filter)
    t1 = time.perf_counter()
    lcc, rot = scan(p, rotations)
    return lcc, rot, t1 - t0, time.perf_counter() - t1, rotations.shape[0]


def cpu_scan_timed(target, template, mask, rotations, laplace_filter=False, nproc=1, pool=None):
    """``cpu_scan`` (same slices and merge) that also returns, per process, the
    set-up seconds, the rotation-loop seconds and the rotations it scanned:
    (lcc, rot, [(prepare_s, scan_s, nrot), ...])."""
    rotations = np.asarray(rotations, dtype=np.float64).reshape(-1, 3, 3)
    nrot = rotations.shape[0]
    per = nrot // nproc
    jobs = []
    for n in range(nproc):
        end = None if n == nproc - 1 else (n + 1) * per
        jobs.append((target, template, mask, laplace_filter, rotations[n * per:end]))
    res = [_timed_worker(jobs[0])] if (pool is None and nproc == 1) else pool.map(_timed_worker, jobs)
    lcc, rot = combine([(r[0], r[1]) for r in res], per)
    return lcc, rot, [(r[2], r[3], r[4]) for r in res]


def cpu_scan(target, template, mask, rotations, laplace_filter=False, nproc=1, pool=None):
    """Restates ``PowerFitter._cpu_scan``: contiguous rotation slices per process,
    then ``_combine``.  ``pool`` is a ``multiprocessing`` pool started with
    ``spawn``; with ``nproc == 1`` and no pool the scan runs in-process."""
    rotations = np.asarray(rotations, dtype=np.float64).reshape(-1, 3, 3)
    nrot = rotations.shape[0]
    per = nrot // nproc
    jobs = []
    for n in range(nproc):
        end = None if n == nproc - 1 else (n + 1) * per
        jobs.append((target, template, mask, laplace_filter, rotations[n * per:end]))
    if pool is None and nproc == 1:
        parts = [_worker(jobs[0])]
    else:
        parts = pool.map(_worker, jobs)
    return combine(parts, per)


# ---------------------------------------------------------------------------
# Top-two scan over contiguous rotation slices on several processes (parity
# checks of the large grids): each slice is ``scan(track_second=True)``; the
# slices merge in rotation order with the strict ``>`` of ``scan`` (lower index
# wins ties), the runner-up of a voxel being the larger of the loser's best and
# the winner's own runner-up.
# ---------------------------------------------------------------------------

def _top2_worker(job):
    target, template, mask, laplace_filter, rots = job
    p = prepare(target, template, mask, laplace_filter)
    return scan(p, rots, track_second=True)


def merge_top2(parts, offsets):
    """Merge per-slice (lcc, rot, second) in slice order; ``offsets[k]`` is the
    first rotation index of slice k."""
    lcc = np.zeros(parts[0][0].shape)
    rot = np.zeros(parts[0][0].shape)
    second = np.zeros(parts[0][0].shape)
    for (pl, pr, ps), off in zip(parts, offsets):
        better = pl > lcc
        second = np.where(better, np.maximum(lcc, ps), np.maximum(second, np.where(pl > second, pl, second)))
        lcc = np.where(better, pl, lcc)
        rot = np.where(better, pr + off, rot)
    return lcc, rot, second


def scan_top2_parallel(target, template, mask, rotations, laplace_filter=False, nproc=None):
    """``scan(track_second=True)`` of the prepared inputs over ``rotations``,
    split into contiguous slices on a ``spawn`` pool of ``nproc`` processes
    (safe after CUDA initialisation in the parent)."""
    import multiprocessing as mp
    rotations = np.asarray(rotations, dtype=np.float64).reshape(-1, 3, 3)
    nrot = rotations.shape[0]
    nproc = max(1, min(nproc or os.cpu_count() or 1, nrot))
    per = -(-nrot // nproc)
    offsets = list(range(0, nrot, per))
    jobs = [(target, template, mask, laplace_filter, rotations[o:o + per]) for o in offsets]
    if len(jobs) == 1:
        parts = [_top2_worker(jobs[0])]
    else:
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            parts = pool.map(_top2_worker, jobs)
    return merge_top2(parts, offsets)
