"""Correlator API: drop-in for the reference's ``BaseCorrelator`` /
``GPUCorrelator`` / ``PowerFitter`` (``powerfitter.py:50-163``, ``:166-255``,
``:396-555``), backed by the CUDA library through its C ABI.

Host-side preprocessing (target normalisation, lcc mask, Laplace filter,
template normalisation over the mask) is done in float64 exactly as the
reference's ``BaseCorrelator`` does it; the per-rotation work (rotation, the
FFT correlations, LCC, running max/argmax) runs on the GPU.
"""
from __future__ import annotations

import os

import numpy as np
from scipy.ndimage import binary_erosion, laplace as _nd_laplace

from . import _lib


class BaseCorrelator:
    """Same contract as the reference ``BaseCorrelator`` (``powerfitter.py:166-255``)."""

    def __init__(self, target, laplace=False):
        target = np.asarray(target)
        self._target = target / target.max()
        self._rotations = None
        self._template = None
        self._mask = None
        self._laplace = laplace
        self._lcc_mask = self._get_lcc_mask(self._target)
        self._rmax = min(target.shape) // 2

    @staticmethod
    def _get_lcc_mask(target):
        return (target > target.max() * 0.05).astype(np.uint8)

    @property
    def target(self):
        return self._target

    @property
    def mask(self):
        return self._mask

    @mask.setter
    def mask(self, mask):
        if self._template is None:
            raise ValueError("First set the template.")
        if self._target.shape != mask.shape:
            raise ValueError("Shape of the mask is different from target.")
        ind = mask != 0
        self._norm_factor = ind.sum()
        if self._norm_factor == 0:
            raise ValueError("Zero-filled mask is not allowed.")
        self._mask = mask.copy()
        if self._laplace:
            self._template = self._laplace_filter(self._template)
        self._template *= self._mask
        self._normalize_template(ind)
        # multiplied again for the core-weighted correlation score
        self._template *= self._mask

    @staticmethod
    def _laplace_filter(array):
        return _nd_laplace(array, mode="wrap")

    def _normalize_template(self, ind):
        self._template[ind] -= self._template[ind].mean()
        self._template[ind] /= self._template[ind].std()

    @property
    def rotations(self):
        return self._rotations

    @rotations.setter
    def rotations(self, rotations):
        self._rotations = np.asarray(rotations, dtype=np.float64).reshape(-1, 3, 3)

    @property
    def template(self):
        return self._template

    @template.setter
    def template(self, template):
        if template.shape != self._target.shape:
            raise ValueError("Shape of template does not match the target.")
        self._mask = None
        self._template = np.array(template, dtype=np.float64, copy=True)

    @property
    def lcc(self):
        return self._lcc

    @property
    def rot(self):
        return self._rot

    def scan(self):
        if any(req is None for req in (self._template, self._mask, self._rotations)):
            raise ValueError("First set the template, mask, and rotations.")


class CUDACorrelator(BaseCorrelator):
    """GB300 correlator: same setters, ``scan()``, ``lcc`` (float32) and ``rot``
    (int32) as the reference ``GPUCorrelator`` (``powerfitter.py:396-555``).

    ``device`` picks the CUDA device; ``flags`` are ``PF_FLAG_*`` values of the
    C ABI (e.g. float64 LCC normalisation).  An optional ``_counter`` with an
    ``increment()`` method is advanced once per rotation, like the reference's
    progress counter.
    """

    def __init__(self, target, laplace=False, device=0, flags=0):
        super().__init__(target, laplace=laplace)
        self._device = device
        self._flags = flags
        self._ctx = _lib.Context(self._target.shape, device)
        ftarget = self._laplace_filter(self._target) if self._laplace else self._target
        self._ctx.set_target(ftarget, self._lcc_mask)

    @staticmethod
    def _laplace_filter(array):
        """Periodic Laplace filter on the GPU (``pf_laplace_wrap``)."""
        return _lib.laplace_wrap(array)

    @BaseCorrelator.mask.setter
    def mask(self, mask):
        BaseCorrelator.mask.fset(self, mask)
        self._ctx.set_template_mask(self._template, self._mask, float(self._norm_factor), self._rmax)

    def scan(self, rot_offset=0):
        self._start(rot_offset)
        while self._launch_next():
            self._wait()
        self._results()

    # The scan in steps, so that several devices run at once (PowerFitter.scan
    # launches the same step on every device before waiting on any).  Without
    # a progress counter the whole set is one asynchronous call.  With one
    # (the reference advances it once per rotation, powerfitter.py:332-333, and
    # its driver polls it, :120-128), the set runs in slices of whole rotation
    # batches, about a hundredth of the set each, and the counter advances as
    # each slice completes; slices of whole batches accumulate to the same
    # results as one call, bit for bit.
    def _start(self, rot_offset=0):
        super().scan()
        self._rot_offset = int(rot_offset)
        self._ctx.set_rotations(self._rotations)
        nrot = self._rotations.shape[0]
        step = nrot
        if getattr(self, "_counter", None) is not None:
            pairs, _, _ = self._ctx.get_tuning()
            batch = 2 * max(1, pairs)
            step = batch * max(1, -(-nrot // (100 * batch)))
        self._slices = [(f, min(step, nrot - f)) for f in range(0, nrot, max(step, 1))] or [(0, 0)]
        self._next = 0

    def _launch_next(self):
        """Queue the next slice (asynchronous); False when none is left."""
        if self._next >= len(self._slices):
            return False
        first, count = self._slices[self._next]
        self._ctx.scan_resident(first, count, self._rot_offset,
                                self._flags | (_lib.PF_FLAG_ACCUMULATE if self._next else 0))
        return True

    def _wait(self):
        """Wait for the slice in flight and advance the progress counter."""
        self._ctx.synchronize()
        counter = getattr(self, "_counter", None)
        if counter is not None:
            for _ in range(self._slices[self._next][1]):
                counter.increment()
        self._next += 1

    def _results(self):
        self._lcc, self._rot = self._ctx.get_results()

    @property
    def context(self):
        return self._ctx


def determine_core_indices(mask):
    """Core weights: number of binary erosions a voxel survives (``helpers.py:26-34``)."""
    core = np.zeros(mask.shape)
    eroded = mask > 0
    while eroded.sum() > 0:
        core += eroded
        eroded = binary_erosion(eroded)
    return core


def combine_shards(parts, nrot_per_job):
    """Merge per-shard (lcc, rot) results: strict ``>``, rotation index of shard n
    offset by ``n * nrot_per_job`` (``PowerFitter._combine``, ``powerfitter.py:146-163``).
    Runs the merge on the GPU."""
    lcc = np.zeros(parts[0][0].shape, dtype=np.float32)
    rot = np.zeros(parts[0][0].shape, dtype=np.int32)
    for n, (plcc, prot) in enumerate(parts):
        _lib.combine_into(lcc.reshape(-1), rot.reshape(-1), np.asarray(plcc, np.float32).reshape(-1),
                          np.asarray(prot, np.int32).reshape(-1), n * nrot_per_job)
    return lcc, rot


class PowerFitter:
    """Search driver with the reference ``PowerFitter`` surface (``powerfitter.py:50-163``).

    ``_queues`` (the reference's list of OpenCL queues) is replaced by
    ``_devices``: CUDA device indices.  With one device the whole rotation set
    is scanned there; with several, contiguous rotation slices are scanned on
    each device and merged with ``_combine`` semantics.
    """

    def __init__(self, target, laplace=False):
        self._target = target
        self._rotations = None
        self._template = None
        self._mask = None
        self._devices = None
        self._nproc = 1
        self._directory = os.path.abspath("./")
        self._laplace = laplace
        self._flags = 0

    @property
    def directory(self):
        return self._directory

    @directory.setter
    def directory(self, directory):
        if os.path.isdir(directory):
            self._directory = os.path.abspath(directory)
        else:
            raise ValueError("Directory does not exist.")

    @staticmethod
    def _array(x):
        return x.array if hasattr(x, "array") else np.asarray(x)

    def scan(self):
        devices = list(self._devices) if self._devices else [0]
        rot = np.asarray(self._rotations, dtype=np.float64).reshape(-1, 3, 3)
        nrot = rot.shape[0]
        per = nrot // len(devices)
        corrs = []
        for n, dev in enumerate(devices):
            end = None if n == len(devices) - 1 else (n + 1) * per
            corr = CUDACorrelator(self._array(self._target), laplace=self._laplace, device=dev,
                                  flags=self._flags)
            corr.template = self._array(self._template)
            corr.mask = self._array(self._mask)
            corr.rotations = rot[n * per:end]
            corrs.append(corr)
        # every device's slice is queued before any is waited on: the devices
        # search their rotations at the same time
        for corr in corrs:
            corr._start()
        while True:
            running = [corr for corr in corrs if corr._launch_next()]
            if not running:
                break
            for corr in running:
                corr._wait()
        parts = []
        for corr in corrs:
            corr._results()
            parts.append((corr.lcc, corr.rot))
        self._corr = corrs[-1]
        if len(parts) == 1:
            self._lcc, self._rot = parts[0]
        else:
            self._lcc, self._rot = combine_shards(parts, per)
