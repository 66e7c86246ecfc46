"""Queue of maps of uneven size scanned together on one GPU, on concurrent
streams or as one captured CUDA graph.

Each map gets its own context (its own compile-time- or runtime-planned
kernels for its grid) on its own CUDA stream; after the per-map setup
(target spectra, template, rotations), every map's scan is queued before any
is awaited, so the kernels of small maps run beside those of large ones and
fill the GPU together.  Results equal per-map scans (same kernels, same
order of rotations per voxel).

Batch and tile shapes: a job's ``pairs`` fixes the rotation pairs per batch;
with ``pairs = 0`` the library's autotuner (``pf_autotune``) picks pairs per
batch and the tile rows of passes 1 and 3 from short timed trial scans.  A
``tuning`` dict shared across calls keeps the choice per grid shape, so a
queue autotunes each size it holds once and reuses the shapes for every later
map of that size.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .correlator import BaseCorrelator


class _Prep(BaseCorrelator):
    """Host preprocessing with the Laplace filter on the GPU (as CUDACorrelator)."""

    @staticmethod
    def _laplace_filter(array):
        return _lib.laplace_wrap(array)


@dataclass
class MapJob:
    target: np.ndarray
    template: np.ndarray
    mask: np.ndarray
    rotations: np.ndarray
    laplace: bool = False
    rot_offset: int = 0
    flags: int = 0
    pairs: int = 0                  # rotation pairs per batch (0: autotune)
    lcc: np.ndarray = field(default=None, repr=False)
    rot: np.ndarray = field(default=None, repr=False)


def _tune(ctx, job, nrot, autotune_trial, tuning):
    """Batch and tile shapes of one map: the job's fixed pairs, the shapes
    already chosen for its grid shape in ``tuning``, or the autotuner's."""
    if job.pairs:
        ctx.set_tuning(pairs=job.pairs)
        return
    key = tuple(job.target.shape)
    if tuning is not None and key in tuning:
        ctx.set_tuning(**{k: tuning[key][k] for k in ("pairs", "rows1", "rows3")})
    elif autotune_trial:
        cfg = ctx.autotune(min(autotune_trial, nrot))
        if tuning is not None:
            tuning[key] = cfg


def scan_queue(jobs, device=0, autotune_trial=256, streams=None, tuning=None):
    """Scan every job; fills ``job.lcc`` / ``job.rot`` and returns the jobs.

    ``streams``: torch CUDA streams or raw ``cudaStream_t`` handles, one per
    job (default: a new torch stream per job).  ``tuning``: a dict of batch and
    tile shapes per grid shape, read and filled (see the module docstring).
    """
    import torch
    torch.cuda.set_device(device)
    if streams is None:
        streams = [torch.cuda.Stream(device=device) for _ in jobs]
    handles = [s.cuda_stream if hasattr(s, "cuda_stream") else int(s) for s in streams]
    contexts = []
    for job, h in zip(jobs, handles):
        base = _Prep(job.target, laplace=job.laplace)
        base.template = job.template
        base.mask = job.mask
        ctx = _lib.Context(base._target.shape, device)
        ctx.set_stream(h)
        ftarget = base._laplace_filter(base._target) if job.laplace else base._target
        ctx.set_target(ftarget, base._lcc_mask)
        ctx.set_template_mask(base._template, base._mask, float(base._norm_factor), base._rmax)
        nrot = ctx.set_rotations(job.rotations)
        _tune(ctx, job, nrot, autotune_trial, tuning)
        contexts.append((ctx, nrot))
    # queue every scan before waiting for any
    for job, (ctx, nrot) in zip(jobs, contexts):
        ctx.scan_resident(0, nrot, job.rot_offset, job.flags)
    for job, (ctx, _) in zip(jobs, contexts):
        job.lcc, job.rot = ctx.get_results()
    for ctx, _ in contexts:
        ctx.close()
    return jobs


class QueueGraph:
    """A queue whose scans are captured once into one CUDA graph.

    Every map keeps its context and stream; the capture forks each map's
    stream from one capture stream and joins it back, so a replay launches the
    whole queue -- every map's kernels on its own stream, concurrent as in
    ``scan_queue`` -- with one graph launch.  Setup (spectra, template,
    rotations, tuning) and one uncaptured warm-up scan per map, which makes
    every device buffer, come before the capture.  Each replay recomputes the
    results from scratch.
    """

    def __init__(self, jobs, device=0, autotune_trial=256, tuning=None):
        import torch
        torch.cuda.set_device(device)
        self.device = device
        self.jobs = list(jobs)
        self.streams = [torch.cuda.Stream(device=device) for _ in self.jobs]
        self.contexts = []
        for job, st in zip(self.jobs, self.streams):
            base = _Prep(job.target, laplace=job.laplace)
            base.template = job.template
            base.mask = job.mask
            ctx = _lib.Context(base._target.shape, device)
            ctx.set_stream(st.cuda_stream)
            ftarget = base._laplace_filter(base._target) if job.laplace else base._target
            ctx.set_target(ftarget, base._lcc_mask)
            ctx.set_template_mask(base._template, base._mask, float(base._norm_factor), base._rmax)
            nrot = ctx.set_rotations(job.rotations)
            _tune(ctx, job, nrot, autotune_trial, tuning)
            self.contexts.append((ctx, nrot))
        self._scan_all()                        # warm-up: allocates every buffer the scans use
        torch.cuda.synchronize(device)
        self.graph = torch.cuda.CUDAGraph()
        main = torch.cuda.Stream(device=device)
        with torch.cuda.graph(self.graph, stream=main):
            for st, (ctx, nrot), job in zip(self.streams, self.contexts, self.jobs):
                st.wait_stream(main)
                ctx.scan_resident(0, nrot, job.rot_offset, job.flags)
                main.wait_stream(st)

    def _scan_all(self):
        for (ctx, nrot), job in zip(self.contexts, self.jobs):
            ctx.scan_resident(0, nrot, job.rot_offset, job.flags)

    def replay(self):
        self.graph.replay()

    def results(self):
        """Fill every job's ``lcc`` / ``rot`` from the last replay."""
        import torch
        torch.cuda.synchronize(self.device)
        for job, (ctx, _) in zip(self.jobs, self.contexts):
            job.lcc, job.rot = ctx.get_results()
        return self.jobs

    def close(self):
        for ctx, _ in self.contexts:
            ctx.close()
        self.contexts = []


# The uneven-map workload: 16 seeded maps of 48^3-160^3.
QUEUE_SIZES = (48, 64, 96, 128, 160)


def make_queue(nmaps=16, seed=0):
    """Seeded maps of uneven size (1.2-2.5 A/voxel, 800-6000 atoms, 5-9 A, SNR 2-6)."""
    from . import synth
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(nmaps):
        n = int(QUEUE_SIZES[i % len(QUEUE_SIZES)])
        vs = float(rng.uniform(1.2, 2.5))
        natoms = int(rng.integers(800, 6001))
        res = float(rng.uniform(5.0, 9.0))
        snr = float(rng.uniform(2.0, 6.0))
        # keep the chain inside the box
        natoms = min(natoms, int(1500 * (n * vs / 2.0 / 30.0) ** 3))
        cases.append(synth.make_case((n, n, n), vs, max(natoms, 200), 1, res, snr, seed * 100 + i))
    return cases
