"""Learned rotation proposal: rank rotations from a coarse search, re-search
only the top fraction at full resolution.

The exhaustive search scores every rotation of a set at full resolution.  The
proposal path instead

1. searches a coarse copy of the map (32^3: the target and template low-passed
   to the coarse grid's Nyquist resolution, as the reference's
   ``lower_resolution`` does (``volume.py:129-141``), then decimated; the
   mask max-pooled) over the whole set, keeping each rotation's best LCC
   (``PF_FLAG_ROT_MAX``);
2. builds per-rotation features from those coarse scores: the rotation's own
   score and its nearest rotations' scores in SO(3), z-scored over the map,
   how well the voxels holding the neighbours' maxima agree with the
   rotation's own (a true fit puts neighbouring rotations' peaks at one
   place, noise scatters them), and how many of the map's top rotations put
   their peak where this rotation puts its own (peak-position votes);
3. scores the features with a small network (bfloat16 weights, float32
   accumulation; forward, gradient and Adam are this project's CUDA kernels,
   ``csrc/pf_learn.cu``), trained on pairs of coarse features and
   full-resolution per-rotation best LCC that the exhaustive search generates;
4. searches the top fraction of the rotations at full resolution: the
   operating fraction chosen on validation maps when the network was trained
   and stored with its weights (0.2% for the shipped network).

The exhaustive search stays the fallback (``fraction=1``) and the measure of
the proposal: recall is whether the proposal's rotations contain the
exhaustive best fit.  PyTorch holds the device tensors and does the gathers and top-k
around the kernels.
"""
from __future__ import annotations

import math
import os
import time

import numpy as np

from . import _lib

COARSE_EDGE = 32
NEIGHBOURS = 12
BASE_FEATURES = 1 + NEIGHBOURS + 4  # own score, neighbour scores (descending), their mean and std,
                                    # peak agreement and the agreement-weighted neighbour score
FEATURES = BASE_FEATURES + 2        # and the peak-position votes (count and score-weighted)
VOTE_TOP = 0.02                     # the map's top 2% of rotations (coarse score) cast the votes
AGREE_SIGMA = 1.0                  # coarse voxels
HIDDEN = 32
TOP_FRACTION = 0.05


# ---------------------------------------------------------------------------
# rotation-set geometry
# ---------------------------------------------------------------------------

def rotmat_to_quat(rotmats):
    """Unit quaternions (w, x, y, z) of rotation matrices (Shepperd's method)."""
    R = np.asarray(rotmats, dtype=np.float64).reshape(-1, 3, 3)
    tr = R[:, 0, 0] + R[:, 1, 1] + R[:, 2, 2]
    q = np.empty((R.shape[0], 4))
    d = np.stack([tr, R[:, 0, 0], R[:, 1, 1], R[:, 2, 2]], axis=1)
    k = np.argmax(d, axis=1)
    for case in range(4):
        s = k == case
        if not s.any():
            continue
        r = R[s]
        if case == 0:
            t = np.sqrt(1.0 + tr[s]) * 2
            q[s] = np.stack([0.25 * t, (r[:, 2, 1] - r[:, 1, 2]) / t, (r[:, 0, 2] - r[:, 2, 0]) / t,
                             (r[:, 1, 0] - r[:, 0, 1]) / t], axis=1)
        else:
            i = case - 1
            j, l = (i + 1) % 3, (i + 2) % 3
            t = np.sqrt(1.0 + r[:, i, i] - r[:, j, j] - r[:, l, l]) * 2
            qq = np.empty((r.shape[0], 4))
            qq[:, 0] = (r[:, l, j] - r[:, j, l]) / t
            qq[:, 1 + i] = 0.25 * t
            qq[:, 1 + j] = (r[:, j, i] + r[:, i, j]) / t
            qq[:, 1 + l] = (r[:, l, i] + r[:, i, l]) / t
            q[s] = qq
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def rotation_neighbours(rotmats, k=NEIGHBOURS):
    """(R, k) indices of each rotation's k nearest rotations in SO(3) (q and -q
    are the same rotation), nearest first, the rotation itself excluded."""
    from scipy.spatial import cKDTree
    q = rotmat_to_quat(rotmats)
    n = q.shape[0]
    if n < 2:
        return np.zeros((n, k), dtype=np.int64)
    tree = cKDTree(np.concatenate([q, -q]))
    _, idx = tree.query(q, k=min(k + 1, 2 * n))
    idx = (idx % n).astype(np.int64)
    # q_j and -q_j are 2 apart, so no rotation shows up twice; drop the rotation itself
    rows = np.arange(n)[:, None]
    keep = idx != rows
    order = np.argsort(~keep, axis=1, kind="stable")
    idx = np.take_along_axis(idx, order, axis=1)[:, :k]
    if idx.shape[1] < k:
        idx = np.concatenate([idx, np.repeat(idx[:, -1:], k - idx.shape[1], axis=1)], axis=1)
    return idx


# ---------------------------------------------------------------------------
# coarse maps
# ---------------------------------------------------------------------------

def coarse_factor(n, edge=COARSE_EDGE):
    """Integer decimation factor that brings an edge of n voxels to about `edge`."""
    k = max(1, int(round(n / float(edge))))
    while k > 1 and n % k:
        k -= 1
    return k


def coarsen(target, template, mask, voxelspacing, resolution, edge=COARSE_EDGE):
    """Coarse (target, template, mask, voxel spacing, resolution) for the proposal search.

    Target and template are low-passed from `resolution` to the coarse grid's
    Nyquist resolution (2 coarse voxels) with a periodic Gaussian -- the
    kernel width sqrt(s_low^2 - s_high^2) of ``lower_resolution`` -- and
    decimated so that coarse voxel i is fine voxel k*i (the rotation centre
    stays voxel 0); the mask is max-pooled over the k-voxel neighbourhood.
    """
    from scipy.ndimage import gaussian_filter, maximum_filter
    from .volume import res_to_sigma
    n = np.asarray(target).shape
    k = coarse_factor(min(n), edge)
    if any(s % k for s in n):
        raise ValueError("grid %s not divisible by the coarse factor %d" % (n, k))
    cs = voxelspacing * k
    res_low = max(resolution, 2.0 * cs)
    sk = math.sqrt(max(res_to_sigma(res_low) ** 2 - res_to_sigma(resolution) ** 2, 0.0)) / voxelspacing

    def low(a):
        a = np.asarray(a, dtype=np.float64)
        a = gaussian_filter(a, sk, mode="wrap") if sk > 0 else a
        return np.ascontiguousarray(a[::k, ::k, ::k])

    m = maximum_filter(np.asarray(mask, dtype=np.float64), size=k, mode="wrap")[::k, ::k, ::k]
    return low(target), low(template), np.ascontiguousarray((m > 0).astype(np.float64)), cs, res_low


# ---------------------------------------------------------------------------
# one map prepared for both searches
# ---------------------------------------------------------------------------

# batch and tile shapes chosen by the autotuner, per (grid shape, set size):
# a run over many maps of one size tunes each search once
_TUNING = {}


def _tuned(ctx, shape, nrot, trial):
    key = (tuple(shape), int(nrot))
    if key in _TUNING:
        ctx.set_tuning(**_TUNING[key])
    else:
        cfg = ctx.autotune(trial)
        _TUNING[key] = {k: cfg[k] for k in ("pairs", "rows1", "rows3")}


class SearchPair:
    """A map's fine and coarse searches (contexts on one device) over one rotation set."""

    def __init__(self, target, template, mask, voxelspacing, resolution, rotmats, laplace=False,
                 core_weighted=False, device=0):
        from .correlator import BaseCorrelator
        self.rotmats = np.ascontiguousarray(rotmats, dtype=np.float64).reshape(-1, 3, 3)
        self.nrot = self.rotmats.shape[0]
        ct, ctm, cm, _, _ = coarsen(target, template, mask, voxelspacing, resolution)
        if core_weighted:
            mask = _lib.core_indices(np.asarray(mask, dtype=np.float64))
            cm = _lib.core_indices(cm)
        self.fine = self._context(BaseCorrelator, target, template, mask, laplace, device)
        self.coarse = self._context(BaseCorrelator, ct, ctm, cm, laplace, device)
        self.coarse.set_rotations(self.rotmats)
        # batch and tile shapes for both grids (short timed trial scans, once per grid shape)
        _tuned(self.coarse, cm.shape, self.nrot, min(2048, self.nrot))
        self.fine.set_rotations(self.rotmats[:min(512, self.nrot)])
        _tuned(self.fine, np.asarray(target).shape, self.nrot, min(512, self.nrot))

    @staticmethod
    def _context(Base, target, template, mask, laplace, device):
        base = Base(np.asarray(target, dtype=np.float64), laplace=laplace)
        base.template = template
        base.mask = mask
        ctx = _lib.Context(base._target.shape, device)
        ft = _lib.laplace_wrap(base._target) if laplace else base._target
        ctx.set_target(ft, base._lcc_mask)
        ctx.set_template_mask(base._template, base._mask, float(base._norm_factor), base._rmax)
        return ctx

    def coarse_scores(self):
        """Best coarse LCC of every rotation of the set and the coarse voxel holding it."""
        self.coarse.scan_resident(0, self.nrot, 0, _lib.PF_FLAG_ROT_MAX)
        return self.coarse.rotation_best(0, self.nrot)

    def fine_exhaustive(self, rotation_max=False):
        """Full-resolution search of the whole set: (lcc, rot[, per-rotation best])."""
        self.fine.set_rotations(self.rotmats)
        self.fine.scan_resident(0, self.nrot, 0, _lib.PF_FLAG_ROT_MAX if rotation_max else 0)
        lcc, rot = self.fine.get_results()
        if rotation_max:
            return lcc, rot, self.fine.rotation_max(0, self.nrot)
        return lcc, rot

    def fine_subset(self, sel):
        """Full-resolution search of rotations `sel` (ascending indices of the
        set); rot holds indices of the set."""
        sel = np.asarray(sel, dtype=np.int64)
        self.fine.set_rotations(self.rotmats[sel])
        self.fine.scan_resident(0, sel.size, 0, 0)
        lcc, rot = self.fine.get_results()
        hit = lcc > 0
        rot = rot.copy()
        rot[hit] = sel[rot[hit]].astype(np.int32)
        return lcc, rot

    def close(self):
        self.fine.close()
        self.coarse.close()


# ---------------------------------------------------------------------------
# features and the network
# ---------------------------------------------------------------------------

def zscore(a, rel=1e-6):
    """(a - mean) / std, or zeros where `a` has no spread: a feature that is the
    same for every rotation of a map (all peaks at one voxel, say) carries no
    information, and dividing its rounding residue by a zero spread would
    give inputs of 1e5 and more."""
    import torch
    m = a.mean()
    sd = a.std()
    if not bool(torch.isfinite(sd)) or float(sd) <= rel * max(1.0, abs(float(m))):
        return torch.zeros_like(a)
    return (a - m) / sd


FEATURE_CLIP = 20.0   # features are clamped to +-20 (z-scores of a well-spread feature stay far inside)


def peak_votes(z, v, shape):
    """Peak-position votes of every rotation: how many of the map's top
    rotations (coarse z-score in the top VOTE_TOP) hold their best coarse LCC
    within one coarse voxel (periodic) of this rotation's own peak voxel, as
    log(1 + count) and as the sum of those rotations' z-scores.  A copy of
    the template in the map draws the peaks of many rotations near the true
    one to its position; noise scatters them."""
    import torch
    nz, ny, nx = shape
    n = nz * ny * nx
    top = z >= torch.quantile(z, 1.0 - VOTE_TOP)
    cnt = torch.bincount(v[top], minlength=n).float().reshape(1, 1, nz, ny, nx)
    wsum = torch.bincount(v[top], weights=z[top], minlength=n).float().reshape(1, 1, nz, ny, nx)
    grid = torch.cat([cnt, wsum], dim=1)
    # 3x3x3 periodic box sum
    box = sum(torch.roll(grid, (a, b, c), dims=(2, 3, 4)) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1))
    flat = box.reshape(2, n)
    return torch.log1p(flat[0][v]), flat[1][v]


def features(coarse, nbr, shape, device=0, votes=True):
    """(R, FEATURES) float32 CUDA tensor from the coarse search's per-rotation
    (best LCC, voxel) and the neighbour table (R, k); `shape` is the coarse
    grid.  ``votes=False`` leaves out the two vote features (BASE_FEATURES
    columns, the input of networks trained without them)."""
    import torch
    scores, voxels = coarse
    dev = "cuda:%d" % device
    s = torch.as_tensor(np.asarray(scores, dtype=np.float32), device=dev)
    finite = torch.isfinite(s)
    lo = s[finite].min() if bool(finite.any()) else torch.tensor(0.0, device=s.device)
    s = torch.where(finite, s, lo)
    z = zscore(s)
    nb = torch.as_tensor(nbr, device=dev)
    ns = z[nb]
    srt = torch.sort(ns, dim=1, descending=True).values
    # agreement of the neighbours' peak positions with the rotation's own (periodic distance)
    v = torch.as_tensor(np.asarray(voxels, dtype=np.int64), device=dev).clamp(min=0)
    nz, ny, nx = shape
    pos = torch.stack([v // (ny * nx), (v // nx) % ny, v % nx], dim=1).float()
    ext = torch.tensor([nz, ny, nx], dtype=torch.float32, device=dev)
    d = (pos[nb] - pos[:, None, :]).abs()
    d = torch.minimum(d, ext - d)
    agree = torch.exp(-(d * d).sum(-1) / (2.0 * AGREE_SIGMA ** 2))
    wz = (agree * ns).sum(1, keepdim=True) / (agree.sum(1, keepdim=True) + 1e-6)
    cols = [z[:, None], srt, ns.mean(1, keepdim=True), ns.std(1, keepdim=True), agree.mean(1, keepdim=True), wz]
    if votes:
        vc, vw = peak_votes(z, v, shape)
        cols += [zscore(vc)[:, None], zscore(vw)[:, None]]
    x = torch.cat(cols, dim=1)
    return torch.nan_to_num(x, nan=0.0, posinf=FEATURE_CLIP, neginf=-FEATURE_CLIP).clamp_(-FEATURE_CLIP,
                                                                                       FEATURE_CLIP).contiguous()


def targets(fine_scores, device=0):
    """z-scored full-resolution per-rotation best LCC and loss weights that
    stress the top 5% (the rotations the proposal must not miss)."""
    import torch
    t = torch.as_tensor(np.asarray(fine_scores, dtype=np.float32), device="cuda:%d" % device)
    finite = torch.isfinite(t)
    lo = t[finite].min() if bool(finite.any()) else torch.tensor(0.0, device=t.device)
    t = torch.where(finite, t, lo)
    z = (t - t.mean()) / (t.std() + 1e-12)
    thr = torch.quantile(z, 1.0 - TOP_FRACTION)
    w = 1.0 + 9.0 * (z >= thr).float()
    return z.contiguous(), w.contiguous()


def default_weights():
    """The trained network shipped with the package (see data/proposal_net_report.json)."""
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "proposal_net.npz")


class ProposalNet:
    """The scoring network: float32 master parameters, bfloat16 copy, Adam state."""

    def __init__(self, nin=FEATURES, nh=HIDDEN, device=0, seed=0, params=None):
        import torch
        self.nin, self.nh, self.device = int(nin), int(nh), int(device)
        self.count = _lib.mlp_param_count(self.nin, self.nh)
        dev = "cuda:%d" % self.device
        if params is None:
            rng = np.random.default_rng(seed)
            nh, nin = self.nh, self.nin
            parts = [rng.normal(0, math.sqrt(2.0 / nin), nh * nin), np.zeros(nh),
                     rng.normal(0, math.sqrt(2.0 / nh), nh * nh), np.zeros(nh),
                     rng.normal(0, math.sqrt(1.0 / nh), nh), np.zeros(1)]
            params = np.concatenate(parts)
        params = np.asarray(params, dtype=np.float32)
        if params.size != self.count:
            raise ValueError("expected %d parameters, got %d" % (self.count, params.size))
        self.p = torch.as_tensor(params, device=dev).contiguous()
        self.pb = self.p.to(torch.bfloat16).contiguous()
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.grad = torch.zeros_like(self.p)
        self.loss = torch.zeros(1, dtype=torch.float32, device=dev)
        self.step = 0
        self.fraction = TOP_FRACTION     # operating fraction of the proposal search

    def _stream(self):
        import torch
        return torch.cuda.current_stream(self.device).cuda_stream

    def forward(self, x):
        import torch
        y = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        _lib.mlp_forward(x, self.nin, self.nh, self.pb, y, self._stream())
        return y

    def train(self, x, t, w, epochs=30, batch=65536, lr=2e-3, seed=0, log=None):
        """Adam on L = sum_i w_i (net(x_i) - t_i)^2 / sum_i w_i over minibatches."""
        import torch
        n = x.shape[0]
        gen = torch.Generator(device=x.device)
        gen.manual_seed(seed)
        wmean = float(w.mean())
        history = []
        for ep in range(epochs):
            perm = torch.randperm(n, device=x.device, generator=gen)
            tot = 0.0
            for b0 in range(0, n, batch):
                idx = perm[b0:b0 + batch]
                xb, tb, wb = x[idx].contiguous(), t[idx].contiguous(), w[idx].contiguous()
                self.grad.zero_()
                self.loss.zero_()
                _lib.mlp_grad(xb, tb, wb, self.nin, self.nh, self.pb, 1.0 / (idx.numel() * wmean), self.grad,
                              self.loss, self._stream())
                self.step += 1
                _lib.mlp_adam(self.p, self.pb, self.grad, self.m, self.v, lr, self.step, stream=self._stream())
                tot += float(self.loss.item()) * idx.numel()
            history.append(tot / n)
            if log:
                log("epoch %d loss %.5f" % (ep, history[-1]))
        return history

    def params(self):
        return self.p.detach().cpu().numpy()

    def save(self, path, meta=None):
        np.savez(path, params=self.params(), nin=self.nin, nh=self.nh, meta=np.array(repr(meta or {})))

    @classmethod
    def load(cls, path, device=0):
        """Weights saved by `save`; ``fraction`` is the operating fraction
        stored with them (chosen on validation maps when the network was
        trained), else TOP_FRACTION."""
        import ast
        with np.load(path) as d:
            net = cls(int(d["nin"]), int(d["nh"]), device=device, params=d["params"])
            meta = ast.literal_eval(str(d["meta"])) if "meta" in d.files else {}
        fr = meta.get("fractions") if isinstance(meta, dict) else None
        net.fraction = float(fr["network"]) if fr and "network" in fr else TOP_FRACTION
        return net


# ---------------------------------------------------------------------------
# the proposal search
# ---------------------------------------------------------------------------

def rank_scores(net, coarse, nbr, shape, device=0):
    """Per-rotation proposal scores: the network on the coarse features, or
    the coarse score itself when `net` is None (the method without it)."""
    if net is None:
        import torch
        return torch.as_tensor(np.asarray(coarse[0], dtype=np.float32), device="cuda:%d" % device)
    return net.forward(features(coarse, nbr, shape, device, votes=net.nin > BASE_FEATURES))


def select(score, fraction=TOP_FRACTION):
    """Ascending indices of the top `fraction` of the rotations by `score`."""
    import torch
    k = max(1, int(math.ceil(fraction * score.numel())))
    s = torch.nan_to_num(score, nan=-float("inf"))
    return torch.sort(torch.topk(s, k).indices).values.cpu().numpy()


def proposal_search(pair, net, nbr, fraction=None, timings=None):
    """Coarse search, ranking, full-resolution search of the top fraction
    (default: the network's operating fraction, or TOP_FRACTION for the coarse
    score alone, ``net`` None; 1 is the exhaustive search).
    Returns (lcc, rot, selected rotation indices)."""
    import torch
    if fraction is None:
        fraction = net.fraction if net is not None else TOP_FRACTION
    t0 = time.perf_counter()
    coarse = pair.coarse_scores()
    t1 = time.perf_counter()
    sel = select(rank_scores(net, coarse, nbr, pair.coarse.shape, pair.fine.device), fraction)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    lcc, rot = pair.fine_subset(sel)
    t3 = time.perf_counter()
    if timings is not None:
        timings.update(coarse_s=t1 - t0, rank_s=t2 - t1, fine_s=t3 - t2, total_s=t3 - t0)
    return lcc, rot, sel
