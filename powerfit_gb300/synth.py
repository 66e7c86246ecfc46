"""Seeded synthetic inputs for the LCC search: chains, density maps, templates.

No public dataset is involved: every map is generated here from a seed.

* Chains: a confined self-avoiding random walk with 3.8 A steps; a step closer
  than 3.0 A to any earlier atom is rejected; the walk stays inside a sphere of
  radius sqrt(5/3) * Rg_target, with Rg_target = 18 A * (atoms / 1500)^(1/3),
  widened to keep the exclusion-sphere packing at or below 0.2 (a random
  walk cannot fill the 0.41 packing the narrower sphere would need).  On a
  dead end the walk backs up and continues.  Elements
  C/N/O/S are drawn at 62/17/20/1 %; template weights are atomic numbers.
* Maps: seeded rigid copies of the chain (random rotations, centres kept
  apart), blurred with sigma = resolution / (sqrt(2) pi) (reference
  ``volume.py:121-122``) using the 4-sigma truncated Gaussian splat of
  ``_powerfit.pyx:75-140`` (``blur_points``) with wraparound, plus Gaussian
  noise with sigma = std(clean map over voxels > 1 % of max) / SNR.
* Template and mask: copy 0 in its own frame, centroid moved to the map origin
  (reference ``powerfit.py:244-255``); mask = balls of 5 A (``dilate_points``,
  ``_powerfit.pyx:143-206``, ``volume.py:204-211``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .rotations import quat_to_rotmat

ELEMENTS = np.array([6, 7, 8, 16])            # C, N, O, S (atomic numbers)
ELEMENT_P = np.array([0.62, 0.17, 0.20, 0.01])


def res_to_sigma(resolution):
    """Gaussian sigma (A) of a map at ``resolution`` (reference ``volume.py:121-122``)."""
    return resolution / (math.sqrt(2.0) * math.pi)


def _splat_indices(points, extend, shape, wraparound):
    """Voxel offsets around each point within ``extend`` (per-point radius).

    Restates the index bounds of ``_powerfit.pyx:117-131`` / ``:180-197``: the
    box [ceil(p - e), floor(p + e)] clipped to [-(n-1), n-1] with wraparound
    (negative indices wrap, large ones are clipped) or to [0, n-1] without.
    Returns flat indices (C order over z, y, x), squared distances and a
    validity mask, atom-major then z, y, x as the reference loops.
    """
    pts = np.asarray(points, dtype=np.float64)          # (3, N) as x, y, z
    ext = np.broadcast_to(np.asarray(extend, dtype=np.float64), (pts.shape[1],))
    k = int(np.floor(2.0 * ext.max())) + 2
    off = np.arange(k)
    nz, ny, nx = shape
    per_axis = []
    for n, axis in ((nx, 0), (ny, 1), (nz, 2)):
        p = pts[axis][:, None]
        lo = np.ceil(p - ext[:, None]).astype(np.int64)
        hi = np.floor(p + ext[:, None]).astype(np.int64)
        lo = np.maximum(lo, -(n - 1) if wraparound else 0)
        hi = np.minimum(hi, n - 1)
        c = lo + off[None, :]                                 # (N, k)
        per_axis.append((np.where(c < 0, c + n, c), (c - p) ** 2, c <= hi))
    (ix, dx2, okx), (iy, dy2, oky), (iz, dz2, okz) = per_axis
    d2 = dz2[:, :, None, None] + dy2[:, None, :, None] + dx2[:, None, None, :]
    valid = okz[:, :, None, None] & oky[:, None, :, None] & okx[:, None, None, :]
    flat = (iz[:, :, None, None] * ny + iy[:, None, :, None]) * nx + ix[:, None, None, :]
    return flat, d2, valid


def blur_points(points, weights, sigma, out, wraparound=True, chunk=2048):
    """Add w * exp(-d^2 / 2 sigma^2) within 4 sigma of every point (voxel units).

    Restates ``_powerfit.pyx:75-140``; ``points`` is (3, N) in x, y, z order.
    """
    pts = np.asarray(points, dtype=np.float64)
    w = np.asarray(weights, dtype=np.float64)
    extend = 4.0 * sigma
    flat_out = out.reshape(-1)
    for s in range(0, pts.shape[1], chunk):
        flat, d2, valid = _splat_indices(pts[:, s:s + chunk], extend, out.shape, wraparound)
        valid &= d2 <= extend * extend
        val = w[s:s + chunk, None, None, None] * np.exp(-d2 / (2.0 * sigma * sigma))
        np.add.at(flat_out, flat[valid], val[valid])
    return out


def dilate_points(points, radii, out, wraparound=True, chunk=2048):
    """Set voxels within ``radii`` of every point to 1 (``_powerfit.pyx:143-206``)."""
    pts = np.asarray(points, dtype=np.float64)
    r = np.broadcast_to(np.asarray(radii, dtype=np.float64), (pts.shape[1],))
    flat_out = out.reshape(-1)
    for s in range(0, pts.shape[1], chunk):
        rr = r[s:s + chunk]
        flat, d2, valid = _splat_indices(pts[:, s:s + chunk], rr, out.shape, wraparound)
        valid &= d2 <= (rr * rr)[:, None, None, None]
        flat_out[flat[valid]] = 1.0
    return out


def make_chain(natoms, rng, step=3.8, min_dist=3.0, rg_target=None, packing=0.2):
    """Confined self-avoiding walk: (natoms, 3) coordinates in A and elements.

    The confining radius is sqrt(5/3) * Rg_target, widened where needed so that
    the 3.0 A exclusion spheres fill at most ``packing`` of the confining ball
    (a sequential walk jams well below random close packing).  On a dead end
    the walk backs up by a growing number of atoms; a walk that stays jammed
    widens the sphere by 2 %.
    """
    if rg_target is None:
        rg_target = 18.0 * (natoms / 1500.0) ** (1.0 / 3.0)
    rconf = max(math.sqrt(5.0 / 3.0) * rg_target,
                (natoms * min_dist ** 3 / (8.0 * packing)) ** (1.0 / 3.0))
    cell = min_dist
    grid: dict = {}
    pos = np.zeros((natoms, 3))

    def key(p):
        return (int(math.floor(p[0] / cell)), int(math.floor(p[1] / cell)),
                int(math.floor(p[2] / cell)))

    def clash(p, upto):
        kx, ky, kz = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get((kx + dx, ky + dy, kz + dz), ()):
                        if j < upto - 1:
                            d = pos[j] - p
                            if d[0] * d[0] + d[1] * d[1] + d[2] * d[2] < min_dist * min_dist:
                                return True
        return False

    grid.setdefault(key(pos[0]), []).append(0)
    i = 1
    best = 1
    stuck = 0
    budget = 400 * natoms
    while i < natoms:
        budget -= 1
        if budget < 0:
            raise RuntimeError("chain generation did not converge")
        if stuck > 24:
            # persistently jammed: widen the confining sphere a little
            rconf *= 1.02
            stuck = 0
        placed = False
        for _ in range(60):
            v = rng.normal(size=3)
            cand = pos[i - 1] + step * v / np.linalg.norm(v)
            if cand @ cand > rconf * rconf:
                continue
            if clash(cand, i):
                continue
            pos[i] = cand
            grid.setdefault(key(cand), []).append(i)
            placed = True
            break
        if placed:
            i += 1
            if i > best:
                best, stuck = i, 0
            continue
        stuck += 1
        back = min(i - 1, 1 << min(stuck, 7))
        for j in range(i - back, i):
            grid[key(pos[j])].remove(j)
        i -= back
    elements = rng.choice(ELEMENTS, size=natoms, p=ELEMENT_P)
    return pos, elements


def random_rotmat(rng, n=1):
    q = rng.normal(size=(n, 4))
    return quat_to_rotmat(q / np.linalg.norm(q, axis=1, keepdims=True))


@dataclass
class Case:
    """One synthetic search problem (arrays in C order z, y, x)."""
    target: np.ndarray       # float32 map
    template: np.ndarray     # float64 blurred copy-0 chain at the origin
    mask: np.ndarray         # float64 0/1 (balls of 5 A)
    voxelspacing: float
    resolution: float
    chain: np.ndarray        # (natoms, 3) copy-0 chain, centroid at the origin
    elements: np.ndarray
    copy_rotmats: np.ndarray  # (ncopies, 3, 3) rotations applied to each copy
    copy_centres: np.ndarray  # (ncopies, 3) centres (A, x y z)
    meta: dict = field(default_factory=dict)


def make_case(shape, voxelspacing, natoms, ncopies, resolution, snr, seed):
    """Build a seeded synthetic map + template + mask (see module docstring)."""
    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in shape)
    chain, elements = make_chain(natoms, rng)
    chain = chain - chain.mean(axis=0)
    radius = float(np.sqrt((chain ** 2).sum(axis=1)).max())
    box = np.array(shape[::-1], dtype=np.float64) * voxelspacing   # x, y, z extents
    sigma = res_to_sigma(resolution) / voxelspacing
    weights = elements.astype(np.float64)
    rots = random_rotmat(rng, ncopies)
    centres = []
    for c in range(ncopies):
        for attempt in range(2000):
            lo = np.minimum(radius, box / 2)
            cen = lo + rng.random(3) * np.maximum(box - 2 * lo, 0.0)
            sep = 2.0 * radius if attempt < 1000 else 1.2 * radius
            if all(np.linalg.norm(cen - o) >= sep for o in centres):
                break
        centres.append(cen)
    centres = np.array(centres)
    clean = np.zeros(shape)
    for c in range(ncopies):
        xyz = (chain @ rots[c].T + centres[c]) / voxelspacing
        blur_points(xyz.T, weights, sigma, clean, True)
    sel = clean > 0.01 * clean.max()
    noise_sigma = clean[sel].std() / snr
    target = (clean + rng.normal(0.0, noise_sigma, size=shape)).astype(np.float32)
    template = np.zeros(shape)
    blur_points((chain / voxelspacing).T, weights, sigma, template, True)
    mask = np.zeros(shape)
    dilate_points((chain / voxelspacing).T, 5.0 / voxelspacing, mask, True)
    return Case(target, template, mask, float(voxelspacing), float(resolution),
                chain, elements, rots, centres,
                dict(shape=shape, natoms=natoms, ncopies=ncopies, snr=snr, seed=seed))


# The measured configurations (sizes, spacings, atoms, copies, resolution, SNR).
CONFIGS = {
    "lcc64": dict(shape=(64, 64, 64), voxelspacing=2.0, natoms=1500, ncopies=3,
                  resolution=8.0, snr=5.0, angle=10.0, laplace=False, core_weighted=False),
    "lcc128_filtered": dict(shape=(128, 128, 128), voxelspacing=1.5, natoms=4000, ncopies=6,
                            resolution=6.0, snr=3.0, angle=4.71, laplace=True, core_weighted=True),
    "lcc192_precision": dict(shape=(192, 192, 192), voxelspacing=1.2, natoms=10000, ncopies=8,
                             resolution=4.5, snr=2.0, angle=4.71, laplace=False, core_weighted=False),
}


def make_config(name, seed=0):
    cfg = CONFIGS[name]
    return make_case(cfg["shape"], cfg["voxelspacing"], cfg["natoms"], cfg["ncopies"],
                     cfg["resolution"], cfg["snr"], seed)
