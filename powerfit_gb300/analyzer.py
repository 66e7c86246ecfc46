"""Peak extraction from the search's (lcc, rot) volumes.

Mirrors the reference's ``Analyzer`` (``analyzer.py:7-113``): a threshold
ladder of ``steps`` cut-offs from max(lcc) down towards 0.5 max(lcc); at each
cut-off the connected (6-connected) regions of ``lcc >= cut-off`` are labelled
and the position of each region's maximum is kept.  Every distinct position
becomes a solution: LCC, Fisher z, z relative to ``z_sigma``, the position in
A (x, y, z) and the best rotation matrix there; solutions are sorted by LCC,
highest first, and written in the reference's ``solutions.out`` format.

This runs on the host once per search on the two output volumes (it is the
consumer of the search, not part of it).
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import label, maximum_position


class Analyzer:
    def __init__(self, corr, rotmat, rotmat_ind, steps=5, voxelspacing=1, origin=(0, 0, 0), z_sigma=1):
        self._corr = np.asarray(corr)
        self._rotmat = np.asarray(rotmat)
        self._rotmat_ind = np.asarray(rotmat_ind)
        self._voxelspacing = voxelspacing
        self._origin = origin
        self._z_sigma = z_sigma
        self._solutions = None
        self.steps = steps

    @property
    def corr(self):
        return self._corr

    @property
    def steps(self):
        return self._steps

    @steps.setter
    def steps(self, steps):
        self._steps = steps
        self._watershed()
        self._solutions = None

    @property
    def voxelspacing(self):
        return self._voxelspacing

    @voxelspacing.setter
    def voxelspacing(self, v):
        self._solutions = None
        self._voxelspacing = v

    @property
    def origin(self):
        return self._origin

    @origin.setter
    def origin(self, o):
        self._solutions = None
        self._origin = o

    @property
    def solutions(self):
        if self._solutions is None:
            self._generate_solutions()
        return self._solutions

    def _watershed(self):
        corr = self._corr
        max_cc = corr.max()
        min_cc = 0.5 * max_cc
        stepsize = (max_cc - min_cc) / self._steps
        cutoff = max_cc
        positions = []
        for _ in range(self._steps):
            cutoff -= stepsize
            labels, nfeat = label(corr >= cutoff)
            if nfeat:
                positions += maximum_position(corr, labels, list(range(1, nfeat + 1)))
        self._positions = set(tuple(int(p) for p in pos) for pos in positions)

    def _generate_solutions(self):
        sols = []
        for pos in self._positions:
            lcc = float(self._corr[pos])
            with np.errstate(divide="ignore", invalid="ignore"):
                fz = 0.5 * (np.log(1 + lcc) - np.log(1 - lcc))
            z, y, x = [c * self._voxelspacing + s for c, s in zip(pos, self._origin[::-1])]
            rot = self._rotmat[int(self._rotmat_ind[pos])]
            sols.append([lcc, fz, fz / self._z_sigma, x, y, z] + list(np.ravel(rot)))
        self._solutions = sorted(sols, key=lambda s: s[0], reverse=True)

    def tofile(self, out="solutions.out"):
        sols = self.solutions
        with open(out, "w") as f:
            head = "#rank cc Fish-z rel-z x y z a11 a12 a13 a21 a22 a23 a31 a32 a33".split()
            fmt_h = " ".join(["{:<6s}"] + ["{:>6s}"] * 3 + ["{:>8s}"] * 3 + ["{:>6s}"] * 9) + "\n"
            f.write(fmt_h.format(*head))
            fmt = " ".join(["{:<6d}"] + ["{:6.3f}"] * 3 + ["{:8.3f}"] * 3 + ["{:6.3f}"] * 9) + "\n"
            for n, s in enumerate(sols):
                f.write(fmt.format(n + 1, *s))
