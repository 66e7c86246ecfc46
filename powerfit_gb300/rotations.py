"""Rotation sets for the 6D search.

``quat_to_rotmat`` and ``euler`` follow ``rotations.py:9-61`` of the reference
(including the rounding of every matrix element to 8 decimals, ``:59``), so a
rotation list built here is element-for-element the list the reference scans.

``proportional_orientations`` keeps the reference's angle -> orientation-set
table (``rotations.py:88-131``).  The sets themselves are Karney's published
SO(3) orientation files (one ``.npy`` per set, ``(N, 5)`` rows of quaternion +
weight); they are data that ships with the reference package, so this module
reads them from a directory the caller names (or ``$POWERFIT_ROTATION_DATA``).

``super_fibonacci`` generates a seeded-free, deterministic low-discrepancy SO(3)
sample of any size (M. Alexa, "Super-Fibonacci Spirals: Fast, Low-Discrepancy
Sampling of SO(3)", CVPR 2022).  It stands in for a Karney set of the same size
where the set file is not available (benchmark workloads, missing sets).
"""
from __future__ import annotations

import math
import os

import numpy as np

# angle (degrees) -> (file, number of orientations); reference rotations.py:91-112
ROTATION_SETS = {
    "E.npy": (1, 360.0),
    "c48u1.npy": (24, 62.8),
    "c600v.npy": (60, 44.48),
    "c48n9.npy": (216, 36.47),
    "c600vc.npy": (360, 27.78),
    "c48u27.npy": (648, 20.83),
    "c48u83.npy": (1992, 16.29),
    "c48u181.npy": (4344, 12.29),
    "c48n309.npy": (7416, 9.72),
    "c48n527.npy": (12648, 8.17),
    "c48u815.npy": (19560, 7.4),
    "c48u1153.npy": (27672, 6.6),
    "c48u1201.npy": (28824, 6.48),
    "c48u1641.npy": (39384, 5.75),
    "c48u2219.npy": (53256, 5.27),
    "c48u2947.npy": (70728, 4.71),
    "c48u3733.npy": (89592, 4.37),
    "c48u4749.npy": (113976, 4.0),
    "c48u5879.npy": (141096, 3.74),
    "c48u7111.npy": (170664, 3.53),
    "c48u8649.npy": (207576, 3.26),
}


def euler(angle, axis):
    """Rotation matrix about one axis (reference ``rotations.py:9-20``)."""
    c, s = math.cos(angle), math.sin(angle)
    if axis == "x":
        m = [[1, 0, 0], [0, c, -s], [0, s, c]]
    elif axis == "y":
        m = [[c, 0, s], [0, 1, 0], [-s, 0, c]]
    elif axis == "z":
        m = [[c, -s, 0], [s, c, 0], [0, 0, 1]]
    else:
        raise ValueError("Axis is not recognized.")
    return np.asarray(m, dtype=np.float64)


def quat_to_rotmat(quaternions):
    """(N,4) quaternions (w, x, y, z) -> (N,3,3) matrices rounded to 8 decimals.

    Same formula and rounding as the reference ``rotations.py:30-61``; a zero
    quaternion maps to the identity, as there.
    """
    q = np.asarray(quaternions, dtype=np.float64).reshape(-1, 4)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    nq = w * w + x * x + y * y + z * z
    s = np.zeros_like(nq)
    pos = nq > 0.0
    s[pos] = 2.0 / nq[pos]
    X, Y, Z = x * s, y * s, z * s
    r = np.empty((q.shape[0], 3, 3), dtype=np.float64)
    r[:, 0, 0] = 1.0 - (y * Y + z * Z)
    r[:, 0, 1] = x * Y - w * Z
    r[:, 0, 2] = x * Z + w * Y
    r[:, 1, 0] = x * Y + w * Z
    r[:, 1, 1] = 1.0 - (x * X + z * Z)
    r[:, 1, 2] = y * Z - w * X
    r[:, 2, 0] = x * Z - w * Y
    r[:, 2, 1] = y * Z + w * X
    r[:, 2, 2] = 1.0 - (x * X + y * Y)
    np.around(r, decimals=8, out=r)
    return r


def nearest_set(angle):
    """Name, size and angle of the set the reference would pick for ``angle``."""
    best = None
    for fname, (count, alpha) in ROTATION_SETS.items():
        d = abs(angle - alpha)
        if best is None or d < best[0]:
            best = (d, fname, count, alpha)
    return best[1], best[2], best[3]


def proportional_orientations(angle, data_dir=None):
    """Quaternions, weights and real angle of the Karney set nearest ``angle``.

    Mirrors ``rotations.py:88-131``.  ``data_dir`` (or the environment variable
    ``POWERFIT_ROTATION_DATA``) is the directory holding the set files.
    """
    fname, _, alpha = nearest_set(angle)
    data_dir = data_dir or os.environ.get("POWERFIT_ROTATION_DATA")
    if not data_dir:
        raise FileNotFoundError(
            "orientation set %s needs a data directory: pass data_dir= or set "
            "POWERFIT_ROTATION_DATA to the directory of the Karney .npy sets" % fname)
    qw = np.load(os.path.join(data_dir, fname))
    return qw[:, :4], qw[:, -1], alpha


# Alexa (2022): phi = sqrt(2), psi is the real root of psi^4 = psi + 4.
_SF_PHI = math.sqrt(2.0)
_SF_PSI = 1.533751168755204288118041


def super_fibonacci(n):
    """(n,4) unit quaternions (w, x, y, z) on a super-Fibonacci spiral."""
    i = np.arange(n, dtype=np.float64) + 0.5
    s = i / n
    r = np.sqrt(s)
    R = np.sqrt(1.0 - s)
    alpha = 2.0 * np.pi * i / _SF_PHI
    beta = 2.0 * np.pi * i / _SF_PSI
    return np.stack([r * np.sin(alpha), r * np.cos(alpha),
                     R * np.sin(beta), R * np.cos(beta)], axis=1)


def rotation_set(angle=None, count=None, data_dir=None):
    """(R,3,3) rotation matrices.

    With a Karney data directory available the reference's set for ``angle`` is
    used; otherwise a super-Fibonacci set with the same number of rotations
    (or ``count``) is generated.  Returns (rotmats, description).
    """
    if angle is not None:
        fname, n, alpha = nearest_set(angle)
        try:
            q, _, _ = proportional_orientations(angle, data_dir)
            return quat_to_rotmat(q), "karney:%s (%d, %.2f deg)" % (fname, n, alpha)
        except FileNotFoundError:
            count = n if count is None else count
            return quat_to_rotmat(super_fibonacci(count)), \
                "super-fibonacci:%d (size of %s, %.2f deg)" % (count, fname, alpha)
    if count is None:
        raise ValueError("give angle or count")
    return quat_to_rotmat(super_fibonacci(count)), "super-fibonacci:%d" % count
