"""Density volumes: MRC/CCP4 I/O, the CLI's map preprocessing and the
template/mask builders (on the GPU).

Mirrors the reference's ``volume.py``:
* ``Volume`` (``:13-54``), ``resample`` / ``trim`` / ``extend`` /
  ``nearest_multiple2357`` (``:66-118``), ``res_to_sigma`` (``:121-122``);
* ``structure_to_shape_like`` (``:192-224``), whose Gaussian splat and ball
  dilation run on the GPU (``pf_blur_points`` / ``pf_dilate_points``);
* MRC / CCP4 reading and writing (``:228-500``).  Files are written with the
  reference's header layout (float32 data, ``mapc/mapr/maps = 1 2 3``, cell
  = shape x voxel spacing, origin in words 50-52 for ``.mrc``, start indices
  for ``.map``/``.ccp4``).  Reading honours any ``mapc/mapr/maps`` order
  (the reference's parser uses the density before assigning it for
  non-standard orders, ``volume.py:366-377``).
"""
from __future__ import annotations

import os
import struct
import sys
import warnings

import numpy as np

_HEADER = struct.Struct("<10i6f3i3f3i27f4s4sfi800s")  # 1024 bytes, little-endian view


class Volume:
    def __init__(self, array, voxelspacing=1.0, origin=(0, 0, 0)):
        self.array = array
        self.voxelspacing = voxelspacing
        self.origin = origin

    @classmethod
    def fromfile(cls, fid, fmt=None):
        array, vs, origin = read_map(fid, fmt)
        return cls(array, vs, origin)

    @property
    def shape(self):
        return self.array.shape

    @property
    def dimensions(self):
        return np.asarray([x * self.voxelspacing for x in self.array.shape][::-1])

    @property
    def start(self):
        return np.asarray([x / self.voxelspacing for x in self.origin])

    def duplicate(self):
        return Volume(self.array.copy(), self.voxelspacing, self.origin)

    def tofile(self, fid, fmt=None):
        fmt = fmt or os.path.splitext(fid)[-1][1:]
        if fmt in ("ccp4", "map", "mrc"):
            write_map(fid, self, fmt)
        else:
            raise RuntimeError("Format is not supported.")


def zeros_like(volume):
    return Volume(np.zeros_like(volume.array), volume.voxelspacing, volume.origin)


# ---------------------------------------------------------------------------
# MRC / CCP4
# ---------------------------------------------------------------------------

def read_map(fid, fmt=None):
    """Return (array (z, y, x) float64, voxel spacing, origin (x, y, z))."""
    fname = getattr(fid, "name", fid)
    fmt = fmt or os.path.splitext(fname)[-1][1:]
    if fmt not in ("ccp4", "map", "mrc"):
        raise ValueError("Extension of file is not supported.")
    if hasattr(fid, "read"):
        raw = fid.read()
    else:
        with open(fid, "rb") as f:
            raw = f.read()
    if len(raw) < 1024:
        raise ValueError("file too short for a map header")
    stamp = raw[212]
    if stamp == 0x44:
        endian = "<"
    elif stamp == 0x11:
        endian = ">"
    else:
        raise RuntimeError("Endiannes is not properly set in file. Check the file format.")
    h = struct.unpack(endian + _HEADER.format[1:], raw[:1024])
    nc, nr, ns, mode, ncstart, nrstart, nsstart, mx, my, mz = h[:10]
    xl, yl, zl, alpha, beta, gamma = h[10:16]
    mapc, mapr, maps = h[16:19]
    if any(abs(a - 90.0) > 1e-3 for a in (alpha, beta, gamma)):
        raise RuntimeError("Only densities in rectangular boxes are supported.")
    spacings = [xl / float(mx), yl / float(my), zl / float(mz)]
    if max(spacings) - min(spacings) > 1e-4 * 3:
        raise RuntimeError("Voxel spacing is not equal in all directions.")
    vs = spacings[0]
    nsymbt = h[23]
    dtypes = {0: "i1", 1: "i2", 2: "f4", 6: "u2"}
    if mode not in dtypes:
        raise RuntimeError("Unsupported map mode %d" % mode)
    data = np.frombuffer(raw, dtype=endian + dtypes[mode], count=nc * nr * ns, offset=1024 + nsymbt)
    data = data.reshape(ns, nr, nc)
    # file axes: columns = mapc, rows = mapr, sections = maps (1 = x, 2 = y, 3 = z)
    order = (mapc, mapr, maps)
    if sorted(order) != [1, 2, 3]:
        raise RuntimeError("invalid axis order %s" % (order,))
    # array axes (0, 1, 2) hold (maps, mapr, mapc); move to (z, y, x)
    axis_of = {maps: 0, mapr: 1, mapc: 2}
    density = np.transpose(data, (axis_of[3], axis_of[2], axis_of[1])).astype(np.float64)
    if fmt == "mrc":
        origin = np.asarray(h[49:52], dtype=np.float64)
    else:
        start = {mapc: ncstart, mapr: nrstart, maps: nsstart}
        origin = np.asarray([start[1], start[2], start[3]], dtype=np.float64) * vs
    return np.ascontiguousarray(density), vs, origin


def write_map(fid, volume, fmt=None):
    fmt = fmt or os.path.splitext(fid)[-1][1:]
    if fmt not in ("ccp4", "mrc", "map"):
        raise ValueError("Format is not recognized. Use ccp4, mrc, or map.")
    arr = np.asarray(volume.array)
    nz, ny, nx = arr.shape
    name = arr.dtype.name
    if name == "int8":
        mode, out_dtype = 0, np.int8
    elif name in ("int16", "int32"):
        mode, out_dtype = 1, np.int16
    elif name in ("float32", "float64"):
        mode, out_dtype = 2, np.float32
    else:
        raise TypeError("Data type ({:})is not supported.".format(name))
    vs = volume.voxelspacing
    if fmt in ("ccp4", "map"):
        starts = [int(round(x)) for x in volume.start]
        origin = [0.0, 0.0, 0.0]
    else:
        starts = [0, 0, 0]
        origin = [float(x) for x in volume.origin]
    xl, yl, zl = (float(x) for x in volume.dimensions)
    header = _HEADER.pack(
        nx, ny, nz, mode, starts[0], starts[1], starts[2], nx, ny, nz,
        xl, yl, zl, 90.0, 90.0, 90.0, 1, 2, 3,
        float(arr.min()), float(arr.max()), float(arr.mean()), 1, 0, 0,
        *([0.0] * 24), *origin, b"MAP ", b"\x44\x41\x00\x00", float(arr.std()), 0, b" " * 800)
    with open(fid, "wb") as out:
        out.write(header)
        out.write(np.ascontiguousarray(arr.astype(out_dtype)).astype("<" + np.dtype(out_dtype).str[1:]).tobytes())


# ---------------------------------------------------------------------------
# map preprocessing used by the CLI (host, once per job)
# ---------------------------------------------------------------------------

def res_to_sigma(resolution):
    return resolution / (np.sqrt(2.0) * np.pi)


def resample(volume, factor, order=1):
    from scipy.ndimage import zoom
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        arr = zoom(volume.array, factor, order=order)
    return Volume(arr, volume.voxelspacing / factor, volume.origin)


def trim(volume, cutoff, margin=2):
    a = volume.array
    if a.max() <= cutoff:
        raise ValueError("Cutoff value should be lower than density max.")
    extent = []
    for axis in range(a.ndim):
        other = tuple(i for i in range(a.ndim) if i != axis)
        above = np.nonzero(a.max(axis=other) > cutoff)[0]
        lo = max(0, int(above[0]) - margin)
        hi = min(a.shape[axis], int(above[-1]) + 1 + margin)
        extent.append(slice(lo, hi))
    origin = [o + volume.voxelspacing * e.start for o, e in zip(volume.origin, extent[::-1])]
    return Volume(a[tuple(extent)], volume.voxelspacing, origin)


def extend(volume, shape):
    out = np.zeros(shape)
    out[tuple(slice(n) for n in volume.shape)] = volume.array
    return Volume(out, volume.voxelspacing, volume.origin)


def is_multiple2357(num):
    for p in (2, 3, 5, 7):
        while num % p == 0:
            num //= p
    return num == 1


def nearest_multiple2357(num):
    n = int(num)
    while not is_multiple2357(n):
        n += 1
    return n


# ---------------------------------------------------------------------------
# template / mask from atoms (GPU splat)
# ---------------------------------------------------------------------------

def structure_to_shape_like(vol, xyz, resolution, weights=None, radii=None, shape="vol"):
    """Blur atoms into a map (``shape='vol'``) or dilate them into a 0/1 mask
    (``shape='mask'``, default radius 5 A) on ``vol``'s grid; ``xyz`` is
    (3, N) in A.  Mirrors ``volume.py:192-224``."""
    from . import _lib
    xyz = np.asarray(xyz, dtype=np.float64).reshape(3, -1)
    grid = (xyz - np.asarray(vol.origin, dtype=np.float64).reshape(3, 1)) / vol.voxelspacing
    out = zeros_like(vol)
    out.array = np.zeros(vol.shape, dtype=np.float64)
    if shape == "vol":
        w = np.ones(xyz.shape[1]) if weights is None else np.asarray(weights, dtype=np.float64)
        if w.size != xyz.shape[1]:
            raise ValueError("weights array is of incorrect size")
        sigma = res_to_sigma(resolution) / vol.voxelspacing
        _lib.blur_points(grid, w, sigma, out.array, True)
    elif shape == "mask":
        r = np.full(xyz.shape[1], 5.0) if radii is None else np.asarray(radii, dtype=np.float64)
        if r.size != xyz.shape[1]:
            raise ValueError("radii array is of incorrect size")
        _lib.dilate_points(grid, r / vol.voxelspacing, out.array, True)
    else:
        raise ValueError("shape should either be 'vol' or 'mask'")
    return out
