"""Map I/O and the peak analyzer (CPU) against the reference's outputs."""
import os

import numpy as np

from powerfit_gb300.analyzer import Analyzer
from powerfit_gb300.volume import (Volume, extend, is_multiple2357, nearest_multiple2357, read_map, trim,
                                   write_map)

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reads_reference_written_map():
    arr, vs, origin = read_map(os.path.join(GOLD, "ref_map.mrc"))
    rng = np.random.default_rng(41)
    ref = rng.random((10, 12, 14)).astype(np.float32).astype(np.float64)
    assert np.array_equal(arr, ref)
    assert abs(vs - 1.5) < 1e-6 and np.allclose(origin, [3.0, -2.0, 5.0])


def _read(path):
    with open(path, "rb") as f:
        return f.read()


def test_written_map_matches_reference_bytes(tmp_path):
    rng = np.random.default_rng(41)
    arr = rng.random((10, 12, 14)).astype(np.float32).astype(np.float64)
    out = str(tmp_path / "m.mrc")
    write_map(out, Volume(arr, 1.5, np.array([3.0, -2.0, 5.0])))
    assert _read(out) == _read(os.path.join(GOLD, "ref_map.mrc"))


def test_round_trip_and_axis_order(tmp_path):
    arr = np.arange(4 * 5 * 6, dtype=np.float64).reshape(4, 5, 6)
    for ext in ("mrc", "map", "ccp4"):
        path = str(tmp_path / ("v." + ext))
        Volume(arr, 2.0, (4.0, 6.0, 8.0)).tofile(path)
        a, vs, origin = read_map(path)
        assert np.array_equal(a, arr) and vs == 2.0
        assert np.allclose(origin, (4.0, 6.0, 8.0))
    # a file stored with sections along x (mapc, mapr, maps = 3, 2, 1)
    path = str(tmp_path / "swap.mrc")
    write_map(path, Volume(arr, 1.0))
    raw = bytearray(_read(path))
    import struct
    struct.pack_into("<3i", raw, 0, 4, 5, 6)          # nc, nr, ns
    struct.pack_into("<3i", raw, 64, 3, 2, 1)         # mapc, mapr, maps
    struct.pack_into("<3i", raw, 28, 6, 5, 4)         # mx, my, mz
    struct.pack_into("<3f", raw, 40, 6.0, 5.0, 4.0)   # cell lengths (x, y, z)
    data = np.transpose(arr, (2, 1, 0)).astype("<f4").tobytes()   # (x, y, z) sections
    raw[1024:] = data
    with open(path, "wb") as f:
        f.write(bytes(raw))
    a, _, _ = read_map(path)
    assert np.array_equal(a, arr)


def test_trim_extend_multiples():
    v = Volume(np.zeros((20, 20, 20)), 1.0, (0.0, 0.0, 0.0))
    v.array[5:9, 6:12, 7:8] = 1.0
    t = trim(v, 0.5)
    assert t.shape == (8, 10, 5) and np.allclose(t.origin, (5.0, 4.0, 3.0))
    assert nearest_multiple2357(121) == 125 and is_multiple2357(210) and not is_multiple2357(11)
    e = extend(t, (9, 10, 6))
    assert e.shape == (9, 10, 6) and e.array[:8, :10, :5].sum() == t.array.sum()


def test_analyzer_matches_reference_solutions(tmp_path):
    d = np.load(os.path.join(GOLD, "analyzer.npz"))
    an = Analyzer(d["lcc"], d["rotmats"], d["rot_ind"], voxelspacing=1.7, origin=(1.0, 2.0, 3.0), z_sigma=0.12)
    sols = np.array(an.solutions)
    assert sols.shape == d["solutions"].shape
    assert np.allclose(sols, d["solutions"])
    out = str(tmp_path / "solutions.out")
    an.tofile(out)
    lines = _read(out).decode().splitlines()
    assert lines[0].startswith("#rank") and len(lines) == 1 + len(sols)
