"""The bench line's byte model and its ncu traffic lookup (CPU only).

The roofline the bench reports divides a fixed algorithmic byte count by the
measured time; these tests pin that count to the streaming model of the
three-pass pipeline (8N + 8H(2F+6) + (16H + 17N)/B per rotation, H =
n*n*(n/2+1), F = 3) at the figures the design notes quote, and the DRAM
traffic lookup to the committed ncu summary and its scaling by pairs."""
import os

import pytest

import bench


@pytest.mark.parametrize("n,B,mb", [(128, 1, 171.7), (128, 256, 119.2), (64, 1, 21.7), (64, 256, 15.1)])
def test_bytes_per_rotation(n, B, mb):
    assert round(bench.bytes_per_rotation(n, B) / 1e6, 1) == mb


def test_bytes_per_rotation_formula():
    n, B = 96, 64
    N, H = n ** 3, n * n * (n // 2 + 1)
    assert bench.bytes_per_rotation(n, B) == 8 * N + 8 * H * 12 + (16 * H + 17 * N) / B


def test_dram_traffic_scales_with_pairs():
    rows = {}
    with open(os.path.join(bench.ROOT, "profiles", "dram_traffic.txt")) as f:
        lines = f.readlines()
    for ln in lines:
        if ln.strip() and not ln.startswith("#"):
            p = ln.split()
            rows[(p[0], int(p[1]))] = (int(p[2]), int(p[3]) + int(p[4]))
    pairs, total = rows[("k_pass2_ct", 128)]
    got, note = bench.dram_traffic("k_pass2_ct", 128, pairs)
    assert got == total and "scaled" not in note
    got, note = bench.dram_traffic("k_pass2_ct", 128, 8 * pairs)
    assert got == pytest.approx(8 * total) and "scaled" in note
    assert bench.dram_traffic("k_pass2_ct", 96, 16)[0] is None


def test_metric_names_the_grid():
    assert bench.metric_for((128, 128, 128)) == "rotations/s at 128^3 LCC (1 GB300)"
    assert bench.metric_for((192, 192, 12)) == "rotations/s at 192x192x12 LCC (1 GB300)"
