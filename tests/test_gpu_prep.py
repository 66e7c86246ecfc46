"""GPU preprocessing (template/mask builders, periodic Laplace, core weights)
against the reference's own outputs (tests/golden/prep.npz)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "prep.npz")


@pytest.fixture(scope="module")
def d():
    return np.load(GOLD)


def test_blur_points(d):
    from powerfit_gb300 import _lib
    for wrap in (1, 0):
        out = np.zeros(d["blur_%d" % wrap].shape)
        _lib.blur_points(d["points"], d["weights"], 1.3, out, bool(wrap))
        ref = d["blur_%d" % wrap]
        assert np.max(np.abs(out - ref)) <= 1e-12 * max(1.0, np.abs(ref).max())


def test_dilate_points(d):
    from powerfit_gb300 import _lib
    for wrap in (1, 0):
        out = np.zeros(d["dilate_%d" % wrap].shape)
        _lib.dilate_points(d["points"], d["radii_%d" % wrap], out, bool(wrap))
        assert np.array_equal(out, d["dilate_%d" % wrap])


def test_laplace_wrap(d):
    from powerfit_gb300 import _lib
    out = _lib.laplace_wrap(d["lap_in"])
    assert np.max(np.abs(out - d["lap_out"])) < 1e-13


def test_core_indices(d):
    from powerfit_gb300 import _lib
    assert np.array_equal(_lib.core_indices(d["core_in"]), d["core_out"])


def test_blur_adds_into_existing_grid():
    from powerfit_gb300 import _lib
    out = np.full((8, 8, 8), 2.0)
    _lib.blur_points(np.zeros((3, 1)), np.ones(1), 0.5, out, True)
    assert out[0, 0, 0] == 3.0 and out.min() == 2.0
