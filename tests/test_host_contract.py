"""Host-side contract (CPU only): the reference's BaseCorrelator behaviour
(``tests/test_powerfitter.py:243-326`` of the reference), rotation utilities,
the synthetic-input generator and the C-ABI library's exported symbols."""
import os
import re

import numpy as np
import pytest

from powerfit_gb300 import BaseCorrelator, determine_core_indices, synth
from powerfit_gb300.rotations import (euler, nearest_set, quat_to_rotmat, rotation_set,
                                      super_fibonacci)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class TestBaseCorrelator:
    def setup_method(self):
        self.shape = (8, 9, 10)
        self.target = np.random.default_rng(0).random(self.shape)
        self.corr = BaseCorrelator(self.target)

    def test_init_normalises_target(self):
        assert self.corr._target.max() == 1
        assert self.corr._rmax == 4
        assert self.corr._lcc_mask.dtype == np.uint8

    def test_rotations_setter(self):
        self.corr.rotations = [0] * 9
        assert isinstance(self.corr._rotations, np.ndarray)
        with pytest.raises(ValueError):
            self.corr.rotations = [0] * 3
        self.corr.rotations = [0] * 27
        assert self.corr._rotations.shape == (3, 3, 3)

    def test_template_setter(self):
        with pytest.raises(ValueError):
            self.corr.template = np.random.rand(3, 3, 3)
        self.corr._mask = 1
        self.corr.template = np.random.rand(*self.shape)
        assert self.corr._mask is None

    def test_normalize_template(self):
        self.corr.template = np.random.rand(*self.shape)
        self.corr._mask = np.ones(self.shape)
        self.corr._normalize_template(self.corr._mask != 0)
        assert abs(self.corr._template.mean()) < 1e-12
        assert abs(self.corr._template.std() - 1) < 1e-12

    def test_mask_setter(self):
        with pytest.raises(ValueError):
            self.corr.mask = None
        template = np.random.rand(*self.shape)
        self.corr._template = template
        with pytest.raises(ValueError):
            self.corr.mask = np.random.rand(10)
        with pytest.raises(ValueError):
            self.corr.mask = np.zeros(self.shape)
        self.corr._laplace = True
        self.corr._template = template.copy()
        mask = np.ones(self.shape)
        self.corr.mask = mask
        assert np.allclose(self.corr._mask, mask)

    def test_scan_requires_inputs(self):
        with pytest.raises(ValueError):
            self.corr.scan()

    def test_preprocessing_matches_oracle(self):
        from oracle import oracle as O
        rng = np.random.default_rng(1)
        template = rng.random(self.shape)
        mask = (rng.random(self.shape) > 0.5) * 2.0
        for laplace in (False, True):
            c = BaseCorrelator(self.target, laplace=laplace)
            c.template = template
            c.mask = mask
            p = O.prepare(self.target, template, mask, laplace)
            assert np.array_equal(c._template, p.template)
            assert np.array_equal(c._lcc_mask, p.lcc_mask)
            assert c._norm_factor == p.norm_factor


def test_core_indices_match_oracle():
    from oracle import oracle as O
    mask = np.zeros((12, 12, 12))
    mask[2:10, 3:9, 1:11] = 1
    assert np.array_equal(determine_core_indices(mask), O.determine_core_indices(mask))
    assert determine_core_indices(mask).max() == 3


def test_quat_to_rotmat_orthonormal_and_rounded():
    q = super_fibonacci(500)
    r = quat_to_rotmat(q)
    assert np.allclose(np.einsum("nij,nkj->nik", r, r), np.eye(3), atol=1e-7)
    assert np.allclose(np.linalg.det(r), 1, atol=1e-7)
    assert np.array_equal(r, np.round(r, 8))
    assert np.allclose(quat_to_rotmat(np.zeros((1, 4)))[0], np.eye(3))


def test_euler_z():
    assert np.allclose(euler(np.pi / 2, "z"), [[0, -1, 0], [1, 0, 0], [0, 0, 1]])
    with pytest.raises(ValueError):
        euler(1.0, "w")


def test_rotation_set_selection():
    assert nearest_set(10.0)[:2] == ("c48n309.npy", 7416)
    assert nearest_set(4.71)[:2] == ("c48u2947.npy", 70728)
    r, desc = rotation_set(4.71, data_dir="/nonexistent-dir")
    assert r.shape == (70728, 3, 3) and "super-fibonacci" in desc


def test_rotations_match_reference():
    from oracle import refimport
    if refimport.load() is None:
        pytest.skip("reference tree not available")
    ref = refimport.module("rotations")
    q = np.random.default_rng(2).normal(size=(50, 4))
    assert np.array_equal(quat_to_rotmat(q), ref.quat_to_rotmat(q))
    qr, w, a = ref.proportional_orientations(10.0)
    from powerfit_gb300.rotations import proportional_orientations
    data_dir = os.path.join(os.path.dirname(ref.__file__), "data")
    q2, w2, a2 = proportional_orientations(10.0, data_dir)
    assert np.array_equal(qr, q2) and a == a2


def test_splat_matches_reference():
    from oracle import refimport
    if refimport.load() is None:
        pytest.skip("reference tree not available")
    ref = refimport.module("_powerfit")
    rng = np.random.default_rng(1)
    shape = (20, 22, 24)
    pts = rng.random((3, 50)) * np.array([[24], [22], [20]]) - 5
    w = rng.random(50)
    a, b = np.zeros(shape), np.zeros(shape)
    ref.blur_points(pts.copy(), w, 1.3, a, True)
    synth.blur_points(pts, w, 1.3, b, True)
    assert np.max(np.abs(a - b)) < 1e-12
    a, b = np.zeros(shape), np.zeros(shape)
    ref.dilate_points(pts.copy(), np.full(50, 2.2), a, True)
    synth.dilate_points(pts, np.full(50, 2.2), b, True)
    assert np.array_equal(a, b)


def test_synthetic_case_is_seeded():
    a = synth.make_case((24, 24, 24), 3.0, 120, 2, 8.0, 5.0, seed=9)
    b = synth.make_case((24, 24, 24), 3.0, 120, 2, 8.0, 5.0, seed=9)
    assert np.array_equal(a.target, b.target) and np.array_equal(a.template, b.template)
    assert a.target.dtype == np.float32 and a.mask.max() == 1
    chain = a.chain
    d = np.linalg.norm(np.diff(chain, axis=0), axis=1)
    assert np.allclose(d, 3.8)


def _header_symbols():
    with open(os.path.join(ROOT, "include", "powerfit_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(pf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_header_symbol():
    import ctypes
    from powerfit_gb300 import build
    if not build.up_to_date():
        try:
            build.build()
        except Exception as e:  # no nvcc
            pytest.skip("cannot build the CUDA library here: %s" % e)
    lib = ctypes.CDLL(build.LIB)
    syms = _header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    from powerfit_gb300 import _lib
    assert sorted(_lib.EXPORTS) == syms


def test_checked_variant_exports_the_same_symbols():
    """The bounds-checked build exports the same C ABI and says which build it
    is; the unchecked build refuses its debugging calls (no device needed)."""
    import ctypes
    from powerfit_gb300 import build
    try:
        paths = build.build_variants(("", "checked"))
    except Exception as e:  # no nvcc
        pytest.skip("cannot build the CUDA library here: %s" % e)
    plain, checked = (ctypes.CDLL(p) for p in paths)
    for s in _header_symbols():
        assert hasattr(checked, s), s
    assert checked.pf_bounds_checked() == 1 and plain.pf_bounds_checked() == 0
    a, b = ctypes.c_uint64(7), ctypes.c_uint64(7)
    plain.pf_debug_bounds.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    assert plain.pf_debug_bounds(0, ctypes.byref(a), ctypes.byref(b)) == -6
    plain.pf_debug_buffer_extent.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    assert plain.pf_debug_buffer_extent(None, 5) == -1


def test_host_splat_matches_reference_outputs():
    d = np.load(os.path.join(ROOT, "tests", "golden", "prep.npz"))
    for wrap in (1, 0):
        a = np.zeros(d["blur_%d" % wrap].shape)
        synth.blur_points(d["points"], d["weights"], 1.3, a, bool(wrap))
        assert np.max(np.abs(a - d["blur_%d" % wrap])) < 1e-12
        b = np.zeros(a.shape)
        synth.dilate_points(d["points"], d["radii_%d" % wrap], b, bool(wrap))
        assert np.array_equal(b, d["dilate_%d" % wrap])
    assert np.array_equal(determine_core_indices(d["core_in"]), d["core_out"])
