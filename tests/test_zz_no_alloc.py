"""The scan entry point that allocates no device memory (pf_scan_noalloc).

Some callers cannot call cudaMalloc while they run -- a host that owns all
device memory through its own allocator, or a plugin that may only use the
buffers it is handed.  pf_scan_noalloc serves them from one fixed device
array inside the library.  This test gives it device buffers it did not
allocate, calls it twice in a row through the C ABI, and checks both results
against the allocating entry point (pf_scan through a context) and the
float64 oracle within the parity tolerance the other GPU tests use (best LCC
within 1e-4; best rotation equal to the oracle's wherever its top-two gap
exceeds 1e-4).  The file is named so that pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LCC_TOL = 1e-4


def _case(seed, shape, nrot):
    from powerfit_gb300 import synth
    from powerfit_gb300.correlator import BaseCorrelator
    from powerfit_gb300.rotations import quat_to_rotmat, super_fibonacci
    c = synth.make_case(shape, 2.0, 600, 2, 8.0, 5.0, seed)
    b = BaseCorrelator(c.target.astype(np.float64))
    b.template = c.template
    b.mask = c.mask
    rot = quat_to_rotmat(super_fibonacci(nrot + seed))[:nrot]
    return b, rot


def _noalloc_scan(lib, b, rot, rot_offset):
    import torch
    dev = torch.device("cuda", 0)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).to(dev)
    target = t(b._target, np.float32)
    lmask = t(b._lcc_mask, np.uint8)
    tmpl = t(b._template, np.float32)
    mask = t(b._mask, np.float32)
    rots = t(rot.reshape(-1, 9), np.float64)
    lcc = torch.full(b._target.shape, -1.0, dtype=torch.float32, device=dev)
    rr = torch.full(b._target.shape, -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    nz, ny, nx = b._target.shape
    p = lambda x: ctypes.c_void_p(x.data_ptr())
    rc = lib.load().pf_scan_noalloc(nz, ny, nx, p(target), p(lmask), p(tmpl), p(mask), float(b._norm_factor),
                                    int(b._rmax), p(rots), rot.shape[0], int(rot_offset), p(lcc), p(rr),
                                    ctypes.c_void_p(stream.cuda_stream))
    lib.check(rc)
    torch.cuda.synchronize(dev)
    return lcc.cpu().numpy(), rr.cpu().numpy()


@pytest.mark.parametrize("seed,shape,nrot,off", [
    (1, (48, 48, 48), 23, 0),
    (2, (40, 48, 36), 16, 500),
    # more rotations than one chunk of the converted-rotation scratch (1,024):
    # the later chunks' offsets into the rotations, the rotation indices and
    # the reused chunk scratch
    (3, (16, 16, 16), 1100, 70000),
])
def test_noalloc_scan_matches_scan_twice(seed, shape, nrot, off):
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    from powerfit_gb300 import _lib
    b, rot = _case(seed, shape, nrot)
    ctx = _lib.Context(shape)
    ctx.set_target(b._target, b._lcc_mask)
    ctx.set_template_mask(b._template, b._mask, float(b._norm_factor), b._rmax)
    ref_lcc, ref_rot = ctx.scan(rot, rot_offset=off)
    # the oracle's best rotation and runner-up: the rotation must match it
    # wherever the top-two gap exceeds the tolerance
    p = O.Prepared(b._target, b._lcc_mask, b._rmax, b._template, b._mask, int(b._norm_factor),
                   np.fft.rfftn(b._target), np.fft.rfftn(b._target ** 2), b._target)
    o_lcc, o_rot, o_second = O.scan(p, rot, track_second=True)
    clear = (o_lcc - o_second) > LCC_TOL
    assert clear.sum() > 0.5 * np.sum(o_lcc > 0)
    for _ in range(2):                       # two calls in a row share the scratch
        lcc, r = _noalloc_scan(_lib, b, rot, off)
        assert np.max(np.abs(lcc - ref_lcc)) < LCC_TOL
        assert np.max(np.abs(lcc - o_lcc)) < LCC_TOL
        assert np.array_equal(r[clear], o_rot[clear].astype(np.int32) + off)
        assert np.all(r[ref_lcc == 0] == 0)
    assert torch.cuda.is_available()


def test_noalloc_rejects_oversized_grid():
    pytest.importorskip("torch")
    from powerfit_gb300 import _lib
    null = ctypes.c_void_p(1)
    rc = _lib.load().pf_scan_noalloc(128, 128, 128, null, null, null, null, 1.0, 8, null, 1, 0, null, null,
                                     ctypes.c_void_p(0))
    assert rc == -5
