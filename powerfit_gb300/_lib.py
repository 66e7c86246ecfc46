"""ctypes binding of ``libpowerfit_gb300.so`` (C ABI in ``include/powerfit_gb300.h``).

There is no CPU fallback: if the library is missing or cannot be loaded every
call raises ``NativeLibraryError``.

With ``POWERFIT_GB300_VARIANT=checked`` in the environment the process loads
``libpowerfit_gb300_checked.so`` instead: the same library built with bounds
checks in the search kernels (``bounds_checked()``, ``debug_bounds()``).
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
VARIANT = os.environ.get("POWERFIT_GB300_VARIANT", "")
if VARIANT not in ("", "checked"):
    raise ValueError("POWERFIT_GB300_VARIANT must be empty or 'checked', got %r" % VARIANT)
LIB_PATH = os.path.join(_HERE, "libpowerfit_gb300_checked.so" if VARIANT == "checked" else "libpowerfit_gb300.so")

PF_FLAG_FP64_NORM = 1
PF_FLAG_NO_PRUNE = 2
PF_FLAG_ACCUMULATE = 4
PF_FLAG_GENERIC = 8
PF_FLAG_ROT_MAX = 16
PF_FLAG_TENSOR_DFT = 32
PF_FLAG_TENSOR_TC05 = 64

EXPORTS = [
    "pf_create", "pf_destroy", "pf_last_error", "pf_global_error", "pf_set_target",
    "pf_set_template_mask", "pf_scan", "pf_set_rotations", "pf_reset_results",
    "pf_scan_resident", "pf_get_results", "pf_synchronize", "pf_set_stream", "pf_set_tuning", "pf_get_tuning", "pf_autotune",
    "pf_get_geometry", "pf_set_profiling", "pf_get_kernel_times", "pf_fft3d",
    "pf_rotate_grid3d", "pf_conj_multiply", "pf_calc_lcc", "pf_combine",
    "pf_blur_points", "pf_dilate_points", "pf_laplace_wrap", "pf_core_indices", "pf_prep_error",
    "pf_scan_noalloc", "pf_get_rotation_max", "pf_get_rotation_best",
    "pf_mlp_param_count", "pf_mlp_forward", "pf_mlp_grad", "pf_mlp_adam", "pf_mlp_error",
    "pf_set_results", "pf_debug_fail_alloc", "pf_bounds_checked", "pf_debug_bounds", "pf_debug_buffer_extent",
]

# sites of a bounds-check violation (pf_debug_bounds)
CHECK_SITES = {
    1: "twiddle table", 2: "shared-memory array", 3: "template/mask gather", 4: "pass-1 row list",
    5: "spectra store", 6: "spectra load", 7: "target spectrum", 8: "output spectra", 9: "cluster push",
    10: "voxel array", 11: "pass-3 voxel list", 12: "per-rotation maximum",
}


class NativeLibraryError(RuntimeError):
    pass


class PowerFitError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


_lock = threading.Lock()
_lib = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_i64 = ctypes.c_int64
_d = ctypes.c_double
_sz = ctypes.c_size_t


def load(path=None):
    """Load the shared library (once) and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise NativeLibraryError(
                "%s not built: run powerfit_gb300.build.build() "
                "(or __graft_entry__.build()) first; there is no CPU fallback" % os.path.basename(path))
        try:
            lib = ctypes.CDLL(path)
        except OSError as e:
            raise NativeLibraryError("cannot load %s: %s" % (path, e)) from e
        sig = {
            "pf_create": (_vp, [_i, _i, _i, _i, ctypes.POINTER(_i)]),
            "pf_destroy": (_i, [_vp]),
            "pf_last_error": (_i, [_vp, ctypes.c_char_p, _sz]),
            "pf_global_error": (_i, [ctypes.c_char_p, _sz]),
            "pf_set_target": (_i, [_vp, _vp, _vp]),
            "pf_set_template_mask": (_i, [_vp, _vp, _vp, _d, _i]),
            "pf_scan": (_i, [_vp, _vp, _i64, _i64, _vp, _vp, _i]),
            "pf_set_rotations": (_i, [_vp, _vp, _i64]),
            "pf_reset_results": (_i, [_vp]),
            "pf_scan_resident": (_i, [_vp, _i64, _i64, _i64, _i]),
            "pf_get_results": (_i, [_vp, _vp, _vp]),
            "pf_synchronize": (_i, [_vp]),
            "pf_set_stream": (_i, [_vp, _vp]),
            "pf_set_tuning": (_i, [_vp, _i, _i, _i]),
            "pf_get_tuning": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
            "pf_autotune": (_i, [_vp, _i64, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i),
                                 ctypes.POINTER(_d)]),
            "pf_get_geometry": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
            "pf_set_profiling": (_i, [_vp, _i]),
            "pf_get_kernel_times": (_i, [_vp, _vp, _vp]),
            "pf_fft3d": (_i, [_vp, _vp, _vp]),
            "pf_rotate_grid3d": (_i, [_vp, _i, _i, _i, _vp, _i, _vp, _i]),
            "pf_conj_multiply": (_i, [_vp, _vp, _vp, _i64]),
            "pf_calc_lcc": (_i, [_vp, _vp, _vp, _vp, _vp, _i64]),
            "pf_combine": (_i, [_vp, _vp, _vp, _vp, _i64, _i64]),
            "pf_blur_points": (_i, [_vp, _vp, _i64, _d, _vp, _i, _i, _i, _i]),
            "pf_dilate_points": (_i, [_vp, _vp, _i64, _vp, _i, _i, _i, _i]),
            "pf_laplace_wrap": (_i, [_vp, _vp, _i, _i, _i]),
            "pf_core_indices": (_i, [_vp, _vp, _i, _i, _i]),
            "pf_prep_error": (_i, [ctypes.c_char_p, _sz]),
            "pf_scan_noalloc": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _d, _i, _vp, _i64, _i64, _vp, _vp, _vp]),
            "pf_get_rotation_max": (_i, [_vp, _vp, _i64, _i64]),
            "pf_get_rotation_best": (_i, [_vp, _vp, _vp, _i64, _i64]),
            "pf_mlp_param_count": (_i64, [_i, _i]),
            "pf_mlp_forward": (_i, [_vp, _i64, _i, _i, _vp, _vp, _vp]),
            "pf_mlp_grad": (_i, [_vp, _vp, _vp, _i64, _i, _i, _vp, ctypes.c_float, _vp, _vp, _vp]),
            "pf_mlp_adam": (_i, [_vp, _vp, _vp, _vp, _vp, _i64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_float, _i, _vp]),
            "pf_mlp_error": (_i, [ctypes.c_char_p, _sz]),
            "pf_set_results": (_i, [_vp, _vp, _vp]),
            "pf_debug_fail_alloc": (_i, [_i64]),
            "pf_bounds_checked": (_i, []),
            "pf_debug_bounds": (_i, [_i, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
            "pf_debug_buffer_extent": (_i, [_vp, _i64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def global_error():
    buf = ctypes.create_string_buffer(512)
    load().pf_global_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc, ctx=None):
    if rc != 0:
        buf = ctypes.create_string_buffer(512)
        load().pf_last_error(ctx, buf, 512)
        raise PowerFitError(rc, buf.value.decode(errors="replace"))


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def c64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != tuple(shape):
        raise ValueError("expected shape %s, got %s" % (tuple(shape), a.shape))
    return a


class Context:
    """Owns one ``pf_ctx`` (one grid shape on one device)."""

    def __init__(self, shape, device=0):
        lib = load()
        nz, ny, nx = (int(s) for s in shape)
        st = ctypes.c_int(0)
        h = lib.pf_create(nz, ny, nx, int(device), ctypes.byref(st))
        if not h:
            raise PowerFitError(st.value, global_error())
        self._h = ctypes.c_void_p(h)
        self.shape = (nz, ny, nx)
        self.device = int(device)
        self.nrot = 0

    @property
    def handle(self):
        if self._h is None:
            raise PowerFitError(-4, "context destroyed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            load().pf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        check(getattr(load(), name)(self.handle, *args), self.handle)

    def set_target(self, target, lcc_mask):
        t = c64(target, self.shape)
        m = np.ascontiguousarray(lcc_mask, dtype=np.uint8)
        if m.shape != self.shape:
            raise ValueError("lcc mask shape mismatch")
        self._call("pf_set_target", ptr(t), ptr(m))

    def set_template_mask(self, template, mask, norm_factor, rmax):
        t = c64(template, self.shape)
        m = c64(mask, self.shape)
        self._call("pf_set_template_mask", ptr(t), ptr(m), float(norm_factor), int(rmax))

    def scan(self, rotmats, rot_offset=0, flags=0):
        r = np.ascontiguousarray(rotmats, dtype=np.float64).reshape(-1, 9)
        self.nrot = r.shape[0]
        lcc = np.empty(self.shape, dtype=np.float32)
        rot = np.empty(self.shape, dtype=np.int32)
        self._call("pf_scan", ptr(r), r.shape[0], int(rot_offset), ptr(lcc), ptr(rot), int(flags))
        return lcc, rot

    def set_rotations(self, rotmats):
        r = np.ascontiguousarray(rotmats, dtype=np.float64).reshape(-1, 9)
        self._call("pf_set_rotations", ptr(r), r.shape[0])
        self.nrot = r.shape[0]
        return r.shape[0]

    def reset_results(self):
        self._call("pf_reset_results")

    def scan_resident(self, first, count, rot_offset=0, flags=0):
        self._call("pf_scan_resident", int(first), int(count), int(rot_offset), int(flags))

    def get_results(self, out_lcc=None, out_rot=None):
        lcc = out_lcc if out_lcc is not None else np.empty(self.shape, dtype=np.float32)
        rot = out_rot if out_rot is not None else np.empty(self.shape, dtype=np.int32)
        self._call("pf_get_results", ptr(lcc), ptr(rot))
        return lcc, rot

    def rotation_max(self, first=0, count=None):
        """Per-rotation best LCC over the lcc-mask voxels (scans with PF_FLAG_ROT_MAX)."""
        if count is None:
            count = self.nrot - first
        out = np.empty(int(count), dtype=np.float32)
        self._call("pf_get_rotation_max", ptr(out), int(first), int(count))
        return out

    def rotation_best(self, first=0, count=None):
        """(best LCC, voxel index) per rotation (scans with PF_FLAG_ROT_MAX; voxel -1: none)."""
        if count is None:
            count = self.nrot - first
        val = np.empty(int(count), dtype=np.float32)
        vox = np.empty(int(count), dtype=np.int32)
        self._call("pf_get_rotation_best", ptr(val), ptr(vox), int(first), int(count))
        return val, vox

    def debug_buffer_extent(self, elements):
        """Bounds-checked build: tell the kernels the intermediate buffer holds
        only `elements` values (-1: all); accesses beyond count as violations."""
        self._call("pf_debug_buffer_extent", int(elements))

    def set_results(self, lcc, rot):
        """Load a running best (checkpoint) to continue with PF_FLAG_ACCUMULATE."""
        l = np.ascontiguousarray(lcc, dtype=np.float32)
        r = np.ascontiguousarray(rot, dtype=np.int32)
        if l.shape != self.shape or r.shape != self.shape:
            raise ValueError("checkpoint shape mismatch")
        self._call("pf_set_results", ptr(l), ptr(r))

    def synchronize(self):
        self._call("pf_synchronize")

    def set_stream(self, stream_handle):
        """Launch on a caller stream (an int cudaStream_t, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); None restores the context's own."""
        self._call("pf_set_stream", ctypes.c_void_p(stream_handle or None))

    def set_tuning(self, pairs=0, rows1=0, rows3=0):
        self._call("pf_set_tuning", int(pairs), int(rows1), int(rows3))

    def get_tuning(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._call("pf_get_tuning", ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def autotune(self, trial_rotations=512):
        """Pick pairs per batch and tile rows by timing short scans (resets results)."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = ctypes.c_double()
        self._call("pf_autotune", int(trial_rotations), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                   ctypes.byref(ms))
        return dict(pairs=a.value, rows1=b.value, rows3=c.value, trial_ms=ms.value)

    def get_geometry(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._call("pf_get_geometry", ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return dict(reff=a.value, valid_planes=b.value, rmax=c.value)

    def set_profiling(self, enable):
        self._call("pf_set_profiling", int(bool(enable)))

    def kernel_times(self):
        ms = np.zeros(3, dtype=np.float64)
        n = np.zeros(3, dtype=np.int64)
        self._call("pf_get_kernel_times", ptr(ms), ptr(n))
        return ms, n

    def fft3d(self, real):
        a = np.ascontiguousarray(real, dtype=np.float32)
        if a.shape != self.shape:
            raise ValueError("shape mismatch")
        out = np.empty(self.shape, dtype=np.complex64)
        self._call("pf_fft3d", ptr(a), ptr(out))
        return out


# ---- unit-level mirrors ----------------------------------------------------

def rotate_grid3d(grid, rotmat, radius, out, nearest):
    """GPU mirror of ``_extensions.rotate_grid3d`` (writes ``out`` in place)."""
    g = c64(grid)
    if out.dtype != np.float64 or not out.flags.c_contiguous or out.shape != g.shape:
        raise ValueError("out must be a C-contiguous float64 array of the grid's shape")
    r = c64(rotmat).reshape(9)
    nz, ny, nx = g.shape
    check(load().pf_rotate_grid3d(ptr(g), nz, ny, nx, ptr(r), int(radius), ptr(out), int(bool(nearest))))
    return out


def conj_multiply(in1, in2, out):
    a = np.ascontiguousarray(in1, dtype=np.complex128)
    b = np.ascontiguousarray(in2, dtype=np.complex128)
    if out.dtype != np.complex128 or not out.flags.c_contiguous or out.size != a.size or b.size != a.size:
        raise ValueError("conj_multiply: size/dtype mismatch")
    check(load().pf_conj_multiply(ptr(a), ptr(b), ptr(out), a.size))
    return out


def calc_lcc(gcc, ave, ave2, mask, lcc):
    g, a, a2 = (np.ascontiguousarray(x, dtype=np.float64) for x in (gcc, ave, ave2))
    m = np.ascontiguousarray(mask, dtype=np.uint8)
    if lcc.dtype != np.float64 or not lcc.flags.c_contiguous or not (g.size == a.size == a2.size == m.size == lcc.size):
        raise ValueError("calc_lcc: size/dtype mismatch")
    check(load().pf_calc_lcc(ptr(g), ptr(a), ptr(a2), ptr(m), ptr(lcc), g.size))
    return lcc


def combine_into(lcc, rot, part_lcc, part_rot, rot_add):
    """GPU merge of one rotation shard (``PowerFitter._combine`` semantics)."""
    pl = np.ascontiguousarray(part_lcc, dtype=np.float32)
    pr = np.ascontiguousarray(part_rot, dtype=np.int32)
    if lcc.dtype != np.float32 or rot.dtype != np.int32 or lcc.size != pl.size or rot.size != pr.size:
        raise ValueError("combine: dtype/size mismatch")
    check(load().pf_combine(ptr(lcc), ptr(rot), ptr(pl), ptr(pr), lcc.size, int(rot_add)))
    return lcc, rot


# ---- preprocessing on the GPU ---------------------------------------------

def _check_prep(rc):
    if rc != 0:
        buf = ctypes.create_string_buffer(256)
        load().pf_prep_error(buf, 256)
        raise PowerFitError(rc, buf.value.decode(errors="replace"))


def _grid_out(out):
    if out.dtype != np.float64 or not out.flags.c_contiguous or out.ndim != 3:
        raise ValueError("out must be a C-contiguous 3D float64 array")
    return out.shape


def blur_points(points, weights, sigma, out, wraparound=True):
    """GPU mirror of ``_powerfit.blur_points`` (adds into ``out``)."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(3, -1)
    w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
    if w.size != pts.shape[1]:
        raise ValueError("weights array is of incorrect size")
    nz, ny, nx = _grid_out(out)
    _check_prep(load().pf_blur_points(ptr(pts), ptr(w), pts.shape[1], float(sigma), ptr(out), nz, ny, nx,
                                      int(bool(wraparound))))
    return out


def dilate_points(points, radii, out, wraparound=True):
    """GPU mirror of ``_powerfit.dilate_points`` (sets balls to 1 in ``out``)."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(3, -1)
    r = np.ascontiguousarray(np.broadcast_to(np.asarray(radii, dtype=np.float64), (pts.shape[1],)))
    nz, ny, nx = _grid_out(out)
    _check_prep(load().pf_dilate_points(ptr(pts), ptr(r), pts.shape[1], ptr(out), nz, ny, nx,
                                        int(bool(wraparound))))
    return out


def laplace_wrap(array):
    """GPU ``scipy.ndimage.laplace(array, mode='wrap')`` (float64)."""
    a = c64(array)
    if a.ndim != 3:
        raise ValueError("laplace_wrap expects a 3D array")
    out = np.empty_like(a)
    _check_prep(load().pf_laplace_wrap(ptr(a), ptr(out), *a.shape))
    return out


def core_indices(mask):
    """GPU ``determine_core_indices``: erosions survived per voxel (float64)."""
    m = c64(mask)
    if m.ndim != 3:
        raise ValueError("core_indices expects a 3D array")
    out = np.empty_like(m)
    _check_prep(load().pf_core_indices(ptr(m), ptr(out), *m.shape))
    return out


# ---- learned proposal: network kernels on device memory --------------------

def check_mlp(rc):
    if rc != 0:
        buf = ctypes.create_string_buffer(256)
        load().pf_mlp_error(buf, 256)
        raise PowerFitError(rc, buf.value.decode(errors="replace"))


def mlp_param_count(nin, nh):
    return int(load().pf_mlp_param_count(int(nin), int(nh)))


def _dp(t):
    """Device pointer of a CUDA tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def mlp_forward(x, nin, nh, params_bf16, y, stream=None):
    """y[i] = net(x[i]) for x (n, nin) float32 on the device (tensors or pointers)."""
    check_mlp(load().pf_mlp_forward(_dp(x), int(x.shape[0]), int(nin), int(nh), _dp(params_bf16), _dp(y),
                                    ctypes.c_void_p(stream)))


def mlp_grad(x, t, w, nin, nh, params_bf16, scale, grad, loss, stream=None):
    """grad += dL/dp and loss += L for L = sum_i scale * w_i * (net(x_i) - t_i)^2."""
    check_mlp(load().pf_mlp_grad(_dp(x), _dp(t), _dp(w), int(x.shape[0]), int(nin), int(nh), _dp(params_bf16),
                                 float(scale), _dp(grad), _dp(loss), ctypes.c_void_p(stream)))


def mlp_adam(params, params_bf16, grad, m, v, lr, step, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
    check_mlp(load().pf_mlp_adam(_dp(params), _dp(params_bf16), _dp(grad), _dp(m), _dp(v), int(params.numel()),
                                 float(lr), float(beta1), float(beta2), float(eps), int(step),
                                 ctypes.c_void_p(stream)))


def debug_fail_alloc(after):
    """Make the `after`-th device allocation from now on fail (-1: off); error-path tests."""
    check(load().pf_debug_fail_alloc(int(after)))


def bounds_checked():
    """Whether the loaded library is the bounds-checked build."""
    return bool(load().pf_bounds_checked())


def debug_bounds(device=0):
    """Violations the bounds checks recorded on `device` since the last call
    (waits for the device; clears them): ``(count, site, index)`` with the
    site's name and index of one of them (``(0, None, None)`` when none).
    Raises PowerFitError (PF_E_UNSUPPORTED) on the unchecked build."""
    first = ctypes.c_uint64(0)
    count = ctypes.c_uint64(0)
    check(load().pf_debug_bounds(int(device), ctypes.byref(first), ctypes.byref(count)))
    if count.value == 0:
        return 0, None, None
    code = first.value
    index = code & ((1 << 48) - 1)
    if index >= 1 << 47:
        index -= 1 << 48
    return int(count.value), CHECK_SITES.get(code >> 48, "site %d" % (code >> 48)), int(index)
