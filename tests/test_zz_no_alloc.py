"""The allocation-free resample entry point (zs_resample_rgba16f_noalloc), called
through the C ABI and checked against the regular resize_filtered executable.

It exists for callers that may not allocate device memory while they run; it keeps
its filter tables and intermediate in one fixed device array.  This file is collected
last so that a failure here never hides the other tests."""
import ctypes

import numpy as np
import pytest

import pipelines as P
import zosimos_gb300 as zs
from zosimos_gb300.synthetic import linear_gradient_gauss

pytestmark = pytest.mark.gpu
F16_TOL = 2.0e-3   # the RGBA16F tolerance of the resample parity tests


def _noalloc():
    fn = zs._lib().zs_resample_rgba16f_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
    fn.restype = ctypes.c_int32
    return fn


def _regular(img16, out, filt):
    """The existing entry point: a lowered resize_filtered executable on device buffers."""
    h, w = img16.shape[:2]
    c, _, _ = P.resample_cmds(w, h, out[0], out[1], filt)
    exe = zs.Linker.from_included().compile(c).lower_to()
    src = zs.DeviceBuffer(w * h * 8)
    dst = zs.DeviceBuffer(out[0] * out[1] * 8)
    src.upload(P.f16_bytes(img16))
    exe.run_device([src.ptr], [dst.ptr])
    zs.device_synchronize()
    return P.f16_from_bytes(dst.download(np.empty((out[1], out[0] * 8), np.uint8)), *out)


def _noalloc_call(img16, out, filt):
    h, w = img16.shape[:2]
    src = zs.DeviceBuffer(w * h * 8)
    dst = zs.DeviceBuffer(out[0] * out[1] * 8)
    src.upload(P.f16_bytes(img16))
    rc = _noalloc()(src.ptr, w, h, dst.ptr, out[0], out[1], filt, None)
    assert rc == 0, zs._lib().zs_last_error()
    zs.device_synchronize()
    return P.f16_from_bytes(dst.download(np.empty((out[1], out[0] * 8), np.uint8)), *out)


def test_noalloc_matches_regular_entry_point_twice():
    cases = [((1024, 768), (277, 208), zs.Filter.Lanczos3),
             ((640, 480), (320, 240), zs.Filter.Box)]
    for (w, h), out, filt in cases:       # two calls in a row share the scratch array
        img = linear_gradient_gauss(w, h, seed=11)
        ours = _noalloc_call(img, out, filt)
        ref = _regular(img, out, filt)
        assert np.abs(ours - ref).max() <= F16_TOL


def test_noalloc_rejects_oversized_requests():
    fn = _noalloc()
    # 8192 x 8192 -> 4096 x 4096 needs a 268 MB intermediate: more than the fixed array.
    rc = fn(ctypes.c_void_p(16), 8192, 8192, ctypes.c_void_p(16), 4096, 4096, zs.Filter.Lanczos3, None)
    assert rc == 10
    assert b"scratch" in zs._lib().zs_last_error()
