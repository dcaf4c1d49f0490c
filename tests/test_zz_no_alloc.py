"""The allocation-free resample entry point (zs_resample_rgba16f_noalloc), called
through the C ABI and checked against the regular resize_filtered executable and
against the FP64 oracle.

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


class _Buffers:
    """Source and destination device buffers, allocated before the calls under test."""

    def __init__(self, img16, out):
        h, w = img16.shape[:2]
        self.w, self.h, self.out = w, h, out
        self.src = zs.DeviceBuffer(w * h * 8)
        self.dst = zs.DeviceBuffer(out[0] * out[1] * 8)
        self.src.upload(P.f16_bytes(img16))

    def call(self, filt, stream=None):
        rc = _noalloc()(self.src.ptr, self.w, self.h, self.dst.ptr, self.out[0], self.out[1], filt, stream)
        assert rc == 0, zs._lib().zs_last_error()

    def result(self):
        zs.device_synchronize()
        return P.f16_from_bytes(self.dst.download(np.empty((self.out[1], self.out[0] * 8), np.uint8)), *self.out)


CASES = [((1024, 768), (277, 208), zs.Filter.Lanczos3),
         ((640, 480), (320, 240), zs.Filter.Box),
         ((333, 250), (100, 80), zs.Filter.Triangle),
         ((100, 80), (333, 250), zs.Filter.Lanczos3)]      # upscale: the windows do not widen


def test_noalloc_matches_regular_entry_point_and_oracle_twice():
    for (w, h), out, filt in CASES:
        img = linear_gradient_gauss(w, h, seed=11)
        bufs = _Buffers(img, out)
        ref = _regular(img, out, filt)
        exact = P.oracle_resample(P.f16_from_bytes(P.f16_bytes(img), w, h), out, filt)
        for _ in range(2):              # two calls in a row share the scratch array
            bufs.call(filt)
            ours = bufs.result()
            assert np.abs(ours - ref).max() <= F16_TOL
            assert np.abs(ours - exact).max() <= F16_TOL


def test_noalloc_allocates_nothing_and_runs_on_a_stream():
    """After a warm-up call, calls allocate no device memory.  Every call here is ordered on
    one created stream: calls share the scratch array, so calls that overlap on the GPU
    (e.g. the legacy default stream against a non-blocking stream such as torch's) race."""
    import torch
    img = linear_gradient_gauss(512, 384, seed=12)
    bufs = _Buffers(img, (200, 150))
    stream = torch.cuda.Stream()        # the caller's stream exists before the calls under test
    handle = ctypes.c_void_p(stream.cuda_stream)
    bufs.call(zs.Filter.Lanczos3, handle)   # warm-up: loads the module, reserves the fixed array
    stream.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        bufs.call(zs.Filter.Box, handle)
        bufs.call(zs.Filter.Lanczos3, handle)
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    exact = P.oracle_resample(P.f16_from_bytes(P.f16_bytes(img), 512, 384), (200, 150), zs.Filter.Lanczos3)
    assert np.abs(bufs.result() - exact).max() <= F16_TOL


def test_noalloc_rejects_oversized_requests():
    fn = _noalloc()
    # 8192 x 8192 -> 4096 x 4096 needs a 268 MB intermediate: more than the fixed array.
    rc = fn(ctypes.c_void_p(16), 8192, 8192, ctypes.c_void_p(16), 4096, 4096, zs.Filter.Lanczos3, None)
    assert rc == 10
    assert b"scratch" in zs._lib().zs_last_error()
