"""Parity at the benchmark configurations' full sizes, against the FP64 oracle.

* Fused colour chain (4096 x 4096 RGBA8 sRGB): every one of the 2^24 RGB triples once,
  through the fused kernel on device buffers and zero copy from pinned host buffers, and
  through the per-op FP32 and FP16 programs.  8-bit outputs within 1 LSB, alpha exact.
* Resample sweep (8192 x 8192 RGBA16F): Lanczos-3 and box at /2, /3.7, /8 on the
  tensor-core and SIMT kernels, and the 17 degree bilinear rotation, checked on bands of
  output rows (top, middle, bottom) computed by the oracle with the full image's weights
  and pixel centres.  Max-abs error within 2e-3.
* Layer stack (32 distinct 4096 x 4096 premultiplied RGBA16F layers): bands of rows, fused
  and plain per-op FP32, within 2e-3.
* Batched thumbnails (1024 RGBA8 images, sides log-uniform in [64, 4096]): every
  thumbnail of the one-launch batch within 1 LSB of the oracle.
"""
import numpy as np
import pytest

import oracle as O
import pipelines as P
import zosimos_gb300 as zs
from zosimos_gb300.synthetic import (layer_transforms, linear_gradient_gauss, premultiplied_layer,
                                     srgb_gradient_noise, thumbnail_sizes)
from zosimos_gb300.workloads import color_chain, layer_stack, resample, rgba_bytes, rotation

pytestmark = pytest.mark.gpu
F16_TOL = 2.0e-3


def lsb(a, b):
    return int(np.abs(a.astype(np.int16) - b.astype(np.int16)).max())


def bands(n, rows=16):
    return [(0, rows), (n // 2 - rows // 2, n // 2 + rows // 2), (n - rows, n)]


# ---------------------------------------------------------------- colour chain, 4096^2: every RGB triple


@pytest.fixture(scope="module")
def cube():
    img = P.rgb_cube_image()
    ref = P.oracle_chain(img).reshape(4096, 4096 * 4)
    return img, ref


def _check_cube(img, got, ref):
    got = got.reshape(4096, 4096, 4)
    assert lsb(got[..., :3], ref.reshape(4096, 4096, 4)[..., :3]) <= 1
    assert np.array_equal(got[..., 3], img[..., 3])


def test_chain_every_rgb_triple_fused_device(cube):
    img, ref = cube
    c, _, _ = color_chain(4096, 4096)
    exe = zs.Linker.from_included().compile(c).lower_to()
    assert exe.kernel_count() == 1
    src, dst = zs.DeviceBuffer(img.nbytes), zs.DeviceBuffer(img.nbytes)
    src.upload(rgba_bytes(img))
    exe.run_device([src.ptr], [dst.ptr])
    zs.device_synchronize()
    _check_cube(img, dst.download(np.empty(img.nbytes, np.uint8)), ref)


def test_chain_every_rgb_triple_zero_copy_host(cube):
    img, ref = cube
    c, _, _ = color_chain(4096, 4096)
    exe = zs.Linker.from_included().compile(c).lower_to()
    hin, hout = zs.PinnedBuffer(img.nbytes), zs.PinnedBuffer(img.nbytes)
    hin.array[:] = img.reshape(-1)
    exe.run_host([hin.array], [hout.array])
    _check_cube(img, hout.array.copy(), ref)


@pytest.mark.parametrize("mode", [zs.Mode.PerOpF32, zs.Mode.PerOpF16])
def test_chain_every_rgb_triple_per_op(cube, mode):
    img, ref = cube
    got = P.ours_chain(img, mode)
    _check_cube(img, got, ref)


# ---------------------------------------------------------------- resample sweep of an 8192^2 RGBA16F image


@pytest.fixture(scope="module")
def big16():
    img = linear_gradient_gauss(8192, 8192, seed=3)
    src = zs.DeviceBuffer(img.nbytes)
    src.upload(img.view(np.uint8))
    return img, img.astype(np.float64), src


def _run_resample(src, n, ow, filt, **caps):
    c, _, _ = resample(n, n, ow, ow, filt)
    exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(**caps))
    dst = zs.DeviceBuffer(ow * ow * 8)
    exe.run_device([src.ptr], [dst.ptr])
    zs.device_synchronize()
    return P.f16_from_bytes(dst.download(np.empty((ow, ow * 8), np.uint8)), ow, ow), exe.describe()


@pytest.mark.parametrize("filt", [zs.Filter.Lanczos3, zs.Filter.Box])
@pytest.mark.parametrize("factor", [2.0, 3.7, 8.0])
@pytest.mark.parametrize("kernel", ["tensor", "simt"])
def test_resample_8192(big16, filt, factor, kernel):
    img, img64, src = big16
    ow = int(round(8192 / factor))
    got, plan = _run_resample(src, 8192, ow, filt, simt_resample=kernel == "simt")
    assert ("tensor cores" in plan) == (kernel == "tensor")
    for y0, y1 in bands(ow):
        exact = O.resample_rows(img64, ow, ow, y0, y1, filt)
        assert np.abs(got[y0:y1] - exact).max() <= F16_TOL, (y0, y1)


def test_resample_8192_per_op_f32(big16):
    img, img64, src = big16
    got, _ = _run_resample(src, 8192, 2214, zs.Filter.Lanczos3, mode=zs.Mode.PerOpF32)
    for y0, y1 in bands(2214):
        assert np.abs(got[y0:y1] - O.resample_rows(img64, 2214, 2214, y0, y1, zs.Filter.Lanczos3)).max() <= F16_TOL


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_rotation_8192(big16, mode):
    img, img64, src = big16
    c, _, _, _ = rotation(8192, 8192, 17.0)
    exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=mode))
    dst = zs.DeviceBuffer(8192 * 8192 * 8)
    exe.run_device([src.ptr], [dst.ptr])
    zs.device_synchronize()
    got = P.f16_from_bytes(dst.download(np.empty((8192, 8192 * 8), np.uint8)), 8192, 8192)
    for y0, y1 in bands(8192) + [(2000, 2016), (6100, 6116)]:
        assert np.abs(got[y0:y1] - P.oracle_rotation_rows(img64, 17.0, y0, y1)).max() <= F16_TOL, (y0, y1)


# ---------------------------------------------------------------- layer stack: 32 distinct 4096^2 layers


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_layer_stack_32_distinct_4096(mode):
    n, w = 32, 4096
    layers = [premultiplied_layer(w, w, seed=5, image=i) for i in range(n)]
    transforms = layer_transforms(n, seed=5)
    c, inputs, _ = layer_stack(w, w, transforms)
    exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=mode))
    if mode == zs.Mode.Fused:
        assert exe.kernel_count() == 1
    bufs = []
    for img in layers:
        b = zs.DeviceBuffer(img.nbytes)
        b.upload(img.view(np.uint8))
        bufs.append(b)
    dst = zs.DeviceBuffer(w * w * 8)
    exe.run_device([b.ptr for b in bufs], [dst.ptr])
    zs.device_synchronize()
    got = P.f16_from_bytes(dst.download(np.empty((w, w * 8), np.uint8)), w, w)
    for y0, y1 in bands(w, 8) + [(1234, 1242)]:
        exact = P.oracle_layer_stack_rows(layers, transforms, y0, y1)
        assert np.abs(got[y0:y1] - exact).max() <= F16_TOL, (y0, y1)


# ---------------------------------------------------------------- 1024 uneven thumbnails


def test_thumbnails_1024_all_images():
    ws, hs = thumbnail_sizes(1024, seed=4)
    images = [srgb_gradient_noise(int(w), int(h), seed=4, image=i) for i, (w, h) in enumerate(zip(ws, hs))]
    got = P.ours_thumbnails(images)
    worst = 0
    for i in range(0, 1024, 64):
        ref = P.oracle_thumbnails(images[i:i + 64])
        for k, r in enumerate(ref):
            d = lsb(got[i + k], r)
            assert d <= 1, (i + k, ws[i + k], hs[i + k], d)
            worst = max(worst, d)
    assert worst <= 1
