"""The custom-operation plugin point (the reference's ShaderCommand through construct_dynamic /
unary_dynamic / binary_dynamic, command/dynamic.rs and command.rs:2933-3048): kernels compiled
from tests/dynamic_ops.cu are registered, used inside programs, fused with the built-in ops around
them in every executor mode, and checked against the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
import pipelines as P
import zosimos_gb300 as zs
from zosimos_gb300.synthetic import srgb_gradient_noise

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ops(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = tmp_path_factory.mktemp("dyn") / "dynamic_ops.cubin"
    subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", str(out),
                    os.path.join(HERE, "dynamic_ops.cu")], check=True)
    image = out.read_bytes()
    return {name: zs.register_op(image, "zs_test_" + name) for name in ("invert", "mix", "gradient")}


def decode(img):
    h, w = img.shape[:2]
    return O.decode(O.SRGB_RGBA8, P.rgba_bytes(img), w, h)


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32, zs.Mode.PerOpF16])
def test_unary_and_binary_custom_ops(ops, mode):
    a = srgb_gradient_noise(97, 61, seed=50, image=0)
    b = srgb_gradient_noise(97, 61, seed=50, image=1)
    pool = zs.Pool()
    ka, kb = pool.insert_srgb(a), pool.insert_srgb(b)
    c = zs.CommandBuffer()
    ia, ib = c.input(pool.descriptor(ka)), c.input(pool.descriptor(kb))
    lin = zs.Descriptor.linear_rgba_f32(97, 61)
    inv = c.unary_dynamic(ia, ops["invert"], lin)
    mixed = c.binary_dynamic(inv, ib, ops["mix"], lin, np.array([0.25], np.float32))
    scaled = c.color_matrix(mixed, [0.9, 0.05, 0.0, 0.0, 1.0, 0.1, 0.02, 0.0, 0.95])
    o, _ = c.output(c.color_convert(scaled, zs.Descriptor.srgb_rgba8(97, 61)))
    got = P.run(c, pool, [(ia, ka), (ib, kb)], [o], mode)[0]
    la, lb = decode(a), decode(b)
    x = la.copy()
    x[..., :3] = 1.0 - la[..., :3]
    x = x + 0.25 * (lb - x)
    O.mat3(x, np.array([0.9, 0.05, 0.0, 0.0, 1.0, 0.1, 0.02, 0.0, 0.95]).reshape(3, 3))
    want = O.encode(O.SRGB_RGBA8, np.ascontiguousarray(x))
    assert np.abs(got.astype(int) - want.astype(int)).max() <= 1


def test_constructor_custom_op_and_its_uniforms(ops):
    c = zs.CommandBuffer()
    g = c.construct_dynamic(ops["gradient"], zs.Descriptor.linear_rgba_f32(40, 30), np.array([0.75], np.float32))
    o, _ = c.output(c.color_convert(g, zs.Descriptor.srgb_rgba8(40, 30)))
    exe = zs.Linker.from_included().compile(c).lower_to()
    assert "custom op" in exe.describe()
    dst = zs.DeviceBuffer(40 * 30 * 4)
    exe.run_device([], [dst.ptr])
    exe.run_device([], [dst.ptr])          # replayed graph
    zs.device_synchronize()
    got = dst.download(np.empty((30, 160), np.uint8))
    y, x = np.mgrid[0:30, 0:40].astype(np.float64)
    lin = np.stack([(x.astype(np.float32) + 0.5) / 40, (y.astype(np.float32) + 0.5) / 30,
                    np.full_like(x, 0.75), np.ones_like(x)], -1)
    assert np.abs(got.astype(int) - O.encode(O.SRGB_RGBA8, lin).astype(int)).max() <= 1


def test_custom_op_arguments(ops):
    c = zs.CommandBuffer()
    i = c.input(zs.Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(zs.ZosimosError) as e:
        c.unary_dynamic(i, 10 ** 6, zs.Descriptor.srgb_rgba8(8, 8))
    assert e.value.code == 10
    buf = c.buffer_zero(64)
    with pytest.raises(zs.ZosimosError):
        c.unary_dynamic(buf, ops["invert"], zs.Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(zs.ZosimosError) as e:
        zs.register_op(b"not a module", "zs_test_invert")
    assert e.value.code in (8, 10)
