"""Knobs and buffer-parameterised operations on the GPU, the reference's tests/knobs.rs and
the knob / with_buffer cases of tests/buffer.rs: a compiled executable is relaunched with new
parameter blocks and the results match the oracle byte for byte and the reference's goldens."""
import numpy as np
import pytest

import oracle as O
import pipelines as P
import zosimos_gb300 as zs
from imgutil import blockhash256

pytestmark = pytest.mark.gpu

BASE = dict(u_min=[0.0, 0.0, 1.0, 1.0], u_max=[1.0, 1.0, 1.0, 1.0], v_min=[0.0, 0.0, 1.0, 1.0],
            v_max=[1.0, 1.0, 1.0, 1.0], uv_min=[0.0, 0.0, 0.0, 0.0], uv_max=[0.0, 0.0, 0.0, 0.0])
# tests/knobs.rs:48-94: five parameterisations of the knob.
KNOBS = [
    ([0.0, 0.0, 0.5, 0.5], [0.5, 0.5, 0.5, 0.5], [0.0, 0.0, 0.5, 0.5], [0.5, 0.5, 0.5, 0.5]),
    ([0.2, 0.0, 0.5, 0.5], [0.5, 0.5, 0.5, 0.5], [0.2, 0.0, 0.5, 0.5], [0.5, 0.5, 0.5, 0.5]),
    ([0.4, 0.0, 0.5, 0.5], [0.5, 0.5, 0.5, 0.5], [0.4, 0.0, 0.5, 0.5], [0.5, 0.5, 0.5, 0.5]),
    ([0.5, 0.0, 0.4, 0.5], [0.5, 0.5, 0.5, 0.5], [0.5, 0.0, 0.4, 0.5], [0.5, 0.5, 0.5, 0.5]),
    ([0.5, 0.0, 0.2, 0.5], [0.5, 0.5, 0.5, 0.5], [0.5, 0.0, 0.2, 0.5], [0.5, 0.5, 0.5, 0.5]),
]


def std430(u_min, u_max, v_min, v_max, uv_min=(0, 0, 0, 0), uv_max=(0, 0, 0, 0)):
    return np.array([u_min, u_max, v_min, v_max, uv_min, uv_max], np.float32)


def oracle_bilinear_srgb8(w, h, block):
    """bilinear.frag in f32 (the GPU's operation order) encoded to sRGB8 exactly."""
    b = block.reshape(6, 4)
    img = O.bilinear_construct(w, h, *[list(map(float, r)) for r in b], f32=True).astype(np.float64)
    return O.encode(O.SRGB_RGBA8, img)


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_knob_on_bilinear(background, foreground, goldens, mode):
    pool = zs.Pool()
    kb, kf = pool.insert_srgb(background), pool.insert_srgb(foreground)
    c = zs.CommandBuffer()
    b = c.input(pool.descriptor(kb))
    f = c.input(pool.descriptor(kf))
    r = c.with_knob().bilinear(zs.Descriptor.srgb_rgba8(512, 512), **BASE)
    o, _ = c.output(r)
    exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=mode))
    knob, nbytes = exe.query_knob(r)
    assert nbytes == 96
    for idx, (u_min, u_max, v_min, v_max) in enumerate(KNOBS):
        block = std430(u_min, u_max, v_min, v_max)
        (key,) = zs.run_executable(exe, pool, [(b, kb), (f, kf)], [(knob, block)], [o])
        got = pool.read(key)
        assert (got == oracle_bilinear_srgb8(512, 512, block)).all(), idx
        assert blockhash256(got.reshape(512, 512, 4)) in goldens[f"bilinear-knob-{idx}"]
    # a launch without knob data uses the static parameters
    (key,) = zs.run_executable(exe, pool, [(b, kb), (f, kf)], [], [o])
    assert (pool.read(key) == oracle_bilinear_srgb8(512, 512, std430(**BASE))).all()


def test_from_buffer_with_knob(goldens):
    """tests/buffer.rs:67-110: a knob on buffer_init, read by from_buffer; the launch's knob
    zeroes row 1 of the 8 x 8 Luma8 image."""
    luma = zs.Descriptor(8, 8, zs.Bits.UInt8, zs.Parts.Luma, zs.ColorKind.Rgb, zs.Primaries.Bt709,
                         zs.Transfer.Srgb, zs.Whitepoint.D65)
    a = np.full(8 * 256, 0xFF, np.uint8)
    c = zs.CommandBuffer()
    buf = c.with_knob().buffer_init(a)
    o, _ = c.output(c.from_buffer(buf, luma))
    exe = zs.Linker.from_included().compile(c).lower_to()
    knob, nbytes = exe.query_knob(buf)
    assert nbytes == a.nbytes
    patched = a.copy()
    patched[256:264] = 0
    pool = zs.Pool()
    (key,) = zs.run_executable(exe, pool, [], [(knob, patched)], [o])
    got = pool.read(key).reshape(8, 8)
    want = np.full((8, 8), 0xFF, np.uint8)
    want[1] = 0
    assert (got == want).all()
    (key,) = zs.run_executable(exe, pool, [], [], [o])          # static bytes again
    assert (pool.read(key) == 0xFF).all()


def test_bilinear_from_buffer(goldens):
    """tests/buffer.rs:112-149: bilinear parameters read from a buffer_init buffer."""
    a = np.array([[0.0, 0.0, 0.0, 1.0], [0.0, 0.0, 0.7, 1.0], [0.0, 0.0, 0.3, 1.0], [0.0, 1.0, 0.3, 1.0],
                  [0.0, 0.0, 0.0, 1.0], [0.0, 0.0, 0.0, 1.0]], np.float32)
    c = zs.CommandBuffer()
    buf = c.buffer_init(a)
    zero = dict(u_min=[0] * 4, u_max=[0] * 4, v_min=[0] * 4, v_max=[0] * 4, uv_min=[0] * 4, uv_max=[0] * 4)
    r = c.with_buffer(buf).bilinear(zs.Descriptor.srgb_rgba8(256, 256), **zero)
    o, _ = c.output(r)
    got = P.run(c, zs.Pool(), [], [o])[0]
    assert (got == oracle_bilinear_srgb8(256, 256, a)).all()
    h = blockhash256(got.reshape(256, 256, 4))
    assert min(bin(int(h, 16) ^ int(g, 16)).count("1") for g in goldens["bilinear_from_buffer"]) <= 8


def test_set_knob_on_the_one_call_path():
    """zs_executable_set_knob: a solid colour knob changes every later zs_run_device result,
    including after a CUDA graph of the plan was captured."""
    c = zs.CommandBuffer()
    d = zs.Descriptor.linear_rgba_f32(64, 32)
    r = c.with_knob().solid_rgba(d, [0.25, 0.5, 0.75, 1.0])
    o, _ = c.output(c.color_convert(r, zs.Descriptor.srgb_rgba8(64, 32)))
    exe = zs.Linker.from_included().compile(c).lower_to()
    knob, nbytes = exe.query_knob(r)
    assert nbytes == 16
    dst = zs.DeviceBuffer(64 * 32 * 4)
    for color in ([0.25, 0.5, 0.75, 1.0], [1.0, 0.0, 0.5, 0.5], [0.0, 0.1, 0.2, 0.3]):
        if color[0] != 0.25:
            exe.set_knob(knob, np.array(color, np.float32))
        exe.run_device([], [dst.ptr])
        exe.run_device([], [dst.ptr])
        zs.device_synchronize()
        got = dst.download(np.empty((32, 256), np.uint8))
        want = O.encode(O.SRGB_RGBA8, np.broadcast_to(np.array(color, np.float64), (32, 64, 4)).copy())
        assert (got == want).all(), color


def test_knob_inside_a_linked_function(goldens):
    """tests/knobs.rs's knob, recorded inside a function that main invokes (two levels: main ->
    outer -> inner) and reached through its link index (RegisterKnob { link_idx, register })."""
    inner = zs.CommandBuffer()
    g = inner.generic()
    x = inner.input_generic(g)
    r = inner.with_knob().bilinear(zs.Descriptor.srgb_rgba8(512, 512), **BASE)
    inner.output(r)
    outer = zs.CommandBuffer()
    h = outer.generic()
    y = outer.input_generic(h)
    fi = outer.function(inner)
    (res,) = outer.invoke(fi, generics=[h], arguments=[y])
    outer.output(res)
    main = zs.CommandBuffer()
    fo = main.function(outer)
    pool = zs.Pool()
    ks = pool.insert(zs.Descriptor.srgb_rgba8(8, 8), np.zeros((8, 32), np.uint8))
    m = main.input(pool.descriptor(ks))
    (out,) = main.invoke(fo, generics=[main.register_descriptor(m)], arguments=[m])
    o, _ = main.output(out)
    exe = zs.Linker.from_included().link(main, [], [outer, inner], [[1], [2], []]).lower_to()
    knob, nbytes = exe.query_knob(r, link_idx=2)
    assert nbytes == 96
    for idx, (u_min, u_max, v_min, v_max) in enumerate(KNOBS[:3]):
        block = std430(u_min, u_max, v_min, v_max)
        (key,) = zs.run_executable(exe, pool, [(m, ks)], [(knob, block)], [o])
        got = pool.read(key)
        assert (got == oracle_bilinear_srgb8(512, 512, block)).all(), idx
        assert blockhash256(got.reshape(512, 512, 4)) in goldens[f"bilinear-knob-{idx}"]
