"""Generic functions and the linker without a device: CommandBuffer::generic / input_generic /
register_descriptor / derive_descriptor / function / invoke (lib/zosimos/src/command.rs:756-922)
and Linker::link (command.rs:2083-2185).  Calls are monomorphised and inlined when linking, so
a linked program lowers (and fuses) like a flat one; lowering needs no GPU."""
import numpy as np
import pytest

import pipelines as P
import zosimos_gb300 as zs
from zosimos_gb300 import Bits, ColorKind, CommandBuffer, Descriptor, Linker, Parts, Transfer, ZosimosError


def lower(prog, mode=zs.Mode.Fused):
    return prog.lower_to(zs.Capabilities(mode=mode))


def resize_function(size=(64, 64)) -> CommandBuffer:
    """A generic function: its input resized to `size`."""
    f = CommandBuffer()
    a = f.generic()
    i = f.input_generic(a)
    f.output(f.resize(i, size))
    return f


def test_generic_palette_signature_and_link():
    fn = P.generic_palette_function()
    assert fn.computed_signature() == (1, 1, 1)
    c = CommandBuffer()
    conv = c.function(fn)
    i = c.input(Descriptor.srgb_rgba8(512, 512))
    ty = c.register_descriptor(i)
    (res,) = c.invoke(conv, generics=[ty], arguments=[i])
    # the result takes the index grid's size and the generic palette's colour (command.rs:1466-1470)
    d = c.describe(res)
    assert (d.width, d.height) == (2048, 2048) and d == Descriptor.srgb_rgba8(2048, 2048)
    o, outformat = c.output(res)
    assert outformat == d
    # a program with calls must be linked: Linker::compile has no definitions
    with pytest.raises(ZosimosError) as e:
        Linker.from_included().compile(c)
    assert e.value.code == 2
    exe = lower(Linker.from_included().link(c, [], [fn], [[1], []]))
    assert exe.output_count() == 1
    assert "palette" in exe.describe()


def test_invoke_checks_its_arguments():
    fn = resize_function()
    c = CommandBuffer()
    f = c.function(fn)
    i = c.input(Descriptor.srgb_rgba8(32, 32))
    ty = c.register_descriptor(i)
    with pytest.raises(ZosimosError) as e:              # INVALID_CALL: argument count
        c.invoke(f, generics=[ty], arguments=[])
    assert e.value.code == 4
    with pytest.raises(ZosimosError) as e:              # INVALID_CALL: generic count
        c.invoke(f, generics=[], arguments=[i])
    assert e.value.code == 4
    with pytest.raises(ZosimosError) as e:              # BAD_REGISTER: no such descriptor variable
        c.invoke(f, generics=[ty + 7], arguments=[i])
    assert e.value.code == 3
    # the argument must match the input rewritten with the generics (command.rs:899-906)
    j = c.input(Descriptor.linear_rgba_f32(32, 32))
    with pytest.raises(ZosimosError) as e:
        c.invoke(f, generics=[ty], arguments=[j])
    assert e.value.code == 4
    (r,) = c.invoke(f, generics=[ty], arguments=[i])
    assert c.describe(r) == Descriptor.srgb_rgba8(64, 64)
    # the call itself is no value
    with pytest.raises(ZosimosError):
        c.output(r - 1)


def test_concrete_function_input_is_checked():
    g = CommandBuffer()
    x = g.input(Descriptor.srgb_rgba8(16, 16))
    g.output(g.color_convert(x, Descriptor.linear_rgba_f32(16, 16)))
    c = CommandBuffer()
    f = c.function(g)
    ok = c.input(Descriptor.srgb_rgba8(16, 16))
    bad = c.input(Descriptor.srgb_rgba8(16, 17))
    with pytest.raises(ZosimosError) as e:
        c.invoke(f, arguments=[bad])
    assert e.value.code == 4
    (r,) = c.invoke(f, arguments=[ok])
    assert c.describe(r) == Descriptor.linear_rgba_f32(16, 16)


def test_one_function_instantiated_for_two_descriptors():
    fn = resize_function((40, 24))
    c = CommandBuffer()
    f = c.function(fn)
    a = c.input(Descriptor.srgb_rgba8(128, 96))
    b = c.input(Descriptor.linear_rgba_f32(300, 200))
    (ra,) = c.invoke(f, generics=[c.register_descriptor(a)], arguments=[a])
    (rb,) = c.invoke(f, generics=[c.register_descriptor(b)], arguments=[b])
    assert c.describe(ra) == Descriptor.srgb_rgba8(40, 24)
    assert c.describe(rb) == Descriptor.linear_rgba_f32(40, 24)
    c.output(ra)
    c.output(rb)
    exe = lower(Linker.from_included().link(c, [], [fn], [[1], []]))
    assert exe.output_count() == 2


def test_link_table_errors():
    fn = resize_function()
    c = CommandBuffer()
    f = c.function(fn)
    i = c.input(Descriptor.srgb_rgba8(32, 32))
    (r,) = c.invoke(f, generics=[c.register_descriptor(i)], arguments=[i])
    c.output(r)
    L = Linker.from_included()
    with pytest.raises(ZosimosError) as e:              # declaration without definition
        L.link(c, [], [fn], [])
    assert e.value.code == 2
    with pytest.raises(ZosimosError) as e:              # more link lists than buffers
        L.link(c, [], [fn], [[1], [], []])
    assert e.value.code == 2
    with pytest.raises(ZosimosError) as e:              # link target out of range
        L.link(c, [], [fn], [[5], []])
    assert e.value.code == 2
    with pytest.raises(ZosimosError) as e:              # main's generics must be given
        L.link(c, [Descriptor.srgb_rgba8(8, 8)], [fn], [[1], []])
    assert e.value.code == 4
    L.link(c, [], [fn], [[1], []])


def test_recursive_link_is_rejected():
    # buffer 1 declares a function with its own signature and is linked to itself
    inner = resize_function()
    rec = CommandBuffer()
    a = rec.generic()
    i = rec.input_generic(a)
    f = rec.function(inner)
    (r,) = rec.invoke(f, generics=[a], arguments=[i])
    rec.output(r)
    c = CommandBuffer()
    g = c.function(rec)
    x = c.input(Descriptor.srgb_rgba8(32, 32))
    (y,) = c.invoke(g, generics=[c.register_descriptor(x)], arguments=[x])
    c.output(y)
    with pytest.raises(ZosimosError) as e:
        Linker.from_included().link(c, [], [rec], [[1], [1]])
    assert e.value.code == 2
    # linked to a real definition instead, the nested call inlines
    exe = lower(Linker.from_included().link(c, [], [rec, inner], [[1], [2], []]))
    assert exe.output_count() == 1


def test_chain_fuses_across_the_call():
    # function: sRGB -> Oklab; caller: back to sRGB -- one fused chain kernel after inlining
    f = CommandBuffer()
    a = f.generic()
    i = f.input_generic(a)
    lab = Descriptor(1, 1, Bits.Float32x4, Parts.LabA, ColorKind.Oklab, transfer=Transfer.Linear)
    f.output(f.color_convert(i, lab))
    c = CommandBuffer()
    fn = c.function(f)
    x = c.input(Descriptor.srgb_rgba8(256, 256))
    (y,) = c.invoke(fn, generics=[c.register_descriptor(x)], arguments=[x])
    z = c.color_convert(y, Descriptor.srgb_rgba8(256, 256))
    c.output(z)
    exe = lower(Linker.from_included().link(c, [], [f], [[1], []]))
    assert exe.kernel_count() == 1 and "fused chain kernel" in exe.describe()


def test_generic_entry_point_takes_link_descriptors():
    m = CommandBuffer()
    a = m.generic()
    i = m.input_generic(a)
    m.output(m.resize(i, (16, 16)))
    with pytest.raises(ZosimosError):
        Linker.from_included().link(m)
    exe = lower(Linker.from_included().link(m, [Descriptor.linear_rgba_f32(64, 48)]))
    assert exe.output_count() == 1


def test_derived_descriptor_replaces_the_size():
    # inputs: an image of the generic descriptor and a 32x32 tile of its texel and colour
    f = CommandBuffer()
    a = f.generic()
    small = f.derive_descriptor(a, (32, 32))
    big = f.input_generic(a)
    tile = f.input_generic(small)
    f.output(f.resize(big, (16, 16)))
    f.output(f.resize(tile, (8, 8)))
    assert f.computed_signature() == (1, 2, 2)
    c = CommandBuffer()
    fn = c.function(f)
    x = c.input(Descriptor.linear_rgba_f16(128, 128))
    t = c.input(Descriptor.linear_rgba_f16(32, 32))
    wrong = c.input(Descriptor.linear_rgba_f16(64, 64))
    ty = c.register_descriptor(x)
    with pytest.raises(ZosimosError) as e:
        c.invoke(fn, generics=[ty], arguments=[x, wrong])
    assert e.value.code == 4
    r0, r1 = c.invoke(fn, generics=[ty], arguments=[x, t])
    assert c.describe(r0) == Descriptor.linear_rgba_f16(16, 16)
    assert c.describe(r1) == Descriptor.linear_rgba_f16(8, 8)


def test_knob_of_a_linked_function_is_found_by_link_index():
    f = CommandBuffer()
    a = f.generic()
    i = f.input_generic(a)
    d = Descriptor.srgb_rgba8(64, 64)
    ramp = f.with_knob().bilinear(d, [0] * 4, [1] * 4, [0] * 4, [1] * 4, [0] * 4, [0] * 4)
    f.output(f.palette(i, 0, 1, ramp))
    c = CommandBuffer()
    fn = c.function(f)
    x = c.input(Descriptor.srgb_rgba8(32, 32))
    (y,) = c.invoke(fn, generics=[c.register_descriptor(x)], arguments=[x])
    c.output(y)
    exe = lower(Linker.from_included().link(c, [], [f], [[1], []]))
    knob, n = exe.query_knob(ramp, link_idx=1)
    assert n == 96
    with pytest.raises(ZosimosError) as e:
        exe.query_knob(ramp, link_idx=2)
    assert e.value.code == 3
    exe.set_knob(knob, np.zeros(24, np.float32))
