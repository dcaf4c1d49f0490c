"""Host-side behaviour of the C ABI that needs no GPU: the library loads and exports
every symbol include/zosimos.h declares; command type checks mirror the reference's
CommandBuffer errors (lib/zosimos/src/command.rs); compile/lower plans have the
expected shape (fusion) -- lowering is host work and runs without a device."""
import math
import os
import re

import numpy as np
import pytest

import zosimos_gb300 as zs
from zosimos_gb300 import (Affine, AffineSample, Bits, ColorKind, CommandBuffer, Descriptor, Linker, Parts,
                           Rectangle, Transfer, Whitepoint, ZosimosError)
from zosimos_gb300.workloads import blend_resize, color_chain, resample, rotation

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "zosimos.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(zs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = zs._lib()
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert len(header_symbols()) > 60


def test_library_path_is_in_tree():
    assert zs.library_path().startswith(os.path.join(ROOT, "zosimos_gb300"))


def lower(c, mode=zs.Mode.Fused):
    return Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=mode))


def test_colour_chain_fuses_to_one_kernel():
    c, _, _ = color_chain(4096, 4096)
    fused = lower(c)
    assert fused.kernel_count() == 1 and "fused chain kernel" in fused.describe()
    # the Oklab L/C scaling between cube root and cube is detected as d I + (1,1,1)^T v
    assert "rank-1 L/C scaling" in fused.describe()
    assert lower(c, zs.Mode.PerOpF32).kernel_count() == 7
    assert lower(c, zs.Mode.PerOpF16).kernel_count() == 7


def test_blend_resize_plan():
    c, _, _, _ = blend_resize()
    fused = lower(c)
    # one launch: the affine gather evaluates the blend at each bilinear tap, encodes, and the
    # constant canvas is never stored
    assert fused.kernel_count() == 1 and "evaluates blend per tap" in fused.describe()
    assert lower(c, zs.Mode.PerOpF32).kernel_count() == 6


def test_resample_and_rotation_plans():
    c, _, _ = resample(1024, 768, 512, 384, zs.Filter.Lanczos3)
    fused = lower(c)
    assert fused.kernel_count() == 1 and "resample 2d" in fused.describe()
    assert lower(c, zs.Mode.PerOpF32).kernel_count() == 2
    # A downscale whose tile span does not fit shared memory keeps the two-pass form.
    c, _, _ = resample(65536, 64, 128, 64, zs.Filter.Lanczos3)
    assert lower(c).kernel_count() == 2
    c, _, _, _ = rotation(640, 480, 17.0)
    assert lower(c).kernel_count() == 1


def test_inscribe_requires_upper_rectangle():
    # command.rs:1196-1198
    c = CommandBuffer()
    b = c.input(Descriptor.srgb_rgba8(64, 64))
    a = c.input(Descriptor.srgb_rgba8(16, 8))
    with pytest.raises(ZosimosError) as e:
        c.inscribe(b, Rectangle(4, 4, 20, 12), a)
    assert e.value.code == 4
    c.inscribe(b, Rectangle(0, 0, 16, 8), a)
    c.inscribe_placed(b, Rectangle(4, 4, 20, 12), a)


def test_inscribe_conflicting_types():
    c = CommandBuffer()
    b = c.input(Descriptor.srgb_rgba8(64, 64))
    a = c.input(Descriptor.linear_rgba_f32(16, 8))
    with pytest.raises(ZosimosError) as e:
        c.inscribe(b, Rectangle(0, 0, 16, 8), a)
    assert e.value.is_type_err


def test_affine_rejects_degenerate_matrix():
    c = CommandBuffer()
    b = c.input(Descriptor.srgb_rgba8(64, 64))
    a = c.input(Descriptor.srgb_rgba8(16, 8))
    with pytest.raises(ZosimosError):
        c.affine(b, Affine.new().scale(0.0, 1.0), a)
    c.affine(b, Affine.new(AffineSample.BiLinear).rotate(math.pi / 4), a)


def test_color_convert_needs_same_whitepoint():
    c = CommandBuffer()
    i = c.input(Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(ZosimosError):
        c.color_convert(i, Descriptor.srgb_rgba8(8, 8).with_color(whitepoint=Whitepoint.D50))
    c.color_convert(i, Descriptor.srgb_rgba8(8, 8).with_color(transfer=Transfer.Bt709))


def test_bradford_nonlinear_is_unimplemented():
    c = CommandBuffer()
    i = c.input(Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(ZosimosError) as e:
        c.chromatic_adaptation(i, zs.ChromaticAdaptationMethod.BradfordNonLinear, Whitepoint.D50)
    assert e.value.code == 2


def test_transmute_checks_texel_size():
    c = CommandBuffer()
    i = c.input(Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(ZosimosError):
        c.transmute(i, Descriptor.linear_rgba_f16(8, 8))
    c.transmute(i, Descriptor(8, 8, Bits.UInt16x2, Parts.LumaA))


def test_blend_unimplemented_upstream_is_built_here():
    c = CommandBuffer()
    b = c.input(Descriptor.srgb_rgba8(8, 8))
    a = c.input(Descriptor.srgb_rgba8(8, 8))
    for mode in (zs.Blend.Alpha, zs.Blend.Multiply, zs.Blend.Screen, zs.Blend.Add):
        c.blend(b, Rectangle(0, 0, 8, 8), a, mode)


def test_inconsistent_descriptors_rejected():
    assert not Descriptor(0, 8).is_consistent()
    assert not Descriptor(8, 8, Bits.UInt8x4, Parts.RgbA, ColorKind.Oklab).is_consistent()
    assert Descriptor(8, 8, Bits.UInt8x4, Parts.LchA, ColorKind.Oklab).is_consistent()
    with pytest.raises(ZosimosError):
        CommandBuffer().input(Descriptor(0, 8))


def test_bad_register_and_missing_output():
    c = CommandBuffer()
    with pytest.raises(ZosimosError) as e:
        c.crop(7, Rectangle(0, 0, 1, 1))
    assert e.value.code == 3
    c.input(Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(ZosimosError):
        Linker.from_included().compile(c)          # no output


def test_pool_roundtrip_and_binding_checks():
    pool = zs.Pool()
    img = (np.arange(8 * 8 * 4) % 251).astype(np.uint8).reshape(8, 8, 4)
    k = pool.insert_srgb(img)
    assert (pool.read(k).reshape(8, 8, 4) == img).all()
    assert pool.descriptor(k).width == 8
    c = CommandBuffer()
    i = c.input(Descriptor.srgb_rgba8(8, 8))
    o, _ = c.output(c.color_convert(i, Descriptor.linear_rgba_f32(8, 8)))
    exe = Linker.from_included().compile(c).lower_to()
    env = exe.from_pool(pool)
    env.bind(i, k)
    k2 = pool.insert_srgb(np.zeros((4, 4, 4), np.uint8))
    with pytest.raises(ZosimosError) as e:
        env.bind(i, k2)                     # StartError::MismatchedDescriptor
    assert e.value.code == 6
    with pytest.raises(ZosimosError) as e:
        env.bind(o, k)                      # not an input register
    assert e.value.code == 3
    pool.remove(k2)
    with pytest.raises(ZosimosError):
        pool.remove(k2)


def test_noalloc_rejects_oversized_without_device():
    import ctypes
    fn = zs._lib().zs_resample_rgba16f_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
    fn.restype = ctypes.c_int32
    assert fn(ctypes.c_void_p(16), 8192, 8192, ctypes.c_void_p(16), 4096, 4096, 1, None) == 10
    # Misaligned texel pointers and sides above 2^24 are argument errors, rejected before
    # anything reaches a device.
    assert fn(ctypes.c_void_p(20), 64, 64, ctypes.c_void_p(16), 32, 32, 1, None) == 10
    assert b"aligned" in zs._lib().zs_last_error()
    assert fn(ctypes.c_void_p(16), 64, 64, ctypes.c_void_p(17), 32, 32, 1, None) == 10
    assert fn(ctypes.c_void_p(16), (1 << 24) + 1, 4, ctypes.c_void_p(16), 32, 4, 1, None) == 10
    # A ratio whose filter tables alone exceed the array is rejected, not computed from garbage.
    assert fn(ctypes.c_void_p(16), 1 << 24, 4, ctypes.c_void_p(16), 1 << 20, 4, 1, None) == 10


def test_derivative_plan_and_unimplemented_methods():
    c = CommandBuffer()
    i = c.input(Descriptor.srgb_rgba8(64, 64))
    c.output(c.derivative(i, zs.DerivativeMethod.Sobel, zs.Direction.Height))
    assert Linker.from_included().compile(c).lower_to().kernel_count() == 1
    for m in (zs.DerivativeMethod.Roberts, zs.DerivativeMethod.Scharr4, zs.DerivativeMethod.Scharr5,
              zs.DerivativeMethod.Scharr5Tab):
        c = CommandBuffer()
        i = c.input(Descriptor.srgb_rgba8(8, 8))
        c.output(c.derivative(i, m))                 # the command is accepted ...
        with pytest.raises(ZosimosError) as e:
            Linker.from_included().compile(c)       # ... compiling it is NotYetImplemented
        assert e.value.code == 2


def test_from_buffer_checks():
    # command.rs:937-968: a buffer register is required, and it must hold `height` rows
    # aligned to 256 bytes.
    c = CommandBuffer()
    b = c.buffer_init(np.zeros(8 * 256, np.uint8))
    luma = zs.Descriptor(8, 8, zs.Bits.UInt8, zs.Parts.Luma, zs.ColorKind.Rgb, zs.Primaries.Bt709,
                         zs.Transfer.Srgb, zs.Whitepoint.D65)
    c.output(c.from_buffer(b, luma))
    exe = Linker.from_included().compile(c).lower_to()
    assert exe.kernel_count() == 0 and "copy" in exe.describe()     # a row copy, no kernel
    with pytest.raises(zs.ZosimosError) as e:
        c.from_buffer(b, Descriptor.srgb_rgba8(65, 8))       # 512-byte rows: 4096 bytes needed
    assert e.value.code == 4                                 # ZS_ERR_OTHER: INVALID_CALL upstream
    with pytest.raises(zs.ZosimosError):
        c.color_convert(b, Descriptor.srgb_rgba8(8, 8))      # a buffer is not an image
    i = c.input(Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(zs.ZosimosError):
        c.from_buffer(i, luma)                              # an image is not a buffer
    z = c.buffer_zero(4096)
    c.output(c.from_buffer(z, Descriptor.srgb_rgba8(64, 16)))


def test_fractal_noise_parameters_follow_the_reference_constructors():
    import oracle as O
    for n in (1, 4, 7):
        assert (zs.fractal_noise_with_octaves(n) == O.fractal_noise_with_octaves(n)).all()
        for d in (0.5, 0.8, 1.0):
            got = zs.fractal_noise_set_damping(zs.fractal_noise_with_octaves(n), d)
            assert (got == O.fractal_noise_set_damping(O.fractal_noise_with_octaves(n), d)).all()
    c = CommandBuffer()
    c.output(c.distribution_fractal_noise(Descriptor.srgb_rgba8(32, 16), zs.fractal_noise_with_octaves(4)))
    assert Linker.from_included().compile(c).lower_to().kernel_count() == 1
    bad = zs.fractal_noise_with_octaves(4)
    bad[4] = 33.0
    with pytest.raises(zs.ZosimosError):
        CommandBuffer().distribution_fractal_noise(Descriptor.srgb_rgba8(8, 8), bad)


def test_normal2d_parameters_follow_the_reference_constructors():
    import oracle as O
    assert (zs.normal2d_with_diagonal(0.2, 0.2) == O.normal2d_with_diagonal(0.2, 0.2)).all()
    assert (zs.normal2d_with_direction(0.04998, 0.0501) == O.normal2d_with_direction(0.04998, 0.0501)).all()
    c = CommandBuffer()
    c.output(c.distribution_normal2d(Descriptor.srgb_rgba8(32, 16), zs.normal2d_with_diagonal(0.2, 0.2)))
    assert Linker.from_included().compile(c).lower_to().kernel_count() == 1


def test_batch_entry_points_check_arguments_without_device():
    import ctypes
    lib = zs._lib()
    c, _, _ = color_chain(16, 16)
    exe = lower(c)
    assert exe.output_count() == 1
    # an empty batch is a no-op; null handles and tables are argument errors
    assert lib.zs_batch_run_device(exe._h, None, None, 0, None) == 0
    assert lib.zs_batch_run_device(None, None, None, 1, None) == 10
    assert lib.zs_batch_run_device(exe._h, None, None, 1, None) == 10
    pool = zs.Pool()
    assert lib.zs_batch_run(exe._h, pool._h, None, 1, None) == 10
    assert lib.zs_batch_run(exe._h, pool._h, None, 0, None) == 0


def test_knobs_and_buffer_parameters_host_side():
    c = CommandBuffer()
    d = Descriptor.srgb_rgba8(16, 16)
    plain = c.bilinear(d, [0] * 4, [1] * 4, [0] * 4, [1] * 4, [0] * 4, [0] * 4)
    knobbed = c.with_knob().bilinear(d, [0] * 4, [1] * 4, [0] * 4, [1] * 4, [0] * 4, [0] * 4)
    # with_knob on an operation without a parameter block fails and is not left pending
    with pytest.raises(ZosimosError) as e:
        c.with_knob().color_convert(plain, Descriptor.linear_rgba_f32(16, 16))
    assert e.value.code == 2
    later = c.bilinear(d, [0] * 4, [1] * 4, [0] * 4, [1] * 4, [0] * 4, [0] * 4)
    short = c.buffer_init(np.zeros(32, np.uint8))
    with pytest.raises(ZosimosError) as e:
        c.with_buffer(short).bilinear(d, [0] * 4, [1] * 4, [0] * 4, [1] * 4, [0] * 4, [0] * 4)
    assert e.value.code == 4            # CommandError::INVALID_CALL: buffer too short
    with pytest.raises(ZosimosError) as e:
        c.with_buffer(plain)
    assert e.value.is_type_err
    outs = [c.output(r)[0] for r in (plain, knobbed, later)]
    exe = Linker.from_included().compile(c).lower_to()
    knob, n = exe.query_knob(knobbed)
    assert n == 96 and "[knob]" in exe.describe()
    for reg in (plain, later):
        with pytest.raises(ZosimosError) as e:
            exe.query_knob(reg)
        assert e.value.code == 3
    env = exe.from_pool(zs.Pool())
    with pytest.raises(ZosimosError) as e:
        env.knob(knob, np.zeros(95, np.uint8))
    assert e.value.code == 10
    env.knob(knob, np.zeros(24, np.float32))
    assert len(outs) == 3


def test_tuning_cache_and_keys(tmp_path):
    c, _, _ = color_chain(4096, 4096)
    exe = lower(c)
    key = exe.tune_key(zs.Tune.ChainThreads)
    # kernel family / chain specialisation / size class / device
    parts = key.split("/")
    assert parts[0] == "chain" and parts[1].startswith("flags") and parts[2] == "px2^24"
    assert exe.tune_key(zs.Tune.BatchRows, 256).startswith("batch/flags")
    assert exe.get_launch(zs.Tune.ChainThreads) == 1024          # untuned default
    assert exe.get_launch(zs.Tune.ChainVectors) == 2
    assert exe.tune_key(zs.Tune.ChainVectors).startswith("chain_vectors/flags")
    exe.set_launch(zs.Tune.ChainVectors, 1)
    assert exe.get_launch(zs.Tune.ChainVectors) == 1
    with pytest.raises(ZosimosError) as e:
        exe.set_launch(zs.Tune.ChainVectors, 3)
    assert e.value.code == 10
    exe.set_launch(zs.Tune.ChainThreads, 512)
    assert exe.get_launch(zs.Tune.ChainThreads) == 512
    with pytest.raises(ZosimosError) as e:
        exe.set_launch(zs.Tune.ChainThreads, 300)
    assert e.value.code == 10
    with pytest.raises(ZosimosError) as e:
        exe.set_launch(zs.Tune.BatchRows, 17)
    assert e.value.code == 10
    assert exe.tune_key(zs.Tune.BatchThreads, 256).startswith("batch_threads/flags")
    # the tensor-core resample's tile width: the planned width, candidates only
    rc, _, _ = resample(1024, 1024, 512, 512, zs.Filter.Lanczos3)
    rexe = lower(rc)
    assert "tensor cores" in rexe.describe()
    assert rexe.get_launch(zs.Tune.ResampleTile) == 16
    assert rexe.tune_key(zs.Tune.ResampleTile).startswith("resample_tc/taps")
    for tw in (8, 32, 16):
        rexe.set_launch(zs.Tune.ResampleTile, tw)
        assert rexe.get_launch(zs.Tune.ResampleTile) == tw
    with pytest.raises(ZosimosError) as e:
        rexe.set_launch(zs.Tune.ResampleTile, 24)
    assert e.value.code == 10
    with pytest.raises(ZosimosError) as e:
        exe.set_launch(zs.Tune.ResampleTile, 16)          # the chain has no resample step
    assert e.value.code == 2
    exe.set_launch(zs.Tune.BatchThreads, 640)
    assert exe.get_launch(zs.Tune.BatchThreads) == 640
    with pytest.raises(ZosimosError) as e:
        exe.set_launch(zs.Tune.BatchThreads, 1024)
    assert e.value.code == 10
    # the process-wide cache: values, a file round trip, and misses
    zs.tune_cache_put("test/a/b", 7)
    zs.tune_cache_put("test/c", 16)
    path = tmp_path / "tune.txt"
    zs.tune_cache_save(path)
    zs.tune_cache_put("test/a/b", 1)
    zs.tune_cache_load(path)
    assert zs.tune_cache_get("test/a/b") == 7 and zs.tune_cache_get("test/c") == 16
    assert "test/c 16" in path.read_text()
    with pytest.raises(ZosimosError) as e:
        zs.tune_cache_get("test/missing")
    assert e.value.code == 7
    bad = tmp_path / "bad.txt"
    bad.write_text("oops\n")
    with pytest.raises(ZosimosError):
        zs.tune_cache_load(bad)


def test_custom_op_ids_are_checked_without_device():
    c = CommandBuffer()
    i = c.input(Descriptor.srgb_rgba8(8, 8))
    with pytest.raises(ZosimosError) as e:
        c.unary_dynamic(i, 12345, Descriptor.srgb_rgba8(8, 8))
    assert e.value.code == 10
    c.output(i)
