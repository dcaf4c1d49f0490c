"""zosimos_gb300 -- a GB300 (sm_103a) executor for zosimos' compiled raster pipeline.

Python mirror of the reference's Rust API (lib/zosimos/src: ``Pool``,
``CommandBuffer``, ``Linker``/``Program``, ``Executable``, ``Environment``,
``Execution``, ``Retire``) over the C ABI of ``libzosimos_gb300.so``
(include/zosimos.h).  All pixel work runs in hand-written CUDA kernels; there is
no CPU fallback: importing this package on a machine without the built library
raises, and launching without a CUDA device returns a device error.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field, replace
from typing import List, Optional, Sequence

import numpy as np

from . import build as _build

__all__ = [
    "Descriptor", "Rectangle", "Affine", "AffineSample", "Pool", "CommandBuffer", "Linker", "Program",
    "Capabilities", "Executable", "Environment", "Execution", "ZosimosError", "Bits", "Parts", "Transfer",
    "ColorKind", "Primaries", "Whitepoint", "ChromaticAdaptationMethod", "Blend", "Filter", "Mode",
    "library_path", "kernel_launch_count",
]

# ---------------------------------------------------------------- vocabulary (include/zosimos.h)


class Bits:
    UInt8, UInt332, UInt233, UInt16, UInt4x4, UInt_444, UInt444_, UInt565 = range(8)
    UInt8x2, UInt8x3, UInt8x4, UInt16x2, UInt16x3, UInt16x4 = range(8, 14)
    UInt1010102, UInt2101010, UInt101010_, UInt_101010, Float16x4, Float32x4 = range(14, 20)


class Parts:
    A, R, G, B, Luma, LumaA, Rgb, Bgr, RgbA, Rgbx, BgrA, Bgrx = range(12)
    ARgb, Xrgb, ABgr, Xbgr, Yuv, Lab, LabA, Lch, LchA = range(12, 21)


class Transfer:
    Bt709, Bt470M, Bt601, Smpte240, Linear, Srgb, Bt2020_10bit, Bt2020_12bit = range(8)
    Smpte2084, Bt2100Pq, Bt2100Hlg, LinearScene = range(8, 12)


class ColorKind:
    Rgb, Oklab, SrLab2, Scalars = range(4)


class Primaries:
    Bt601_525, Bt601_625, Bt709, Smpte240, Bt2020, Bt2100, P3, AdobeRgb, Xyz = range(9)


class Whitepoint:
    A, B, C, D50, D55, D65, D75, E, F2, F7, F11 = range(11)


class ChromaticAdaptationMethod:
    Xyz, VonKries, BradfordVonKries, BradfordNonLinear = range(4)


class AffineSample:
    Nearest, BiLinear = range(2)


class Blend:
    Alpha = Over = 0
    Multiply, Screen, Add = 1, 2, 3


class Filter:
    Box, Lanczos3, Triangle = range(3)


class DerivativeMethod:
    """command.rs DerivativeMethod (Roberts, Scharr4, Scharr5, Scharr5Tab: not yet implemented)."""
    Roberts, Prewitt, Sobel, Scharr3, Scharr4, Scharr5, Scharr3To4Bit, Scharr5Tab, Scharr3To8Bit = range(9)


class Direction:
    Width, Height = range(2)


class Mode:
    Fused, PerOpF32, PerOpF16 = range(3)


class Tune:
    """Launch parameters the autotuner chooses (ZS_TUNE_*)."""
    ChainThreads, BatchRows, BatchThreads, ResampleTile, ChainVectors = range(5)


STATUS = {0: "ok", 1: "type error", 2: "unimplemented", 3: "bad register", 4: "other", 5: "launch error",
          6: "mismatched descriptor", 7: "missing key", 8: "device error", 9: "timeout", 10: "invalid argument",
          11: "out of memory", 12: "step limit"}

TEXEL_BYTES = [1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 4, 4, 6, 8, 4, 4, 4, 4, 8, 16]


class ZosimosError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code

    @property
    def is_type_err(self) -> bool:
        return self.code == 1


# ---------------------------------------------------------------- C structures


class _CDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("row_stride", ctypes.c_uint64),
                ("bits", ctypes.c_uint32), ("parts", ctypes.c_uint32), ("color", ctypes.c_uint32),
                ("primaries", ctypes.c_uint32), ("transfer", ctypes.c_uint32), ("whitepoint", ctypes.c_uint32),
                ("alpha", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class _CRect(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint32), ("y", ctypes.c_uint32), ("max_x", ctypes.c_uint32),
                ("max_y", ctypes.c_uint32)]


class _CCaps(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("mode", ctypes.c_uint32), ("use_graph", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


_LIB = None


def library_path() -> str:
    return _build.LIB


def _lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        P, U32, U64, I32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
        pU32, pU64 = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint64)
        pD, pR = ctypes.POINTER(_CDesc), ctypes.POINTER(_CRect)
        sig = {
            "zs_last_error": ([], ctypes.c_char_p), "zs_version": ([], ctypes.c_char_p),
            "zs_pool_new": ([], P), "zs_pool_free": ([P], None),
            "zs_pool_insert": ([P, pD, P, pU64], I32), "zs_pool_declare": ([P, pD, pU64], I32),
            "zs_pool_descriptor": ([P, U64, pD], I32), "zs_pool_read": ([P, U64, P, U64], I32),
            "zs_pool_write": ([P, U64, P, U64], I32), "zs_pool_upload": ([P, U64], I32),
            "zs_pool_device_ptr": ([P, U64, ctypes.POINTER(P)], I32), "zs_pool_remove": ([P, U64], I32),
            "zs_pool_set_descriptor": ([P, U64, pD], I32), "zs_pool_clear_cache": ([P], I32),
            "zs_cmd_new": ([], P), "zs_cmd_free": ([P], None),
            "zs_cmd_input": ([P, pD, pU32], I32), "zs_cmd_crop": ([P, U32, pR, pU32], I32),
            "zs_cmd_color_convert": ([P, U32, pD, pU32], I32),
            "zs_cmd_chromatic_adaptation": ([P, U32, U32, U32, pU32], I32),
            "zs_cmd_inscribe": ([P, U32, pR, U32, pU32], I32),
            "zs_cmd_inscribe_placed": ([P, U32, pR, U32, pU32], I32),
            "zs_cmd_extract": ([P, U32, U32, pU32], I32), "zs_cmd_inject": ([P, U32, U32, U32, pU32], I32),
            "zs_cmd_transmute": ([P, U32, pD, pU32], I32), "zs_cmd_palette": ([P, U32, I32, I32, U32, pU32], I32),
            "zs_cmd_bilinear": ([P, pD, P, pU32], I32), "zs_cmd_solid_rgba": ([P, pD, P, pU32], I32),
            "zs_cmd_affine": ([P, U32, P, U32, U32, pU32], I32), "zs_cmd_resize": ([P, U32, U32, U32, pU32], I32),
            "zs_cmd_resize_filtered": ([P, U32, U32, U32, U32, pU32], I32),
            "zs_cmd_blend": ([P, U32, pR, U32, U32, pU32], I32), "zs_cmd_color_matrix": ([P, U32, P, pU32], I32),
            "zs_cmd_derivative": ([P, U32, U32, U32, pU32], I32),
            "zs_cmd_distribution_normal2d": ([P, pD, P, pU32], I32),
            "zs_normal2d_with_diagonal": ([ctypes.c_float, ctypes.c_float, P], I32),
            "zs_normal2d_with_direction": ([ctypes.c_float, ctypes.c_float, P], I32),
            "zs_cmd_distribution_fractal_noise": ([P, pD, P, pU32], I32),
            "zs_cmd_buffer_init": ([P, P, U64, pU32], I32),
            "zs_cmd_buffer_zero": ([P, U64, pU32], I32),
            "zs_cmd_from_buffer": ([P, U32, pD, pU32], I32),
            "zs_fractal_noise_with_octaves": ([U32, P], I32),
            "zs_fractal_noise_set_damping": ([P, ctypes.c_float], I32),
            "zs_cmd_output": ([P, U32, pU32, pD], I32), "zs_cmd_describe": ([P, U32, pD], I32),
            "zs_compile": ([P, ctypes.POINTER(P)], I32), "zs_program_free": ([P], None),
            "zs_lower": ([P, ctypes.POINTER(_CCaps), ctypes.POINTER(P)], I32), "zs_executable_free": ([P], None),
            "zs_executable_kernel_count": ([P, pU32], I32), "zs_executable_describe": ([P], ctypes.c_char_p),
            "zs_env_new": ([P, P, ctypes.POINTER(P)], I32), "zs_env_free": ([P], None),
            "zs_env_bind": ([P, U32, U64], I32), "zs_env_bind_output": ([P, U32, U64], I32),
            "zs_launch": ([P, P, ctypes.POINTER(P)], I32), "zs_exec_is_running": ([P], I32),
            "zs_exec_step": ([P], I32), "zs_exec_sync": ([P], I32), "zs_retire_output": ([P, U32, pU64], I32),
            "zs_exec_free": ([P], None),
            "zs_run_host": ([P, P, U32, P, U32], I32), "zs_run_device": ([P, P, U32, P, U32, P], I32),
            "zs_host_alloc": ([U64], P), "zs_host_free": ([P], None), "zs_device_alloc": ([U64], P),
            "zs_device_free": ([P], None), "zs_memcpy_h2d": ([P, P, U64], I32), "zs_memcpy_d2h": ([P, P, U64], I32),
            "zs_device_synchronize": ([], I32), "zs_kernel_launch_count": ([], U64),
            "zs_device_status": ([ctypes.c_int32, pU32], I32),
            "zs_selftest_wait_timeout": ([ctypes.c_int32, U32], I32),
            "zs_descriptor_is_consistent": ([pD], I32), "zs_descriptor_byte_len": ([pD], U64),
            "zs_texel_bytes": ([U32], U32),
            "zs_batch_thumbnails": ([P, P, P, P, U32, U32, P, P], I32),
            "zs_batch_run_device": ([P, P, P, U32, P], I32), "zs_batch_run": ([P, P, P, U32, P], I32),
            "zs_executable_io_count": ([P, P, P], I32),
            "zs_cmd_with_knob": ([P], I32), "zs_cmd_with_buffer": ([P, U32], I32),
            "zs_register_op": ([P, U64, ctypes.c_char_p, pU32], I32),
            "zs_cmd_construct_dynamic": ([P, U32, P, U64, pD, pU32], I32),
            "zs_cmd_unary_dynamic": ([P, U32, U32, P, U64, pD, pU32], I32),
            "zs_cmd_binary_dynamic": ([P, U32, U32, U32, P, U64, pD, pU32], I32),
            "zs_autotune": ([P, P, U32, P, U32, P, U32, P], I32),
            "zs_autotune_batch_thumbnails": ([P, P, P, P, U32, U32, P, P, U32, P], I32),
            "zs_executable_set_launch": ([P, U32, I32], I32), "zs_executable_get_launch": ([P, U32, P], I32),
            "zs_executable_tune_key": ([P, U32, U32, P, U64], I32),
            "zs_tune_cache_get": ([ctypes.c_char_p, P], I32), "zs_tune_cache_put": ([ctypes.c_char_p, I32], I32),
            "zs_tune_cache_save": ([ctypes.c_char_p], I32), "zs_tune_cache_load": ([ctypes.c_char_p], I32),
            "zs_executable_query_knob": ([P, U32, U32, pU32, pU64], I32),
            "zs_executable_set_knob": ([P, U32, P, U64], I32), "zs_env_knob": ([P, U32, P, U64], I32),
            "zs_exec_step_to": ([P, U32, pU32], I32), "zs_retire_input": ([P, U32, pU64], I32),
            "zs_env_recover_buffers": ([P, pU64], I32),
            "zs_cmd_generic": ([P, pU32], I32), "zs_cmd_input_generic": ([P, U32, pU32], I32),
            "zs_cmd_derive_descriptor": ([P, U32, U32, U32, pU32], I32),
            "zs_cmd_register_descriptor": ([P, U32, pU32], I32),
            "zs_cmd_signature": ([P, pU32, pU32, pU32], I32), "zs_cmd_function": ([P, P, pU32], I32),
            "zs_cmd_invoke": ([P, U32, pU32, U32, pU32, U32, pU32, U32], I32),
            "zs_link": ([P, pD, U32, ctypes.POINTER(P), U32, ctypes.POINTER(pU32), pU32, U32, ctypes.POINTER(P)], I32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = lib
    return _LIB


def _check(rc: int) -> None:
    if rc != 0:
        msg = _lib().zs_last_error()
        raise ZosimosError(rc, msg.decode() if msg else "")


def kernel_launch_count() -> int:
    return int(_lib().zs_kernel_launch_count())


def selftest_wait_timeout(device: int = 0, limit_us: int = 2000) -> None:
    """Run a kernel whose bounded wait nothing completes (it gives up after `limit_us` and
    sets bit 0 of the device status word, as a real timeout would)."""
    _check(_lib().zs_selftest_wait_timeout(device, limit_us))


def normal2d_with_diagonal(var0: float, var1: float) -> np.ndarray:
    """DistributionNormal2d::with_diagonal: parameters of a centred normal density."""
    p = np.zeros(7, np.float32)
    _check(_lib().zs_normal2d_with_diagonal(var0, var1, p.ctypes.data))
    return p


def fractal_noise_with_octaves(num_octaves: int) -> np.ndarray:
    """FractalNoise::with_octaves: [grid x, grid y, initial amplitude, damping, octaves]."""
    p = np.zeros(5, np.float32)
    _check(_lib().zs_fractal_noise_with_octaves(num_octaves, p.ctypes.data))
    return p


def fractal_noise_set_damping(params, damping: float) -> np.ndarray:
    """FractalNoise::set_damping: amplitudes of all octaves sum to 1."""
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(5)).copy()
    _check(_lib().zs_fractal_noise_set_damping(p.ctypes.data, damping))
    return p


def normal2d_with_direction(x: float, y: float) -> np.ndarray:
    """DistributionNormal2d::with_direction: a 1-D normal density along (x, y)."""
    p = np.zeros(7, np.float32)
    _check(_lib().zs_normal2d_with_direction(x, y, p.ctypes.data))
    return p


def device_status(device: int = 0) -> int:
    """Synchronise `device` and return (and clear) its status word: bit 0 set means a
    kernel's bounded wait on its own bulk copies gave up and its output is incomplete."""
    flags = ctypes.c_uint32(0)
    _check(_lib().zs_device_status(device, ctypes.byref(flags)))
    return int(flags.value)


# ---------------------------------------------------------------- value types


@dataclass
class Descriptor:
    """buffer.rs Descriptor: layout + colour + texel (row_stride 0 = tight rows)."""
    width: int
    height: int
    bits: int = Bits.UInt8x4
    parts: int = Parts.RgbA
    color: int = ColorKind.Rgb
    primaries: int = Primaries.Bt709
    transfer: int = Transfer.Srgb
    whitepoint: int = Whitepoint.D65
    alpha: int = 0
    row_stride: int = 0

    @staticmethod
    def srgb_rgba8(width: int, height: int) -> "Descriptor":
        """Descriptor::with_srgb_image of an RGBA8 image."""
        return Descriptor(width, height)

    @staticmethod
    def linear_rgba_f32(width: int, height: int, primaries=Primaries.Bt709, whitepoint=Whitepoint.D65):
        return Descriptor(width, height, Bits.Float32x4, Parts.RgbA, ColorKind.Rgb, primaries, Transfer.Linear,
                          whitepoint)

    @staticmethod
    def linear_rgba_f16(width: int, height: int, primaries=Primaries.Bt709, whitepoint=Whitepoint.D65):
        return Descriptor(width, height, Bits.Float16x4, Parts.RgbA, ColorKind.Rgb, primaries, Transfer.Linear,
                          whitepoint)

    def with_size(self, width: int, height: int) -> "Descriptor":
        return replace(self, width=width, height=height, row_stride=0)

    def with_color(self, **kw) -> "Descriptor":
        return replace(self, **kw)

    @property
    def texel_bytes(self) -> int:
        return TEXEL_BYTES[self.bits]

    @property
    def byte_len(self) -> int:
        return (self.row_stride or self.width * self.texel_bytes) * self.height

    def is_consistent(self) -> bool:
        return bool(_lib().zs_descriptor_is_consistent(ctypes.byref(self._c())))

    def _c(self) -> _CDesc:
        return _CDesc(self.width, self.height, self.row_stride, self.bits, self.parts, self.color, self.primaries,
                      self.transfer, self.whitepoint, self.alpha, 0)

    @staticmethod
    def _from_c(c: _CDesc) -> "Descriptor":
        return Descriptor(c.width, c.height, c.bits, c.parts, c.color, c.primaries, c.transfer, c.whitepoint,
                          c.alpha, c.row_stride)


@dataclass
class Rectangle:
    """command.rs Rectangle: [x, max_x) x [y, max_y)."""
    x: int
    y: int
    max_x: int
    max_y: int

    @staticmethod
    def with_width_height(w: int, h: int) -> "Rectangle":
        return Rectangle(0, 0, w, h)

    def width(self) -> int:
        return max(self.max_x - self.x, 0)

    def height(self) -> int:
        return max(self.max_y - self.y, 0)

    def contains(self, o: "Rectangle") -> bool:
        if not (self.x <= o.x and self.y <= o.y):
            return False
        rw, rh = self.width() - (o.x - self.x), self.height() - (o.y - self.y)
        return rw >= 0 and rh >= 0 and rw >= o.width() and rh >= o.height()

    def join(self, o: "Rectangle") -> "Rectangle":
        return Rectangle(min(self.x, o.x), min(self.y, o.y), max(self.max_x, o.max_x), max(self.max_y, o.max_y))

    def meet(self, o: "Rectangle") -> "Rectangle":
        return Rectangle(max(self.x, o.x), max(self.y, o.y), min(self.max_x, o.max_x), min(self.max_y, o.max_y))

    def _c(self) -> _CRect:
        return _CRect(self.x, self.y, self.max_x, self.max_y)


def _f32(v) -> np.float32:
    return np.float32(v)


@dataclass
class Affine:
    """command.rs Affine: a row-major homogeneous matrix in pixel units, built in f32
    exactly like Affine::{new, scale, rotate, shift} (command.rs:3420-3485)."""
    transformation: np.ndarray = field(default_factory=lambda: np.eye(3, dtype=np.float32))
    sampling: int = AffineSample.Nearest

    @staticmethod
    def new(sampling: int = AffineSample.Nearest) -> "Affine":
        return Affine(np.eye(3, dtype=np.float32), sampling)

    def _post(self, m) -> "Affine":
        m = np.asarray(m, dtype=np.float32).reshape(3, 3)
        t = self.transformation.astype(np.float32)
        out = np.zeros((3, 3), dtype=np.float32)
        for i in range(3):
            for j in range(3):
                out[i, j] = _f32(_f32(_f32(m[i, 0] * t[0, j]) + _f32(m[i, 1] * t[1, j])) + _f32(m[i, 2] * t[2, j]))
        return Affine(out, self.sampling)

    def scale(self, x: float, y: float) -> "Affine":
        return self._post([x, 0, 0, 0, y, 0, 0, 0, 1])

    def rotate(self, rad: float) -> "Affine":
        r = _f32(rad)
        c, s = _f32(math.cos(r)), _f32(math.sin(r))
        return self._post([c, s, 0, -s, c, 0, 0, 0, 1])

    def shift(self, x: float, y: float) -> "Affine":
        return self._post([1, 0, x, 0, 1, y, 0, 0, 1])


@dataclass
class Capabilities:
    """Lowering options (program.rs Capabilities): device, executor mode, graph replay and
    `simt_resample` (resize_filtered on the FP32 SIMT kernel instead of the tensor cores)."""
    device: int = 0
    mode: int = Mode.Fused
    use_graph: bool = True
    simt_resample: bool = False
    zero_copy: bool = True        # run_host of a lone chain on pinned host buffers: no staging copies


# ---------------------------------------------------------------- pool


class Pool:
    """pool.rs Pool: owns images in pinned host memory, optionally device resident."""

    def __init__(self):
        self._h = _lib().zs_pool_new()
        if not self._h:
            raise ZosimosError(11, "pool allocation failed")

    def __del__(self):
        if getattr(self, "_h", None):
            _lib().zs_pool_free(self._h)
            self._h = None

    def insert(self, desc: Descriptor, data) -> int:
        arr = np.ascontiguousarray(data)
        if arr.nbytes != desc.byte_len:
            raise ZosimosError(10, f"expected {desc.byte_len} bytes, got {arr.nbytes}")
        key = ctypes.c_uint64()
        _check(_lib().zs_pool_insert(self._h, ctypes.byref(desc._c()), arr.ctypes.data, ctypes.byref(key)))
        return key.value

    def insert_srgb(self, rgba: np.ndarray) -> int:
        """Pool::insert_srgb for an (H, W, 4) uint8 image."""
        h, w = rgba.shape[:2]
        return self.insert(Descriptor.srgb_rgba8(w, h), np.ascontiguousarray(rgba, dtype=np.uint8))

    def declare(self, desc: Descriptor) -> int:
        key = ctypes.c_uint64()
        _check(_lib().zs_pool_declare(self._h, ctypes.byref(desc._c()), ctypes.byref(key)))
        return key.value

    def descriptor(self, key: int) -> Descriptor:
        c = _CDesc()
        _check(_lib().zs_pool_descriptor(self._h, key, ctypes.byref(c)))
        return Descriptor._from_c(c)

    def set_descriptor(self, key: int, desc: Descriptor) -> None:
        _check(_lib().zs_pool_set_descriptor(self._h, key, ctypes.byref(desc._c())))

    def read(self, key: int) -> np.ndarray:
        """The image bytes as (H, row_bytes) uint8."""
        d = self.descriptor(key)
        out = np.empty((d.height, d.row_stride or d.width * d.texel_bytes), dtype=np.uint8)
        _check(_lib().zs_pool_read(self._h, key, out.ctypes.data, out.nbytes))
        return out

    def write(self, key: int, data) -> None:
        arr = np.ascontiguousarray(data)
        _check(_lib().zs_pool_write(self._h, key, arr.ctypes.data, arr.nbytes))

    def upload(self, key: int) -> None:
        _check(_lib().zs_pool_upload(self._h, key))

    def device_ptr(self, key: int) -> int:
        p = ctypes.c_void_p()
        _check(_lib().zs_pool_device_ptr(self._h, key, ctypes.byref(p)))
        return p.value

    def remove(self, key: int) -> None:
        _check(_lib().zs_pool_remove(self._h, key))

    def clear_cache(self) -> None:
        _check(_lib().zs_pool_clear_cache(self._h))


# ---------------------------------------------------------------- command buffer


class CommandBuffer:
    """command.rs CommandBuffer: SSA image ops; each method returns the result register."""

    def __init__(self):
        self._h = _lib().zs_cmd_new()

    def __del__(self):
        if getattr(self, "_h", None):
            _lib().zs_cmd_free(self._h)
            self._h = None

    def _reg(self, fn, *args) -> int:
        reg = ctypes.c_uint32()
        _check(fn(self._h, *args, ctypes.byref(reg)))
        return reg.value

    def input(self, desc: Descriptor) -> int:
        return self._reg(_lib().zs_cmd_input, ctypes.byref(desc._c()))

    def crop(self, src: int, rect: Rectangle) -> int:
        return self._reg(_lib().zs_cmd_crop, src, ctypes.byref(rect._c()))

    def color_convert(self, src: int, target: Descriptor) -> int:
        """color_convert(src, color, texel): `target` supplies colour and texel."""
        return self._reg(_lib().zs_cmd_color_convert, src, ctypes.byref(target._c()))

    def chromatic_adaptation(self, src: int, method: int, target: int) -> int:
        return self._reg(_lib().zs_cmd_chromatic_adaptation, src, method, target)

    def inscribe(self, below: int, rect: Rectangle, above: int) -> int:
        return self._reg(_lib().zs_cmd_inscribe, below, ctypes.byref(rect._c()), above)

    def inscribe_placed(self, below: int, rect: Rectangle, above: int) -> int:
        return self._reg(_lib().zs_cmd_inscribe_placed, below, ctypes.byref(rect._c()), above)

    def extract(self, src: int, channel: int) -> int:
        return self._reg(_lib().zs_cmd_extract, src, channel)

    def inject(self, below: int, channel: int, above: int) -> int:
        return self._reg(_lib().zs_cmd_inject, below, channel, above)

    def transmute(self, src: int, target: Descriptor) -> int:
        return self._reg(_lib().zs_cmd_transmute, src, ctypes.byref(target._c()))

    def palette(self, palette: int, width_channel: Optional[int], height_channel: Optional[int],
                indices: int) -> int:
        wc = -1 if width_channel is None else width_channel
        hc = -1 if height_channel is None else height_channel
        return self._reg(_lib().zs_cmd_palette, palette, wc, hc, indices)

    def bilinear(self, desc: Descriptor, u_min, u_max, v_min, v_max, uv_min, uv_max) -> int:
        p = np.ascontiguousarray(np.concatenate([u_min, u_max, v_min, v_max, uv_min, uv_max]).astype(np.float32))
        return self._reg(_lib().zs_cmd_bilinear, ctypes.byref(desc._c()), p.ctypes.data)

    def solid_rgba(self, desc: Descriptor, color) -> int:
        c = np.ascontiguousarray(np.asarray(color, dtype=np.float32))
        return self._reg(_lib().zs_cmd_solid_rgba, ctypes.byref(desc._c()), c.ctypes.data)

    def affine(self, below: int, affine: Affine, above: int) -> int:
        m = np.ascontiguousarray(affine.transformation.astype(np.float32).reshape(9))
        return self._reg(_lib().zs_cmd_affine, below, m.ctypes.data, affine.sampling, above)

    def resize(self, src: int, size) -> int:
        return self._reg(_lib().zs_cmd_resize, src, size[0], size[1])

    def resize_filtered(self, src: int, size, filt: int) -> int:
        return self._reg(_lib().zs_cmd_resize_filtered, src, size[0], size[1], filt)

    def distribution_normal2d(self, desc: Descriptor, params) -> int:
        """params: the 7 floats of normal2d_with_diagonal / normal2d_with_direction."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(7))
        return self._reg(_lib().zs_cmd_distribution_normal2d, ctypes.byref(desc._c()), p.ctypes.data)

    def buffer_init(self, data) -> int:
        """A byte buffer register holding a copy of `data` (bytes, or the raw bytes of an array)."""
        if isinstance(data, np.ndarray):
            b = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
        else:
            b = np.frombuffer(bytes(data), np.uint8)
        return self._reg(_lib().zs_cmd_buffer_init, b.ctypes.data, b.nbytes)

    def buffer_zero(self, length: int) -> int:
        return self._reg(_lib().zs_cmd_buffer_zero, length)

    def from_buffer(self, buffer: int, desc: Descriptor) -> int:
        """The buffer's bytes as an image of `desc`, rows 256-byte aligned."""
        return self._reg(_lib().zs_cmd_from_buffer, buffer, ctypes.byref(desc._c()))

    def distribution_fractal_noise(self, desc: Descriptor, params) -> int:
        """params: the 5 floats of fractal_noise_with_octaves / fractal_noise_set_damping."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(5))
        return self._reg(_lib().zs_cmd_distribution_fractal_noise, ctypes.byref(desc._c()), p.ctypes.data)

    def derivative(self, src: int, method: int, direction: int = Direction.Width) -> int:
        return self._reg(_lib().zs_cmd_derivative, src, method, direction)

    def blend(self, below: int, rect: Rectangle, above: int, mode: int) -> int:
        return self._reg(_lib().zs_cmd_blend, below, ctypes.byref(rect._c()), above, mode)

    def color_matrix(self, src: int, matrix) -> int:
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float32).reshape(9))
        return self._reg(_lib().zs_cmd_color_matrix, src, m.ctypes.data)

    def with_knob(self) -> "CommandBuffer":
        """CommandBuffer::with_knob: the next operation's parameters become a run-time knob."""
        _check(_lib().zs_cmd_with_knob(self._h))
        return self

    def with_buffer(self, buffer: int) -> "CommandBuffer":
        """CommandBuffer::with_buffer: the next operation reads its parameters from `buffer`."""
        _check(_lib().zs_cmd_with_buffer(self._h, buffer))
        return self

    def construct_dynamic(self, op: int, desc: Descriptor, uniforms=b"") -> int:
        """CommandBuffer::construct_dynamic: a registered custom kernel with no operand."""
        u = _uniform_bytes(uniforms)
        return self._reg(_lib().zs_cmd_construct_dynamic, op, u, len(u), ctypes.byref(desc._c()))

    def unary_dynamic(self, src: int, op: int, desc: Descriptor, uniforms=b"") -> int:
        u = _uniform_bytes(uniforms)
        return self._reg(_lib().zs_cmd_unary_dynamic, src, op, u, len(u), ctypes.byref(desc._c()))

    def binary_dynamic(self, lhs: int, rhs: int, op: int, desc: Descriptor, uniforms=b"") -> int:
        u = _uniform_bytes(uniforms)
        return self._reg(_lib().zs_cmd_binary_dynamic, lhs, rhs, op, u, len(u), ctypes.byref(desc._c()))

    # -- generic functions (command.rs:756-922)

    def generic(self) -> int:
        """CommandBuffer::generic: a generic descriptor parameter; returns its descriptor variable."""
        ty = ctypes.c_uint32()
        _check(_lib().zs_cmd_generic(self._h, ctypes.byref(ty)))
        return ty.value

    def input_generic(self, ty: int) -> int:
        return self._reg(_lib().zs_cmd_input_generic, ty)

    def derive_descriptor(self, base: int, size=None) -> int:
        """CommandBuffer::derive_descriptor: variable `base` with its size replaced (None: kept)."""
        w, h = size if size is not None else (0, 0)
        return self._reg(_lib().zs_cmd_derive_descriptor, base, w, h)

    def register_descriptor(self, reg: int) -> int:
        return self._reg(_lib().zs_cmd_register_descriptor, reg)

    def computed_signature(self):
        """(generics, inputs, outputs) counts of this buffer as a function."""
        g, i, o = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _check(_lib().zs_cmd_signature(self._h, ctypes.byref(g), ctypes.byref(i), ctypes.byref(o)))
        return g.value, i.value, o.value

    def function(self, signature: "CommandBuffer") -> int:
        """CommandBuffer::function: declares a function with `signature`'s computed signature."""
        f = self._reg(_lib().zs_cmd_function, signature._h)
        if not hasattr(self, "_fn_outputs"):
            self._fn_outputs = {}
        self._fn_outputs[f] = signature.computed_signature()[2]
        return f

    def invoke(self, function: int, generics: Sequence[int] = (), arguments: Sequence[int] = ()) -> List[int]:
        """CommandBuffer::invoke: returns the result registers."""
        sig = self._functions_outputs(function)
        g = (ctypes.c_uint32 * max(len(generics), 1))(*generics)
        a = (ctypes.c_uint32 * max(len(arguments), 1))(*arguments)
        r = (ctypes.c_uint32 * max(sig, 1))()
        _check(_lib().zs_cmd_invoke(self._h, function, g, len(generics), a, len(arguments), r, sig))
        return list(r[:sig])

    def _functions_outputs(self, function: int) -> int:
        outs = getattr(self, "_fn_outputs", {})
        if function not in outs:
            raise ZosimosError(3, "no such function")
        return outs[function]

    def output(self, src: int):
        reg = ctypes.c_uint32()
        d = _CDesc()
        _check(_lib().zs_cmd_output(self._h, src, ctypes.byref(reg), ctypes.byref(d)))
        return reg.value, Descriptor._from_c(d)

    def describe(self, reg: int) -> Descriptor:
        d = _CDesc()
        _check(_lib().zs_cmd_describe(self._h, reg, ctypes.byref(d)))
        return Descriptor._from_c(d)


# ---------------------------------------------------------------- program / executable


class Linker:
    """command.rs Linker (only the included standard library exists here)."""

    @staticmethod
    def from_included() -> "Linker":
        return Linker()

    def compile(self, commands: CommandBuffer) -> "Program":
        h = ctypes.c_void_p()
        _check(_lib().zs_compile(commands._h, ctypes.byref(h)))
        return Program(h)

    def link(self, main: CommandBuffer, tys: Sequence[Descriptor] = (), functions: Sequence[CommandBuffer] = (),
             links: Sequence[Sequence[int]] = ()) -> "Program":
        """Linker::link: links[i] lists, for each function declared in buffer i (0 = main, then
        `functions`), the buffer index (0 = main) that defines it."""
        nt = len(tys)
        ct = (_CDesc * max(nt, 1))(*[d._c() for d in tys])
        fs = (ctypes.c_void_p * max(len(functions), 1))(*[f._h for f in functions])
        rows = [(ctypes.c_uint32 * max(len(l), 1))(*l) for l in links]
        lp = (ctypes.POINTER(ctypes.c_uint32) * max(len(links), 1))(
            *[ctypes.cast(r, ctypes.POINTER(ctypes.c_uint32)) for r in rows])
        lc = (ctypes.c_uint32 * max(len(links), 1))(*[len(l) for l in links])
        h = ctypes.c_void_p()
        _check(_lib().zs_link(main._h, ct, nt, fs, len(functions), lp, lc, len(links), ctypes.byref(h)))
        return Program(h)


class Program:
    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        if getattr(self, "_h", None):
            _lib().zs_program_free(self._h)
            self._h = None

    def lower_to(self, caps: Optional[Capabilities] = None) -> "Executable":
        caps = caps or Capabilities()
        c = _CCaps(caps.device, caps.mode, int(caps.use_graph),
                   (1 if caps.simt_resample else 0) | (0 if caps.zero_copy else 2))
        h = ctypes.c_void_p()
        _check(_lib().zs_lower(self._h, ctypes.byref(c), ctypes.byref(h)))
        return Executable(h)


class Executable:
    """run.rs Executable: a lowered program, reusable across launches."""

    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        if getattr(self, "_h", None):
            _lib().zs_executable_free(self._h)
            self._h = None

    def kernel_count(self) -> int:
        n = ctypes.c_uint32()
        _check(_lib().zs_executable_kernel_count(self._h, ctypes.byref(n)))
        return n.value

    def describe(self) -> str:
        return _lib().zs_executable_describe(self._h).decode()

    def from_pool(self, pool: Pool) -> "Environment":
        h = ctypes.c_void_p()
        _check(_lib().zs_env_new(self._h, pool._h, ctypes.byref(h)))
        return Environment(h, pool, self)

    def launch(self, env: "Environment") -> "Execution":
        h = ctypes.c_void_p()
        envh, env._h = env._h, None          # consumed
        _check(_lib().zs_launch(self._h, envh, ctypes.byref(h)))
        return Execution(h, env.pool)

    def run_host(self, inputs: Sequence[np.ndarray], outputs: Sequence[np.ndarray]) -> None:
        """One launch from host arrays into host arrays (C-contiguous, exact byte sizes)."""
        ins = (ctypes.c_void_p * len(inputs))(*[np.ascontiguousarray(a).ctypes.data for a in inputs])
        outs = (ctypes.c_void_p * len(outputs))(*[a.ctypes.data for a in outputs])
        _check(_lib().zs_run_host(self._h, ins, len(inputs), outs, len(outputs)))

    def batch_thumbnails(self, images: Sequence[int], widths: Sequence[int], heights: Sequence[int], canvas: int,
                         out: int, stream: int = 0) -> None:
        """One persistent launch over many device-resident RGBA8 sRGB images: this
        executable's fused colour chain, box fit-resize to `canvas`, centred on a
        transparent canvas x canvas image; `out` receives n * canvas^2 * 4 bytes."""
        n = len(images)
        ptrs = (ctypes.c_void_p * n)(*images)
        ws = (ctypes.c_uint32 * n)(*widths)
        hs = (ctypes.c_uint32 * n)(*heights)
        _check(_lib().zs_batch_thumbnails(self._h, ptrs, ws, hs, n, canvas, out, stream or None))

    def batch_run_device(self, inputs: Sequence[Sequence[int]], outputs: Sequence[Sequence[int]],
                         stream: int = 0) -> None:
        """zs_batch_run_device: one run per row of device pointers, recorded into one CUDA
        graph (cached per pointer table, replayed when the same table comes again)."""
        n = len(inputs)
        flat_in = [p for row in inputs for p in row]
        flat_out = [p for row in outputs for p in row]
        ins = (ctypes.c_void_p * max(len(flat_in), 1))(*flat_in)
        outs = (ctypes.c_void_p * max(len(flat_out), 1))(*flat_out)
        _check(_lib().zs_batch_run_device(self._h, ins, outs, n, stream or None))

    def batch_run(self, pool: "Pool", keys: Sequence[Sequence[int]]):
        """zs_batch_run: one run per row of pool keys; returns the output keys per run."""
        n = len(keys)
        flat = [k for row in keys for k in row]
        arr = (ctypes.c_uint64 * max(len(flat), 1))(*flat)
        nout = self.output_count()
        out = (ctypes.c_uint64 * max(n * nout, 1))()
        _check(_lib().zs_batch_run(self._h, pool._h, arr, n, out))
        return [list(out[i * nout:(i + 1) * nout]) for i in range(n)]

    def query_knob(self, register: int, link_idx: int = 0):
        """Executable::query_knob: (knob id, byte length of its parameter block)."""
        k, n = ctypes.c_uint32(), ctypes.c_uint64()
        _check(_lib().zs_executable_query_knob(self._h, link_idx, register, ctypes.byref(k), ctypes.byref(n)))
        return k.value, n.value

    def set_knob(self, knob: int, data) -> None:
        """The knob's parameter block for every later launch (one-call paths included)."""
        b = bytes(np.ascontiguousarray(data).view(np.uint8).reshape(-1)) if isinstance(data, np.ndarray) else bytes(data)
        _check(_lib().zs_executable_set_knob(self._h, knob, b, len(b)))

    def autotune(self, inputs: Sequence[int], outputs: Sequence[int], stream: int = 0, reps: int = 10) -> int:
        """zs_autotune on device buffers (which receive the result); returns the chain block size."""
        ins = (ctypes.c_void_p * max(len(inputs), 1))(*inputs)
        outs = (ctypes.c_void_p * max(len(outputs), 1))(*outputs)
        t = ctypes.c_int32()
        _check(_lib().zs_autotune(self._h, ins, len(inputs), outs, len(outputs), stream or None, reps, ctypes.byref(t)))
        return t.value

    def autotune_batch_thumbnails(self, images, widths, heights, canvas: int, out: int, stream: int = 0,
                                  reps: int = 3) -> int:
        """zs_autotune_batch_thumbnails: returns the chosen output rows per work item."""
        n = len(images)
        rows = ctypes.c_uint32()
        _check(_lib().zs_autotune_batch_thumbnails(self._h, (ctypes.c_void_p * n)(*images), (ctypes.c_uint32 * n)(*widths),
                                                   (ctypes.c_uint32 * n)(*heights), n, canvas, out, stream or None,
                                                   reps, ctypes.byref(rows)))
        return rows.value

    def set_launch(self, param: int, value: int) -> None:
        _check(_lib().zs_executable_set_launch(self._h, param, value))

    def get_launch(self, param: int) -> int:
        v = ctypes.c_int32()
        _check(_lib().zs_executable_get_launch(self._h, param, ctypes.byref(v)))
        return v.value

    def tune_key(self, param: int, canvas: int = 0) -> str:
        buf = ctypes.create_string_buffer(512)
        _check(_lib().zs_executable_tune_key(self._h, param, canvas, buf, 512))
        return buf.value.decode()

    def output_count(self) -> int:
        n = ctypes.c_uint32()
        _check(_lib().zs_executable_io_count(self._h, None, ctypes.byref(n)))
        return n.value

    def run_device(self, inputs: Sequence[int], outputs: Sequence[int], stream: int = 0) -> None:
        """One launch on device pointers (no host copies); graph-replayed when enabled."""
        ins = (ctypes.c_void_p * len(inputs))(*inputs)
        outs = (ctypes.c_void_p * len(outputs))(*outputs)
        _check(_lib().zs_run_device(self._h, ins, len(inputs), outs, len(outputs), stream or None))


class Environment:
    """run.rs Environment: bindings of pool images to input / output registers."""

    def __init__(self, handle, pool: Pool, exe: Executable):
        self._h = handle
        self.pool = pool
        self.exe = exe

    def __del__(self):
        if getattr(self, "_h", None):
            _lib().zs_env_free(self._h)
            self._h = None

    def bind(self, reg: int, key: int) -> None:
        _check(_lib().zs_env_bind(self._h, reg, key))

    def bind_output(self, reg: int, key: int) -> None:
        _check(_lib().zs_env_bind_output(self._h, reg, key))

    def recover_buffers(self) -> int:
        """Environment::recover_buffers: bytes of intermediate buffers the executable holds."""
        n = ctypes.c_uint64()
        _check(_lib().zs_env_recover_buffers(self._h, ctypes.byref(n)))
        return n.value

    def knob(self, knob: int, data) -> None:
        """Environment::knob: this launch's parameter block for `knob`."""
        b = bytes(np.ascontiguousarray(data).view(np.uint8).reshape(-1)) if isinstance(data, np.ndarray) else bytes(data)
        _check(_lib().zs_env_knob(self._h, knob, b, len(b)))


class Execution:
    """run.rs Execution + Retire: step-wise execution on one CUDA stream."""

    def __init__(self, handle, pool: Pool):
        self._h = handle
        self.pool = pool

    def __del__(self):
        if getattr(self, "_h", None):
            _lib().zs_exec_free(self._h)
            self._h = None

    def is_running(self) -> bool:
        return bool(_lib().zs_exec_is_running(self._h))

    def step(self) -> None:
        _check(_lib().zs_exec_step(self._h))

    def step_to(self, max_steps: int) -> int:
        """Execution::step_to(StepLimits::new().with_steps(max_steps)): steps enqueued."""
        n = ctypes.c_uint32()
        _check(_lib().zs_exec_step_to(self._h, max_steps, ctypes.byref(n)))
        return n.value

    def sync(self) -> None:
        _check(_lib().zs_exec_sync(self._h))

    def retire_input(self, reg: int) -> int:
        key = ctypes.c_uint64()
        _check(_lib().zs_retire_input(self._h, reg, ctypes.byref(key)))
        return key.value

    def retire_output(self, reg: int) -> int:
        key = ctypes.c_uint64()
        _check(_lib().zs_retire_output(self._h, reg, ctypes.byref(key)))
        return key.value


# ---------------------------------------------------------------- device memory helpers


class DeviceBuffer:
    """A raw device allocation (for device-resident IO with Executable.run_device)."""

    def __init__(self, nbytes: int):
        self.nbytes = nbytes
        self.ptr = _lib().zs_device_alloc(nbytes)
        if not self.ptr:
            raise ZosimosError(11, f"device allocation of {nbytes} bytes failed")

    def upload(self, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        assert a.nbytes == self.nbytes
        _check(_lib().zs_memcpy_h2d(self.ptr, a.ctypes.data, a.nbytes))

    def download(self, out: np.ndarray) -> np.ndarray:
        assert out.nbytes == self.nbytes and out.flags["C_CONTIGUOUS"]
        _check(_lib().zs_memcpy_d2h(out.ctypes.data, self.ptr, out.nbytes))
        return out

    def free(self) -> None:
        if self.ptr:
            _lib().zs_device_free(self.ptr)
            self.ptr = None

    def __del__(self):
        self.free()


class PinnedBuffer:
    """Page-locked, device-mapped host memory (zs_host_alloc) viewed as a numpy array;
    Executable.run_host streams such buffers directly where the plan allows it."""

    def __init__(self, shape, dtype=np.uint8):
        dt = np.dtype(dtype)
        self.nbytes = int(np.prod(shape)) * dt.itemsize
        self.ptr = _lib().zs_host_alloc(self.nbytes)
        if not self.ptr:
            raise ZosimosError(11, f"pinned host allocation of {self.nbytes} bytes failed")
        buf = (ctypes.c_uint8 * self.nbytes).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dt).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            _lib().zs_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        self.free()


def device_synchronize() -> None:
    _check(_lib().zs_device_synchronize())


def _uniform_bytes(data) -> bytes:
    if isinstance(data, np.ndarray):
        return bytes(np.ascontiguousarray(data).view(np.uint8).reshape(-1))
    return bytes(data)


def register_op(image: bytes, kernel_name: str) -> int:
    """zs_register_op: a custom operation's compiled module (PTX text or cubin) and kernel name
    (the analogue of a ShaderCommand's SPIR-V source); returns its op id."""
    data = bytes(image)
    if not data.endswith(b"\0"):
        data += b"\0"          # PTX text must be terminated; a cubin ignores the extra byte
    op = ctypes.c_uint32()
    _check(_lib().zs_register_op(data, len(data), kernel_name.encode(), ctypes.byref(op)))
    return op.value


def tune_cache_get(key: str) -> int:
    v = ctypes.c_int32()
    _check(_lib().zs_tune_cache_get(key.encode(), ctypes.byref(v)))
    return v.value


def tune_cache_put(key: str, value: int) -> None:
    _check(_lib().zs_tune_cache_put(key.encode(), value))


def tune_cache_save(path: str) -> None:
    _check(_lib().zs_tune_cache_save(str(path).encode()))


def tune_cache_load(path: str) -> None:
    _check(_lib().zs_tune_cache_load(str(path).encode()))


def run_executable(exe: Executable, pool: Pool, binds, knobs, outputs):
    """tests/util.rs run_executable_with_output: bind, set this launch's knobs, step to the end,
    retire the outputs into the pool."""
    env = exe.from_pool(pool)
    for reg, key in binds:
        env.bind(reg, key)
    for knob, data in knobs:
        env.knob(knob, data)
    execution = exe.launch(env)
    while execution.is_running():
        execution.step()
    return [execution.retire_output(r) for r in outputs]


def run_pipeline(commands: CommandBuffer, pool: Pool, binds, outputs, caps: Optional[Capabilities] = None):
    """tests/util.rs run_once_with_output: compile, lower, bind, step to the end, retire."""
    exe = Linker.from_included().compile(commands).lower_to(caps)
    env = exe.from_pool(pool)
    for reg, key in binds:
        env.bind(reg, key)
    execution = exe.launch(env)
    while execution.is_running():
        execution.step()
    keys = [execution.retire_output(r) for r in outputs]
    return keys
