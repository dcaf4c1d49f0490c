// zs_device.cuh -- device-side pixel arithmetic of the executor (FP32).
//
// Restates, for sm_103a, the per-texel work the reference does in its staging and
// colour fragment shaders:
//   lib/std/src/stage.frag   transfer functions (:279-425), demux/mux (:533-641),
//                            parts order (:654-747)
//   lib/std/src/oklab.frag, srlab2.frag, linear.frag, inject.frag
// plus the native Rgba8UnormSrgb decode/encode the texture unit / ROP performs
// (lib/zosimos/src/program.rs:794-838), done here with two exact tables.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "zs_shared.h"

// sRGB8 -> linear f32 (correctly rounded from FP64) and the bucketed rounding
// thresholds of linear f32 -> sRGB8 (built by zs_tables.cu, uploaded once per
// device).  Each kernel file is its own translation unit (compiled in parallel, no
// relocatable device code), so every one holds its own copy of these variables;
// ZS_TU_HOOKS at the end of each file exports the host functions that fill its tables
// and read its status word, and zs_tables.cu calls them all.
static __device__ float zs_srgb_decode_lut[256];
static __device__ uint32_t zs_srgb_encode_tab[ZS_ENC_ENTRIES];
static __device__ uint32_t zs_srgb_encode_tab_shifted[ZS_ENCS_ENTRIES];
// Sticky error bits set by kernels whose bounded waits gave up (ZS_DEVSTAT_*); the host
// reads and clears them after synchronising.
static __device__ unsigned int zs_device_status_word;

// The kernel files, one translation unit each (ZS_TU_HOOKS(name) in every one).
#define ZS_DEVICE_TUS(X) X(raster) X(resample) X(resample_tc) X(chain) X(layers) X(batch) X(noalloc) X(selftest)

#define ZS_TU_DECLARE_HOOKS(NAME)                                                                   \
    cudaError_t tu_upload_tables_##NAME(const float *dec, const uint32_t *enc, const uint32_t *encs); \
    cudaError_t tu_device_status_##NAME(unsigned int *flags, bool clear);

// Host functions of this translation unit: upload the sRGB tables into its copies, and
// read (and optionally clear) its status word.  The current device must be selected.
#define ZS_TU_HOOKS(NAME)                                                                            \
    namespace zs {                                                                                   \
    cudaError_t tu_upload_tables_##NAME(const float *dec, const uint32_t *enc, const uint32_t *encs) { \
        cudaError_t e = cudaMemcpyToSymbol(zs_srgb_decode_lut, dec, sizeof(zs_srgb_decode_lut));     \
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(zs_srgb_encode_tab, enc, sizeof(zs_srgb_encode_tab)); \
        if (e == cudaSuccess)                                                                        \
            e = cudaMemcpyToSymbol(zs_srgb_encode_tab_shifted, encs, sizeof(zs_srgb_encode_tab_shifted)); \
        return e;                                                                                    \
    }                                                                                                \
    cudaError_t tu_device_status_##NAME(unsigned int *flags, bool clear) {                          \
        unsigned int v = 0;                                                                          \
        cudaError_t e = cudaMemcpyFromSymbol(&v, zs_device_status_word, sizeof(v));                  \
        if (e == cudaSuccess && clear && v) {                                                        \
            const unsigned int zero = 0;                                                             \
            e = cudaMemcpyToSymbol(zs_device_status_word, &zero, sizeof(zero));                      \
        }                                                                                            \
        *flags = v;                                                                                  \
        return e;                                                                                    \
    }                                                                                                \
    }

// ---------------------------------------------------------------- transfer functions

__device__ __forceinline__ float zs_oe_bt709(float v) {
    return v >= 0.018f ? 1.099f * powf(v, 0.45f) - 0.099f : 4.5f * v;
}
__device__ __forceinline__ float zs_eo_bt709(float v) {
    return v >= 0.081247944f ? powf((v + 0.099f) / 1.099f, 1.0f / 0.45f) : v / 4.5f;  // threshold = oe(0.018)
}
__device__ __forceinline__ float zs_oe_srgb(float v) {
    if (v < -0.0031308f) return -1.055f * powf(-v, 1.0f / 2.4f) + 0.055f;
    if (v <= 0.0031308f) return v * 12.92f;
    return 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ float zs_eo_srgb(float v) {
    if (v < -0.04045f) return -powf((-v + 0.055f) / 1.055f, 2.4f);
    if (v <= 0.04045f) return v / 12.92f;
    return powf((v + 0.055f) / 1.055f, 2.4f);
}
__device__ __forceinline__ float zs_eo_pq(float v) {
    const float m1 = 2610.0f / 16384.0f, m2 = 2523.0f / 4096.0f, c1 = 3424.0f / 4096.0f,
                c2 = 2413.0f / 128.0f, c3 = 2392.0f / 128.0f;
    float n = powf(v, 1.0f / m2);
    float num = fmaxf(n - c1, 0.0f);
    return powf(num / (c2 - c3 * n), 1.0f / m1);
}
__device__ __forceinline__ float zs_oe_pq(float v) {
    const float m1 = 2610.0f / 16384.0f, m2 = 2523.0f / 4096.0f, c1 = 3424.0f / 4096.0f,
                c2 = 2413.0f / 128.0f, c3 = 2392.0f / 128.0f;
    float e = zs_oe_bt709(59.5208f * v);
    float y = powf(powf(e, 2.4f) / 100.0f, m1);
    return powf((c1 + c2 * y) / (c3 * y + 1.0f), m2);
}

// parts_transfer / parts_untransfer on one channel (stage.frag:750-809).  BT.601
// reuses BT.709 with the directions swapped exactly as the reference does.
__device__ __forceinline__ float zs_oe(uint32_t t, float v) {
    switch (t) {
    case 0: return zs_oe_bt709(v);
    case 1: return powf(v, 1.0f / 2.2f);
    case 2: return zs_eo_bt709(v);
    case 3: return v < 0.0228f ? 4.0f * v : 1.1115f * powf(v, 0.45f) - 0.1115f;
    case 5: return zs_oe_srgb(v);
    case 6: case 7: return zs_oe_bt709(v);
    case 8: return zs_oe_pq(v);
    default: return v;
    }
}
__device__ __forceinline__ float zs_eo(uint32_t t, float v) {
    switch (t) {
    case 0: return zs_eo_bt709(v);
    case 1: return powf(v, 2.2f);
    case 2: return zs_oe_bt709(v);
    case 3: return v < 0.0913f ? v / 4.0f : powf((v - 0.1115f) / 1.1115f, 1.0f / 0.45f);
    case 5: return zs_eo_srgb(v);
    case 6: case 7: return zs_eo_bt709(v);
    case 8: return zs_eo_pq(v);
    default: return v;
    }
}

__device__ __forceinline__ void zs_lab_to_lch(float4 &c) {   // stage.frag:415-420
    const float pi = 3.14159265358979323846f;
    float ch = sqrtf(c.y * c.y + c.z * c.z);
    float h = (atan2f(c.z, c.y) * 180.0f / pi) / 360.0f + 0.5f;
    c.y = ch;
    c.z = h;
}
__device__ __forceinline__ void zs_lch_to_lab(float4 &c) {   // stage.frag:422-425
    const float pi = 3.14159265358979323846f;
    float angle = (360.0f * (c.z - 0.5f)) * pi / 180.0f;
    float ch = c.y;
    c.y = ch * cosf(angle);
    c.z = ch * sinf(angle);
}

__device__ __forceinline__ void zs_untransfer4(float4 &c, uint32_t t) {
    if (t == 0x100u) { zs_lch_to_lab(c); return; }
    if (t == 4u || t == 11u || t == 10u || t == 9u) return;
    c.x = zs_eo(t, c.x); c.y = zs_eo(t, c.y); c.z = zs_eo(t, c.z);
}
__device__ __forceinline__ void zs_transfer4(float4 &c, uint32_t t) {
    if (t == 0x100u) { zs_lab_to_lch(c); return; }
    if (t == 4u || t == 11u || t == 10u || t == 9u) return;
    c.x = zs_oe(t, c.x); c.y = zs_oe(t, c.y); c.z = zs_oe(t, c.z);
}

// ---------------------------------------------------------------- demux / mux

__device__ __forceinline__ float zs_u(uint32_t v, float maxv) { return (float)v / maxv; }

__device__ inline float4 zs_demux(uint32_t n, uint32_t bits) {   // stage.frag:533-582
    switch (bits) {
    case 0: { float x = zs_u(n, 255.0f); return make_float4(x, x, x, x); }
    case 1: return make_float4(zs_u(n & 3, 3.f), zs_u((n >> 2) & 7, 7.f), zs_u(n >> 5, 7.f), 1.f);
    case 2: return make_float4(zs_u(n & 7, 7.f), zs_u((n >> 3) & 7, 7.f), zs_u(n >> 6, 3.f), 1.f);
    case 3: { float x = zs_u(n, 65535.0f); return make_float4(x, x, x, x); }
    case 4: return make_float4(zs_u(n & 15, 15.f), zs_u((n >> 4) & 15, 15.f), zs_u((n >> 8) & 15, 15.f),
                               zs_u(n >> 12, 15.f));
    case 5: return make_float4(zs_u(n & 15, 15.f), zs_u((n >> 4) & 15, 15.f), zs_u((n >> 8) & 15, 15.f), 1.f);
    case 6: return make_float4(zs_u((n >> 4) & 15, 15.f), zs_u((n >> 8) & 15, 15.f),
                               zs_u((n >> 12) & 15, 15.f), 1.f);
    case 7: return make_float4(zs_u(n & 31, 31.f), zs_u((n >> 5) & 63, 63.f), zs_u(n >> 11, 31.f), 1.f);
    case 8: return make_float4(zs_u(n & 255, 255.f), 0.f, 0.f, zs_u((n >> 8) & 255, 255.f));
    case 9: return make_float4(zs_u(n & 255, 255.f), zs_u((n >> 8) & 255, 255.f),
                               zs_u((n >> 16) & 255, 255.f), 1.f);
    case 10: return make_float4(zs_u(n & 255, 255.f), zs_u((n >> 8) & 255, 255.f),
                                zs_u((n >> 16) & 255, 255.f), zs_u(n >> 24, 255.f));
    case 11: return make_float4(zs_u(n & 65535, 65535.f), zs_u(n >> 16, 65535.f), 0.f, 1.f);
    case 14: return make_float4(zs_u(n & 3, 3.f), zs_u((n >> 2) & 1023, 1023.f),
                                zs_u((n >> 12) & 1023, 1023.f), zs_u(n >> 22, 1023.f));
    case 15: return make_float4(zs_u(n & 1023, 1023.f), zs_u((n >> 10) & 1023, 1023.f),
                                zs_u((n >> 20) & 1023, 1023.f), zs_u(n >> 30, 3.f));
    case 16: return make_float4(zs_u((n >> 2) & 1023, 1023.f), zs_u((n >> 12) & 1023, 1023.f),
                                zs_u(n >> 22, 1023.f), 1.f);
    case 17: return make_float4(zs_u(n & 1023, 1023.f), zs_u((n >> 10) & 1023, 1023.f),
                                zs_u((n >> 20) & 1023, 1023.f), 1.f);
    default: return make_float4(1.f, 0.f, 0.f, 1.f);             // BIT_DECODE_FAIL
    }
}

__device__ __forceinline__ uint32_t zs_q(float v, float maxv) { return (uint32_t)(v * maxv); }

__device__ inline uint32_t zs_mux(float4 c, uint32_t bits) {   // stage.frag:590-641
    switch (bits) {
    case 0: return zs_q(c.x, 255.f);
    case 1: return zs_q(c.x, 3.f) + (zs_q(c.y, 7.f) << 2) + (zs_q(c.z, 7.f) << 5);
    case 2: return zs_q(c.x, 7.f) + (zs_q(c.y, 7.f) << 3) + (zs_q(c.z, 3.f) << 6);
    case 3: return zs_q(c.x, 65535.f);
    case 4: return zs_q(c.x, 15.f) + (zs_q(c.y, 15.f) << 4) + (zs_q(c.z, 15.f) << 8) + (zs_q(c.w, 15.f) << 12);
    case 5: return zs_q(c.x, 15.f) + (zs_q(c.y, 15.f) << 4) + (zs_q(c.z, 15.f) << 8);
    case 6: return (zs_q(c.x, 15.f) << 4) + (zs_q(c.y, 15.f) << 8) + (zs_q(c.z, 15.f) << 12);
    case 7: return zs_q(c.x, 31.f) + (zs_q(c.y, 63.f) << 5) + (zs_q(c.z, 31.f) << 11);
    case 8: return zs_q(c.x, 255.f) + (zs_q(c.w, 255.f) << 8);
    case 9: return zs_q(c.x, 255.f) + (zs_q(c.y, 255.f) << 8) + (zs_q(c.z, 255.f) << 16);
    case 10: return zs_q(c.x, 255.f) + (zs_q(c.y, 255.f) << 8) + (zs_q(c.z, 255.f) << 16) + (zs_q(c.w, 255.f) << 24);
    case 11: return zs_q(c.x, 65535.f) + (zs_q(c.w, 65535.f) << 16);
    case 14: return zs_q(c.x, 3.f) + (zs_q(c.y, 1023.f) << 2) + (zs_q(c.z, 1023.f) << 12) + (zs_q(c.w, 1023.f) << 22);
    case 15: return zs_q(c.x, 1023.f) + (zs_q(c.y, 1023.f) << 10) + (zs_q(c.z, 1023.f) << 20) + (zs_q(c.w, 3.f) << 30);
    case 16: return (zs_q(c.x, 1023.f) << 2) + (zs_q(c.y, 1023.f) << 12) + (zs_q(c.z, 1023.f) << 22);
    case 17: return zs_q(c.x, 1023.f) + (zs_q(c.y, 1023.f) << 10) + (zs_q(c.z, 1023.f) << 20);
    default: return 0x55445544u;                                   // BIT_ENCODE_FAIL
    }
}

// parts_normalize (stage.frag:654-699).  BgrA is reordered (the shader leaves it as is).
__device__ inline float4 zs_parts_normalize(float4 c, uint32_t parts) {
    switch (parts) {
    case 0: return make_float4(0.f, 0.f, 0.f, c.x);
    case 1: return make_float4(c.x, 0.f, 0.f, 1.f);
    case 2: return make_float4(0.f, c.x, 0.f, 1.f);
    case 3: return make_float4(0.f, 0.f, c.x, 1.f);
    case 4: return make_float4(c.x, c.x, c.x, 1.f);
    case 5: return make_float4(c.x, c.x, c.x, c.w);
    case 6: case 9: case 17: case 19: return make_float4(c.x, c.y, c.z, 1.f);
    case 7: case 11: return make_float4(c.z, c.y, c.x, 1.f);
    case 10: return make_float4(c.z, c.y, c.x, c.w);
    case 12: return make_float4(c.y, c.z, c.w, c.x);
    case 13: return make_float4(c.y, c.z, c.w, 1.f);
    case 14: return make_float4(c.w, c.z, c.y, c.x);
    case 15: return make_float4(c.w, c.z, c.y, 1.f);
    default: return c;
    }
}

// parts_denormalize (stage.frag:703-747).
__device__ inline float4 zs_parts_denormalize(float4 c, uint32_t parts) {
    switch (parts) {
    case 0: return make_float4(c.w, 0.f, 0.f, 1.f);
    case 1: return make_float4(c.x, 0.f, 0.f, 1.f);
    case 2: return make_float4(c.y, 0.f, 0.f, 1.f);
    case 3: return make_float4(c.z, 0.f, 0.f, 1.f);
    case 4: return make_float4(c.x, c.x, c.x, 1.f);
    case 5: return make_float4(c.x, c.x, c.x, c.w);
    case 6: case 9: case 17: case 19: return make_float4(c.x, c.y, c.z, 1.f);
    case 7: case 11: return make_float4(c.z, c.y, c.x, 1.f);
    case 10: return make_float4(c.z, c.y, c.x, c.w);
    case 12: return make_float4(c.w, c.x, c.y, c.z);
    case 13: return make_float4(1.f, c.x, c.y, c.z);
    case 14: return make_float4(c.w, c.z, c.y, c.x);
    case 15: return make_float4(1.f, c.z, c.y, c.x);
    default: return c;
    }
}

// ---------------------------------------------------------------- sRGB8 tables

__device__ __forceinline__ uint32_t zs_enc_srgb8(const uint32_t *tab, float x) {
    // Exact round-to-nearest sRGB8 encode of x (clamped to [0, 1]): the table entry of
    // the bucket (float bits >> 16) folds the code at the bucket start, the rounding
    // threshold inside the bucket and the bucket base, so that (entry + bits) >> 24
    // is the code.
    uint32_t b = __float_as_uint(__saturatef(x));
    b = max(b, ZS_ENC_BASE << 16);
    return (tab[(b >> 16) - ZS_ENC_BASE] + b) >> 24;
}

__device__ __forceinline__ uint32_t zs_unorm8(float x) { return __float2uint_rn(__saturatef(x) * 255.0f); }

// ---------------------------------------------------------------- raw texel IO

__device__ __forceinline__ uint4 zs_load_raw(const uint8_t *p, uint32_t bpp) {
    uint4 r = make_uint4(0, 0, 0, 0);
    switch (bpp) {
    case 1: r.x = p[0]; break;
    case 2: r.x = *(const uint16_t *)p; break;
    case 3: r.x = p[0] | (p[1] << 8) | (p[2] << 16); break;
    case 4: r.x = *(const uint32_t *)p; break;
    case 6: r.x = *(const uint16_t *)p | ((uint32_t) * (const uint16_t *)(p + 2) << 16);
            r.y = *(const uint16_t *)(p + 4); break;
    case 8: { uint2 v = *(const uint2 *)p; r.x = v.x; r.y = v.y; } break;
    case 16: r = *(const uint4 *)p; break;
    default: break;
    }
    return r;
}

__device__ __forceinline__ void zs_store_raw(uint8_t *p, uint32_t bpp, uint4 r) {
    switch (bpp) {
    case 1: p[0] = (uint8_t)r.x; break;
    case 2: *(uint16_t *)p = (uint16_t)r.x; break;
    case 3: p[0] = (uint8_t)r.x; p[1] = (uint8_t)(r.x >> 8); p[2] = (uint8_t)(r.x >> 16); break;
    case 4: *(uint32_t *)p = r.x; break;
    case 6: *(uint16_t *)p = (uint16_t)r.x; *(uint16_t *)(p + 2) = (uint16_t)(r.x >> 16);
            *(uint16_t *)(p + 4) = (uint16_t)r.y; break;
    case 8: *(uint2 *)p = make_uint2(r.x, r.y); break;
    case 16: *(uint4 *)p = r; break;
    default: break;
    }
}

__device__ __forceinline__ float zs_h2f(uint32_t h) { return __half2float(__ushort_as_half((unsigned short)h)); }
__device__ __forceinline__ uint32_t zs_f2h(float f) { return __half_as_ushort(__float2half_rn(f)); }

// Raw texel bytes -> linear value (the value the reference's shaders see).
__device__ inline float4 zs_decode_raw(const ZsFormat &f, uint4 r) {
    switch (f.fast) {
    case ZS_FAST_RGBA8_SRGB:
        return make_float4(zs_srgb_decode_lut[r.x & 255], zs_srgb_decode_lut[(r.x >> 8) & 255],
                           zs_srgb_decode_lut[(r.x >> 16) & 255], (float)(r.x >> 24) / 255.0f);
    case ZS_FAST_BGRA8_SRGB:
        return make_float4(zs_srgb_decode_lut[(r.x >> 16) & 255], zs_srgb_decode_lut[(r.x >> 8) & 255],
                           zs_srgb_decode_lut[r.x & 255], (float)(r.x >> 24) / 255.0f);
    case ZS_FAST_RGBA8_UNORM:
        return make_float4((float)(r.x & 255) / 255.0f, (float)((r.x >> 8) & 255) / 255.0f,
                           (float)((r.x >> 16) & 255) / 255.0f, (float)(r.x >> 24) / 255.0f);
    case ZS_FAST_BGRA8_UNORM:
        return make_float4((float)((r.x >> 16) & 255) / 255.0f, (float)((r.x >> 8) & 255) / 255.0f,
                           (float)(r.x & 255) / 255.0f, (float)(r.x >> 24) / 255.0f);
    case ZS_FAST_F16X4:
        return make_float4(zs_h2f(r.x & 0xffff), zs_h2f(r.x >> 16), zs_h2f(r.y & 0xffff), zs_h2f(r.y >> 16));
    case ZS_FAST_F32X4:
        return make_float4(__uint_as_float(r.x), __uint_as_float(r.y), __uint_as_float(r.z), __uint_as_float(r.w));
    default: break;
    }
    float4 c;
    if (f.bits == 13) {
        c = make_float4((float)(r.x & 0xffff) / 65535.0f, (float)(r.x >> 16) / 65535.0f,
                        (float)(r.y & 0xffff) / 65535.0f, (float)(r.y >> 16) / 65535.0f);
    } else if (f.bits == 18) {
        c = make_float4(zs_h2f(r.x & 0xffff), zs_h2f(r.x >> 16), zs_h2f(r.y & 0xffff), zs_h2f(r.y >> 16));
    } else if (f.bits == 19) {
        c = make_float4(__uint_as_float(r.x), __uint_as_float(r.y), __uint_as_float(r.z), __uint_as_float(r.w));
    } else {
        c = zs_demux(r.x, f.bits);
    }
    c = zs_parts_normalize(c, f.parts);
    zs_untransfer4(c, f.transfer);
    return c;
}

__device__ __forceinline__ float zs_clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// Linear value -> raw texel bytes.
__device__ inline uint4 zs_encode_raw(const ZsFormat &f, float4 c) {
    uint4 r = make_uint4(0, 0, 0, 0);
    switch (f.fast) {
    case ZS_FAST_RGBA8_SRGB:
        r.x = zs_enc_srgb8(zs_srgb_encode_tab, c.x) | (zs_enc_srgb8(zs_srgb_encode_tab, c.y) << 8) |
              (zs_enc_srgb8(zs_srgb_encode_tab, c.z) << 16) | (zs_unorm8(c.w) << 24);
        return r;
    case ZS_FAST_BGRA8_SRGB:
        r.x = zs_enc_srgb8(zs_srgb_encode_tab, c.z) | (zs_enc_srgb8(zs_srgb_encode_tab, c.y) << 8) |
              (zs_enc_srgb8(zs_srgb_encode_tab, c.x) << 16) | (zs_unorm8(c.w) << 24);
        return r;
    case ZS_FAST_RGBA8_UNORM:
        r.x = zs_unorm8(c.x) | (zs_unorm8(c.y) << 8) | (zs_unorm8(c.z) << 16) | (zs_unorm8(c.w) << 24);
        return r;
    case ZS_FAST_BGRA8_UNORM:
        r.x = zs_unorm8(c.z) | (zs_unorm8(c.y) << 8) | (zs_unorm8(c.x) << 16) | (zs_unorm8(c.w) << 24);
        return r;
    case ZS_FAST_F16X4:
        r.x = zs_f2h(c.x) | (zs_f2h(c.y) << 16);
        r.y = zs_f2h(c.z) | (zs_f2h(c.w) << 16);
        return r;
    case ZS_FAST_F32X4:
        return make_uint4(__float_as_uint(c.x), __float_as_uint(c.y), __float_as_uint(c.z), __float_as_uint(c.w));
    default: break;
    }
    zs_transfer4(c, f.transfer);
    c = zs_parts_denormalize(c, f.parts);
    if (f.bits == 18) {
        r.x = zs_f2h(c.x) | (zs_f2h(c.y) << 16);
        r.y = zs_f2h(c.z) | (zs_f2h(c.w) << 16);
        return r;
    }
    if (f.bits == 19) {
        return make_uint4(__float_as_uint(c.x), __float_as_uint(c.y), __float_as_uint(c.z), __float_as_uint(c.w));
    }
    c = make_float4(zs_clamp01(c.x), zs_clamp01(c.y), zs_clamp01(c.z), zs_clamp01(c.w));
    if (f.native) {
        r.x = zs_unorm8(c.x) | (zs_unorm8(c.y) << 8) | (zs_unorm8(c.z) << 16) | (zs_unorm8(c.w) << 24);
        return r;
    }
    if (f.bits == 13) {
        r.x = zs_q(c.x, 65535.f) | (zs_q(c.y, 65535.f) << 16);
        r.y = zs_q(c.z, 65535.f) | (zs_q(c.w, 65535.f) << 16);
        return r;
    }
    r.x = zs_mux(c, f.bits);
    return r;
}

// One RGBA16F texel (8 bytes) as FP32.
__device__ __forceinline__ float4 zs_h4(uint2 v) {
    const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&v.x));
    const float2 hi = __half22float2(*reinterpret_cast<const __half2 *>(&v.y));
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

__device__ __forceinline__ float4 zs_load_px(const ZsSource &s, int x, int y) {
    const uint8_t *p = s.ptr + (int64_t)y * s.stride + (int64_t)x * s.fmt.bpp;
    return zs_decode_raw(s.fmt, zs_load_raw(p, s.fmt.bpp));
}

// ---------------------------------------------------------------- pixel program

__device__ __forceinline__ float zs_scbrt(float v) {
    // sign(v) * |v|^(1/3) through the hardware base-2 log / exp (relative error ~1e-6).
    float r = exp2f(__log2f(fabsf(v)) * (1.0f / 3.0f));
    return copysignf(r, v);
}

__device__ __forceinline__ void zs_mat3(const float *m, float4 &c) {
    float x = c.x, y = c.y, z = c.z;
    c.x = fmaf(m[0], x, fmaf(m[1], y, m[2] * z));
    c.y = fmaf(m[3], x, fmaf(m[4], y, m[5] * z));
    c.z = fmaf(m[6], x, fmaf(m[7], y, m[8] * z));
}

__device__ __forceinline__ float zs_srl_nl(float v) {
    if (fabsf(v) < 216.0f / 24389.0f) return v * 24389.0f / 2700.0f;
    return 1.16f * powf(v, 1.0f / 3.0f) - 0.16f;
}
__device__ __forceinline__ float zs_srl_nlinv(float v) {
    if (fabsf(v) < 0.08f) return v * 2700.0f / 24389.0f;
    float vp = (v + 0.16f) / 1.16f;
    return vp * vp * vp;
}

__device__ inline void zs_blend_px(float4 &b, float4 s, uint32_t mode, uint32_t straight) {
    float ab = b.w, as = s.w;
    if (straight) {
        b.x *= ab; b.y *= ab; b.z *= ab;
        s.x *= as; s.y *= as; s.z *= as;
    }
    float ao;
    switch (mode) {
    case 1:
        b.x = s.x * (1.f - ab) + b.x * (1.f - as) + s.x * b.x;
        b.y = s.y * (1.f - ab) + b.y * (1.f - as) + s.y * b.y;
        b.z = s.z * (1.f - ab) + b.z * (1.f - as) + s.z * b.z;
        ao = as + ab * (1.f - as);
        break;
    case 2:
        b.x = s.x + b.x - s.x * b.x;
        b.y = s.y + b.y - s.y * b.y;
        b.z = s.z + b.z - s.z * b.z;
        ao = as + ab * (1.f - as);
        break;
    case 3:
        b.x = fminf(s.x + b.x, 1.f);
        b.y = fminf(s.y + b.y, 1.f);
        b.z = fminf(s.z + b.z, 1.f);
        ao = fminf(as + ab, 1.f);
        break;
    default:
        b.x = s.x + b.x * (1.f - as);
        b.y = s.y + b.y * (1.f - as);
        b.z = s.z + b.z * (1.f - as);
        ao = as + ab * (1.f - as);
        break;
    }
    b.w = ao;
    if (straight) {
        if (ao > 0.f) { b.x /= ao; b.y /= ao; b.z /= ao; }
        else { b.x = 0.f; b.y = 0.f; b.z = 0.f; }
    }
}

__device__ inline void zs_run_program(const ZsPixelProgram &P, const ZsFormat *fmts, float4 &r, float4 &r2) {
    for (int i = 0; i < P.n; ++i) {
        const ZsPInstr I = P.ins[i];
        const float *m = P.prm + I.p;
        switch (I.op) {
        case ZS_P_MAT3: zs_mat3(m, r); break;
        case ZS_P_CBRT: r.x = zs_scbrt(r.x); r.y = zs_scbrt(r.y); r.z = zs_scbrt(r.z); break;
        case ZS_P_CUBE: r.x = r.x * r.x * r.x; r.y = r.y * r.y * r.y; r.z = r.z * r.z * r.z; break;
        case ZS_P_CLAMP01: r.x = zs_clamp01(r.x); r.y = zs_clamp01(r.y); r.z = zs_clamp01(r.z); break;
        case ZS_P_SRL_NL: r.x = zs_srl_nl(r.x); r.y = zs_srl_nl(r.y); r.z = zs_srl_nl(r.z); break;
        case ZS_P_SRL_NLINV: r.x = zs_srl_nlinv(r.x); r.y = zs_srl_nlinv(r.y); r.z = zs_srl_nlinv(r.z); break;
        case ZS_P_SRL_ENC_DIFF: {
            float x = r.x, y = r.y, z = r.z;
            r.x = y;
            r.y = (x - y) * 5.0f / 1.16f;
            r.z = (z - y) * 2.0f / 1.16f;
        } break;
        case ZS_P_SRL_DEC_DIFF: {
            float L = r.x, a = r.y, b = r.z;
            r.x = a * 1.16f / 5.0f + L;
            r.y = L;
            r.z = b * 1.16f / 2.0f + L;
        } break;
        case ZS_P_QUANT: r = zs_decode_raw(fmts[I.a], zs_encode_raw(fmts[I.a], r)); break;
        case ZS_P_TRANSMUTE: r = zs_decode_raw(fmts[I.b], zs_encode_raw(fmts[I.a], r)); break;
        case ZS_P_INJECT: {
            float d = r2.x * m[4] + r2.y * m[5] + r2.z * m[6] + r2.w * m[7];
            r.x = r.x * (1.f - m[0]) + d * m[0];
            r.y = r.y * (1.f - m[1]) + d * m[1];
            r.z = r.z * (1.f - m[2]) + d * m[2];
            r.w = r.w * (1.f - m[3]) + d * m[3];
        } break;
        case ZS_P_BLEND: zs_blend_px(r, r2, I.a, I.b); break;
        case ZS_P_MOV2: r2 = r; break;
        case ZS_P_SWAP: { float4 t = r; r = r2; r2 = t; } break;
        case ZS_P_PREMUL: r.x *= r.w; r.y *= r.w; r.z *= r.w; break;
        case ZS_P_UNPREMUL:
            if (r.w > 0.f) { r.x /= r.w; r.y /= r.w; r.z /= r.w; } else { r.x = 0.f; r.y = 0.f; r.z = 0.f; }
            break;
        default: break;
        }
    }
}

// ---------------------------------------------------------------- geometry (raster and layer kernels)

__device__ __forceinline__ int zs_quad_src(int p, int t0, int t1, int s0, int s1) {
    // floor(s0 + (p - t0 + 0.5) * (s1 - s0) / (t1 - t0)) in exact integer arithmetic.
    long long num = (2LL * (p - t0) + 1) * (long long)(s1 - s0);
    return s0 + (int)(num / (2LL * (t1 - t0)));
}

__device__ __forceinline__ void zs_affine_map(const float *inv, int x, int y, float &qx, float &qy) {
    float cx = (float)x + 0.5f, cy = (float)y + 0.5f;
    float X = fmaf(inv[0], cx, fmaf(inv[1], cy, inv[2]));
    float Y = fmaf(inv[3], cx, fmaf(inv[4], cy, inv[5]));
    float Z = fmaf(inv[6], cx, fmaf(inv[7], cy, inv[8]));
    if (Z != 1.0f) { X = __fdiv_rn(X, Z); Y = __fdiv_rn(Y, Z); }
    qx = X;
    qy = Y;
}

// Pixel of work item i in 32 x 8 tiles of 256 items: warp w of the tile covers columns
// 8 (w % 4) .. +8 and rows 4 (w / 4) .. +4, lane l column l % 8 and row l / 8.
__device__ __forceinline__ void zs_tile_pixel(int64_t i, int tiles_x, int &x, int &y) {
    const int64_t tile = i >> 8;
    const int t = (int)(i & 255), w = t >> 5, l = t & 31;
    const int ty = (int)(tile / tiles_x), tx = (int)(tile - (int64_t)ty * tiles_x);
    x = (tx << 5) + ((w & 3) << 3) + (l & 7);
    y = (ty << 3) + ((w >> 2) << 2) + (l >> 3);
}

__device__ __forceinline__ int zs_clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// The common ending of the RGBA16F kernels: no pixel program after the producer and an RGBA16F
// destination, stored as one 8-byte texel with two packing conversions (the bits zs_encode_raw
// gives for ZS_FAST_F16X4, without its format dispatch).
__device__ __forceinline__ bool zs_plain_f16_out(const ZsPixelProgram &P, const ZsFormat &f) {
    return P.n == 0 && f.fast == ZS_FAST_F16X4;
}
__device__ __forceinline__ void zs_store_f16x4(uint8_t *p, float4 c) {
    const __half2 lo = __floats2half2_rn(c.x, c.y), hi = __floats2half2_rn(c.z, c.w);
    *(uint2 *)p = make_uint2(*reinterpret_cast<const uint32_t *>(&lo), *reinterpret_cast<const uint32_t *>(&hi));
}

__device__ __forceinline__ float4 zs_lerp4(float4 a, float4 b, float t) {
    return make_float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t,
                       a.w + (b.w - a.w) * t);
}
