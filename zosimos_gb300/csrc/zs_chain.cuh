// zs_chain.cuh -- pixel-pair arithmetic of the fused colour chain (FP32x2), shared by
// the chain kernel (k_chain.cu) and the batched thumbnail kernel (k_batch.cu).
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "zs_shared.h"

// Lane copies of each sRGB encode bucket in shared memory (lane & 7 reads copy lane & 7):
// at most 4 lanes share a copy, so a warp's 32 random bucket lookups rarely conflict.
#define ZS_ENC_REP 8

__device__ __forceinline__ float zs_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float zs_lg2(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

template <bool NONNEG>
__device__ __forceinline__ float zs_cbrt1(float x) {
    if (NONNEG) return zs_ex2(zs_lg2(x) * (1.0f / 3.0f));
    return copysignf(zs_ex2(zs_lg2(fabsf(x)) * (1.0f / 3.0f)), x);
}

// saturate(x) as a saturating add on the FMA pipe (the ALU pipe is the busier one).
__device__ __forceinline__ float zs_sat(float x) {
    float y;
    asm("add.rn.sat.f32 %0, %1, 0f00000000;" : "=f"(y) : "f"(x));
    return y;
}

// saturate(a * b + c) in one FMA-pipe instruction.
__device__ __forceinline__ float zs_fma_sat(float a, float b, float c) {
    float y;
    asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(a), "f"(b), "f"(c));
    return y;
}

// rgb' = M rgb on a pixel pair; SAT saturates the results to [0, 1] in the last FMA of
// each row (scalar fma.sat: the packed FP32x2 FMA has no saturating form).
template <bool SAT>
__device__ __forceinline__ float2 zs_row2(const float2 *c, float2 x, float2 y, float2 z) {
    const float2 t = __ffma2_rn(c[1], y, __fmul2_rn(c[2], z));
    if (SAT) return make_float2(zs_fma_sat(c[0].x, x.x, t.x), zs_fma_sat(c[0].y, x.y, t.y));
    return __ffma2_rn(c[0], x, t);
}

template <bool SAT>
__device__ __forceinline__ void zs_m3x2(const float (*m)[2], float2 &r, float2 &g, float2 &b) {
    const float2 *c = reinterpret_cast<const float2 *>(m);
    const float2 x = r, y = g, z = b;
    r = zs_row2<SAT>(c, x, y, z);
    g = zs_row2<SAT>(c + 3, x, y, z);
    b = zs_row2<SAT>(c + 6, x, y, z);
}

// xs = x + 2^-12 for x in [0, 1] -> table entry + bits of xs; the sRGB8 code is byte 3
// of the result.  The shift (added to a pixel pair by one packed add) keeps the argument
// inside the table without an integer clamp.  `ebase` is the 32-bit shared address of this
// lane's copy of bucket 0 minus ZS_ENCS_BASE buckets, so the lookup is one shift, one
// shift-add, one shared load and one add.
__device__ __forceinline__ uint32_t zs_enc_q(uint32_t ebase, float xs) {
    static_assert(ZS_ENC_REP == 8, "32-byte buckets");
    const uint32_t b = __float_as_uint(xs);
    uint32_t e;
    asm("{\n\t.reg .u32 t, a;\n\t"
        "shr.u32 t, %1, 16;\n\t"
        "shl.b32 t, t, 5;\n\t"
        "add.u32 a, t, %2;\n\t"
        "ld.shared.u32 %0, [a];\n\t}"
        : "=r"(e)
        : "r"(b), "r"(ebase));
    return e + b;
}

// Shared address base for zs_enc_q: copy (lane & 7) of the replicated table at `enc`.
__device__ __forceinline__ uint32_t zs_enc_base(const uint32_t *enc, int lane) {
    return (uint32_t)__cvta_generic_to_shared(enc + (lane & (ZS_ENC_REP - 1))) - ZS_ENCS_BASE * ZS_ENC_REP * 4u;
}

// Decoded value of byte K of texel w for this lane: (code << 8) | (lane << 2) is the
// byte offset of the lane-replicated table entry, built by one byte permute.
template <int K>
__device__ __forceinline__ float zs_dec(const unsigned char *lut, uint32_t w, uint32_t lane4) {
    const uint32_t off = __byte_perm(w, lane4, 0x5504u | (K << 4));
    return *reinterpret_cast<const float *>(lut + off);
}

// The same lookup when the table sits at shared address ZS_DEC_ABS (64 KiB aligned): the
// PRMT also copies the table's address bits (bytes 2 and 3 of lane4abs = ZS_DEC_ABS | lane
// << 2), so its result is the shared address itself and the load needs no add.
#define ZS_DEC_ABS 0x10000u
template <int K>
__device__ __forceinline__ float zs_dec_abs(uint32_t w, uint32_t lane4abs) {
    const uint32_t addr = __byte_perm(w, lane4abs, 0x7604u | (K << 4));
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

__device__ __forceinline__ void zs_cbrt2(float2 &v) {
    // NONNEG: both arguments are >= 0 (the MUFU log of 0 is -inf, its exp2 is 0).
    float2 l = make_float2(zs_lg2(v.x), zs_lg2(v.y));
    l = __fmul2_rn(l, make_float2(1.0f / 3.0f, 1.0f / 3.0f));
    v = make_float2(zs_ex2(l.x), zs_ex2(l.y));
}
