// k_batch.cu -- many RGBA8 sRGB images of uneven sizes turned into thumbnails by one
// launch over a static work list (the reference's batch-reuse case runs one Executable per
// image, lib/zosimos/tests/loop.rs:84-95).
//
// Per image: decode -> the fused colour chain of a lowered Program (canonical form
// M_a, [cbrt], M_b, [cube], M_c, [clamp], M_d, linear result) -> box (area coverage)
// fit-resize so the long side is `canvas` -> centred inscribe on a transparent
// canvas x canvas image -> exact sRGB8 encode.  The canvases are zero-filled (the
// transparent margins) by one memset; the fitted pixels are cut into work items, one item per
// warp at a time, which warps take from a queue (one atomic add per item, no block barriers)
// over all images, ordered largest items first, so that every image's cost spreads over all
// warps and they finish together.
//
// The colour chain is nonlinear, so it runs on every source texel before the box filter.
// Downscaled images (both scale factors >= 1, the bulk of the work) use streaming items that
// put each texel through the chain exactly once, reading source rows coalesced:
//  * an item is a band of output rows x a run of output columns whose box windows span at most
//    128 source columns; lane l owns source columns c0 + l + 32 k, k = 0..3, so every row load
//    of the warp is 128 contiguous bytes;
//  * the warp walks the band's source rows top to bottom, texels go through the chain two
//    at a time in FP32x2 registers (decode from the lane-replicated shared table, MUFU cube
//    roots, the rank-1 Oklab L/C form when planned), and each lane keeps the vertical box sums
//    of its four columns in registers; the next row's loads are issued before this row's
//    arithmetic;
//  * when the last row of an output row's window has been added, the column sums go to the
//    warp's 2 KiB slice of shared memory and the lanes owning output columns apply the
//    horizontal box weights, normalise, encode and store; a boundary row shared with the next
//    output row seeds the next sums with its own weight.
// Upscaled images (few texels) use per-output items: lane l owns one output column of 32 and
// walks its 2 x 2 (or wider) window directly.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "host/zs_host.hpp"
#include "zs_chain.cuh"
#include "zs_device.cuh"
#include "zs_kernels.h"

#define ZS_BATCH_SPAN 128         // source columns of a streaming item: 4 per lane
#define ZS_BATCH_SMEM (2 * ZS_DEC_ABS)   // dynamic shared memory per block
#define ZS_BATCH_ROWS_DEFAULT 4   // work-item height until the autotuner chose (see batch_thumbnails)

struct ZsBatchImage {
    const uint8_t *ptr;
    int32_t width, height;     // source
    int32_t tw, th;            // fitted size
    int32_t x0, y0;            // placement on the canvas
    float sx, sy;              // source pixels per fitted pixel
    float fx, fy;              // filter widths: max(sx, 1), max(sy, 1)
    int32_t stream;            // 1: streaming items, 0: per-output items
    int32_t kx;                // output columns per item
    int32_t chunks;            // items across the fitted width
    int32_t ry;                // output rows per item
    int32_t index;             // the image's position in the caller's list (its canvas)
    int32_t pad;
};

struct ZsBatchArgs {
    const ZsBatchImage *images;
    const int32_t *prefix;     // [n + 1]: first work item of each image, total at [n]
    int32_t *queue;            // next work item (zeroed before every batch)
    uint8_t *out;
    int32_t n;
    int32_t canvas;
    int32_t flags;
    int32_t pad;
    float m2[4][9][2];         // the chain's matrices with every coefficient duplicated (f32x2 operands)
    float mb_v[3][2];          // ZS_CHAIN_MB_RANK1: M_b = d I + (1,1,1)^T v
    float mb_d[2];
};

// Chain specialisations: LAB = cube root, cube and clamp all present (the Oklab / SrLab2
// chains), NONNEG and RANK1 as in the chain kernel; GENERIC reads the flags at run time.
enum { ZS_BATCH_GENERIC = 0, ZS_BATCH_LAB = 1, ZS_BATCH_LAB_NONNEG = 2, ZS_BATCH_LAB_RANK1 = 3,
       ZS_BATCH_LAB_NONNEG_RANK1 = 4 };

template <int SPEC> struct ZsBatchSpec {
    static constexpr bool generic = SPEC == ZS_BATCH_GENERIC;
    static constexpr bool nonneg = SPEC == ZS_BATCH_LAB_NONNEG || SPEC == ZS_BATCH_LAB_NONNEG_RANK1;
    static constexpr bool rank1 = SPEC == ZS_BATCH_LAB_RANK1 || SPEC == ZS_BATCH_LAB_NONNEG_RANK1;
};

// rgb' = M rgb on two pixel pairs, every coefficient read once for both.
template <bool SAT>
__device__ __forceinline__ void zs_m3x2x2(const float (*m)[2], float2 (&v)[2][3]) {
    const float2 *c = reinterpret_cast<const float2 *>(m);
    const float2 x0 = v[0][0], y0 = v[0][1], z0 = v[0][2], x1 = v[1][0], y1 = v[1][1], z1 = v[1][2];
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        v[0][row] = zs_row2<SAT>(c + 3 * row, x0, y0, z0);
        v[1][row] = zs_row2<SAT>(c + 3 * row, x1, y1, z1);
    }
}

template <bool NONNEG>
__device__ __forceinline__ void zs_cbrt_pair(float2 &x) {
    if (NONNEG) zs_cbrt2(x);
    else x = make_float2(zs_cbrt1<false>(x.x), zs_cbrt1<false>(x.y));
}

// The canonical chain on four texels (two FP32x2 pairs: (w0, w1) and (w2, w3)), linear
// result in v[pair][channel]: decode through the lane-replicated shared table at shared
// address ZS_DEC_ABS (lane4 = ZS_DEC_ABS | lane << 2), matrix products, MUFU cube roots.
template <int SPEC>
__device__ __forceinline__ void zs_batch_chain4(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3,
                                                const unsigned char *lut, uint32_t lane4, const ZsBatchArgs &a,
                                                float2 (&v)[2][3]) {
    using S = ZsBatchSpec<SPEC>;
    (void)lut;
    v[0][0] = make_float2(zs_dec_abs<0>(w0, lane4), zs_dec_abs<0>(w1, lane4));
    v[0][1] = make_float2(zs_dec_abs<1>(w0, lane4), zs_dec_abs<1>(w1, lane4));
    v[0][2] = make_float2(zs_dec_abs<2>(w0, lane4), zs_dec_abs<2>(w1, lane4));
    v[1][0] = make_float2(zs_dec_abs<0>(w2, lane4), zs_dec_abs<0>(w3, lane4));
    v[1][1] = make_float2(zs_dec_abs<1>(w2, lane4), zs_dec_abs<1>(w3, lane4));
    v[1][2] = make_float2(zs_dec_abs<2>(w2, lane4), zs_dec_abs<2>(w3, lane4));
    zs_m3x2x2<false>(a.m2[0], v);
    const bool cbrt = S::generic ? (a.flags & ZS_CHAIN_CBRT) != 0 : true;
    if (cbrt) {
        const bool nonneg = S::generic ? ((a.flags & ZS_CHAIN_CBRT_NONNEG) != 0) : S::nonneg;
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                if (nonneg) zs_cbrt_pair<true>(v[p][ch]);
                else zs_cbrt_pair<false>(v[p][ch]);
            }
    }
    if (!S::generic && S::rank1) {
        const float2 *mv = reinterpret_cast<const float2 *>(a.mb_v);
        const float2 d = *reinterpret_cast<const float2 *>(a.mb_d);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const float2 t = __ffma2_rn(mv[0], v[p][0], __ffma2_rn(mv[1], v[p][1], __fmul2_rn(mv[2], v[p][2])));
            v[p][0] = __ffma2_rn(d, v[p][0], t);
            v[p][1] = __ffma2_rn(d, v[p][1], t);
            v[p][2] = __ffma2_rn(d, v[p][2], t);
        }
    } else {
        zs_m3x2x2<false>(a.m2[1], v);
    }
    const bool cube = S::generic ? (a.flags & ZS_CHAIN_CUBE) != 0 : true;
    if (cube) {
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) v[p][ch] = __fmul2_rn(__fmul2_rn(v[p][ch], v[p][ch]), v[p][ch]);
    }
    const bool clamp = S::generic ? (a.flags & ZS_CHAIN_CLAMP) != 0 : true;
    if (clamp) zs_m3x2x2<true>(a.m2[2], v);
    else zs_m3x2x2<false>(a.m2[2], v);
    zs_m3x2x2<false>(a.m2[3], v);
}

// Alpha codes of a texel pair as floats: byte 3 of each texel under the exponent of 2^23
// (one byte permute), minus 2^23 by one packed add.
__device__ __forceinline__ float2 zs_alpha2(uint32_t w0, uint32_t w1) {
    const float2 biased = make_float2(__uint_as_float(__byte_perm(w0, 0x4B000000u, 0x7443u)),
                                      __uint_as_float(__byte_perm(w1, 0x4B000000u, 0x7443u)));
    return __fadd2_rn(biased, make_float2(-8388608.0f, -8388608.0f));
}

// Box (area coverage) window of output index u along one axis.
__device__ __forceinline__ void zs_box_window(int u, float s, float f, int len, int &j0, int &j1, float &lo, float &hi) {
    const float c = ((float)u + 0.5f) * s;
    lo = c - 0.5f * f;
    hi = c + 0.5f * f;
    j0 = max((int)floorf(lo), 0);
    j1 = min((int)ceilf(hi), len);
}

// Coverage of texel j by the window [lo, hi).
__device__ __forceinline__ float zs_cover(float lo, float hi, int j) {
    return fmaxf(fminf(hi, (float)j + 1.f) - fmaxf(lo, (float)j), 0.f);
}

__device__ __forceinline__ uint32_t zs_batch_encode(float4 acc, float inv) {
    return zs_enc_srgb8(zs_srgb_encode_tab, acc.x * inv) | (zs_enc_srgb8(zs_srgb_encode_tab, acc.y * inv) << 8) |
           (zs_enc_srgb8(zs_srgb_encode_tab, acc.z * inv) << 16) | (zs_unorm8(acc.w * inv * (1.0f / 255.0f)) << 24);
}

// A streaming item: output rows [v0, v1) x output columns [u0, u1) of image I.
template <int SPEC>
__device__ __forceinline__ void zs_batch_stream(const ZsBatchImage &I, int band, int chunk, float4 *hb,
                                                const unsigned char *lut, uint32_t lane4, int lane,
                                                const ZsBatchArgs &a, uint32_t *out) {
    const int u0 = chunk * I.kx, u1 = min(u0 + I.kx, I.tw);
    int xs, xe, t0, t1;
    float tlo, thi;
    zs_box_window(u0, I.sx, I.fx, I.width, xs, t1, tlo, thi);
    zs_box_window(u1 - 1, I.sx, I.fx, I.width, t0, xe, tlo, thi);
    xe = min(xe, xs + ZS_BATCH_SPAN);
    const int v0 = band * I.ry, v1 = min(v0 + I.ry, I.th);
    int jy0, jy1, ye;
    float loy, hiy;
    zs_box_window(v1 - 1, I.sy, I.fy, I.height, t0, ye, tlo, thi);
    zs_box_window(v0, I.sy, I.fy, I.height, jy0, jy1, loy, hiy);
    const uint32_t *img = reinterpret_cast<const uint32_t *>(I.ptr);
    const int W = I.width;
    // This lane's columns xs + lane + 32 k; those past the span re-read its last column
    // (computed, never used), so every load is unconditional.
    const int c0 = xs + lane;
    const int o0 = min(c0, xe - 1), o1 = min(c0 + 32, xe - 1), o2 = min(c0 + 64, xe - 1), o3 = min(c0 + 96, xe - 1);
    // Column sums: pair 0 = columns (c0, c0 + 32), pair 1 = (c0 + 64, c0 + 96).
    float2 sr0 = make_float2(0.f, 0.f), sg0 = sr0, sb0 = sr0, sa0 = sr0, sr1 = sr0, sg1 = sr0, sb1 = sr0, sa1 = sr0;
    int v = v0;
    int y = jy0;
    // Rows y + 1 and y + 2 are in flight during row y's arithmetic; prefetches stop at the
    // band's last row (ylast).  The band ends when its last output row is stored; should it
    // run past ylast, the row is loaded when it is needed (ny tracks the prefetched row).
    const int ylast = max(min(ye, I.height) - 1, jy0);
    const uint32_t *p = img + (size_t)y * W;
    uint32_t w0 = __ldg(p + o0), w1 = __ldg(p + o1), w2 = __ldg(p + o2), w3 = __ldg(p + o3);
    int ny = min(y + 1, ylast);
    p = img + (size_t)ny * W;
    uint32_t n0 = __ldg(p + o0), n1 = __ldg(p + o1), n2 = __ldg(p + o2), n3 = __ldg(p + o3);
    for (;;) {
        const int my = min(y + 2, ylast);
        p = img + (size_t)my * W;
        const uint32_t m0 = __ldg(p + o0), m1 = __ldg(p + o1), m2 = __ldg(p + o2), m3 = __ldg(p + o3);
        float2 cv[2][3];
        zs_batch_chain4<SPEC>(w0, w1, w2, w3, lut, lane4, a, cv);
        const float2 r0 = cv[0][0], g0 = cv[0][1], b0 = cv[0][2], r1 = cv[1][0], g1 = cv[1][1], b1 = cv[1][2];
        const float2 al0 = zs_alpha2(w0, w1), al1 = zs_alpha2(w2, w3);
        const float wy = zs_cover(loy, hiy, y);
        const float2 wy2 = make_float2(wy, wy);
        sr0 = __ffma2_rn(wy2, r0, sr0);
        sg0 = __ffma2_rn(wy2, g0, sg0);
        sb0 = __ffma2_rn(wy2, b0, sb0);
        sa0 = __ffma2_rn(wy2, al0, sa0);
        sr1 = __ffma2_rn(wy2, r1, sr1);
        sg1 = __ffma2_rn(wy2, g1, sg1);
        sb1 = __ffma2_rn(wy2, b1, sb1);
        sa1 = __ffma2_rn(wy2, al1, sa1);
        // Output rows whose window ends with this row (uniform across the warp).
        while (y == jy1 - 1 && v < v1) {
            hb[lane] = make_float4(sr0.x, sg0.x, sb0.x, sa0.x);
            hb[lane + 32] = make_float4(sr0.y, sg0.y, sb0.y, sa0.y);
            hb[lane + 64] = make_float4(sr1.x, sg1.x, sb1.x, sa1.x);
            hb[lane + 96] = make_float4(sr1.y, sg1.y, sb1.y, sa1.y);
            const int vd = v, dy0 = jy0, dy1 = jy1;
            const float dlo = loy, dhi = hiy;
            // The next output row starts with this row's share of it.
            ++v;
            float wn = 0.f;
            if (v < v1) {
                zs_box_window(v, I.sy, I.fy, I.height, jy0, jy1, loy, hiy);
                wn = zs_cover(loy, hiy, y);
            }
            const float2 wn2 = make_float2(wn, wn);
            sr0 = __fmul2_rn(wn2, r0);
            sg0 = __fmul2_rn(wn2, g0);
            sb0 = __fmul2_rn(wn2, b0);
            sa0 = __fmul2_rn(wn2, al0);
            sr1 = __fmul2_rn(wn2, r1);
            sg1 = __fmul2_rn(wn2, g1);
            sb1 = __fmul2_rn(wn2, b1);
            sa1 = __fmul2_rn(wn2, al1);
            __syncwarp();
            for (int k = lane; k < u1 - u0; k += 32) {
                const int u = u0 + k;
                int jx0, jx1;
                float lox, hix;
                zs_box_window(u, I.sx, I.fx, I.width, jx0, jx1, lox, hix);
                const float wxsum = fmaxf(fminf(hix, (float)jx1) - fmaxf(lox, (float)jx0), 0.f);
                jx0 = max(jx0, xs);
                jx1 = min(jx1, xe);
                float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int j = jx0; j < jx1; ++j) {
                    const float wx = zs_cover(lox, hix, j);
                    const float4 c = hb[j - xs];
                    acc.x = fmaf(wx, c.x, acc.x);
                    acc.y = fmaf(wx, c.y, acc.y);
                    acc.z = fmaf(wx, c.z, acc.z);
                    acc.w = fmaf(wx, c.w, acc.w);
                }
                const float wsum = wxsum * fmaxf(fminf(dhi, (float)dy1) - fmaxf(dlo, (float)dy0), 0.f);
                out[(size_t)(I.y0 + vd) * a.canvas + I.x0 + u] = zs_batch_encode(acc, wsum > 0.f ? 1.0f / wsum : 0.f);
            }
            __syncwarp();
        }
        if (v >= v1 || y + 1 >= I.height) break;
        ++y;
        if (ny != y) {
            p = img + (size_t)y * W;
            n0 = __ldg(p + o0);
            n1 = __ldg(p + o1);
            n2 = __ldg(p + o2);
            n3 = __ldg(p + o3);
        }
        w0 = n0;
        w1 = n1;
        w2 = n2;
        w3 = n3;
        n0 = m0;
        n1 = m1;
        n2 = m2;
        n3 = m3;
        ny = my;
    }
}

// A per-output item (upscaled images): lane l owns output column u of 32, rows [v0, v1).
template <int SPEC>
__device__ __forceinline__ void zs_batch_direct(const ZsBatchImage &I, int band, int chunk, const unsigned char *lut,
                                                uint32_t lane4, int lane, const ZsBatchArgs &a, uint32_t *out) {
    const int u = chunk * I.kx + lane;
    if (u >= I.tw) return;
    int jx0, jx1;
    float lox, hix;
    zs_box_window(u, I.sx, I.fx, I.width, jx0, jx1, lox, hix);
    const float wxsum = fmaxf(fminf(hix, (float)jx1) - fmaxf(lox, (float)jx0), 0.f);
    const uint32_t *img = reinterpret_cast<const uint32_t *>(I.ptr);
    const int v0 = band * I.ry, v1 = min(v0 + I.ry, I.th);
    for (int v = v0; v < v1; ++v) {
        int jy0, jy1;
        float loy, hiy;
        zs_box_window(v, I.sy, I.fy, I.height, jy0, jy1, loy, hiy);
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int jy = jy0; jy < jy1; ++jy) {
            const float wy = zs_cover(loy, hiy, jy);
            const uint32_t *row = img + (size_t)jy * I.width;
            for (int jx = jx0; jx < jx1; jx += 2) {
                const bool two = jx + 1 < jx1;
                const uint32_t t0 = __ldg(row + jx), t1 = two ? __ldg(row + jx + 1) : t0;
                float2 v[2][3];
                zs_batch_chain4<SPEC>(t0, t1, t0, t1, lut, lane4, a, v);
                const float2 al = zs_alpha2(t0, t1);
                const float wa = wy * zs_cover(lox, hix, jx), wb = two ? wy * zs_cover(lox, hix, jx + 1) : 0.f;
                acc.x = fmaf(wb, v[0][0].y, fmaf(wa, v[0][0].x, acc.x));
                acc.y = fmaf(wb, v[0][1].y, fmaf(wa, v[0][1].x, acc.y));
                acc.z = fmaf(wb, v[0][2].y, fmaf(wa, v[0][2].x, acc.z));
                acc.w = fmaf(wb, al.y, fmaf(wa, al.x, acc.w));
            }
        }
        const float wsum = wxsum * fmaxf(fminf(hiy, (float)jy1) - fmaxf(loy, (float)jy0), 0.f);
        out[(size_t)(I.y0 + v) * a.canvas + I.x0 + u] = zs_batch_encode(acc, wsum > 0.f ? 1.0f / wsum : 0.f);
    }
}

// One block per SM (the 64 KiB decode table once per SM); THREADS is 768 or 640 (autotuned:
// 24 warps with a few spilled registers or 20 warps without).
template <int THREADS, int SPEC>
__global__ void __launch_bounds__(THREADS, 1) zs_batch_kernel(const __grid_constant__ ZsBatchArgs a) {
    // From the start of the dynamic window: one 128-column slice of float4 column sums per
    // warp; at shared address ZS_DEC_ABS .. 2 * ZS_DEC_ABS: the decode table, [code][64] floats
    // (lanes 32..63 unused), so that one PRMT forms each decode's load address.  The host
    // launches with ZS_BATCH_SMEM bytes after checking that the slices fit below ZS_DEC_ABS;
    // should the window start higher, the block flags it and does nothing.
    extern __shared__ __align__(16) float zs_batch_smem[];
    const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(zs_batch_smem);
    uint32_t dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    if (s0 + (uint32_t)(THREADS / 32 * ZS_BATCH_SPAN * sizeof(float4)) > ZS_DEC_ABS ||
        ZS_DEC_ABS + 256u * 64u * 4u > s0 + dyn) {
        if (threadIdx.x == 0) atomicOr(&zs_device_status_word, ZS_DEVSTAT_LAYOUT);
        return;
    }
    float *table = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(zs_batch_smem) + (ZS_DEC_ABS - s0));
    for (int i = threadIdx.x; i < 256 * 8; i += blockDim.x) {
        const float d = zs_srgb_decode_lut[i >> 3];
        reinterpret_cast<float4 *>(table)[(i >> 3) * 16 + (i & 7)] = make_float4(d, d, d, d);
    }
    __syncthreads();
    const unsigned char *lut = reinterpret_cast<const unsigned char *>(table);
    float4 *hb = reinterpret_cast<float4 *>(zs_batch_smem) + (threadIdx.x >> 5) * ZS_BATCH_SPAN;
    const int lane = threadIdx.x & 31;
    const uint32_t lane4 = ZS_DEC_ABS | ((uint32_t)lane << 2);
    const int total = a.prefix[a.n];
    int img = 0;   // entry of the current item: a warp's items only move forward, so scan on
    for (;;) {
        // Each warp takes the next item of the queue: the images are ordered by item cost,
        // largest first, so the last items handed out are the cheapest.
        int it = 0;
        if (lane == 0) it = atomicAdd(a.queue, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= total) break;
        while (a.prefix[img + 1] <= it) ++img;
        const ZsBatchImage I = a.images[img];
        const int local = it - a.prefix[img];
        const int band = local / I.chunks, chunk = local - band * I.chunks;
        uint32_t *out = reinterpret_cast<uint32_t *>(a.out + (size_t)I.index * a.canvas * a.canvas * 4);
        if (I.stream) zs_batch_stream<SPEC>(I, band, chunk, hb, lut, lane4, lane, a, out);
        else zs_batch_direct<SPEC>(I, band, chunk, lut, lane4, lane, a, out);
    }
}

namespace zs {

int batch_thumbnails(Executable *chain, const void *const *images, const uint32_t *widths, const uint32_t *heights,
                     uint32_t n, uint32_t canvas, void *out, cudaStream_t stream) {
    const Step *cs = nullptr;
    for (const Step &s : chain->steps)
        if (s.kind == StepKind::Chain) cs = &s;
    if (!cs || chain->steps.size() != 1) {
        set_last_error("zs_batch_thumbnails: the executable must be one fused RGBA8 sRGB colour chain");
        return ZS_ERR_UNIMPLEMENTED;
    }
    if (canvas == 0 || canvas > 16384) {
        set_last_error("zs_batch_thumbnails: canvas size out of range");
        return ZS_ERR_INVALID_ARG;
    }
    if (n == 0) return ZS_OK;
    chain->ensure_buffers();
    std::vector<ZsBatchImage> host(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (!images[i] || widths[i] == 0 || heights[i] == 0) {
            set_last_error("zs_batch_thumbnails: null image or empty size");
            return ZS_ERR_INVALID_ARG;
        }
        ZsBatchImage &I = host[i];
        I.ptr = (const uint8_t *)images[i];
        I.width = (int)widths[i];
        I.height = (int)heights[i];
        if (widths[i] >= heights[i]) {
            I.tw = (int)canvas;
            I.th = std::max(1, (int)std::lround((double)heights[i] * canvas / widths[i]));
        } else {
            I.th = (int)canvas;
            I.tw = std::max(1, (int)std::lround((double)widths[i] * canvas / heights[i]));
        }
        I.x0 = ((int)canvas - I.tw) / 2;
        I.y0 = ((int)canvas - I.th) / 2;
        I.sx = (float)((double)I.width / I.tw);
        I.sy = (float)((double)I.height / I.th);
        I.fx = I.sx > 1.f ? I.sx : 1.f;
        I.fy = I.sy > 1.f ? I.sy : 1.f;
    }
    // Work-item height `rows` (the tuned value for this chain, canvas and device when the
    // autotuner has seen them): a streaming item covers about 16 x rows source rows, a
    // per-output item `rows` output rows.  Every choice gives the same bytes: each output
    // pixel's sums run over the same texels in the same order.
    if (chain->batch_rows <= 0) {
        int tuned;
        if (tune_get(batch_tune_key(*chain, canvas, chain->device), tuned) && tuned >= 1 && tuned <= 16)
            chain->batch_rows = tuned;
    }
    const int rows = chain->batch_rows > 0 ? chain->batch_rows : ZS_BATCH_ROWS_DEFAULT;
    std::vector<double> cost(n);
    for (uint32_t i = 0; i < n; ++i) {
        ZsBatchImage &I = host[i];
        I.index = (int32_t)i;
        I.pad = 0;
        // Streaming when both axes shrink and the box windows of at least one output column
        // fit the 128-column span (2 columns of slack for the window rounding).
        const int kx = (int)std::floor((ZS_BATCH_SPAN - 4) / (double)I.sx);
        I.stream = I.sx >= 1.f && I.sy >= 1.f && kx >= 1;
        if (I.stream) {
            I.kx = std::min(kx, I.tw);
            I.ry = std::max(1, (int)std::lround(16.0 * rows / I.sy));
        } else {
            I.kx = 32;
            I.ry = rows;
        }
        I.chunks = (I.tw + I.kx - 1) / I.kx;
        // Texels one item puts through the chain.
        cost[i] = I.stream ? std::min((double)ZS_BATCH_SPAN, I.kx * (double)I.sx + 2.0) * (I.ry * (double)I.sy + 1.0)
                           : 32.0 * I.ry * (std::ceil(I.fx) + 1.0) * (std::ceil(I.fy) + 1.0);
    }
    // Work list: images by item cost, largest first (ties in the caller's order), so that the
    // queue ends with its cheapest items and the warps finish together.
    std::vector<uint32_t> order(n);
    for (uint32_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return cost[x] > cost[y]; });
    std::vector<ZsBatchImage> sorted(n);
    std::vector<int32_t> prefix(n + 1, 0);
    for (uint32_t k = 0; k < n; ++k) {
        const ZsBatchImage &I = host[order[k]];
        sorted[k] = I;
        const int64_t items = (int64_t)((I.th + I.ry - 1) / I.ry) * I.chunks;
        if ((int64_t)prefix[k] + items > INT32_MAX) {
            set_last_error("zs_batch_thumbnails: too many output pixels in one batch");
            return ZS_ERR_INVALID_ARG;
        }
        prefix[k + 1] = prefix[k] + (int32_t)items;
    }
    // Scratch: image table + item prefix table, kept with the executable in two sets used by
    // alternate batches, uploaded from a pinned staging copy: the batch two calls back (the
    // last user of this set) must have finished with it before it is rewritten, while the
    // previous batch may still run.
    const size_t table_bytes = (sizeof(ZsBatchImage) * n + 255) & ~(size_t)255;
    const size_t prefix_bytes = (sizeof(int32_t) * (n + 1) + 15) & ~(size_t)15;
    const size_t bytes = table_bytes + prefix_bytes + 16;   // + the queue counter
    auto device_error = [](cudaError_t e) {
        set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? ZS_ERR_OUT_OF_MEMORY : ZS_ERR_DEVICE;
    };
    cudaError_t e = cudaSuccess;
    Executable::BatchSet &bs = chain->batch_sets[chain->batch_next];
    chain->batch_next ^= 1;
    if (bs.done && (e = cudaEventSynchronize(bs.done)) != cudaSuccess) return device_error(e);
    if (bs.bytes < bytes) {
        if (bs.scratch) cudaFree(bs.scratch);
        if (bs.staging) cudaFreeHost(bs.staging);
        bs.scratch = bs.staging = nullptr;
        bs.bytes = 0;
        if ((e = cudaMalloc(&bs.scratch, bytes)) != cudaSuccess) return device_error(e);
        if ((e = cudaMallocHost(&bs.staging, bytes)) != cudaSuccess) return device_error(e);
        bs.bytes = bytes;
    }
    if (!bs.done && (e = cudaEventCreateWithFlags(&bs.done, cudaEventDisableTiming)) != cudaSuccess)
        return device_error(e);
    uint8_t *scratch = (uint8_t *)bs.scratch, *staging = (uint8_t *)bs.staging;
    std::memcpy(staging, sorted.data(), sizeof(ZsBatchImage) * n);
    std::memcpy(staging + table_bytes, prefix.data(), sizeof(int32_t) * (n + 1));
    if ((e = cudaMemcpyAsync(scratch, staging, table_bytes + prefix_bytes, cudaMemcpyHostToDevice, stream)) !=
        cudaSuccess)
        return device_error(e);
    ZsBatchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.images = (const ZsBatchImage *)scratch;
    a.prefix = (const int32_t *)(scratch + table_bytes);
    a.queue = (int32_t *)(scratch + table_bytes + prefix_bytes);
    a.out = (uint8_t *)out;
    a.n = (int)n;
    a.canvas = (int)canvas;
    a.flags = cs->chain.flags;
    std::memcpy(a.m2, cs->chain.m2, sizeof(a.m2));
    std::memcpy(a.mb_v, cs->chain.mb_v, sizeof(a.mb_v));
    std::memcpy(a.mb_d, cs->chain.mb_d, sizeof(a.mb_d));
    const bool lab = (a.flags & ZS_CHAIN_CBRT) && (a.flags & ZS_CHAIN_CUBE) && (a.flags & ZS_CHAIN_CLAMP);
    const bool nonneg = (a.flags & ZS_CHAIN_CBRT_NONNEG) != 0;
    const bool rank1 = (a.flags & ZS_CHAIN_MB_RANK1) != 0;
    const int spec = !lab ? ZS_BATCH_GENERIC
                          : (nonneg ? (rank1 ? ZS_BATCH_LAB_NONNEG_RANK1 : ZS_BATCH_LAB_NONNEG)
                                    : (rank1 ? ZS_BATCH_LAB_RANK1 : ZS_BATCH_LAB));
    if (chain->batch_threads <= 0) {
        int tuned;
        if (tune_get(batch_tune_key(*chain, canvas, chain->device, "batch_threads"), tuned) &&
            (tuned == 768 || tuned == 640))
            chain->batch_threads = tuned;
    }
    const int threads = chain->batch_threads > 0 ? chain->batch_threads : 640;
    static void (*const kernels[2][5])(ZsBatchArgs) = {
        {zs_batch_kernel<768, 0>, zs_batch_kernel<768, 1>, zs_batch_kernel<768, 2>, zs_batch_kernel<768, 3>,
         zs_batch_kernel<768, 4>},
        {zs_batch_kernel<640, 0>, zs_batch_kernel<640, 1>, zs_batch_kernel<640, 2>, zs_batch_kernel<640, 3>,
         zs_batch_kernel<640, 4>}};
    void (*kernel)(ZsBatchArgs) = kernels[threads == 640 ? 1 : 0][spec];
    // The column-sum slices below ZS_DEC_ABS, after the driver's reserved shared memory (the
    // kernel has no static shared memory), the decode table above it.
    const size_t smem = ZS_BATCH_SMEM;
    {
        int reserved = 0;
        e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, chain->device);
        if (e != cudaSuccess) return device_error(e);
        if ((size_t)reserved + (size_t)(threads / 32) * ZS_BATCH_SPAN * sizeof(float4) > ZS_DEC_ABS)
            return device_error(cudaErrorNotSupported);
    }
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (e != cudaSuccess) return device_error(e);
    if (per_sm < 1) per_sm = 1;
    // The grid covers every SM: warps take items of all images from the queue.
    long long blocks = (long long)chain->sm_count * per_sm;
    const long long need = ((long long)prefix[n] + threads / 32 - 1) / (threads / 32);
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    // The batch launch (zero the canvases, one kernel) is captured once as a CUDA graph and
    // replayed for every later batch with the same output buffer, count and canvas: the image
    // table the kernel reads is the per-batch data, uploaded above.
    // The key holds every kernel argument byte and the launch shape: a graph is replayed only
    // for a launch it captured exactly.
    std::vector<uint64_t> key = {(uint64_t)(uintptr_t)out, n, canvas, (uint64_t)(uintptr_t)kernel, (uint64_t)blocks};
    {
        static_assert(sizeof(ZsBatchArgs) % 8 == 0, "argument block in 64-bit words");
        const size_t words = sizeof(ZsBatchArgs) / 8;
        const size_t at = key.size();
        key.resize(at + words);
        std::memcpy(key.data() + at, &a, sizeof(ZsBatchArgs));
    }
    auto enqueue = [&]() {
        // The work queue starts at item 0; transparent margins: zero every canvas, the kernel
        // writes the fitted pixels.
        cudaError_t ce = cudaMemsetAsync(a.queue, 0, sizeof(int32_t), stream);
        if (ce == cudaSuccess) ce = cudaMemsetAsync(out, 0, (size_t)n * canvas * canvas * 4, stream);
        if (ce == cudaSuccess) {
            kernel<<<(unsigned)blocks, threads, smem, stream>>>(a);
            ce = cudaGetLastError();
        }
        return ce;
    };
    if (!bs.graph || bs.key != key) {
        if (bs.graph) cudaGraphExecDestroy(bs.graph);
        bs.graph = nullptr;
        bs.key.clear();
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            // A stream that cannot be captured (the legacy default stream): launch directly.
            cudaGetLastError();
            if ((e = enqueue()) != cudaSuccess) return device_error(e);
            if ((e = cudaEventRecord(bs.done, stream)) != cudaSuccess) return device_error(e);
            g_kernel_launches.fetch_add(1);
            return ZS_OK;
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ce = enqueue();
        e = cudaStreamEndCapture(stream, &g);
        if (ce != cudaSuccess || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return device_error(ce != cudaSuccess ? ce : e);
        }
        cudaGraphExec_t ge = nullptr;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return device_error(e);
        bs.graph = ge;
        bs.key = key;
    }
    if ((e = cudaGraphLaunch(bs.graph, stream)) != cudaSuccess) return device_error(e);
    if ((e = cudaEventRecord(bs.done, stream)) != cudaSuccess) return device_error(e);
    g_kernel_launches.fetch_add(1);
    return ZS_OK;
}

}  // namespace zs

ZS_TU_HOOKS(batch)
