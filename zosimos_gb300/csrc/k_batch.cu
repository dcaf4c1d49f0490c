// k_batch.cu -- many RGBA8 sRGB images of uneven sizes turned into thumbnails by one
// persistent launch over a device work queue (the reference's batch-reuse case runs one
// Executable per image, lib/zosimos/tests/loop.rs:84-95).
//
// Per image: decode -> the fused colour chain of a lowered Program (canonical form
// M_a, [cbrt], M_b, [cube], M_c, [clamp], M_d, linear result) -> box (area coverage)
// fit-resize so the long side is `canvas` -> centred inscribe on a transparent
// canvas x canvas image -> exact sRGB8 encode.  The canvases are zero-filled (the
// transparent margins) by one memset; the fitted pixels are cut into work items of 32
// adjacent pixels of one row, one item per warp, so the 32 lanes have windows of the
// same size.  Warps take items by static striding over all images (a prefix table and a
// binary search find the image of an item), which spreads every image's cost over all
// warps without atomics or barriers.  Each lane computes its output pixel from its source
// window: the box weights are separable, the source texels of a window row go through
// the colour chain two at a time in FP32x2 registers.
#include <cstring>
#include <vector>

#include "host/zs_host.hpp"
#include "zs_chain.cuh"
#include "zs_device.cuh"
#include "zs_kernels.h"

#define ZS_BATCH_THREADS 256

struct ZsBatchImage {
    const uint8_t *ptr;
    int32_t width, height;     // source
    int32_t tw, th;            // fitted size
    int32_t x0, y0;            // placement on the canvas
    float sx, sy;              // source pixels per fitted pixel
    float fx, fy;              // filter widths: max(sx, 1), max(sy, 1)
};

struct ZsBatchArgs {
    const ZsBatchImage *images;
    const int32_t *prefix;     // [n + 1]: first work item of each image, total at [n]
    uint8_t *out;
    int32_t n;
    int32_t canvas;
    int32_t flags;
    int32_t pad;
    float m[4][9];
    float m2[4][9][2];         // the same matrices with every coefficient duplicated (f32x2 operands)
};

__device__ __forceinline__ void zs_batch_m3(const float *m, float &r, float &g, float &b) {
    float x = r, y = g, z = b;
    r = fmaf(m[0], x, fmaf(m[1], y, m[2] * z));
    g = fmaf(m[3], x, fmaf(m[4], y, m[5] * z));
    b = fmaf(m[6], x, fmaf(m[7], y, m[8] * z));
}

// Linear result of the canonical chain for one RGBA8 sRGB texel.
__device__ __forceinline__ float4 zs_batch_chain(uint32_t w, const ZsBatchArgs &a) {
    float r = zs_srgb_decode_lut[w & 255u], g = zs_srgb_decode_lut[(w >> 8) & 255u],
          b = zs_srgb_decode_lut[(w >> 16) & 255u];
    zs_batch_m3(a.m[0], r, g, b);
    if (a.flags & ZS_CHAIN_CBRT) { r = zs_scbrt(r); g = zs_scbrt(g); b = zs_scbrt(b); }
    zs_batch_m3(a.m[1], r, g, b);
    if (a.flags & ZS_CHAIN_CUBE) { r = r * r * r; g = g * g * g; b = b * b * b; }
    zs_batch_m3(a.m[2], r, g, b);
    if (a.flags & ZS_CHAIN_CLAMP) { r = __saturatef(r); g = __saturatef(g); b = __saturatef(b); }
    zs_batch_m3(a.m[3], r, g, b);
    return make_float4(r, g, b, (float)(w >> 24) / 255.0f);
}

// The same chain on two texels at once: decode through the lane-replicated shared table
// of the chain kernel, FP32x2 matrix products, MUFU cube roots.
template <bool NONNEG>
__device__ __forceinline__ void zs_batch_chain2(uint32_t w0, uint32_t w1, const unsigned char *lut, uint32_t lane4,
                                                const ZsBatchArgs &a, float2 &r, float2 &g, float2 &b) {
    r = make_float2(zs_dec<0>(lut, w0, lane4), zs_dec<0>(lut, w1, lane4));
    g = make_float2(zs_dec<1>(lut, w0, lane4), zs_dec<1>(lut, w1, lane4));
    b = make_float2(zs_dec<2>(lut, w0, lane4), zs_dec<2>(lut, w1, lane4));
    zs_m3x2<false>(a.m2[0], r, g, b);
    if (a.flags & ZS_CHAIN_CBRT) {
        if (NONNEG) {
            zs_cbrt2(r);
            zs_cbrt2(g);
            zs_cbrt2(b);
        } else {
            r = make_float2(zs_cbrt1<false>(r.x), zs_cbrt1<false>(r.y));
            g = make_float2(zs_cbrt1<false>(g.x), zs_cbrt1<false>(g.y));
            b = make_float2(zs_cbrt1<false>(b.x), zs_cbrt1<false>(b.y));
        }
    }
    zs_m3x2<false>(a.m2[1], r, g, b);
    if (a.flags & ZS_CHAIN_CUBE) {
        r = __fmul2_rn(__fmul2_rn(r, r), r);
        g = __fmul2_rn(__fmul2_rn(g, g), g);
        b = __fmul2_rn(__fmul2_rn(b, b), b);
    }
    if (a.flags & ZS_CHAIN_CLAMP) zs_m3x2<true>(a.m2[2], r, g, b);
    else zs_m3x2<false>(a.m2[2], r, g, b);
    zs_m3x2<false>(a.m2[3], r, g, b);
}

// Box (area coverage) window of output index u along one axis.
__device__ __forceinline__ void zs_box_window(int u, float s, float f, int len, int &j0, int &j1, float &lo, float &hi) {
    const float c = ((float)u + 0.5f) * s;
    lo = c - 0.5f * f;
    hi = c + 0.5f * f;
    j0 = max((int)floorf(lo), 0);
    j1 = min((int)ceilf(hi), len);
}

template <bool NONNEG>
__global__ void __launch_bounds__(ZS_BATCH_THREADS) zs_batch_kernel(const __grid_constant__ ZsBatchArgs a) {
    extern __shared__ __align__(16) float zs_batch_lut[];      // [code][64], lanes 32..63 unused
    for (int i = threadIdx.x; i < 256 * 32; i += blockDim.x) zs_batch_lut[(i >> 5) * 64 + (i & 31)] = zs_srgb_decode_lut[i >> 5];
    __syncthreads();
    const unsigned char *lut = reinterpret_cast<const unsigned char *>(zs_batch_lut);
    const int lane = threadIdx.x & 31;
    const uint32_t lane4 = (uint32_t)lane << 2;
    const int warps = (int)(gridDim.x * (blockDim.x >> 5));
    const int total = a.prefix[a.n];
    int lo = 0;   // image of the current item: items only move forward, so scan from the last one
    for (int it = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); it < total; it += warps) {
        while (a.prefix[lo + 1] <= it) ++lo;
        const ZsBatchImage I = a.images[lo];
        const int segs = (I.tw + 31) >> 5, local = it - a.prefix[lo];
        const int v = local / segs, u = (local - v * segs) * 32 + lane;
        if (u >= I.tw) continue;
        uint32_t *out = reinterpret_cast<uint32_t *>(a.out + (size_t)lo * a.canvas * a.canvas * 4);
        int jx0, jx1, jy0, jy1;
        float lox, hix, loy, hiy;
        zs_box_window(u, I.sx, I.fx, I.width, jx0, jx1, lox, hix);
        zs_box_window(v, I.sy, I.fy, I.height, jy0, jy1, loy, hiy);
        // The weights of a window sum to its length clipped to the image; per row, source
        // texels go through the chain two at a time (the odd tail pairs with itself at weight 0).
        const float wsum = fmaxf(fminf(hix, (float)jx1) - fmaxf(lox, (float)jx0), 0.f) *
                           fmaxf(fminf(hiy, (float)jy1) - fmaxf(loy, (float)jy0), 0.f);
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int jy = jy0; jy < jy1; ++jy) {
            const float wy = fminf(hiy, (float)jy + 1.f) - fmaxf(loy, (float)jy);
            if (wy <= 0.f) continue;
            const uint32_t *row = reinterpret_cast<const uint32_t *>(I.ptr + (size_t)jy * I.width * 4);
            float2 sr = make_float2(0.f, 0.f), sg = sr, sb = sr, sa = sr;
            for (int jx = jx0; jx < jx1; jx += 2) {
                const bool two = jx + 1 < jx1;
                const uint32_t w0 = __ldg(row + jx), w1 = two ? __ldg(row + jx + 1) : w0;
                const float2 wx = make_float2(
                    fmaxf(fminf(hix, (float)jx + 1.f) - fmaxf(lox, (float)jx), 0.f),
                    two ? fmaxf(fminf(hix, (float)jx + 2.f) - fmaxf(lox, (float)jx + 1.f), 0.f) : 0.f);
                float2 r, g, b;
                zs_batch_chain2<NONNEG>(w0, w1, lut, lane4, a, r, g, b);
                const float2 al = make_float2((float)(w0 >> 24) * (1.0f / 255.0f), (float)(w1 >> 24) * (1.0f / 255.0f));
                sr = __ffma2_rn(wx, r, sr);
                sg = __ffma2_rn(wx, g, sg);
                sb = __ffma2_rn(wx, b, sb);
                sa = __ffma2_rn(wx, al, sa);
            }
            acc.x = fmaf(wy, sr.x + sr.y, acc.x);
            acc.y = fmaf(wy, sg.x + sg.y, acc.y);
            acc.z = fmaf(wy, sb.x + sb.y, acc.z);
            acc.w = fmaf(wy, sa.x + sa.y, acc.w);
        }
        const float inv = wsum > 0.f ? 1.0f / wsum : 0.f;
        const uint32_t code = zs_enc_srgb8(zs_srgb_encode_tab, acc.x * inv) | (zs_enc_srgb8(zs_srgb_encode_tab, acc.y * inv) << 8) |
                              (zs_enc_srgb8(zs_srgb_encode_tab, acc.z * inv) << 16) | (zs_unorm8(acc.w * inv) << 24);
        out[(size_t)(I.y0 + v) * a.canvas + I.x0 + u] = code;
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
    // Work items: 32 adjacent fitted pixels of one row.
    std::vector<int32_t> prefix(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) {
        const int64_t items = (int64_t)host[i].th * ((host[i].tw + 31) / 32);
        if ((int64_t)prefix[i] + items > INT32_MAX) {
            set_last_error("zs_batch_thumbnails: too many output pixels in one batch");
            return ZS_ERR_INVALID_ARG;
        }
        prefix[i + 1] = prefix[i] + (int32_t)items;
    }
    // Scratch: image table + item prefix table, kept with the executable.
    const size_t table_bytes = (sizeof(ZsBatchImage) * n + 255) & ~(size_t)255;
    const size_t bytes = table_bytes + sizeof(int32_t) * (n + 1);
    if (chain->batch_bytes < bytes) {
        if (chain->batch_scratch) cudaFree(chain->batch_scratch);
        chain->batch_scratch = nullptr;
        chain->batch_bytes = 0;
        cudaError_t e = cudaMalloc(&chain->batch_scratch, bytes);
        if (e != cudaSuccess) {
            set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
            return ZS_ERR_OUT_OF_MEMORY;
        }
        chain->batch_bytes = bytes;
    }
    uint8_t *scratch = (uint8_t *)chain->batch_scratch;
    ZsBatchImage *table = (ZsBatchImage *)scratch;
    int32_t *dprefix = (int32_t *)(scratch + table_bytes);
    cudaError_t e = cudaMemcpyAsync(table, host.data(), sizeof(ZsBatchImage) * n, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dprefix, prefix.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, stream);
    // Transparent margins: zero every canvas, the kernel writes the fitted pixels.
    if (e == cudaSuccess) e = cudaMemsetAsync(out, 0, (size_t)n * canvas * canvas * 4, stream);
    if (e != cudaSuccess) {
        set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    ZsBatchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.images = table;
    a.prefix = dprefix;
    a.out = (uint8_t *)out;
    a.n = (int)n;
    a.canvas = (int)canvas;
    a.flags = cs->chain.flags;
    std::memcpy(a.m, cs->chain.m, sizeof(a.m));
    std::memcpy(a.m2, cs->chain.m2, sizeof(a.m2));
    auto kernel = (a.flags & ZS_CHAIN_CBRT_NONNEG) ? zs_batch_kernel<true> : zs_batch_kernel<false>;
    const size_t smem = 256 * 64 * sizeof(float);
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, ZS_BATCH_THREADS, smem);
    if (e != cudaSuccess) {
        set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    if (per_sm < 1) per_sm = 1;
    long long blocks = (long long)chain->sm_count * per_sm;
    const long long need = ((long long)prefix[n] + ZS_BATCH_THREADS / 32 - 1) / (ZS_BATCH_THREADS / 32);
    if (blocks > need) blocks = need;
    if (blocks < 1) return ZS_OK;
    kernel<<<(unsigned)blocks, ZS_BATCH_THREADS, smem, stream>>>(a);
    g_kernel_launches.fetch_add(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    return ZS_OK;
}

}  // namespace zs

ZS_TU_HOOKS(batch)
