// k_batch.cu -- many RGBA8 sRGB images of uneven sizes turned into thumbnails by one
// persistent launch over a device work queue (the reference's batch-reuse case runs one
// Executable per image, lib/zosimos/tests/loop.rs:84-95).
//
// Per image: decode -> the fused colour chain of a lowered Program (canonical form
// M_a, [cbrt], M_b, [cube], M_c, [clamp], M_d, linear result) -> box (area coverage)
// fit-resize so the long side is `canvas` -> centred inscribe on a transparent
// canvas x canvas image -> exact sRGB8 encode.  The canvas of image i is cut into
// work items of ZS_BATCH_ROWS rows; CTAs pull items with one atomicAdd each (no
// spinning, no inter-CTA waits), so the uneven cost of the images balances itself.
// Each thread computes output pixels directly from their source window: the box
// weights are separable and every source pixel in the window is decoded and pushed
// through the chain in FP32 registers.
#include <vector>

#include "host/zs_host.hpp"
#include "zs_device.cuh"
#include "zs_kernels.h"

#define ZS_BATCH_ROWS 4
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
    uint32_t *counter;         // work-queue head, zeroed before the launch
    uint8_t *out;
    int32_t n;
    int32_t canvas;
    int32_t items_per_image;
    int32_t flags;
    float m[4][9];
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

// Box (area coverage) window of output index u along one axis.
__device__ __forceinline__ void zs_box_window(int u, float s, float f, int len, int &j0, int &j1, float &lo, float &hi) {
    const float c = ((float)u + 0.5f) * s;
    lo = c - 0.5f * f;
    hi = c + 0.5f * f;
    j0 = max((int)floorf(lo), 0);
    j1 = min((int)ceilf(hi), len);
}

__global__ void __launch_bounds__(ZS_BATCH_THREADS) zs_batch_kernel(const __grid_constant__ ZsBatchArgs a) {
    __shared__ uint32_t item;
    const int total = a.n * a.items_per_image;
    const int cpx = a.canvas * ZS_BATCH_ROWS;
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(a.counter, 1u);
        __syncthreads();
        const int it = (int)item;
        __syncthreads();
        if (it >= total) break;
        const int img = it / a.items_per_image;
        const int band = it - img * a.items_per_image;
        const ZsBatchImage I = a.images[img];
        uint32_t *out = reinterpret_cast<uint32_t *>(a.out + (size_t)img * a.canvas * a.canvas * 4);
        for (int p = threadIdx.x; p < cpx; p += blockDim.x) {
            const int oy = band * ZS_BATCH_ROWS + p / a.canvas;
            const int ox = p % a.canvas;
            if (oy >= a.canvas) continue;
            const int u = ox - I.x0, v = oy - I.y0;
            uint32_t code = 0;   // transparent canvas
            if (u >= 0 && v >= 0 && u < I.tw && v < I.th) {
                int jx0, jx1, jy0, jy1;
                float lox, hix, loy, hiy;
                zs_box_window(u, I.sx, I.fx, I.width, jx0, jx1, lox, hix);
                zs_box_window(v, I.sy, I.fy, I.height, jy0, jy1, loy, hiy);
                float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
                float wsum = 0.f;
                for (int jy = jy0; jy < jy1; ++jy) {
                    const float wy = fminf(hiy, (float)jy + 1.f) - fmaxf(loy, (float)jy);
                    if (wy <= 0.f) continue;
                    const uint32_t *row = reinterpret_cast<const uint32_t *>(I.ptr + (size_t)jy * I.width * 4);
                    for (int jx = jx0; jx < jx1; ++jx) {
                        const float wx = fminf(hix, (float)jx + 1.f) - fmaxf(lox, (float)jx);
                        if (wx <= 0.f) continue;
                        const float wgt = wx * wy;
                        const float4 c = zs_batch_chain(__ldg(row + jx), a);
                        acc.x = fmaf(wgt, c.x, acc.x);
                        acc.y = fmaf(wgt, c.y, acc.y);
                        acc.z = fmaf(wgt, c.z, acc.z);
                        acc.w = fmaf(wgt, c.w, acc.w);
                        wsum += wgt;
                    }
                }
                const float inv = wsum > 0.f ? 1.0f / wsum : 0.f;
                code = zs_enc_srgb8(zs_srgb_encode_tab, acc.x * inv) | (zs_enc_srgb8(zs_srgb_encode_tab, acc.y * inv) << 8) |
                       (zs_enc_srgb8(zs_srgb_encode_tab, acc.z * inv) << 16) | (zs_unorm8(acc.w * inv) << 24);
            }
            out[(size_t)oy * a.canvas + ox] = code;
        }
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
    // Scratch: image table + work-queue counter, kept with the executable.
    const size_t bytes = sizeof(ZsBatchImage) * n + 256;
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
    uint32_t *counter = (uint32_t *)scratch;
    ZsBatchImage *table = (ZsBatchImage *)(scratch + 256);
    cudaError_t e = cudaMemcpyAsync(table, host.data(), sizeof(ZsBatchImage) * n, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) {
        set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    ZsBatchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.images = table;
    a.counter = counter;
    a.out = (uint8_t *)out;
    a.n = (int)n;
    a.canvas = (int)canvas;
    a.items_per_image = ((int)canvas + ZS_BATCH_ROWS - 1) / ZS_BATCH_ROWS;
    a.flags = cs->chain.flags;
    std::memcpy(a.m, cs->chain.m, sizeof(a.m));
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zs_batch_kernel, ZS_BATCH_THREADS, 0);
    if (per_sm < 1) per_sm = 1;
    long long blocks = (long long)chain->sm_count * per_sm;
    const long long items = (long long)n * a.items_per_image;
    if (blocks > items) blocks = items;
    zs_batch_kernel<<<(unsigned)blocks, ZS_BATCH_THREADS, 0, stream>>>(a);
    g_kernel_launches.fetch_add(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    return ZS_OK;
}

}  // namespace zs
