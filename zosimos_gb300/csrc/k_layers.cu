// k_layers.cu -- a stack of affine-transformed layers blended in one HBM pass.
//
// The reference would run, per layer, an affine paint of the layer onto a canvas
// (copy.frag through box.vert, lib/zosimos/src/command.rs:2642-2678) and a blend of
// the result onto the accumulated image (blend is UNIMPLEMENTED upstream,
// command.rs:1509-1519) -- two full-image passes and two stored intermediates per
// layer.  Here every output pixel walks the layer list once: inverse-map the pixel
// centre into the layer (same fixed-order f32 arithmetic as the affine producer),
// sample (nearest or bilinear, clamp-to-edge taps, the layer's canvas colour outside
// it), optionally quantise to the declared texel, blend onto an FP32 accumulator held
// in registers.  Reads: each layer's footprint once (plus bilinear neighbours from
// L1/L2); writes: the output once.
#include "zs_device.cuh"
#include "zs_kernels.h"

__device__ __forceinline__ float4 zs_layer_sample(const ZsLayer &L, int x, int y) {
    float qx, qy;
    zs_affine_map(L.inv, x, y, qx, qy);
    const bool inside = qx >= 0.0f && qx < (float)L.width && qy >= 0.0f && qy < (float)L.height;
    if (!inside) return make_float4(L.canvas[0], L.canvas[1], L.canvas[2], L.canvas[3]);
    ZsSource s;
    s.ptr = L.ptr;
    s.stride = L.stride;
    s.width = L.width;
    s.height = L.height;
    s.fmt = L.fmt;
    if (!L.bilinear) {
        int ix = min((int)floorf(qx), L.width - 1), iy = min((int)floorf(qy), L.height - 1);
        return zs_load_px(s, ix, iy);
    }
    float tx = qx - 0.5f, ty = qy - 0.5f;
    float fx0 = floorf(tx), fy0 = floorf(ty);
    float fx = tx - fx0, fy = ty - fy0;
    int x0 = (int)fx0, y0 = (int)fy0;
    int xa = zs_clampi(x0, 0, L.width - 1), xb = zs_clampi(x0 + 1, 0, L.width - 1);
    int ya = zs_clampi(y0, 0, L.height - 1), yb = zs_clampi(y0 + 1, 0, L.height - 1);
    float4 top = zs_lerp4(zs_load_px(s, xa, ya), zs_load_px(s, xb, ya), fx);
    float4 bot = zs_lerp4(zs_load_px(s, xa, yb), zs_load_px(s, xb, yb), fx);
    return zs_lerp4(top, bot, fy);
}

__global__ void __launch_bounds__(256) zs_layers_kernel(const __grid_constant__ ZsLayersArgs a) {
    // 32 x 8 pixel tiles (8 x 4 per warp): each warp's samples of a layer fall into a
    // compact footprint of that layer.
    const int tiles_x = (a.width + 31) >> 5;
    const int64_t n = (int64_t)tiles_x * ((a.height + 7) >> 3) * 256;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        int x, y;
        zs_tile_pixel(i, tiles_x, x, y);
        if (x >= a.width || y >= a.height) continue;
        float4 acc = a.has_base ? zs_load_px(a.base, x, y)
                                : make_float4(a.base_color[0], a.base_color[1], a.base_color[2], a.base_color[3]);
        for (int l = 0; l < a.nlayers; ++l) {
            const ZsLayer &L = a.layers[l];
            float4 s = zs_layer_sample(L, x, y);
            if (L.quant_sample) s = zs_decode_raw(a.fmts[L.quant_sample - 1], zs_encode_raw(a.fmts[L.quant_sample - 1], s));
            zs_blend_px(acc, s, L.mode, L.straight);
            if (L.quant_acc) acc = zs_decode_raw(a.fmts[L.quant_acc - 1], zs_encode_raw(a.fmts[L.quant_acc - 1], acc));
        }
        float4 r2 = make_float4(0.f, 0.f, 0.f, 0.f);
        zs_run_program(a.prog, a.fmts, acc, r2);
        uint8_t *dp = a.dst + (int64_t)y * a.dst_stride + (int64_t)x * a.dst_fmt.bpp;
        zs_store_raw(dp, a.dst_fmt.bpp, zs_encode_raw(a.dst_fmt, acc));
    }
}

// The common stack: RGBA16F layers sampled bilinearly through affine inverses, premultiplied
// operands, no lossy quantisation (FP32 quantisation is the identity).  Same arithmetic, in
// the same order, as zs_layer_sample + zs_blend_px, without the per-tap format dispatch; each
// thread takes four pixels four rows apart so that a layer's parameters are read once per
// four pixels and four samples are in flight.  Tiles of 32 x 32 pixels, 8 x 16 per warp.
#define ZS_LAY_PX 4   // pixels per thread, four rows apart
__global__ void __launch_bounds__(256) zs_layers_f16_kernel(const __grid_constant__ ZsLayersArgs a) {
    const int tiles_x = (a.width + 31) >> 5;
    const int64_t n = (int64_t)tiles_x * ((a.height + 8 * ZS_LAY_PX - 1) / (8 * ZS_LAY_PX)) * 256;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        const int64_t tile = i >> 8;
        const int t = (int)(i & 255), w = t >> 5, l = t & 31;
        const int ty = (int)(tile / tiles_x), tx = (int)(tile - (int64_t)ty * tiles_x);
        const int x = (tx << 5) + ((w & 3) << 3) + (l & 7);
        const int y0 = ty * (8 * ZS_LAY_PX) + (w >> 2) * (4 * ZS_LAY_PX) + (l >> 3);
        if (x >= a.width || y0 >= a.height) continue;
        float4 acc[ZS_LAY_PX];
#pragma unroll
        for (int p = 0; p < ZS_LAY_PX; ++p)
            acc[p] = a.has_base ? zs_load_px(a.base, x, min(y0 + 4 * p, a.height - 1))
                                : make_float4(a.base_color[0], a.base_color[1], a.base_color[2], a.base_color[3]);
        const float cx = (float)x + 0.5f;
        for (int li = 0; li < a.nlayers; ++li) {
            const ZsLayer &L = a.layers[li];
            const float i0 = L.inv[0], i1 = L.inv[1], i2 = L.inv[2], i3 = L.inv[3], i4 = L.inv[4], i5 = L.inv[5];
            const float fw = (float)L.width, fh = (float)L.height;
            const uint8_t *base = L.ptr;
            const int64_t stride = L.stride;
            float4 s[ZS_LAY_PX];
#pragma unroll
            for (int p = 0; p < ZS_LAY_PX; ++p) {
                const float cy = (float)(y0 + 4 * p) + 0.5f;
                const float qx = fmaf(i0, cx, fmaf(i1, cy, i2));
                const float qy = fmaf(i3, cx, fmaf(i4, cy, i5));
                if (qx >= 0.0f && qx < fw && qy >= 0.0f && qy < fh) {
                    const float txf = qx - 0.5f, tyf = qy - 0.5f;
                    const float fx0 = floorf(txf), fy0 = floorf(tyf);
                    const float fx = txf - fx0, fy = tyf - fy0;
                    const int x0 = (int)fx0, y0i = (int)fy0;
                    // 0 <= q < size puts the first tap in [-1, size - 1]: one bound per tap.
                    const int xa = max(x0, 0), xb = min(x0 + 1, L.width - 1);
                    const int ya = max(y0i, 0), yb = min(y0i + 1, L.height - 1);
                    const uint8_t *ra = base + (int64_t)ya * stride, *rb = base + (int64_t)yb * stride;
                    const float4 t00 = zs_h4(__ldg((const uint2 *)(ra + (int64_t)xa * 8)));
                    const float4 t01 = zs_h4(__ldg((const uint2 *)(ra + (int64_t)xb * 8)));
                    const float4 t10 = zs_h4(__ldg((const uint2 *)(rb + (int64_t)xa * 8)));
                    const float4 t11 = zs_h4(__ldg((const uint2 *)(rb + (int64_t)xb * 8)));
                    s[p] = zs_lerp4(zs_lerp4(t00, t01, fx), zs_lerp4(t10, t11, fx), fy);
                } else {
                    s[p] = make_float4(L.canvas[0], L.canvas[1], L.canvas[2], L.canvas[3]);
                }
            }
            const uint32_t mode = L.mode;
#pragma unroll
            for (int p = 0; p < ZS_LAY_PX; ++p) zs_blend_px(acc[p], s[p], mode, 0);
        }
#pragma unroll
        for (int p = 0; p < ZS_LAY_PX; ++p) {
            const int y = y0 + 4 * p;
            if (y >= a.height) break;
            uint8_t *dp = a.dst + (int64_t)y * a.dst_stride + (int64_t)x * a.dst_fmt.bpp;
            if (zs_plain_f16_out(a.prog, a.dst_fmt)) {
                zs_store_f16x4(dp, acc[p]);
                continue;
            }
            float4 r = acc[p], r2 = make_float4(0.f, 0.f, 0.f, 0.f);
            zs_run_program(a.prog, a.fmts, r, r2);
            zs_store_raw(dp, a.dst_fmt.bpp, zs_encode_raw(a.dst_fmt, r));
        }
    }
}

namespace zs {

cudaError_t launch_layers(const ZsLayersArgs &args, int sm_count, cudaStream_t stream) {
    if (args.width <= 0 || args.height <= 0) return cudaSuccess;
    if (args.f16_bilinear) {
        int64_t blocks = (int64_t)((args.width + 31) / 32) * ((args.height + 8 * ZS_LAY_PX - 1) / (8 * ZS_LAY_PX));
        const int64_t cap = (int64_t)(sm_count > 0 ? sm_count : 148) * 8;
        if (blocks > cap) blocks = cap;
        zs_layers_f16_kernel<<<(unsigned)blocks, 256, 0, stream>>>(args);
        g_kernel_launches.fetch_add(1);
        return cudaGetLastError();
    }
    int64_t blocks = (int64_t)((args.width + 31) / 32) * ((args.height + 7) / 8);
    const int64_t cap = (int64_t)(sm_count > 0 ? sm_count : 148) * 8;
    if (blocks > cap) blocks = cap;
    zs_layers_kernel<<<(unsigned)blocks, 256, 0, stream>>>(args);
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

}  // namespace zs

ZS_TU_HOOKS(layers)
