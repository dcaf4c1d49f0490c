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
    const int64_t n = (int64_t)a.width * a.height;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        const int y = (int)(i / a.width);
        const int x = (int)(i - (int64_t)y * a.width);
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

namespace zs {

cudaError_t launch_layers(const ZsLayersArgs &args, int sm_count, cudaStream_t stream) {
    const int64_t n = (int64_t)args.width * args.height;
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    const int64_t cap = (int64_t)(sm_count > 0 ? sm_count : 148) * 8;
    if (blocks > cap) blocks = cap;
    zs_layers_kernel<<<(unsigned)blocks, 256, 0, stream>>>(args);
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

}  // namespace zs
