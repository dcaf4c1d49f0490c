// k_batch.cu -- many RGBA8 sRGB images of uneven sizes turned into thumbnails by one
// launch over a static work list (the reference's batch-reuse case runs one Executable per
// image, lib/zosimos/tests/loop.rs:84-95).
//
// Per image: decode -> the fused colour chain of a lowered Program (canonical form
// M_a, [cbrt], M_b, [cube], M_c, [clamp], M_d, linear result) -> box (area coverage)
// fit-resize so the long side is `canvas` -> centred inscribe on a transparent
// canvas x canvas image -> exact sRGB8 encode.  The canvases are zero-filled (the
// transparent margins) by one memset; the fitted pixels are cut into work items of 32
// output columns x `rows` output rows (1..16, chosen by the autotuner), one item per warp,
// taken by static striding
// over all images (no atomics, no barriers), so that every image's cost spreads over all warps.
//
// The colour chain is nonlinear, so it runs on every source texel before the box filter;
// the kernel is built so that each texel goes through it once:
//  * lane l owns output column u; its box window covers texels [j0, j1) of a source row, with
//    weight 1 inside and fractional weights only at the two ends;
//  * on a downscale the windows tile the row, so the last texel of lane l is the first texel
//    of lane l + 1: lane l + 1 computes it and hands its unweighted value over with a warp
//    shuffle, lane l applies its own edge weight;
//  * consecutive output rows share one source row: the horizontal sums of the last row of an
//    output row are kept in registers and reused by the next one;
//  * texels go through the chain two at a time in FP32x2 registers (decode from the
//    lane-replicated shared table, MUFU cube roots, the rank-1 Oklab L/C form when planned).
#include <cstring>
#include <vector>

#include "host/zs_host.hpp"
#include "zs_chain.cuh"
#include "zs_device.cuh"
#include "zs_kernels.h"

#define ZS_BATCH_THREADS 256
#define ZS_BATCH_ROWS_DEFAULT 1   // output rows per work item until the autotuner chose

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
    int32_t rows;              // output rows per work item
    float m2[4][9][2];         // the chain's matrices with every coefficient duplicated (f32x2 operands)
    float mb_v[3][2];          // ZS_CHAIN_MB_RANK1: M_b = d I + (1,1,1)^T v
    float mb_d[2];
};

// The canonical chain on two texels at once, linear result: decode through the
// lane-replicated shared table, FP32x2 matrix products, MUFU cube roots.
template <bool NONNEG, bool RANK1>
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
    if (RANK1) {
        const float2 *v = reinterpret_cast<const float2 *>(a.mb_v);
        const float2 d = *reinterpret_cast<const float2 *>(a.mb_d);
        const float2 t = __ffma2_rn(v[0], r, __ffma2_rn(v[1], g, __fmul2_rn(v[2], b)));
        r = __ffma2_rn(d, r, t);
        g = __ffma2_rn(d, g, t);
        b = __ffma2_rn(d, b, t);
    } else {
        zs_m3x2<false>(a.m2[1], r, g, b);
    }
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

// This lane's horizontally weighted sum of one source row (colour in xyz, alpha code sum in
// w): texels [j0, jend) through the chain, weight wfirst at j0, wlast at j1 - 1, 1 between;
// when `share`, texel j1 - 1 is the next lane's first texel and arrives by shuffle.  Every
// lane of the warp calls this together (the shuffles use the full mask).
template <bool NONNEG, bool RANK1>
__device__ __forceinline__ float4 zs_batch_row(const uint32_t *row, int j0, int jend, int j1, float wfirst, float wlast,
                                               bool share, const unsigned char *lut, uint32_t lane4,
                                               const ZsBatchArgs &a) {
    float2 sr = make_float2(0.f, 0.f), sg = sr, sb = sr, sa = sr;
    float4 first = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int jx = j0; jx < jend; jx += 2) {
        const bool two = jx + 1 < jend;
        const uint32_t w0 = __ldg(row + jx), w1 = two ? __ldg(row + jx + 1) : w0;
        float2 r, g, b;
        zs_batch_chain2<NONNEG, RANK1>(w0, w1, lut, lane4, a, r, g, b);
        const float2 al = make_float2(__uint2float_rn(w0 >> 24), __uint2float_rn(w1 >> 24));
        if (jx == j0) first = make_float4(r.x, g.x, b.x, al.x);
        const float2 wx = make_float2(jx == j0 ? wfirst : (jx == j1 - 1 ? wlast : 1.f),
                                      two ? (jx + 1 == j1 - 1 ? wlast : 1.f) : 0.f);
        sr = __ffma2_rn(wx, r, sr);
        sg = __ffma2_rn(wx, g, sg);
        sb = __ffma2_rn(wx, b, sb);
        sa = __ffma2_rn(wx, al, sa);
    }
    float4 rs = make_float4(sr.x + sr.y, sg.x + sg.y, sb.x + sb.y, sa.x + sa.y);
    const float nr = __shfl_down_sync(0xffffffffu, first.x, 1), ng = __shfl_down_sync(0xffffffffu, first.y, 1);
    const float nb = __shfl_down_sync(0xffffffffu, first.z, 1), na = __shfl_down_sync(0xffffffffu, first.w, 1);
    if (share) {
        rs.x = fmaf(wlast, nr, rs.x);
        rs.y = fmaf(wlast, ng, rs.y);
        rs.z = fmaf(wlast, nb, rs.z);
        rs.w = fmaf(wlast, na, rs.w);
    }
    return rs;
}

template <bool NONNEG, bool RANK1>
__global__ void __launch_bounds__(ZS_BATCH_THREADS, 3) zs_batch_kernel(const __grid_constant__ ZsBatchArgs a) {
    extern __shared__ __align__(16) float zs_batch_lut[];      // [code][64], lanes 32..63 unused
    for (int i = threadIdx.x; i < 256 * 8; i += blockDim.x) {
        const float d = zs_srgb_decode_lut[i >> 3];
        reinterpret_cast<float4 *>(zs_batch_lut)[(i >> 3) * 16 + (i & 7)] = make_float4(d, d, d, d);
    }
    __syncthreads();
    const unsigned char *lut = reinterpret_cast<const unsigned char *>(zs_batch_lut);
    const int lane = threadIdx.x & 31;
    const uint32_t lane4 = (uint32_t)lane << 2;
    const int warps = (int)(gridDim.x * (blockDim.x >> 5));
    const int total = a.prefix[a.n];
    int img = 0;   // image of the current item: items only move forward, so scan from the last one
    for (int it = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); it < total; it += warps) {
        while (a.prefix[img + 1] <= it) ++img;
        const ZsBatchImage I = a.images[img];
        const int strips = (I.tw + 31) >> 5, local = it - a.prefix[img];
        const int band = local / strips, u = (local - band * strips) * 32 + lane;
        const bool valid = u < I.tw;
        // Horizontal window of this lane (none for lanes past the fitted width).
        int jx0 = 0, jx1 = 0;
        float lox = 0.f, hix = 0.f;
        if (valid) zs_box_window(u, I.sx, I.fx, I.width, jx0, jx1, lox, hix);
        const int next_j0 = __shfl_down_sync(0xffffffffu, jx0, 1);
        const int next_valid = __shfl_down_sync(0xffffffffu, valid ? 1 : 0, 1);
        const bool share = I.sx >= 1.f && lane < 31 && valid && next_valid && next_j0 == jx1 - 1 && jx1 - 1 > jx0;
        const int jend = share ? jx1 - 1 : jx1;
        const float wfirst = fmaxf(fminf(hix, (float)jx0 + 1.f) - fmaxf(lox, (float)jx0), 0.f);
        const float wlast = fmaxf(fminf(hix, (float)jx1) - fmaxf(lox, (float)jx1 - 1.f), 0.f);
        const float wxsum = fmaxf(fminf(hix, (float)jx1) - fmaxf(lox, (float)jx0), 0.f);
        uint32_t *out = reinterpret_cast<uint32_t *>(a.out + (size_t)img * a.canvas * a.canvas * 4);
        const int v0 = band * a.rows, v1 = min(v0 + a.rows, I.th);
        int carry_row = -1;
        float4 carry = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int v = v0; v < v1; ++v) {
            int jy0, jy1;
            float loy, hiy;
            zs_box_window(v, I.sy, I.fy, I.height, jy0, jy1, loy, hiy);
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int jy = jy0; jy < jy1; ++jy) {
                const float wy = fmaxf(fminf(hiy, (float)jy + 1.f) - fmaxf(loy, (float)jy), 0.f);
                float4 rs = carry;
                if (jy != carry_row) {     // uniform across the warp
                    const uint32_t *row = reinterpret_cast<const uint32_t *>(I.ptr + (size_t)jy * I.width * 4);
                    rs = zs_batch_row<NONNEG, RANK1>(row, jx0, jend, jx1, wfirst, wlast, share, lut, lane4, a);
                    carry_row = jy;
                    carry = rs;
                }
                acc.x = fmaf(wy, rs.x, acc.x);
                acc.y = fmaf(wy, rs.y, acc.y);
                acc.z = fmaf(wy, rs.z, acc.z);
                acc.w = fmaf(wy, rs.w, acc.w);
            }
            if (!valid) continue;
            const float wsum = wxsum * fmaxf(fminf(hiy, (float)jy1) - fmaxf(loy, (float)jy0), 0.f);
            const float inv = wsum > 0.f ? 1.0f / wsum : 0.f;
            const uint32_t code = zs_enc_srgb8(zs_srgb_encode_tab, acc.x * inv) |
                                  (zs_enc_srgb8(zs_srgb_encode_tab, acc.y * inv) << 8) |
                                  (zs_enc_srgb8(zs_srgb_encode_tab, acc.z * inv) << 16) |
                                  (zs_unorm8(acc.w * inv * (1.0f / 255.0f)) << 24);
            out[(size_t)(I.y0 + v) * a.canvas + I.x0 + u] = code;
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
    // Work items: 32 output columns x `rows` output rows (the tuned height for this chain,
    // canvas and device when the autotuner has seen them).
    if (chain->batch_rows <= 0) {
        int tuned;
        if (tune_get(batch_tune_key(*chain, canvas, chain->device), tuned) && tuned >= 1 && tuned <= 16)
            chain->batch_rows = tuned;
    }
    const int rows = chain->batch_rows > 0 ? chain->batch_rows : ZS_BATCH_ROWS_DEFAULT;
    std::vector<int32_t> prefix(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) {
        const int64_t items = (int64_t)((host[i].th + rows - 1) / rows) * ((host[i].tw + 31) / 32);
        if ((int64_t)prefix[i] + items > INT32_MAX) {
            set_last_error("zs_batch_thumbnails: too many output pixels in one batch");
            return ZS_ERR_INVALID_ARG;
        }
        prefix[i + 1] = prefix[i] + (int32_t)items;
    }
    // Scratch: image table + item prefix table, kept with the executable, uploaded from a
    // pinned staging copy.  The previous batch of this executable must have finished with
    // both before they are rewritten.
    const size_t table_bytes = (sizeof(ZsBatchImage) * n + 255) & ~(size_t)255;
    const size_t bytes = table_bytes + sizeof(int32_t) * (n + 1);
    auto device_error = [](cudaError_t e) {
        set_last_error(std::string("zs_batch_thumbnails: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? ZS_ERR_OUT_OF_MEMORY : ZS_ERR_DEVICE;
    };
    cudaError_t e = cudaSuccess;
    if (chain->batch_done && (e = cudaEventSynchronize(chain->batch_done)) != cudaSuccess) return device_error(e);
    if (chain->batch_bytes < bytes) {
        if (chain->batch_scratch) cudaFree(chain->batch_scratch);
        if (chain->batch_staging) cudaFreeHost(chain->batch_staging);
        chain->batch_scratch = chain->batch_staging = nullptr;
        chain->batch_bytes = 0;
        if ((e = cudaMalloc(&chain->batch_scratch, bytes)) != cudaSuccess) return device_error(e);
        if ((e = cudaMallocHost(&chain->batch_staging, bytes)) != cudaSuccess) return device_error(e);
        chain->batch_bytes = bytes;
    }
    if (!chain->batch_done && (e = cudaEventCreateWithFlags(&chain->batch_done, cudaEventDisableTiming)) != cudaSuccess)
        return device_error(e);
    uint8_t *scratch = (uint8_t *)chain->batch_scratch, *staging = (uint8_t *)chain->batch_staging;
    std::memcpy(staging, host.data(), sizeof(ZsBatchImage) * n);
    std::memcpy(staging + table_bytes, prefix.data(), sizeof(int32_t) * (n + 1));
    if ((e = cudaMemcpyAsync(scratch, staging, bytes, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
        return device_error(e);
    ZsBatchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.images = (const ZsBatchImage *)scratch;
    a.prefix = (const int32_t *)(scratch + table_bytes);
    a.out = (uint8_t *)out;
    a.n = (int)n;
    a.canvas = (int)canvas;
    a.flags = cs->chain.flags;
    a.rows = rows;
    std::memcpy(a.m2, cs->chain.m2, sizeof(a.m2));
    std::memcpy(a.mb_v, cs->chain.mb_v, sizeof(a.mb_v));
    std::memcpy(a.mb_d, cs->chain.mb_d, sizeof(a.mb_d));
    const bool nonneg = (a.flags & ZS_CHAIN_CBRT_NONNEG) || !(a.flags & ZS_CHAIN_CBRT);
    const bool rank1 = (a.flags & ZS_CHAIN_MB_RANK1) != 0;
    auto kernel = nonneg ? (rank1 ? zs_batch_kernel<true, true> : zs_batch_kernel<true, false>)
                         : (rank1 ? zs_batch_kernel<false, true> : zs_batch_kernel<false, false>);
    const size_t smem = 256 * 64 * sizeof(float);
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, ZS_BATCH_THREADS, smem);
    if (e != cudaSuccess) return device_error(e);
    if (per_sm < 1) per_sm = 1;
    // The grid covers every SM: warps stride over the items of all images.
    long long blocks = (long long)chain->sm_count * per_sm;
    const long long need = ((long long)prefix[n] + ZS_BATCH_THREADS / 32 - 1) / (ZS_BATCH_THREADS / 32);
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
        // Transparent margins: zero every canvas, the kernel writes the fitted pixels.
        cudaError_t ce = cudaMemsetAsync(out, 0, (size_t)n * canvas * canvas * 4, stream);
        if (ce == cudaSuccess) {
            kernel<<<(unsigned)blocks, ZS_BATCH_THREADS, smem, stream>>>(a);
            ce = cudaGetLastError();
        }
        return ce;
    };
    if (!chain->batch_graph || chain->batch_key != key) {
        if (chain->batch_graph) cudaGraphExecDestroy(chain->batch_graph);
        chain->batch_graph = nullptr;
        chain->batch_key.clear();
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            // A stream that cannot be captured (the legacy default stream): launch directly.
            cudaGetLastError();
            if ((e = enqueue()) != cudaSuccess) return device_error(e);
            if ((e = cudaEventRecord(chain->batch_done, stream)) != cudaSuccess) return device_error(e);
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
        chain->batch_graph = ge;
        chain->batch_key = key;
    }
    if ((e = cudaGraphLaunch(chain->batch_graph, stream)) != cudaSuccess) return device_error(e);
    if ((e = cudaEventRecord(chain->batch_done, stream)) != cudaSuccess) return device_error(e);
    g_kernel_launches.fetch_add(1);
    return ZS_OK;
}

}  // namespace zs

ZS_TU_HOOKS(batch)
