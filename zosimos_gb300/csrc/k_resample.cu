// k_resample.cu -- both passes of a separable resample in one tiled, pipelined launch.
//
// resize_filtered (Lanczos-3 / box / triangle, FP64-normalised weights) as one kernel.
// Each CTA owns output tiles of 64 columns x TH rows (TH = 8, 16 or 32, chosen from the
// vertical scale so that there are several tiles per CTA slot).  A tile's source rows
// stream through shared memory in batches of ZS_RS_RB rows:
//
//   * one thread issues `cp.async.bulk` copies of the raw texel bytes of each row
//     segment the tile's filter windows touch, completing on a per-stage mbarrier; the
//     copies run `stages` batches ahead of the consumers and continue across tile
//     boundaries, so HBM reads are always in flight;
//   * every thread filters horizontally (decode from shared memory, FP32 FMAs over the
//     column's taps) and writes one filtered texel per (row, column) of the batch;
//   * after one barrier, each thread accumulates the filtered rows into the FP32
//     registers of the output rows whose vertical window contains them.
//
// The horizontally filtered intermediate never leaves the SM.  The tile's source
// segment starts at a 16-byte boundary (rounded down; the remainder is skipped when
// reading), so the bulk copies need a 16-byte aligned base and row stride; otherwise all
// threads stage the rows with plain loads.
//
// Every mbarrier wait is bounded (ZS_RS_WAIT_NS of global time): a wait that gives up
// sets ZS_DEVSTAT_WAIT_TIMEOUT in the device status word, the CTA waits (again bounded)
// for the copies it still has in flight and returns.
#include "zs_device.cuh"
#include "zs_kernels.h"
#include "zs_ptx.cuh"

#define ZS_RS_THREADS 256
#define ZS_RS_GROUPS (ZS_RS_THREADS / ZS_RS_TW)   // 4 row groups of 64 columns
#define ZS_RS_HP (ZS_RS_TW + 1)                   // filtered-row pitch (float4): no bank conflicts
static_assert(ZS_RS_RB == 8 && ZS_RS_THREADS == 256 && ZS_RS_TW == 64, "8 warps x (8 rows x 8 columns)");

namespace {

// Geometry of one output tile: its source column segment and source row range.
struct RsTile {
    int x0, y0, x1, y1;   // inclusive output corners
    int cs0, L;           // first source column, source columns
    int rs0, rs1;         // source rows [rs0, rs1)
};

__device__ __forceinline__ RsTile zs_rs_tile(const ZsRasterArgs &a, int tile, int tiles_x, int th) {
    RsTile t;
    t.x0 = (tile % tiles_x) * ZS_RS_TW;
    t.y0 = (tile / tiles_x) * th;
    t.x1 = min(t.x0 + ZS_RS_TW, a.width) - 1;
    t.y1 = min(t.y0 + th, a.height) - 1;
    t.cs0 = a.index_x[t.x0];
    t.L = a.index_x[t.x1] + a.index_y[t.x1] - t.cs0;
    t.rs0 = a.vfirst[t.y0];
    t.rs1 = a.vfirst[t.y1] + a.vcount[t.y1];
    return t;
}

// Source-kind specialisations of the texel decode from shared memory.
enum { ZS_RSK_GENERIC = 0, ZS_RSK_F16X4 = 1 };

template <int SK>
__device__ __forceinline__ float4 zs_rs_texel(const uint8_t *p, const ZsFormat &f) {
    if (SK == ZS_RSK_F16X4) {
        const uint2 v = *(const uint2 *)p;
        const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&v.x));
        const float2 hi = __half22float2(*reinterpret_cast<const __half2 *>(&v.y));
        return make_float4(lo.x, lo.y, hi.x, hi.y);
    }
    return zs_decode_raw(f, zs_load_raw(p, f.bpp));
}

__device__ __forceinline__ void zs_rs_fma(float4 &h, float w, float4 v) {
    h.x = fmaf(w, v.x, h.x); h.y = fmaf(w, v.y, h.y);
    h.z = fmaf(w, v.z, h.z); h.w = fmaf(w, v.w, h.w);
}

__device__ __forceinline__ float4 zs_rs_h2f4(uint32_t lo, uint32_t hi) {
    const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&lo));
    const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&hi));
    return make_float4(a.x, a.y, b.x, b.y);
}

// One horizontally filtered texel: taps p[0 .. cnt) (texels of `bpp` bytes) weighted by
// w[0 .. cnt), accumulated in tap order.  RGBA16F reads two texels per 16-byte load once
// the address is 16-byte aligned.
template <int SK>
__device__ __forceinline__ float4 zs_rs_hfilter(const uint8_t *p, const float *w, int cnt, const ZsFormat &f) {
    float4 h = make_float4(0.f, 0.f, 0.f, 0.f);
    if (SK == ZS_RSK_F16X4) {
        int k = 0;
        if (cnt > 0 && ((uintptr_t)p & 15) != 0) {
            const uint2 v = *(const uint2 *)p;
            zs_rs_fma(h, w[0], zs_rs_h2f4(v.x, v.y));
            k = 1;
        }
#pragma unroll 2
        for (; k + 1 < cnt; k += 2) {
            const uint4 v = *(const uint4 *)(p + k * 8);
            zs_rs_fma(h, w[k], zs_rs_h2f4(v.x, v.y));
            zs_rs_fma(h, w[k + 1], zs_rs_h2f4(v.z, v.w));
        }
        if (k < cnt) {
            const uint2 v = *(const uint2 *)(p + k * 8);
            zs_rs_fma(h, w[k], zs_rs_h2f4(v.x, v.y));
        }
        return h;
    }
    const int bpp = f.bpp;
    for (int k = 0; k < cnt; ++k) zs_rs_fma(h, w[k], zs_rs_texel<SK>(p + k * bpp, f));
    return h;
}

}  // namespace

template <int RPT, int SK>
__global__ void __launch_bounds__(ZS_RS_THREADS, 2) zs_resample2d_kernel(const __grid_constant__ ZsRasterArgs a) {
    constexpr int TH = RPT * ZS_RS_GROUPS;
    extern __shared__ __align__(16) uint8_t zs_rs_smem[];
    const ZsSource &s0 = a.src[0];
    const int bpp = s0.fmt.bpp;
    const int NS = a.stages;
    const int rowbytes = ZS_RS_ROWBYTES(a.max_span, bpp);                        // = 16 (mod 128)
    const int hstride = a.taps | 1;                                               // odd: no bank conflicts
    uint8_t *stage_base = zs_rs_smem;                                             // [NS][RB][rowbytes]
    float4 *hrow = (float4 *)(zs_rs_smem + (size_t)NS * ZS_RS_RB * rowbytes);     // [2][RB][HP]
    float *hws = (float *)(hrow + 2 * ZS_RS_RB * ZS_RS_HP);                       // [TW][hstride]
    float *vws = hws + ((ZS_RS_TW * hstride + 3) & ~3);                           // [TH][vtaps]
    uint64_t *bars = (uint64_t *)(vws + ((TH * a.vtaps + 3) & ~3));               // [NS]
    const int tiles_x = (a.width + ZS_RS_TW - 1) / ZS_RS_TW;
    const int tiles = tiles_x * ((a.height + TH - 1) / TH);
    // Vertical phase: one column and RPT output rows per thread.
    const int col = threadIdx.x % ZS_RS_TW;
    const int rgrp = threadIdx.x / ZS_RS_TW;
    // Horizontal phase: a warp filters 8 rows x 8 columns, lane = (row, column group); the
    // staged rows are 16 (mod 128) bytes apart, so the 8 rows of one column hit 8
    // different bank groups.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int hb = lane & 7;
    const int hc0 = warp * 8 + (lane >> 3), hc1 = hc0 + 4;
    const bool bulk = ((uintptr_t)s0.ptr & 15) == 0 && (s0.stride & 15) == 0;
    const bool producer = threadIdx.x == 0;

    // Producer cursor (thread 0): the next batch to copy, in the consumers' order.
    int ptile = blockIdx.x, pbi = 0, pcached = -1;
    uint32_t issued = 0;
    RsTile pt;
    auto issue_next = [&]() {
        while (ptile < tiles) {
            if (pcached != ptile) {
                pt = zs_rs_tile(a, ptile, tiles_x, TH);
                pcached = ptile;
            }
            const int nbt = (pt.rs1 - pt.rs0 + ZS_RS_RB - 1) / ZS_RS_RB;
            if (pbi < nbt) {
                const int stage = (int)(issued % (uint32_t)NS);
                const uint32_t bar = zs_smem_addr(bars + stage);
                const int r0 = pt.rs0 + pbi * ZS_RS_RB;
                const int nb = min(ZS_RS_RB, pt.rs1 - r0);
                const int64_t cb = ((int64_t)pt.cs0 * bpp) & ~(int64_t)15;
                const uint32_t size = (uint32_t)((pt.cs0 * (int64_t)bpp - cb + (int64_t)pt.L * bpp + 15) & ~(int64_t)15);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                zs_mbar_expect_tx(bar, size * (uint32_t)nb);
                const uint32_t dst = zs_smem_addr(stage_base + (size_t)stage * ZS_RS_RB * rowbytes);
                for (int b = 0; b < nb; ++b)
                    zs_bulk_g2s(dst + (uint32_t)(b * rowbytes), s0.ptr + (int64_t)(r0 + b) * s0.stride + cb, size, bar);
                ++issued;
                ++pbi;
                return;
            }
            ptile += gridDim.x;
            pbi = 0;
        }
    };

    if (bulk) {
        if (producer) {
            for (int s = 0; s < NS; ++s) zs_mbar_init(zs_smem_addr(bars + s), 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
        if (producer)
            for (int s = 0; s < NS; ++s) issue_next();
    }

    uint32_t g = 0;   // batches consumed by this CTA
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const RsTile t = zs_rs_tile(a, tile, tiles_x, TH);
        const int ox = t.x0 + col;
        const bool colok = ox <= t.x1;
        const int shift = bulk ? (int)(((int64_t)t.cs0 * bpp) & 15) : 0;
        int hf0 = 0, hn0 = 0, hf1 = 0, hn1 = 0;
        if (t.x0 + hc0 <= t.x1) {
            hf0 = a.index_x[t.x0 + hc0] - t.cs0;
            hn0 = a.index_y[t.x0 + hc0];
        }
        if (t.x0 + hc1 <= t.x1) {
            hf1 = a.index_x[t.x0 + hc1] - t.cs0;
            hn1 = a.index_y[t.x0 + hc1];
        }
        // The tile's filter weights, staged once (the previous tile's readers are done).
        __syncthreads();
        for (int i = threadIdx.x; i < ZS_RS_TW * a.taps; i += ZS_RS_THREADS) {
            const int c = i / a.taps, k = i - c * a.taps;
            hws[c * hstride + k] = t.x0 + c <= t.x1 ? __ldg(a.weights + (int64_t)t.x0 * a.taps + i) : 0.f;
        }
        for (int i = threadIdx.x; i < TH * a.vtaps; i += ZS_RS_THREADS) {
            const int r = i / a.vtaps;
            vws[i] = t.y0 + r <= t.y1 ? __ldg(a.vweights + (int64_t)t.y0 * a.vtaps + i) : 0.f;
        }
        __syncthreads();
        int vf[RPT], vc[RPT];
        float4 acc[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            const int oy = t.y0 + rgrp + j * ZS_RS_GROUPS;
            vf[j] = oy <= t.y1 ? a.vfirst[oy] : 0;
            vc[j] = oy <= t.y1 ? a.vcount[oy] : 0;
            acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        const int nbt = (t.rs1 - t.rs0 + ZS_RS_RB - 1) / ZS_RS_RB;
        for (int bi = 0; bi < nbt; ++bi, ++g) {
            const int rs = t.rs0 + bi * ZS_RS_RB;
            const int nb = min(ZS_RS_RB, t.rs1 - rs);
            const int stage = (int)(g % (uint32_t)NS);
            const uint8_t *sb = stage_base + (size_t)stage * ZS_RS_RB * rowbytes;
            bool timed_out = false;
            if (bulk) {
                timed_out = !zs_mbar_wait(zs_smem_addr(bars + stage), (g / (uint32_t)NS) & 1u);
            } else {
                // Plain staging: every thread copies texels of the batch's rows.
                uint8_t *sw = stage_base + (size_t)stage * ZS_RS_RB * rowbytes;
                for (int i = threadIdx.x; i < nb * t.L; i += ZS_RS_THREADS) {
                    const int b = i / t.L, c = i - b * t.L;
                    const uint8_t *gp = s0.ptr + (int64_t)(rs + b) * s0.stride + (int64_t)(t.cs0 + c) * bpp;
                    zs_store_raw(sw + b * rowbytes + c * bpp, bpp, zs_load_raw(gp, bpp));
                }
                __syncthreads();
            }
            float4 *hr = hrow + (g & 1u) * (ZS_RS_RB * ZS_RS_HP);
            if (!timed_out && hb < nb) {
                const uint8_t *rp = sb + hb * rowbytes + shift;
                if (hn0 > 0) hr[hb * ZS_RS_HP + hc0] = zs_rs_hfilter<SK>(rp + hf0 * bpp, hws + hc0 * hstride, hn0, s0.fmt);
                if (hn1 > 0) hr[hb * ZS_RS_HP + hc1] = zs_rs_hfilter<SK>(rp + hf1 * bpp, hws + hc1 * hstride, hn1, s0.fmt);
            }
            if (__syncthreads_or(timed_out)) {
                // Give up: record it, let the copies still in flight land, and return.
                if (producer) {
                    atomicOr(&zs_device_status_word, ZS_DEVSTAT_WAIT_TIMEOUT);
                    for (uint32_t j = g; j < issued; ++j)
                        zs_mbar_wait(zs_smem_addr(bars + (j % (uint32_t)NS)), (j / (uint32_t)NS) & 1u);
                }
                return;
            }
            if (bulk && producer) issue_next();
            if (colok) {
                // Each output row takes the filtered rows of this batch inside its window.
#pragma unroll
                for (int j = 0; j < RPT; ++j) {
                    const int lo = max(rs, vf[j]), hi = min(rs + nb, vf[j] + vc[j]);
                    const float *vw = vws + (rgrp + j * ZS_RS_GROUPS) * a.vtaps;
                    for (int sy = lo; sy < hi; ++sy) {
                        const float w = vw[sy - vf[j]];
                        const float4 h = hr[(sy - rs) * ZS_RS_HP + col];
                        acc[j].x = fmaf(w, h.x, acc[j].x); acc[j].y = fmaf(w, h.y, acc[j].y);
                        acc[j].z = fmaf(w, h.z, acc[j].z); acc[j].w = fmaf(w, h.w, acc[j].w);
                    }
                }
            }
        }
        if (colok) {
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const int oy = t.y0 + rgrp + j * ZS_RS_GROUPS;
                if (oy > t.y1) continue;
                float4 r = acc[j], r2 = make_float4(0.f, 0.f, 0.f, 0.f);
                zs_run_program(a.prog, a.fmts, r, r2);
                uint8_t *dp = a.dst + (int64_t)oy * a.dst_stride + (int64_t)ox * a.dst_fmt.bpp;
                zs_store_raw(dp, a.dst_fmt.bpp, zs_encode_raw(a.dst_fmt, r));
            }
        }
    }
}

namespace zs {

namespace {

// Shared memory of one CTA for `stages` staged batches.
size_t rs_smem_bytes(const ZsRasterArgs &a, int stages) {
    const size_t rowbytes = (size_t)ZS_RS_ROWBYTES(a.max_span, a.src[0].fmt.bpp);
    const size_t hw = (size_t)((ZS_RS_TW * (a.taps | 1) + 3) & ~3), vw = (size_t)((a.tile_rows * a.vtaps + 3) & ~3);
    return (size_t)stages * ZS_RS_RB * rowbytes + 2 * ZS_RS_RB * ZS_RS_HP * sizeof(float4) + (hw + vw) * sizeof(float) +
           stages * sizeof(uint64_t);
}

template <int RPT, int SK>
cudaError_t launch_rs(const ZsRasterArgs &args, size_t smem, int sm_count, cudaStream_t stream) {
    auto kern = zs_resample2d_kernel<RPT, SK>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const int th = RPT * ZS_RS_GROUPS;
    const int tiles = ((args.width + ZS_RS_TW - 1) / ZS_RS_TW) * ((args.height + th - 1) / th);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, ZS_RS_THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int blocks = (sm_count > 0 ? sm_count : 148) * per_sm;
    if (blocks > tiles) blocks = tiles;
    kern<<<blocks, ZS_RS_THREADS, smem, stream>>>(args);
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

template <int SK>
cudaError_t launch_rs_rows(const ZsRasterArgs &a, size_t smem, int sm_count, cudaStream_t stream) {
    switch (a.tile_rows) {
    case 8: return launch_rs<2, SK>(a, smem, sm_count, stream);
    case 16: return launch_rs<4, SK>(a, smem, sm_count, stream);
    case 32: return launch_rs<8, SK>(a, smem, sm_count, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_resample2d(const ZsRasterArgs &args, int sm_count, cudaStream_t stream) {
    if (resample_tc_usable(args)) return launch_resample_tc(args, sm_count, stream);
    ZsRasterArgs a = args;
    if (a.max_span < 1 || a.src[0].fmt.bpp < 1) return cudaErrorInvalidValue;
    const size_t one = rs_smem_bytes(a, 1) - rs_smem_bytes(a, 0);
    int stages = (int)(ZS_RS_STAGE_BUDGET / one);
    stages = stages < 2 ? 2 : (stages > 4 ? 4 : stages);
    a.stages = stages;
    const size_t smem = rs_smem_bytes(a, stages);
    if (smem > ZS_RS_MAX_SMEM) return cudaErrorInvalidValue;
    if (a.src[0].fmt.fast == ZS_FAST_F16X4) return launch_rs_rows<ZS_RSK_F16X4>(a, smem, sm_count, stream);
    return launch_rs_rows<ZS_RSK_GENERIC>(a, smem, sm_count, stream);
}

}  // namespace zs

ZS_TU_HOOKS(resample)
