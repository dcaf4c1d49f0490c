// k_affine_tma.cu -- the affine bilinear gather of an RGBA16F image (command.rs:1636-1673, a
// rotation / scale of the source painted over the canvas) with each output tile's source
// footprint staged in shared memory by TMA.
//
// The gather kernel (zs_affine_f16_kernel) reads its four bilinear taps per pixel from
// global memory and is bound by their latency.  Here a CTA walks output tiles of 64 x 32
// pixels; for each tile the rectangle of source pixels its taps can touch (the inverse
// affine of the tile's corner pixel centres, one pixel of margin for rounding, clamped to
// the image, x rounded down to an even pixel for the 16-byte TMA alignment) arrives by one
// cp.async.bulk.tensor.2d copy into one of three shared buffers, the copies of the next two
// tiles in flight while the current one is computed.  The taps are then shared-memory loads; the
// arithmetic (map, coverage, clamp-to-edge taps, lerps, pixel program, encode) is that of
// zs_affine_f16_kernel, in the same order, so the bytes are the same.  A tile whose taps do
// not fit the box (a transform the host did not size it for) reads global memory instead.
//
// Roles: thread 0 issues the copies (tiles 0..2 up front, tile i + 3 once every warp has
// released the buffer of tile i); all eight warps compute.  Every mbarrier wait is bounded
// (one second): a wait that gives up records ZS_DEVSTAT_WAIT_TIMEOUT, the CTA stops taking
// tiles, and thread 0 waits (bounded) for its copies still in flight before returning.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>

#include "zs_device.cuh"
#include "zs_kernels.h"
#include "zs_ptx.cuh"

#define ZS_AT_THREADS 256
#define ZS_AT_TW 64
#define ZS_AT_TH 32
#define ZS_AT_NBUF 3          // staging buffers: two tiles in flight while one is computed
#define ZS_AT_MAX_SMEM (200 * 1024)

struct ZsAffTma {
    int32_t bw, bh;          // box of source pixels (bw even)
    int32_t tiles_x, tiles;
    uint32_t buf_bytes;      // one staging buffer, rounded up to 128 bytes
    int32_t pad;
};

namespace {

// Source box of the output tile [x0, x1) x [y0, y1): origin (bx0, by0) of the bw x bh box
// that holds every tap a pixel of the tile can read; false when the taps do not fit it.
// Called by the issuing thread and by every computing thread with the same arguments;
// not inlined, so that all of them run the same instructions and agree on the box.
__device__ __noinline__ bool zs_at_box(const float *aff, int w, int h, int bw, int bh, int x0, int y0, int x1,
                                       int y1, int &bx0, int &by0) {
    float qx0 = 3.0e38f, qx1 = -3.0e38f, qy0 = 3.0e38f, qy1 = -3.0e38f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float cx = (float)((c & 1) ? x1 - 1 : x0) + 0.5f, cy = (float)((c & 2) ? y1 - 1 : y0) + 0.5f;
        const float qx = fmaf(aff[0], cx, fmaf(aff[1], cy, aff[2]));
        const float qy = fmaf(aff[3], cx, fmaf(aff[4], cy, aff[5]));
        qx0 = fminf(qx0, qx);
        qx1 = fmaxf(qx1, qx);
        qy0 = fminf(qy0, qy);
        qy1 = fmaxf(qy1, qy);
    }
    // Taps of a sample at q: floor(q - 0.5) and the next; one more pixel each side for the
    // rounding of the per-pixel maps; inside the image (taps are clamped to it).
    const float lim = 1.0e9f;
    const int tx0 = max((int)floorf(fmaxf(qx0, -lim) - 0.5f) - 1, 0);
    const int tx1 = min((int)floorf(fminf(qx1, lim) - 0.5f) + 2, w - 1);
    const int ty0 = max((int)floorf(fmaxf(qy0, -lim) - 0.5f) - 1, 0);
    const int ty1 = min((int)floorf(fminf(qy1, lim) - 0.5f) + 2, h - 1);
    bx0 = tx0 & ~1;
    by0 = ty0;
    return tx1 - bx0 < bw && ty1 - by0 < bh;
}

__device__ __forceinline__ bool zs_at_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag) {
    if (zs_mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = zs_globaltimer();
    for (;;) {
        if (zs_mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (zs_globaltimer() - t0 > ZS_WAIT_NS) {
            *abort_flag = 1;
            atomicOr(&zs_device_status_word, ZS_DEVSTAT_WAIT_TIMEOUT);
            return false;
        }
    }
}

__device__ __forceinline__ float4 zs_at_tap(const uint2 *sb, int bw, int bx0, int by0, int tx, int ty) {
    return zs_h4(sb[(ty - by0) * bw + (tx - bx0)]);
}

}  // namespace

__global__ void __launch_bounds__(ZS_AT_THREADS) zs_affine_tma_kernel(const __grid_constant__ ZsRasterArgs a,
                                                                      const __grid_constant__ CUtensorMap tm,
                                                                      const __grid_constant__ ZsAffTma p) {
    extern __shared__ __align__(128) uint8_t zs_at_smem[];
    __shared__ __align__(8) uint64_t full[ZS_AT_NBUF], empty[ZS_AT_NBUF];
    __shared__ int abort_word;
    volatile int *abort_flag = &abort_word;
    const ZsSource &s0 = a.src[0], &s1 = a.src[1];
    const int lane = threadIdx.x & 31;
    const int W = s1.width, H = s1.height;
    const float fw = (float)W, fh = (float)H;

    if (threadIdx.x == 0) {
        for (int b = 0; b < ZS_AT_NBUF; ++b) {
            zs_mbar_init(zs_smem_addr(full + b), 1);
            zs_mbar_init(zs_smem_addr(empty + b), ZS_AT_THREADS / 32);
        }
        abort_word = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    // Thread 0: start the copy of local tile `it` into buffer it % ZS_AT_NBUF (or complete
    // its barrier without data when its taps do not fit the box).
    uint32_t issued = 0;
    auto issue = [&](uint32_t it) {
        const int t = (int)(blockIdx.x + it * gridDim.x);
        const int tyi = t / p.tiles_x, txi = t - tyi * p.tiles_x;
        const int x0 = txi * ZS_AT_TW, y0 = tyi * ZS_AT_TH;
        int bx0, by0;
        const uint32_t b = it % ZS_AT_NBUF, bar = zs_smem_addr(full + b);
        if (zs_at_box(a.aff, W, H, p.bw, p.bh, x0, y0, min(x0 + ZS_AT_TW, a.width), min(y0 + ZS_AT_TH, a.height), bx0,
                      by0)) {
            zs_mbar_expect_tx(bar, (uint32_t)(p.bw * p.bh * 8));
            zs_tma_2d(zs_smem_addr(zs_at_smem + b * p.buf_bytes), &tm, bx0, by0, bar);
        } else {
            zs_mbar_arrive(bar);
        }
        issued = it + 1;
    };
    const uint32_t ntiles = blockIdx.x < (uint32_t)p.tiles ? (p.tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (threadIdx.x == 0)
        for (uint32_t it = 0; it < ZS_AT_NBUF && it < ntiles; ++it) issue(it);

    const int cxl = threadIdx.x & (ZS_AT_TW - 1), ryl = threadIdx.x / ZS_AT_TW;   // column, first row
    uint32_t landed = 0;   // tiles whose copy this thread has seen complete
    for (uint32_t it = 0; it < ntiles; ++it) {
        const uint32_t b = it % ZS_AT_NBUF, parity = (it / ZS_AT_NBUF) & 1u;
        if (!zs_at_wait(zs_smem_addr(full + b), parity, abort_flag)) break;
        landed = it + 1;
        const int t = (int)(blockIdx.x + it * gridDim.x);
        const int tyi = t / p.tiles_x, txi = t - tyi * p.tiles_x;
        const int x0 = txi * ZS_AT_TW, y0 = tyi * ZS_AT_TH;
        int bx0, by0;
        const bool staged = zs_at_box(a.aff, W, H, p.bw, p.bh, x0, y0, min(x0 + ZS_AT_TW, a.width),
                                      min(y0 + ZS_AT_TH, a.height), bx0, by0);
        const uint2 *sb = reinterpret_cast<const uint2 *>(zs_at_smem + b * p.buf_bytes);
        const int x = x0 + cxl;
        if (x < a.width) {
            const float cx = (float)x + 0.5f;
#pragma unroll 2
            for (int k = 0; k < ZS_AT_TH / (ZS_AT_THREADS / ZS_AT_TW); ++k) {
                const int y = y0 + ryl + k * (ZS_AT_THREADS / ZS_AT_TW);
                if (y >= a.height) break;
                const float cy = (float)y + 0.5f;
                const float qx = fmaf(a.aff[0], cx, fmaf(a.aff[1], cy, a.aff[2]));
                const float qy = fmaf(a.aff[3], cx, fmaf(a.aff[4], cy, a.aff[5]));
                float4 r;
                if (qx >= 0.0f && qx < fw && qy >= 0.0f && qy < fh) {
                    const float txf = qx - 0.5f, tyf = qy - 0.5f;
                    const float fx0 = floorf(txf), fy0 = floorf(tyf);
                    const float fx = txf - fx0, fy = tyf - fy0;
                    const int xi = (int)fx0, yi = (int)fy0;
                    const int xa = zs_clampi(xi, 0, W - 1), xb = zs_clampi(xi + 1, 0, W - 1);
                    const int ya = zs_clampi(yi, 0, H - 1), yb = zs_clampi(yi + 1, 0, H - 1);
                    float4 t00, t01, t10, t11;
                    if (staged) {
                        t00 = zs_at_tap(sb, p.bw, bx0, by0, xa, ya);
                        t01 = zs_at_tap(sb, p.bw, bx0, by0, xb, ya);
                        t10 = zs_at_tap(sb, p.bw, bx0, by0, xa, yb);
                        t11 = zs_at_tap(sb, p.bw, bx0, by0, xb, yb);
                    } else {
                        const uint8_t *ra = s1.ptr + (int64_t)ya * s1.stride, *rb = s1.ptr + (int64_t)yb * s1.stride;
                        t00 = zs_h4(__ldg((const uint2 *)(ra + (int64_t)xa * 8)));
                        t01 = zs_h4(__ldg((const uint2 *)(ra + (int64_t)xb * 8)));
                        t10 = zs_h4(__ldg((const uint2 *)(rb + (int64_t)xa * 8)));
                        t11 = zs_h4(__ldg((const uint2 *)(rb + (int64_t)xb * 8)));
                    }
                    r = zs_lerp4(zs_lerp4(t00, t01, fx), zs_lerp4(t10, t11, fx), fy);
                } else if (a.has_below) {
                    r = zs_load_px(s0, x, y);
                } else {
                    r = make_float4(a.cons[0], a.cons[1], a.cons[2], a.cons[3]);
                }
                float4 r2 = make_float4(0.f, 0.f, 0.f, 0.f);
                zs_run_program(a.prog, a.fmts, r, r2);
                uint8_t *dp = a.dst + (int64_t)y * a.dst_stride + (int64_t)x * a.dst_fmt.bpp;
                zs_store_raw(dp, a.dst_fmt.bpp, zs_encode_raw(a.dst_fmt, r));
            }
        }
        // Release the buffer; thread 0 refills it with local tile it + ZS_AT_NBUF once every
        // warp has.
        __syncwarp();
        if (lane == 0) zs_mbar_arrive(zs_smem_addr(empty + b));
        if (threadIdx.x == 0 && it + ZS_AT_NBUF < ntiles) {
            if (!zs_at_wait(zs_smem_addr(empty + b), parity, abort_flag)) break;
            issue(it + ZS_AT_NBUF);
        }
    }
    // A CTA that stops early lets thread 0's copies still in flight land before its shared
    // memory goes (bounded).
    if (threadIdx.x == 0 && *abort_flag) {
        for (uint32_t j = landed; j < issued; ++j)
            zs_mbar_wait(zs_smem_addr(full + j % ZS_AT_NBUF), (j / ZS_AT_NBUF) & 1u);
    }
}

namespace zs {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_at_encode = nullptr;
std::once_flag g_at_once;

PFN_cuTensorMapEncodeTiled_v12000 at_encode() {
    std::call_once(g_at_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_at_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    return g_at_encode;
}

// Box of source pixels that holds the taps of any 64 x 32 output tile under this affine
// inverse: the spread of the corner maps, two taps, a pixel of margin each side, and the
// even rounding of the origin.
bool at_box_size(const float *aff, int &bw, int &bh) {
    const double sx = (ZS_AT_TW - 1) * std::fabs((double)aff[0]) + (ZS_AT_TH - 1) * std::fabs((double)aff[1]);
    const double sy = (ZS_AT_TW - 1) * std::fabs((double)aff[3]) + (ZS_AT_TH - 1) * std::fabs((double)aff[4]);
    if (!(sx < 512.0 && sy < 512.0)) return false;
    bw = (int)std::ceil(sx) + 6;
    bw += bw & 1;
    bh = (int)std::ceil(sy) + 5;
    return bw <= 256 && bh <= 256 && ZS_AT_NBUF * (((size_t)bw * bh * 8 + 127) & ~(size_t)127) <= ZS_AT_MAX_SMEM;
}

}  // namespace

// The staged form of the RGBA16F affine bilinear gather; cudaErrorNotSupported when the
// transform's tile footprint or the source layout does not suit it (the caller then uses
// the direct gather kernel).
cudaError_t launch_affine_tma(const ZsRasterArgs &a, int sm_count, cudaStream_t stream) {
    const ZsSource &s = a.src[1];
    int bw = 0, bh = 0;
    PFN_cuTensorMapEncodeTiled_v12000 enc = at_encode();
    if (!enc || !at_box_size(a.aff, bw, bh) || ((uintptr_t)s.ptr & 15) || (s.stride & 15) || s.width < 1 ||
        s.height < 1)
        return cudaErrorNotSupported;
    alignas(64) CUtensorMap tm;
    const cuuint64_t dims[2] = {(cuuint64_t)s.width, (cuuint64_t)s.height};
    const cuuint64_t strides[1] = {(cuuint64_t)s.stride};
    const cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh}, estr[2] = {1, 1};
    if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, (void *)s.ptr, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorNotSupported;
    ZsAffTma p;
    p.bw = bw;
    p.bh = bh;
    p.tiles_x = (a.width + ZS_AT_TW - 1) / ZS_AT_TW;
    p.tiles = p.tiles_x * ((a.height + ZS_AT_TH - 1) / ZS_AT_TH);
    p.buf_bytes = (uint32_t)(((size_t)bw * bh * 8 + 127) & ~(size_t)127);
    p.pad = 0;
    const size_t smem = ZS_AT_NBUF * (size_t)p.buf_bytes;
    cudaError_t e = cudaFuncSetAttribute(zs_affine_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zs_affine_tma_kernel, ZS_AT_THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    long long blocks = (long long)(sm_count > 0 ? sm_count : 148) * per_sm;
    if (blocks > p.tiles) blocks = p.tiles;
    zs_affine_tma_kernel<<<(unsigned)blocks, ZS_AT_THREADS, smem, stream>>>(a, tm, p);
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

}  // namespace zs

ZS_TU_HOOKS(affine_tma)
