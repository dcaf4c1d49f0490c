// k_resample_tc.cu -- resize_filtered of an RGBA16F image with the vertical pass on the
// 5th-generation tensor cores (tcgen05) and the horizontal pass read out of tensor memory.
//
// The vertical filter of a band of 128 output rows is a banded matrix product
//
//     D[m, n] = sum_k Vw[oy0 + m, r0 + k] * S[r0 + k, n]
//
// with m the output row (the MMA's M = 128), k a source row and n one of the f16 values
// (x, channel) of the source columns a tile of output columns needs (N = 64 * atoms <=
// 256).  A (the band of vertical weights, f16) is precomputed on the host per band and
// chunk of 64 source rows in the K-major 128-byte-swizzled layout and arrives by a bulk
// copy; B (the source rows, exactly f16) is loaded by TMA with 128-byte swizzle, which is
// the MN-major canonical layout, so the image is consumed straight from HBM without
// reformatting.  The FP32 accumulator D lives in tensor memory (two 256-column buffers so
// that the epilogue of one tile overlaps the MMAs of the next).
//
// Epilogue: every output row is one TMEM lane; 16 warps (four per lane quarter) take the
// tile's output columns, read the horizontal taps of their column from TMEM
// (tcgen05.ld 32x32b.x4 = the 4 channels of one source pixel), apply the FP32 horizontal
// weights in tap order, run the fused pixel program and store.  The tile's horizontal
// weights and tap windows arrive in shared memory by bulk copy with the tile (one table
// per accumulator buffer), so the epilogue issues no global loads.
//
// Roles: warp 0 lane 0 issues the row copies (4-stage ring of {A chunk, B atoms}), warp 1
// allocates TMEM and its lane 0 copies each tile's horizontal tables and issues the MMAs,
// warps 2..17 are the epilogue.  All
// mbarrier waits are bounded (one second); a wait that gives up raises an abort flag that
// every role polls, sets ZS_DEVSTAT_WAIT_TIMEOUT, and the CTA drains its own copies and
// MMAs (bounded) and frees its TMEM before returning.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "zs_device.cuh"
#include "zs_kernels.h"
#include "zs_ptx.cuh"

#define ZS_TC_STAGES 4                                                     // ring slots (narrow tiles)
#define ZS_TC_EPI_WARPS 16
#ifndef ZS_TC_TAPB
#define ZS_TC_TAPB 8                                                       // taps per TMEM-load batch
#endif
#define ZS_TC_THREADS (64 + 32 * ZS_TC_EPI_WARPS)
#define ZS_TC_ATOM_BYTES (ZS_TC_K * 128)                                   // 64 rows x 128 B
// Narrow tiles (<= 4 atoms): 4 stages of {A, 4 atoms}, two 256-column accumulators.
// Wide tiles (5..8 atoms): 2 stages of {A, 8 atoms}, one 512-column accumulator filled by
// two N <= 256 MMAs per K step.
#define ZS_TC_STAGE_BYTES (ZS_TC_CHUNK_BYTES + 4 * ZS_TC_ATOM_BYTES)
#define ZS_TC_WIDE_STAGE_BYTES (ZS_TC_CHUNK_BYTES + 8 * ZS_TC_ATOM_BYTES)
#define ZS_TC_TMEM_COLS 512
// Per-tile horizontal tables (weights [tw][tc_taps], first tap [tw], tap count [tw]) for
// tw <= 32, tc_taps <= 64, one per accumulator buffer.
#define ZS_TC_TAB_BYTES ((32 * 64 + 2 * 32) * 4)
#define ZS_TC_SMEM (ZS_TC_STAGES * ZS_TC_STAGE_BYTES + 2 * ZS_TC_TAB_BYTES + 1024 + 256)

static_assert(ZS_TC_STAGE_BYTES % 1024 == 0 && ZS_TC_WIDE_STAGE_BYTES % 1024 == 0,
              "stages stay 1024-byte aligned (128-byte swizzle atoms)");
static_assert(2 * ZS_TC_WIDE_STAGE_BYTES <= ZS_TC_STAGES * ZS_TC_STAGE_BYTES, "both rings fit the stage region");

namespace {

// Bounded wait that also gives up when another role raised the abort flag; on its own
// timeout it raises the flag and records the timeout in the device status word.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag) {
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

// Shared-memory matrix descriptor (tcgen05): start address, leading and stride byte
// offsets (16-byte units), version 1, 128-byte swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46) | (2ull << 61);
}

// Instruction descriptor, kind::f16: D FP32, A and B f16, A K-major, B MN-major, M = 128.
__device__ __forceinline__ uint32_t tc_idesc(int n) {
    return (1u << 4) | (1u << 16) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(ZS_TC_M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_ld4(uint32_t taddr, uint32_t (&r)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

struct TcTile {
    int band, x0, cs0;    // 128-row band, first output column, first staged source column (even)
};

__device__ __forceinline__ TcTile tc_tile(const ZsRasterArgs &a, int t, int tiles_x) {
    TcTile r;
    r.band = t / tiles_x;
    r.x0 = (t % tiles_x) * a.tc_tw;
    r.cs0 = a.index_x[r.x0] & ~1;
    return r;
}

}  // namespace

__global__ void __launch_bounds__(ZS_TC_THREADS, 1)
    zs_resample_tc_kernel(const __grid_constant__ ZsRasterArgs a, const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ __align__(1024) uint8_t zs_tc_smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)zs_tc_smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *tab = smem + ZS_TC_STAGES * ZS_TC_STAGE_BYTES;                // [2][ZS_TC_TAB_BYTES]
    uint64_t *full = (uint64_t *)(tab + 2 * ZS_TC_TAB_BYTES);
    uint64_t *empty = full + ZS_TC_STAGES;
    uint64_t *tfull = empty + ZS_TC_STAGES;    // [2] accumulator ready
    uint64_t *tempty = tfull + 2;              // [2] accumulator drained (and its tables free)
    uint64_t *tabfull = tempty + 2;            // [2] tile tables landed
    uint64_t *drain = tabfull + 2;
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_x = (a.width + a.tc_tw - 1) / a.tc_tw;
    const int tiles = tiles_x * ((a.height + ZS_TC_M - 1) / ZS_TC_M);
    const int atoms = a.tc_atoms;
    const bool wide = atoms > 4;
    const uint32_t NS = wide ? 2u : (uint32_t)ZS_TC_STAGES;                  // ring slots
    const uint32_t SB = wide ? ZS_TC_WIDE_STAGE_BYTES : ZS_TC_STAGE_BYTES;   // bytes per slot
    const uint32_t nbuf = wide ? 1u : 2u;                                     // accumulators
    const uint32_t accw = ZS_TC_TMEM_COLS / nbuf;                            // columns each

    if (threadIdx.x == 0) {
        for (int s = 0; s < ZS_TC_STAGES; ++s) {
            zs_mbar_init(zs_smem_addr(full + s), 1);
            zs_mbar_init(zs_smem_addr(empty + s), 1);
        }
        for (int b = 0; b < 2; ++b) {
            zs_mbar_init(zs_smem_addr(tfull + b), 1);
            zs_mbar_init(zs_smem_addr(tempty + b), ZS_TC_EPI_WARPS);
            zs_mbar_init(zs_smem_addr(tabfull + b), 1);
        }
        zs_mbar_init(zs_smem_addr(drain), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(zs_smem_addr(tmem_slot)),
                     "r"(ZS_TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------------------------------------------------------- copies
        uint32_t it = 0;
        const uint32_t tx = ZS_TC_CHUNK_BYTES + (uint32_t)atoms * ZS_TC_ATOM_BYTES;
        for (int t = blockIdx.x; t < tiles && !*abort_flag; t += gridDim.x) {
            const TcTile tt = tc_tile(a, t, tiles_x);
            const int first = a.vimg_index[2 * tt.band], nk = a.vimg_index[2 * tt.band + 1];
            const int rbase = a.vfirst[tt.band * ZS_TC_M];
            bool ok = true;
            for (int kc = 0; kc < nk; ++kc, ++it) {
                const int s = (int)(it % NS);
                if (!tc_wait(zs_smem_addr(empty + s), ((it / NS) & 1u) ^ 1u, abort_flag)) {
                    ok = false;
                    break;
                }
                const uint32_t bar = zs_smem_addr(full + s);
                const uint32_t st = zs_smem_addr(smem + (size_t)s * SB);
                zs_mbar_expect_tx(bar, tx);
                zs_bulk_g2s(st, a.vimg + (size_t)(first + kc) * ZS_TC_CHUNK_BYTES, ZS_TC_CHUNK_BYTES, bar);
                for (int at = 0; at < atoms; ++at)
                    zs_tma_2d(st + ZS_TC_CHUNK_BYTES + at * ZS_TC_ATOM_BYTES, &tmap, tt.cs0 * 4 + 64 * at,
                              rbase + ZS_TC_K * kc, bar);
            }
            if (!ok) break;
        }
        if (*abort_flag) {
            // Let this thread's copies land before the CTA (and its shared memory) goes.
            const uint32_t lo = it > NS ? it - NS : 0;
            for (uint32_t j = lo; j < it; ++j) zs_mbar_wait(zs_smem_addr(full + (j % NS)), (j / NS) & 1u);
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------------------------------------------------------- MMAs
        uint32_t it = 0, lt = 0, tabs = 0;
        const uint32_t idesc0 = tc_idesc(64 * (wide ? 4 : atoms)), idesc1 = tc_idesc(64 * (wide ? atoms - 4 : 4));
        const uint32_t wbytes = (uint32_t)(a.tc_tw * a.tc_taps * 4), ibytes = (uint32_t)(a.tc_tw * 4);
        for (int t = blockIdx.x; t < tiles && !*abort_flag; t += gridDim.x, ++lt) {
            const TcTile tt = tc_tile(a, t, tiles_x);
            const int nk = a.vimg_index[2 * tt.band + 1];
            const uint32_t ab = lt % nbuf;
            if (!tc_wait(zs_smem_addr(tempty + ab), ((lt / nbuf) & 1u) ^ 1u, abort_flag)) break;
            tc_fence_after();
            {
                // The tile's horizontal weights and tap windows, into the table buffer of its
                // accumulator (free now that the epilogue of the tile two before is done).
                const uint32_t bar = zs_smem_addr(tabfull + ab);
                const uint32_t tb = zs_smem_addr(tab + ab * ZS_TC_TAB_BYTES);
                zs_mbar_expect_tx(bar, wbytes + 2 * ibytes);
                zs_bulk_g2s(tb, a.tc_weights + (int64_t)tt.x0 * a.tc_taps, wbytes, bar);
                zs_bulk_g2s(tb + wbytes, a.index_x + tt.x0, ibytes, bar);
                zs_bulk_g2s(tb + wbytes + ibytes, a.index_y + tt.x0, ibytes, bar);
                ++tabs;
            }
            const uint32_t d = tmem + ab * accw;
            bool ok = true;
            for (int kc = 0; kc < nk; ++kc, ++it) {
                const int s = (int)(it % NS);
                if (!tc_wait(zs_smem_addr(full + s), (it / NS) & 1u, abort_flag)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t sa = zs_smem_addr(smem + (size_t)s * SB);
                const uint32_t sb = sa + ZS_TC_CHUNK_BYTES;
#pragma unroll
                for (int ks = 0; ks < ZS_TC_K / 16; ++ks) {
                    // A: K-major, 16 K-elements = 32 bytes further along each swizzled row.
                    // B: MN-major, 16 K-rows = two 1024-byte groups of 8 rows further.
                    const uint64_t ad = tc_desc(sa + 32 * ks, 16, 1024);
                    tc_mma(d, ad, tc_desc(sb + 2048 * ks, ZS_TC_ATOM_BYTES, 1024), idesc0, (kc | ks) != 0);
                    if (wide)   // atoms 4.. into accumulator columns 256..
                        tc_mma(d + 256, ad, tc_desc(sb + 4 * ZS_TC_ATOM_BYTES + 2048 * ks, ZS_TC_ATOM_BYTES, 1024), idesc1,
                               (kc | ks) != 0);
                }
                tc_commit(zs_smem_addr(empty + s));
            }
            if (!ok) break;
            tc_commit(zs_smem_addr(tfull + ab));
        }
        // Nothing of this thread's may still run when the TMEM and shared memory go.
        tc_commit(zs_smem_addr(drain));
        zs_mbar_wait(zs_smem_addr(drain), 0);
        if (*abort_flag)
            for (uint32_t j = tabs > nbuf ? tabs - nbuf : 0; j < tabs; ++j)
                zs_mbar_wait(zs_smem_addr(tabfull + (j % nbuf)), (j / nbuf) & 1u);
    } else if (warp >= 2) {
        // ---------------------------------------------------------------- epilogue
        const int e = warp - 2;
        const int quarter = warp & 3;      // TMEM lanes this warp may read
        const int part = e >> 2;           // this warp's outputs: x0 + part + 4 i
        const int m = quarter * 32 + lane;
        const bool plain = zs_plain_f16_out(a.prog, a.dst_fmt);
        uint32_t lt = 0;
        for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++lt) {
            const TcTile tt = tc_tile(a, t, tiles_x);
            const uint32_t ab = lt % nbuf;
            if (!tc_wait(zs_smem_addr(tabfull + ab), (lt / nbuf) & 1u, abort_flag)) break;
            if (!tc_wait(zs_smem_addr(tfull + ab), (lt / nbuf) & 1u, abort_flag)) break;
            tc_fence_after();
            const float *tw_w = (const float *)(tab + ab * ZS_TC_TAB_BYTES);
            const int *tw_first = (const int *)(tw_w + a.tc_tw * a.tc_taps);
            const int *tw_cnt = tw_first + a.tc_tw;
            const int oy = tt.band * ZS_TC_M + m;
            const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16) + ab * accw;
            for (int ox = tt.x0 + part; ox < min(tt.x0 + a.tc_tw, a.width); ox += 4) {
                const int oxl = ox - tt.x0;
                const int cnt = tw_cnt[oxl];
                const uint32_t col = (uint32_t)(tw_first[oxl] - tt.cs0) * 4u;
                const float *w = tw_w + oxl * a.tc_taps;   // 16-byte rows
                // Two accumulator pairs (even and odd taps) halve the FMA dependency chains.
                float2 a01 = make_float2(0.f, 0.f), a23 = make_float2(0.f, 0.f);
                float2 b01 = make_float2(0.f, 0.f), b23 = make_float2(0.f, 0.f);
                for (int k0 = 0; k0 < cnt; k0 += ZS_TC_TAPB) {
                    const int n = min(ZS_TC_TAPB, cnt - k0);
                    uint32_t r[ZS_TC_TAPB][4];
                    float wk[ZS_TC_TAPB];
#pragma unroll
                    for (int j = 0; j < ZS_TC_TAPB; ++j)
                        if (j < n) tc_ld4(trow + col + 4u * (uint32_t)(k0 + j), r[j]);
#pragma unroll
                    for (int j = 0; j < ZS_TC_TAPB; j += 4)
                        if (j < n) {
                            // k0 + j < cnt <= tc_taps, both multiples of 4: inside the row.
                            const float4 q = *reinterpret_cast<const float4 *>(w + k0 + j);
                            wk[j] = q.x;
                            wk[j + 1] = q.y;
                            wk[j + 2] = q.z;
                            wk[j + 3] = q.w;
                        }
                    tc_wait_ld();
                    // Tie the loaded registers to the wait so that no use moves above it.
#pragma unroll
                    for (int j = 0; j < ZS_TC_TAPB; ++j)
                        if (j < n)
                            asm volatile("" : "+r"(r[j][0]), "+r"(r[j][1]), "+r"(r[j][2]), "+r"(r[j][3]));
#pragma unroll
                    for (int j = 0; j < ZS_TC_TAPB; ++j)
                        if (j < n) {
                            const float2 w2 = make_float2(wk[j], wk[j]);
                            const float2 v01 = make_float2(__uint_as_float(r[j][0]), __uint_as_float(r[j][1]));
                            const float2 v23 = make_float2(__uint_as_float(r[j][2]), __uint_as_float(r[j][3]));
                            if (j & 1) {
                                b01 = __ffma2_rn(w2, v01, b01);
                                b23 = __ffma2_rn(w2, v23, b23);
                            } else {
                                a01 = __ffma2_rn(w2, v01, a01);
                                a23 = __ffma2_rn(w2, v23, a23);
                            }
                        }
                }
                if (oy < a.height) {
                    float4 acc = make_float4(a01.x + b01.x, a01.y + b01.y, a23.x + b23.x, a23.y + b23.y);
                    uint8_t *dp = a.dst + (int64_t)oy * a.dst_stride + (int64_t)ox * a.dst_fmt.bpp;
                    if (plain) {
                        zs_store_f16x4(dp, acc);
                    } else {
                        float4 r2 = make_float4(0.f, 0.f, 0.f, 0.f);
                        zs_run_program(a.prog, a.fmts, acc, r2);
                        zs_store_raw(dp, a.dst_fmt.bpp, zs_encode_raw(a.dst_fmt, acc));
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) zs_mbar_arrive(zs_smem_addr(tempty + ab));
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    __syncwarp();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ZS_TC_TMEM_COLS)
                     : "memory");
}

namespace zs {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;
std::once_flag g_encode_once;

PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode_tiled = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    return g_encode_tiled;
}

}  // namespace

bool resample_tc_usable(const ZsRasterArgs &a) {
    const ZsSource &s = a.src[0];
    return a.tc_tw > 0 && a.vimg && a.vimg_index && a.tc_weights && a.tc_taps % 4 == 0 && a.tc_taps <= 64 &&
           s.fmt.fast == ZS_FAST_F16X4 && ((uintptr_t)s.ptr & 15) == 0 &&
           (s.stride & 15) == 0 && a.tc_atoms >= 1 && a.tc_atoms <= ZS_TC_MAX_ATOMS && encode_tiled() != nullptr;
}

cudaError_t launch_resample_tc(const ZsRasterArgs &a, int sm_count, cudaStream_t stream) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_tiled();
    if (!enc) return cudaErrorNotSupported;
    alignas(64) CUtensorMap tm;
    const ZsSource &s = a.src[0];
    const cuuint64_t dims[2] = {(cuuint64_t)s.width * 4, (cuuint64_t)s.height};
    const cuuint64_t strides[1] = {(cuuint64_t)s.stride};
    const cuuint32_t box[2] = {64, ZS_TC_K}, estr[2] = {1, 1};
    if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, (void *)s.ptr, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(zs_resample_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ZS_TC_SMEM);
    if (e != cudaSuccess) return e;
    const int tiles = ((a.width + a.tc_tw - 1) / a.tc_tw) * ((a.height + ZS_TC_M - 1) / ZS_TC_M);
    int blocks = sm_count > 0 ? sm_count : 148;
    if (blocks > tiles) blocks = tiles;
    zs_resample_tc_kernel<<<blocks, ZS_TC_THREADS, ZS_TC_SMEM, stream>>>(a, tm);
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

}  // namespace zs

ZS_TU_HOOKS(resample_tc)
