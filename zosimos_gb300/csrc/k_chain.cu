// k_chain.cu -- the fused colour chain in canonical form, RGBA8 sRGB in and out.
//
//   decode -> M_a -> [cbrt] -> M_b -> [cube] -> M_c -> [clamp] -> M_d -> encode
//
// Every chain of the reference's per-pixel colour ops (color_convert between RGB
// spaces, chromatic_adaptation, Oklab encode/decode, colour matrices) folds into
// this form on the host (matrices multiplied in FP64).  Compared with the
// reference, which runs one render pass per op and re-quantises the image after
// every pass (lib/zosimos/src/program.rs:1486-1533), this is one HBM pass:
// 4 bytes read and 4 bytes written per pixel.
//
// The chain is issue-bound on GB300 rather than HBM-bound (about 58 instructions per
// 8 bytes moved), so the data path is built to minimise instructions per pixel:
//  * 16-byte coalesced streaming loads/stores; two vectors (8 pixels) computed while the
//    next two are in flight (software pipeline); one 1024-thread block per SM, so the
//    replicated tables fit beside each other;
//  * sRGB decode from a lane-replicated shared table (lane l reads column l: no bank
//    conflicts whatever the data) at shared address 0x10000, so one PRMT of the texel forms
//    the load address; 32-bit vector indices;
//  * pixels processed in pairs with packed FP32x2 FMA (one instruction, two pixels),
//    the matrix coefficients read as 64-bit constant operands;
//  * cube roots as ex2(lg2(x)/3) on the MUFU pipe (the sign fix-up is dropped when the
//    host proves M_a keeps [0,1]^3 non-negative);
//  * an Oklab L/C scaling between the cube root and the cube (M_b = d I + (1,1,1)^T v,
//    detected on the host in FP64) costs 6 FMAs instead of 9;
//  * clamps folded into the last FMA of each matrix row (fma.sat on the FMA pipe), the
//    encode shift added to a pixel pair by one packed add;
//  * exact round-to-nearest sRGB encode from a bucketed threshold table replicated 8x
//    across lanes (entry + float bits carries the code into byte 3): one shift, one
//    shift-add, one shared load and one add per channel, packed with PRMT;
//  * alpha bytes passed through (unorm8 alpha decode + encode is the identity).
#include <atomic>
#include <cstdint>
#include <type_traits>

#include "zs_chain.cuh"
#include "zs_device.cuh"
#include "zs_kernels.h"

#define ZS_CHAIN_THREADS 1024

// Decode rows are 256 bytes apart so that the byte offset of (code, lane) is
// (code << 8) | (lane << 2): one PRMT builds it from the packed texel.
struct ZsChainSmem {
    float lut[256 * 64];                         // [code][lane], lanes 32..63 unused
    uint32_t enc[ZS_ENCS_ENTRIES * ZS_ENC_REP];   // [bucket][lane & 7], shifted domain
};

// Decode of byte K: from the table at `lut` (lane4 = lane << 2), or with ABS from the table
// at shared address ZS_DEC_ABS (lane4 = ZS_DEC_ABS | lane << 2).
template <int K, bool ABS>
__device__ __forceinline__ float zs_dec_at(const unsigned char *lut, uint32_t w, uint32_t lane4) {
    if (ABS) return zs_dec_abs<K>(w, lane4);
    return zs_dec<K>(lut, w, lane4);
}

template <bool CBRT, bool CUBE, bool CLAMP, bool NONNEG, bool RANK1, bool ABS = false>
__device__ __forceinline__ void zs_chain_pair(uint32_t &wp, uint32_t &wq, const unsigned char *lut,
                                              uint32_t lane4, uint32_t ebase, const ZsChainArgs &a) {
    float2 r = make_float2(zs_dec_at<0, ABS>(lut, wp, lane4), zs_dec_at<0, ABS>(lut, wq, lane4));
    float2 g = make_float2(zs_dec_at<1, ABS>(lut, wp, lane4), zs_dec_at<1, ABS>(lut, wq, lane4));
    float2 b = make_float2(zs_dec_at<2, ABS>(lut, wp, lane4), zs_dec_at<2, ABS>(lut, wq, lane4));
    zs_m3x2<false>(a.m2[0], r, g, b);
    if (CBRT) {
        if (NONNEG) {
            zs_cbrt2(r);
            zs_cbrt2(g);
            zs_cbrt2(b);
        } else {
            r.x = zs_cbrt1<false>(r.x); r.y = zs_cbrt1<false>(r.y);
            g.x = zs_cbrt1<false>(g.x); g.y = zs_cbrt1<false>(g.y);
            b.x = zs_cbrt1<false>(b.x); b.y = zs_cbrt1<false>(b.y);
        }
    }
    if (RANK1) {
        // c' = d c + (v . c) (1, 1, 1)
        const float2 *v = reinterpret_cast<const float2 *>(a.mb_v);
        const float2 d = *reinterpret_cast<const float2 *>(a.mb_d);
        const float2 t = __ffma2_rn(v[0], r, __ffma2_rn(v[1], g, __fmul2_rn(v[2], b)));
        r = __ffma2_rn(d, r, t);
        g = __ffma2_rn(d, g, t);
        b = __ffma2_rn(d, b, t);
    } else {
        zs_m3x2<false>(a.m2[1], r, g, b);
    }
    if (CUBE) {
        r = __fmul2_rn(__fmul2_rn(r, r), r);
        g = __fmul2_rn(__fmul2_rn(g, g), g);
        b = __fmul2_rn(__fmul2_rn(b, b), b);
    }
    zs_m3x2<CLAMP>(a.m2[2], r, g, b);
    zs_m3x2<true>(a.m2[3], r, g, b);
    const float2 sh = make_float2(1.0f / 4096.0f, 1.0f / 4096.0f);
    r = __fadd2_rn(r, sh);
    g = __fadd2_rn(g, sh);
    b = __fadd2_rn(b, sh);
    const uint32_t rp = zs_enc_q(ebase, r.x), gp = zs_enc_q(ebase, g.x), bp = zs_enc_q(ebase, b.x);
    const uint32_t rq = zs_enc_q(ebase, r.y), gq = zs_enc_q(ebase, g.y), bq = zs_enc_q(ebase, b.y);
    wp = __byte_perm(__byte_perm(rp, gp, 0x0073), __byte_perm(bp, wp, 0x0073), 0x5410);
    wq = __byte_perm(__byte_perm(rq, gq, 0x0073), __byte_perm(bq, wq, 0x0073), 0x5410);
}

// Dynamic shared memory of the FAST form: the encode table at the start of the block's
// dynamic window, the decode table at shared address ZS_DEC_ABS .. 2 * ZS_DEC_ABS.
#define ZS_CHAIN_FAST_SMEM (2 * ZS_DEC_ABS)

// VEC: 16-byte vectors per thread and loop iteration (2: two computed while the next two are
// in flight; 1: one computed while the next one is in flight), chosen by the autotuner.
// FAST (VEC 2, one block per SM, fewer than 2^31 vectors plus three grid strides): the decode
// table at a fixed 64 KiB-aligned shared address, so each decode is a PRMT and a load with
// no address add, and 32-bit vector indices; about 5 fewer instructions per pixel.
template <bool CBRT, bool CUBE, bool CLAMP, bool NONNEG, bool RANK1, int VEC, bool FAST>
__global__ void __launch_bounds__(ZS_CHAIN_THREADS, 1) zs_chain_srgb8_kernel(const __grid_constant__ ZsChainArgs a) {
    extern __shared__ __align__(16) unsigned char zs_smem_raw[];
    struct { float *lut; uint32_t *enc; } sm;
    if (FAST) {
        // The host launches this form with ZS_CHAIN_FAST_SMEM bytes when the block's shared
        // window starts below ZS_DEC_ABS - sizeof(enc); should the window start higher, the
        // block flags it and does nothing.
        const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(zs_smem_raw);
        uint32_t dyn;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        if (s0 + (uint32_t)sizeof(ZsChainSmem::enc) > ZS_DEC_ABS || ZS_DEC_ABS + (uint32_t)sizeof(ZsChainSmem::lut) > s0 + dyn) {
            if (threadIdx.x == 0) atomicOr(&zs_device_status_word, ZS_DEVSTAT_LAYOUT);
            return;
        }
        sm.enc = reinterpret_cast<uint32_t *>(zs_smem_raw);
        sm.lut = reinterpret_cast<float *>(zs_smem_raw + (ZS_DEC_ABS - s0));
    } else {
        ZsChainSmem &t = *reinterpret_cast<ZsChainSmem *>(zs_smem_raw);
        sm.enc = t.enc;
        sm.lut = t.lut;
    }
    using IX = typename std::conditional<FAST, int, int64_t>::type;
    const uint4 *in = reinterpret_cast<const uint4 *>(a.src);
    uint4 *out = reinterpret_cast<uint4 *>(a.dst);
    const IX nvec = (IX)(a.npx >> 2);
    const IX stride = (IX)gridDim.x * blockDim.x;
    IX v = (IX)blockIdx.x * blockDim.x + threadIdx.x;
    // Programmatic dependent launch: the next launch in the stream may start as soon as this
    // one runs; its CTAs stage their tables while this grid drains, then wait below.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // Tables: one 16-byte store writes four lane copies of an entry.
    for (int i = threadIdx.x; i < 256 * 8; i += blockDim.x) {
        const float d = zs_srgb_decode_lut[i >> 3];
        reinterpret_cast<float4 *>(sm.lut)[(i >> 3) * 16 + (i & 7)] = make_float4(d, d, d, d);
    }
    static_assert(ZS_ENC_REP == 8, "two uint4 per encode bucket");
    for (int i = threadIdx.x; i < 2 * ZS_ENCS_ENTRIES; i += blockDim.x) {
        const uint32_t e = zs_srgb_encode_tab_shifted[i >> 1];
        reinterpret_cast<uint4 *>(sm.enc)[i] = make_uint4(e, e, e, e);
    }
    // Image data only after the previous grid in the stream has completed and its writes are
    // visible (a no-op without programmatic dependent launch); the first two vectors are
    // requested before the barrier that publishes the tables.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (VEC == 1) {
        uint4 w = make_uint4(0, 0, 0, 0);
        if (v < nvec) w = __ldcs(in + v);
        __syncthreads();
        const int lane = threadIdx.x & 31;
        const unsigned char *lut = reinterpret_cast<const unsigned char *>(sm.lut);
        const uint32_t lane4 = (uint32_t)lane << 2;
        const uint32_t ebase = zs_enc_base(sm.enc, lane);
        for (; v < nvec; v += stride) {
            // The next vector is in flight while this one is computed.
            const uint4 n = v + stride < nvec ? __ldcs(in + v + stride) : w;
            zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1>(w.x, w.y, lut, lane4, ebase, a);
            zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1>(w.z, w.w, lut, lane4, ebase, a);
            __stcs(out + v, w);
            w = n;
        }
        const int64_t tail0 = nvec << 2;
        const int64_t t = tail0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (t < a.npx && t < tail0 + 4) {
            const uint32_t *in32 = reinterpret_cast<const uint32_t *>(a.src);
            uint32_t *out32 = reinterpret_cast<uint32_t *>(a.dst);
            uint32_t p = in32[t], q = p;
            zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1>(p, q, lut, lane4, ebase, a);
            out32[t] = p;
        }
        return;
    }
    const bool piped = v + stride < nvec;
    uint4 w0 = make_uint4(0, 0, 0, 0), w1 = w0;
    if (piped) {
        w0 = __ldcs(in + v);
        w1 = __ldcs(in + v + stride);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned char *lut = reinterpret_cast<const unsigned char *>(sm.lut);
    const uint32_t lane4 = ((uint32_t)lane << 2) | (FAST ? ZS_DEC_ABS : 0u);
    const uint32_t ebase = zs_enc_base(sm.enc, lane);

    if (piped) {
        // Software pipeline: the next two vectors are in flight while the current two are
        // computed, so each thread keeps 32 bytes of reads outstanding at all times.
        for (;;) {
            const IX nx = v + 2 * stride;
            const bool more = nx + stride < nvec;
            uint4 n0 = w0, n1 = w1;
            if (more) {
                n0 = __ldcs(in + nx);
                n1 = __ldcs(in + nx + stride);
            }
            zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1, FAST>(w0.x, w0.y, lut, lane4, ebase, a);
            zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1, FAST>(w0.z, w0.w, lut, lane4, ebase, a);
            __stcs(out + v, w0);
            zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1, FAST>(w1.x, w1.y, lut, lane4, ebase, a);
            zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1, FAST>(w1.z, w1.w, lut, lane4, ebase, a);
            __stcs(out + v + stride, w1);
            v = nx;
            if (!more) break;
            w0 = n0;
            w1 = n1;
        }
    }
    if (v < nvec) {
        uint4 w = __ldcs(in + v);
        zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1, FAST>(w.x, w.y, lut, lane4, ebase, a);
        zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1, FAST>(w.z, w.w, lut, lane4, ebase, a);
        __stcs(out + v, w);
    }
    // Tail pixels (npx not a multiple of 4): block 0, threads 0..3.
    const int64_t tail0 = nvec << 2;
    const int64_t t = tail0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < a.npx && t < tail0 + 4) {
        const uint32_t *in32 = reinterpret_cast<const uint32_t *>(a.src);
        uint32_t *out32 = reinterpret_cast<uint32_t *>(a.dst);
        uint32_t p = in32[t], q = p;
        zs_chain_pair<CBRT, CUBE, CLAMP, NONNEG, RANK1, FAST>(p, q, lut, lane4, ebase, a);
        out32[t] = p;
    }
}

namespace zs {

// Whether the FAST form's layout fits on `dev`: the block's dynamic shared window starts after
// the driver's reserved shared memory, which must leave room for the encode table below
// ZS_DEC_ABS (the kernel has no static shared memory).
static bool fast_layout_fits(int dev) {
    static std::atomic<int> fits_of[ZS_MAX_DEVICES];
    int f = fits_of[dev].load();
    if (f == 0) {
        int reserved = 0, optin = 0;
        if (cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
            (void)cudaGetLastError();
            reserved = 1 << 30;
        }
        const bool ok = (size_t)reserved + sizeof(ZsChainSmem::enc) <= ZS_DEC_ABS && optin >= (int)ZS_CHAIN_FAST_SMEM;
        f = ok ? 1 : 2;
        fits_of[dev].store(f);
    }
    return f == 1;
}

template <bool CBRT, bool CUBE, bool CLAMP, bool NONNEG, bool RANK1 = false>
static cudaError_t launch_chain_t(const ZsChainArgs &args, int sm_count, cudaStream_t stream, int threads,
                                  int vectors) {
    // The shared-memory opt-in is a per-device attribute of the kernel: set it (and size the
    // grid) once per device and block size, on the device that is current for this launch.
    // Block sizes: 1024 threads (one block per SM) or 512, chosen by the autotuner, and 256
    // for the zero-copy host round trip (fewer host reads in flight); all run the same
    // arithmetic per pixel.
    static std::atomic<int> per_sm_of[ZS_MAX_DEVICES][3][3];
    const int which = threads == 512 ? 1 : (threads == 256 ? 2 : 0);
    const int block = which == 1 ? 512 : (which == 2 ? 256 : ZS_CHAIN_THREADS);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= ZS_MAX_DEVICES) return cudaErrorInvalidDevice;
    // The grid is at most one wave (sm_count x blocks per SM, at most 2048 threads per SM); the
    // FAST form needs vector indices that stay below 2^31 over three grid strides.
    const int64_t nvec = (args.npx + 3) / 4;
    const int64_t sms = sm_count > 0 ? sm_count : 148;
    const bool fast = vectors != 1 && block == ZS_CHAIN_THREADS && (args.npx >> 2) + 3 * 2 * sms * block < INT32_MAX &&
                      fast_layout_fits(dev);
    const int form = vectors == 1 ? 1 : (fast ? 2 : 0);
    auto kernel = form == 1 ? zs_chain_srgb8_kernel<CBRT, CUBE, CLAMP, NONNEG, RANK1, 1, false>
                            : (form == 2 ? zs_chain_srgb8_kernel<CBRT, CUBE, CLAMP, NONNEG, RANK1, 2, true>
                                         : zs_chain_srgb8_kernel<CBRT, CUBE, CLAMP, NONNEG, RANK1, 2, false>);
    const size_t smem = form == 2 ? (size_t)ZS_CHAIN_FAST_SMEM : sizeof(ZsChainSmem);
    int per_sm = per_sm_of[dev][which][form].load();
    if (per_sm == 0) {
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        per_sm_of[dev][which][form].store(per_sm);
    }
    int64_t blocks = (nvec + block - 1) / block;
    const int64_t cap = sms * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    // Launched with programmatic stream serialization: the table staging of this launch
    // overlaps the tail of the previous kernel in the stream (the kernel waits for it with
    // griddepcontrol.wait before touching image data).
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kernel, args);
    if (e != cudaSuccess) return e;
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

template <bool NONNEG>
static cudaError_t launch_chain_n(const ZsChainArgs &args, int sm_count, cudaStream_t stream, int threads,
                                  int vectors) {
    const bool cb = args.flags & ZS_CHAIN_CBRT, cu = args.flags & ZS_CHAIN_CUBE, cl = args.flags & ZS_CHAIN_CLAMP;
    // The Oklab form (cube root, L/C scaling, cube) with the rank-1 middle matrix.
    if (cb && cu && (args.flags & ZS_CHAIN_MB_RANK1)) {
        if (cl) return launch_chain_t<true, true, true, NONNEG, true>(args, sm_count, stream, threads, vectors);
        return launch_chain_t<true, true, false, NONNEG, true>(args, sm_count, stream, threads, vectors);
    }
    if (cb && cu && cl) return launch_chain_t<true, true, true, NONNEG>(args, sm_count, stream, threads, vectors);
    if (cb && cu && !cl) return launch_chain_t<true, true, false, NONNEG>(args, sm_count, stream, threads, vectors);
    if (cb && !cu && cl) return launch_chain_t<true, false, true, NONNEG>(args, sm_count, stream, threads, vectors);
    if (cb && !cu && !cl) return launch_chain_t<true, false, false, NONNEG>(args, sm_count, stream, threads, vectors);
    if (!cb && cu && cl) return launch_chain_t<false, true, true, NONNEG>(args, sm_count, stream, threads, vectors);
    if (!cb && cu && !cl) return launch_chain_t<false, true, false, NONNEG>(args, sm_count, stream, threads, vectors);
    if (!cb && !cu && cl) return launch_chain_t<false, false, true, NONNEG>(args, sm_count, stream, threads, vectors);
    return launch_chain_t<false, false, false, NONNEG>(args, sm_count, stream, threads, vectors);
}

cudaError_t launch_chain(const ZsChainArgs &args, uint8_t src_fast, uint8_t dst_fast, int sm_count,
                         cudaStream_t stream, int threads, int vectors) {
    if (src_fast != ZS_FAST_RGBA8_SRGB || dst_fast != ZS_FAST_RGBA8_SRGB) return cudaErrorNotSupported;
    if (args.npx <= 0) return cudaSuccess;
    // 16-byte vector loads and stores: other pointers take the generic raster kernel.
    if (((uintptr_t)args.src | (uintptr_t)args.dst) & 15u) return cudaErrorNotSupported;
    if ((args.flags & ZS_CHAIN_CBRT_NONNEG) || !(args.flags & ZS_CHAIN_CBRT))
        return launch_chain_n<true>(args, sm_count, stream, threads, vectors);
    return launch_chain_n<false>(args, sm_count, stream, threads, vectors);
}

}  // namespace zs

ZS_TU_HOOKS(chain)
