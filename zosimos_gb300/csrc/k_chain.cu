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
// Data path per thread: 16-byte coalesced streaming loads (4 pixels), sRGB decode
// through a lane-replicated shared table (conflict-free: lane l reads column l),
// FP32 arithmetic, exact round-to-nearest sRGB encode through the bucketed
// threshold table, alpha bytes passed through (decode/encode of a unorm8 alpha is
// the identity), 16-byte streaming stores.
#include <atomic>

#include "zs_device.cuh"
#include "zs_kernels.h"

namespace zs {
extern std::atomic<uint64_t> g_kernel_launches;
}

#define ZS_CHAIN_THREADS 256
#define ZS_CHAIN_UNROLL 2

struct ZsChainSmem {
    float lut[256 * 32];
    uint32_t enc[ZS_ENC_ENTRIES];
};

__device__ __forceinline__ void zs_m3(const float *m, float &r, float &g, float &b) {
    float x = r, y = g, z = b;
    r = fmaf(m[0], x, fmaf(m[1], y, m[2] * z));
    g = fmaf(m[3], x, fmaf(m[4], y, m[5] * z));
    b = fmaf(m[6], x, fmaf(m[7], y, m[8] * z));
}

template <bool CBRT, bool CUBE, bool CLAMP>
__device__ __forceinline__ uint32_t zs_chain_px(uint32_t w, const float *lut_lane, const uint32_t *enc,
                                                const ZsChainArgs &a) {
    float r = lut_lane[(w & 255u) << 5];
    float g = lut_lane[((w >> 8) & 255u) << 5];
    float b = lut_lane[((w >> 16) & 255u) << 5];
    zs_m3(a.m[0], r, g, b);
    if (CBRT) { r = zs_scbrt(r); g = zs_scbrt(g); b = zs_scbrt(b); }
    zs_m3(a.m[1], r, g, b);
    if (CUBE) { r = r * r * r; g = g * g * g; b = b * b * b; }
    zs_m3(a.m[2], r, g, b);
    if (CLAMP) { r = __saturatef(r); g = __saturatef(g); b = __saturatef(b); }
    zs_m3(a.m[3], r, g, b);
    return zs_enc_srgb8(enc, r) | (zs_enc_srgb8(enc, g) << 8) | (zs_enc_srgb8(enc, b) << 16) | (w & 0xff000000u);
}

template <bool CBRT, bool CUBE, bool CLAMP>
__global__ void __launch_bounds__(ZS_CHAIN_THREADS) zs_chain_srgb8_kernel(const __grid_constant__ ZsChainArgs a) {
    extern __shared__ __align__(16) unsigned char zs_smem_raw[];
    ZsChainSmem &sm = *reinterpret_cast<ZsChainSmem *>(zs_smem_raw);
    for (int i = threadIdx.x; i < 256 * 32; i += blockDim.x) sm.lut[i] = zs_srgb_decode_lut[i >> 5];
    for (int i = threadIdx.x; i < ZS_ENC_ENTRIES; i += blockDim.x) sm.enc[i] = zs_srgb_encode_tab[i];
    __syncthreads();
    const float *lut_lane = sm.lut + (threadIdx.x & 31);
    const uint32_t *enc = sm.enc;

    const uint4 *in = reinterpret_cast<const uint4 *>(a.src);
    uint4 *out = reinterpret_cast<uint4 *>(a.dst);
    const int64_t nvec = a.npx >> 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; v + (ZS_CHAIN_UNROLL - 1) * stride < nvec; v += ZS_CHAIN_UNROLL * stride) {
        uint4 w[ZS_CHAIN_UNROLL];
#pragma unroll
        for (int u = 0; u < ZS_CHAIN_UNROLL; ++u) w[u] = __ldcs(in + v + u * stride);
#pragma unroll
        for (int u = 0; u < ZS_CHAIN_UNROLL; ++u) {
            uint4 o;
            o.x = zs_chain_px<CBRT, CUBE, CLAMP>(w[u].x, lut_lane, enc, a);
            o.y = zs_chain_px<CBRT, CUBE, CLAMP>(w[u].y, lut_lane, enc, a);
            o.z = zs_chain_px<CBRT, CUBE, CLAMP>(w[u].z, lut_lane, enc, a);
            o.w = zs_chain_px<CBRT, CUBE, CLAMP>(w[u].w, lut_lane, enc, a);
            __stcs(out + v + u * stride, o);
        }
    }
    for (; v < nvec; v += stride) {
        uint4 w = __ldcs(in + v), o;
        o.x = zs_chain_px<CBRT, CUBE, CLAMP>(w.x, lut_lane, enc, a);
        o.y = zs_chain_px<CBRT, CUBE, CLAMP>(w.y, lut_lane, enc, a);
        o.z = zs_chain_px<CBRT, CUBE, CLAMP>(w.z, lut_lane, enc, a);
        o.w = zs_chain_px<CBRT, CUBE, CLAMP>(w.w, lut_lane, enc, a);
        __stcs(out + v, o);
    }
    // Tail pixels (npx not a multiple of 4).
    const int64_t tail0 = nvec << 2;
    const int64_t t = tail0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < a.npx && t < tail0 + 4) {
        const uint32_t *in32 = reinterpret_cast<const uint32_t *>(a.src);
        uint32_t *out32 = reinterpret_cast<uint32_t *>(a.dst);
        out32[t] = zs_chain_px<CBRT, CUBE, CLAMP>(in32[t], lut_lane, enc, a);
    }
}

namespace zs {

template <bool CBRT, bool CUBE, bool CLAMP>
static cudaError_t launch_chain_t(const ZsChainArgs &args, int sm_count, cudaStream_t stream) {
    const size_t smem = sizeof(ZsChainSmem);
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(zs_chain_srgb8_kernel<CBRT, CUBE, CLAMP>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zs_chain_srgb8_kernel<CBRT, CUBE, CLAMP>,
                                                                  ZS_CHAIN_THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const int64_t nvec = (args.npx + 3) / 4;
    int64_t blocks = (nvec + ZS_CHAIN_THREADS - 1) / ZS_CHAIN_THREADS;
    const int64_t cap = (int64_t)(sm_count > 0 ? sm_count : 148) * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    zs_chain_srgb8_kernel<CBRT, CUBE, CLAMP><<<(unsigned)blocks, ZS_CHAIN_THREADS, smem, stream>>>(args);
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

cudaError_t launch_chain(const ZsChainArgs &args, uint8_t src_fast, uint8_t dst_fast, int sm_count,
                         cudaStream_t stream) {
    if (src_fast != ZS_FAST_RGBA8_SRGB || dst_fast != ZS_FAST_RGBA8_SRGB) return cudaErrorNotSupported;
    if (args.npx <= 0) return cudaSuccess;
    const bool cb = args.flags & ZS_CHAIN_CBRT, cu = args.flags & ZS_CHAIN_CUBE, cl = args.flags & ZS_CHAIN_CLAMP;
    if (cb && cu && cl) return launch_chain_t<true, true, true>(args, sm_count, stream);
    if (cb && cu && !cl) return launch_chain_t<true, true, false>(args, sm_count, stream);
    if (cb && !cu && cl) return launch_chain_t<true, false, true>(args, sm_count, stream);
    if (cb && !cu && !cl) return launch_chain_t<true, false, false>(args, sm_count, stream);
    if (!cb && cu && cl) return launch_chain_t<false, true, true>(args, sm_count, stream);
    if (!cb && cu && !cl) return launch_chain_t<false, true, false>(args, sm_count, stream);
    if (!cb && !cu && cl) return launch_chain_t<false, false, true>(args, sm_count, stream);
    return launch_chain_t<false, false, false>(args, sm_count, stream);
}

}  // namespace zs
