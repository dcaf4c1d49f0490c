// k_noalloc.cu -- a resample entry point that never allocates device memory.
//
// Who needs it: code that may not call cudaMalloc at the moment it resamples -- a host
// application whose memory is budgeted up front (it hands every buffer in and forbids
// the library from growing the device footprint), a plugin running inside another
// framework's allocator, or a caller that must not trigger an allocation (and the
// implicit synchronisation some allocators imply) in the middle of a latency-critical
// loop.  Such a caller provides the input and output buffers; everything else this
// path needs lives in one fixed device array defined below.
//
// What it does: the same separable two-pass resample as resize_filtered (horizontal
// pass into an FP16 intermediate, vertical pass into the output), RGBA16F linear in
// and out, tightly packed rows.  The intermediate and the per-output-pixel filter
// tables (first tap, tap count, weights) are carved out of the static scratch array.
// The tables are computed on the GPU: FP64 kernel values normalised to sum 1 in
// FP64, stored as FP32 -- the same rule the host planner uses.
//
// Limits and sharing:
//  * the scratch array holds ZS_NOALLOC_SCRATCH_BYTES (32 MiB) per GPU.  With CUDA's lazy
//    module loading (the default) the driver reserves it when this file's module is first
//    used on a device -- at the first call of this entry point there -- and keeps it until
//    the process exits, so the first call may itself fail with an out-of-memory error.
//    Callers with a fixed device budget make one small warm-up call at start-up, outside
//    any stream capture, and count the 32 MiB in their budget;
//  * src and dst must be 8-byte aligned (the kernels move whole RGBA16F texels), and
//    widths and heights at most ZS_NOALLOC_MAX_SIDE;
//  * a call is rejected (ZS_ERR_INVALID_ARG, with the reason in zs_last_error) when its
//    tables plus the dst_width x src_height x 8-byte intermediate do not fit;
//  * every call on a device uses the same array and leaves its contents behind; nothing
//    in it has to start at zero, because each call writes every byte it later reads;
//  * calls whose work overlaps on the GPU (e.g. issued on different streams without an
//    ordering between them, such as the legacy default stream and a non-blocking stream)
//    race on the array and their results are undefined: order them on one stream or
//    serialise them.  The resample kernels clamp every tap window to their source, so a
//    race corrupts pixels but reads no memory outside the buffers.
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and keeps it for the life of the
//    process; make that first call before any stream capture begins, and do not use this
//    entry point across a reset of the device (cudaDeviceReset), which unloads the module.
#include <math.h>

#include <cstring>
#include <mutex>
#include <string>

#include "host/zs_host.hpp"
#include "zs_device.cuh"
#include "zs_kernels.h"

#define ZS_NOALLOC_SCRATCH_BYTES (32u << 20)
#define ZS_NOALLOC_MAX_DEVICES 64
#define ZS_NOALLOC_MAX_SIDE (1u << 24)

static __device__ __align__(256) unsigned char zs_noalloc_scratch[ZS_NOALLOC_SCRATCH_BYTES];

// Filter tables of one axis: first[dst], count[dst], weights[dst][taps].
__global__ void zs_noalloc_weights_kernel(int src_len, int dst_len, int filter, int taps, int32_t *first,
                                          int32_t *count, float *weights) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dst_len) return;
    const double s = (double)src_len / (double)dst_len, f = s > 1.0 ? s : 1.0;
    const double R = filter == 1 ? 3.0 : (filter == 2 ? 1.0 : 0.5);
    const double r = R * f;
    const double c = ((double)i + 0.5) * s;
    int lo = (int)floor(c - r), hi = (int)ceil(c + r);
    if (lo < 0) lo = 0;
    if (hi > src_len) hi = src_len;
    float *w = weights + (size_t)i * taps;
    double sum = 0.0;
    int n = 0, start = -1;
    // Pass 1: the normalising sum (FP64) and the tap window.
    for (int j = lo; j < hi && n < taps; ++j) {
        double v;
        if (filter == 0) {
            double a = c - 0.5 * f, b = c + 0.5 * f;
            double ov = fmin(b, j + 1.0) - fmax(a, (double)j);
            v = ov > 0 ? ov : 0.0;
        } else {
            double t = (j + 0.5 - c) / f;
            if (filter == 1) {
                double at = fabs(t);
                if (at >= 3.0) v = 0.0;
                else if (at < 1e-12) v = 1.0;
                else {
                    const double pi = 3.14159265358979323846;
                    v = (sin(pi * t) / (pi * t)) * (sin(pi * t / 3.0) / (pi * t / 3.0));
                }
            } else {
                v = fabs(t) < 1.0 ? 1.0 - fabs(t) : 0.0;
            }
        }
        if (start < 0) {
            if (v == 0.0) continue;
            start = j;
        }
        w[n++] = (float)v;     // provisional, rescaled below
        sum += v;
    }
    // Drop trailing zero taps and rescale in FP64 (recomputing each tap to keep FP64).
    while (n > 0 && w[n - 1] == 0.0f) n--;
    if (start < 0 || sum == 0.0) {
        int j = (int)floor(c);
        if (j > src_len - 1) j = src_len - 1;
        first[i] = j;
        count[i] = 1;
        w[0] = 1.0f;
        return;
    }
    for (int t = 0; t < n; ++t) {
        const int j = start + t;
        double v;
        if (filter == 0) {
            double a = c - 0.5 * f, b = c + 0.5 * f;
            double ov = fmin(b, j + 1.0) - fmax(a, (double)j);
            v = ov > 0 ? ov : 0.0;
        } else {
            double tt = (j + 0.5 - c) / f;
            if (filter == 1) {
                double at = fabs(tt);
                if (at >= 3.0) v = 0.0;
                else if (at < 1e-12) v = 1.0;
                else {
                    const double pi = 3.14159265358979323846;
                    v = (sin(pi * tt) / (pi * tt)) * (sin(pi * tt / 3.0) / (pi * tt / 3.0));
                }
            } else {
                v = fabs(tt) < 1.0 ? 1.0 - fabs(tt) : 0.0;
            }
        }
        w[t] = (float)(v / sum);
    }
    first[i] = start;
    count[i] = n;
}

namespace {

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[ZS_NOALLOC_MAX_DEVICES] = {nullptr};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Taps per output pixel of one axis (the host planner's rule); sides are bounded by
// ZS_NOALLOC_MAX_SIDE, so the count fits easily in 64 bits.
int64_t taps_for(uint32_t src, uint32_t dst, uint32_t filter) {
    const double s = (double)src / (double)dst, f = s > 1.0 ? s : 1.0;
    const double R = filter == 1 ? 3.0 : (filter == 2 ? 1.0 : 0.5);
    return (int64_t)ceil(2.0 * R * f) + 2;
}

}  // namespace

extern "C" int zs_resample_rgba16f_noalloc(const void *src, uint32_t src_width, uint32_t src_height, void *dst,
                                           uint32_t dst_width, uint32_t dst_height, uint32_t filter,
                                           void *stream) {
    using namespace zs;
    if (!src || !dst || src_width == 0 || src_height == 0 || dst_width == 0 || dst_height == 0 || filter > 2) {
        set_last_error("zs_resample_rgba16f_noalloc: null buffer, empty size or unknown filter");
        return ZS_ERR_INVALID_ARG;
    }
    if (src_width > ZS_NOALLOC_MAX_SIDE || src_height > ZS_NOALLOC_MAX_SIDE || dst_width > ZS_NOALLOC_MAX_SIDE ||
        dst_height > ZS_NOALLOC_MAX_SIDE) {
        set_last_error("zs_resample_rgba16f_noalloc: a width or height exceeds " +
                       std::to_string((unsigned)ZS_NOALLOC_MAX_SIDE));
        return ZS_ERR_INVALID_ARG;
    }
    if (((uintptr_t)src | (uintptr_t)dst) & 7u) {
        set_last_error("zs_resample_rgba16f_noalloc: src and dst must be 8-byte aligned (whole RGBA16F texels)");
        return ZS_ERR_INVALID_ARG;
    }
    const int64_t tx = taps_for(src_width, dst_width, filter), ty = taps_for(src_height, dst_height, filter);
    if (4ull * (uint64_t)dst_width * (uint64_t)tx > ZS_NOALLOC_SCRATCH_BYTES ||
        4ull * (uint64_t)dst_height * (uint64_t)ty > ZS_NOALLOC_SCRATCH_BYTES) {
        set_last_error("zs_resample_rgba16f_noalloc: the filter tables alone need more scratch than the fixed " +
                       std::to_string((size_t)ZS_NOALLOC_SCRATCH_BYTES) + " bytes");
        return ZS_ERR_INVALID_ARG;
    }
    // Scratch layout: [first_x count_x weights_x][first_y count_y weights_y][intermediate]
    const size_t fx = 0, cx = align256(fx + 4ull * dst_width), wx = align256(cx + 4ull * dst_width);
    const size_t fy = align256(wx + 4ull * dst_width * tx), cy = align256(fy + 4ull * dst_height);
    const size_t wy = align256(cy + 4ull * dst_height), mid = align256(wy + 4ull * dst_height * ty);
    const size_t need = mid + 8ull * dst_width * src_height;
    if (need > ZS_NOALLOC_SCRATCH_BYTES) {
        set_last_error("zs_resample_rgba16f_noalloc: needs " + std::to_string(need) +
                       " bytes of scratch (filter tables + dst_width x src_height x 8-byte intermediate), "
                       "more than the fixed " + std::to_string((size_t)ZS_NOALLOC_SCRATCH_BYTES) + " bytes");
        return ZS_ERR_INVALID_ARG;
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess || device < 0 || device >= ZS_NOALLOC_MAX_DEVICES) {
        set_last_error(std::string("zs_resample_rgba16f_noalloc: no usable current device: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[device]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, zs_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                set_last_error(std::string("zs_resample_rgba16f_noalloc: cudaGetSymbolAddress failed: ") +
                               cudaGetErrorString(e));
                return ZS_ERR_DEVICE;
            }
            g_noalloc_ptr[device] = p;
        }
        base = static_cast<unsigned char *>(g_noalloc_ptr[device]);
    }
    cudaStream_t s = (cudaStream_t)stream;
    int32_t *first_x = (int32_t *)(base + fx), *count_x = (int32_t *)(base + cx);
    int32_t *first_y = (int32_t *)(base + fy), *count_y = (int32_t *)(base + cy);
    float *w_x = (float *)(base + wx), *w_y = (float *)(base + wy);
    zs_noalloc_weights_kernel<<<(dst_width + 127) / 128, 128, 0, s>>>((int)src_width, (int)dst_width, (int)filter,
                                                                       (int)tx, first_x, count_x, w_x);
    zs_noalloc_weights_kernel<<<(dst_height + 127) / 128, 128, 0, s>>>((int)src_height, (int)dst_height, (int)filter,
                                                                        (int)ty, first_y, count_y, w_y);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("zs_resample_rgba16f_noalloc: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    add_kernel_launches(2);

    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const ZsFormat f16 = [] {
        ZsFormat f{};
        f.bits = ZS_BITS_FLOAT16X4;
        f.parts = ZS_PARTS_RGBA;
        f.bpp = 8;
        f.transfer = ZS_TRANSFER_LINEAR;
        f.fast = ZS_FAST_F16X4;
        return f;
    }();
    ZsRasterArgs a;
    memset(&a, 0, sizeof(a));
    a.producer = ZS_PR_RESAMPLE_H;
    a.nsrc = 1;
    a.src[0].ptr = (const uint8_t *)src;
    a.src[0].stride = 8ll * src_width;
    a.src[0].width = (int)src_width;
    a.src[0].height = (int)src_height;
    a.src[0].fmt = f16;
    a.index_x = first_x;
    a.index_y = count_x;
    a.weights = w_x;
    a.taps = (int32_t)tx;
    a.dst = base + mid;
    a.dst_stride = 8ll * dst_width;
    a.width = (int)dst_width;
    a.height = (int)src_height;
    a.dst_fmt = f16;
    e = launch_raster(a, sms, s);
    if (e == cudaSuccess) {
        a.producer = ZS_PR_RESAMPLE_V;
        a.src[0].ptr = base + mid;
        a.src[0].stride = 8ll * dst_width;
        a.src[0].width = (int)dst_width;
        a.src[0].height = (int)src_height;
        a.index_x = first_y;
        a.index_y = count_y;
        a.weights = w_y;
        a.taps = (int32_t)ty;
        a.dst = (uint8_t *)dst;
        a.dst_stride = 8ll * dst_width;
        a.height = (int)dst_height;
        e = launch_raster(a, sms, s);
    }
    if (e != cudaSuccess) {
        set_last_error(std::string("zs_resample_rgba16f_noalloc: ") + cudaGetErrorString(e));
        return ZS_ERR_DEVICE;
    }
    return ZS_OK;
}

ZS_TU_HOOKS(noalloc)
