// zs_tables.cu -- exact sRGB8 <-> linear tables, computed on the host in FP64 and
// uploaded once per device.
//
// The reference decodes and encodes sRGB RGBA8 images in fixed-function hardware
// (Rgba8UnormSrgb, lib/zosimos/src/program.rs:794-805): the texture unit applies the
// sRGB EOTF on sampling and the ROP applies the OETF with round-to-nearest on store.
// Here both directions are table driven:
//   * decode: 256 correctly rounded f32 values of the EOTF (stage.frag:345-352);
//   * encode: for every f32 x in [2^-13, 1] the bucket (bits(x) >> 16) holds the
//     code at the bucket start and at most one rounding threshold of
//     round(255 * OETF(x)); thresholds are EOTF((k + 0.5) / 255) rounded up to f32.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <vector>

#include "zs_device.cuh"
#include "zs_kernels.h"

namespace zs {

ZS_DEVICE_TUS(ZS_TU_DECLARE_HOOKS)

static double eotf_srgb(double v) {
    if (v < -0.04045) return -std::pow((-v + 0.055) / 1.055, 2.4);
    if (v <= 0.04045) return v / 12.92;
    return std::pow((v + 0.055) / 1.055, 2.4);
}

static uint32_t fbits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

// Bucketed threshold table: entry j covers the floats whose bits >> 16 == base + j.
static void build_encode(uint32_t *encode, uint32_t entries, uint32_t base, double shift) {
    uint32_t thr[255];
    for (int k = 0; k < 255; ++k) {
        double x = eotf_srgb((k + 0.5) / 255.0) + shift;
        float f = (float)x;
        if ((double)f < x) f = std::nextafter(f, 2.0f);
        thr[k] = fbits(f);
    }
    for (uint32_t j = 0; j < entries; ++j) {
        uint32_t start = (j + base) << 16, end = start + 0x10000u;
        uint32_t code = 0, inside = 0, nin = 0;
        for (int k = 0; k < 255; ++k) {
            if (thr[k] <= start) code = (uint32_t)k + 1;
            else if (thr[k] < end) { inside = thr[k] & 0xffffu; ++nin; }
        }
        if (nin > 1) throw std::runtime_error("sRGB encode bucket holds two thresholds");
        uint32_t t = nin ? inside : 0x10000u;
        encode[j] = (code << 24) + (1u << 24) - t - start;
    }
}

void build_srgb_tables(float *decode, uint32_t *encode, uint32_t *encode_shifted) {
    for (int v = 0; v < 256; ++v) decode[v] = (float)eotf_srgb(v / 255.0);
    build_encode(encode, ZS_ENC_ENTRIES, ZS_ENC_BASE, 0.0);
    // x' = x + 2^-12 (x in [0, 1]); thresholds move by the same exact shift.
    build_encode(encode_shifted, ZS_ENCS_ENTRIES, ZS_ENCS_BASE, 1.0 / 4096.0);
}

static std::mutex g_tables_mutex;
static std::vector<int> g_tables_ready;

cudaError_t init_device_tables(int device) {
    std::lock_guard<std::mutex> lock(g_tables_mutex);
    if (device < 0) return cudaErrorInvalidDevice;
    if ((int)g_tables_ready.size() <= device) g_tables_ready.resize(device + 1, 0);
    if (g_tables_ready[device]) return cudaSuccess;
    static float dec[256];
    static uint32_t enc[ZS_ENC_ENTRIES], encs[ZS_ENCS_ENTRIES];
    static bool built = false;
    if (!built) {
        build_srgb_tables(dec, enc, encs);
        built = true;
    }
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return e;
    if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
#define ZS_UPLOAD(NAME) \
    if (e == cudaSuccess) e = tu_upload_tables_##NAME(dec, enc, encs);
    ZS_DEVICE_TUS(ZS_UPLOAD)
#undef ZS_UPLOAD
    if (prev != device) cudaSetDevice(prev);
    if (e == cudaSuccess) g_tables_ready[device] = 1;
    return e;
}

cudaError_t read_device_status(int device, uint32_t *flags, bool clear) {
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return e;
    if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
    // The status bits of every kernel file, ORed.
    unsigned int v = 0;
#define ZS_STATUS(NAME)                                        \
    if (e == cudaSuccess) {                                    \
        unsigned int w = 0;                                    \
        e = tu_device_status_##NAME(&w, clear);                \
        v |= w;                                                \
    }
    ZS_DEVICE_TUS(ZS_STATUS)
#undef ZS_STATUS
    if (prev != device) cudaSetDevice(prev);
    *flags = v;
    return e;
}

}  // namespace zs
