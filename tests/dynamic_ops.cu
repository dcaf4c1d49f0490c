// Custom operations for the plugin-point tests (zs_register_op): kernels over the
// zs_dyn_args parameter block of include/zosimos.h, launched with 16 x 16 blocks.
#include "../include/zosimos.h"

__device__ __forceinline__ bool zs_test_pixel(const zs_dyn_args &a, int &x, int &y) {
    x = blockIdx.x * blockDim.x + threadIdx.x;
    y = blockIdx.y * blockDim.y + threadIdx.y;
    return x < a.width && y < a.height;
}

// 1 - rgb, alpha kept.
extern "C" __global__ void zs_test_invert(zs_dyn_args a) {
    int x, y;
    if (!zs_test_pixel(a, x, y)) return;
    const float4 s = reinterpret_cast<const float4 *>(a.src[0])[(size_t)y * a.src_width[0] + x];
    reinterpret_cast<float4 *>(a.dst)[(size_t)y * a.width + x] = make_float4(1.f - s.x, 1.f - s.y, 1.f - s.z, s.w);
}

// lhs + t (rhs - lhs) per channel, t the first uniform float.
extern "C" __global__ void zs_test_mix(zs_dyn_args a) {
    int x, y;
    if (!zs_test_pixel(a, x, y)) return;
    const float t = a.uniform_len >= 4 ? *reinterpret_cast<const float *>(a.uniforms) : 0.5f;
    const float4 p = reinterpret_cast<const float4 *>(a.src[0])[(size_t)y * a.src_width[0] + x];
    const float4 q = reinterpret_cast<const float4 *>(a.src[1])[(size_t)y * a.src_width[1] + x];
    reinterpret_cast<float4 *>(a.dst)[(size_t)y * a.width + x] =
        make_float4(fmaf(t, q.x - p.x, p.x), fmaf(t, q.y - p.y, p.y), fmaf(t, q.z - p.z, p.z), fmaf(t, q.w - p.w, p.w));
}

// A constructor: (x + 0.5) / w, (y + 0.5) / h, the uniform float, 1.
extern "C" __global__ void zs_test_gradient(zs_dyn_args a) {
    int x, y;
    if (!zs_test_pixel(a, x, y)) return;
    const float b = a.uniform_len >= 4 ? *reinterpret_cast<const float *>(a.uniforms) : 0.f;
    reinterpret_cast<float4 *>(a.dst)[(size_t)y * a.width + x] =
        make_float4(((float)x + 0.5f) / (float)a.width, ((float)y + 0.5f) / (float)a.height, b, 1.f);
}
