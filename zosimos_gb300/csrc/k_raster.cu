// k_raster.cu -- the generic raster kernel: one launch per materialised register.
//
// Replaces one render pass of the reference (a quad draw of a fragment shader over
// the target, lib/zosimos/src/program.rs:1486-1533, run.rs:2678-2739) *plus* every
// per-pixel op the planner fused behind it, so that intermediates never round-trip
// through HBM.  Producers:
//   LOAD      pixel-aligned operands (colour ops, inject)            linear/inject.frag
//   BILINEAR  bilinear.frag:14-20                                     construct
//   SOLID     solid_rgb                                               construct
//   QUAD      copy.frag + box.vert:43-59 (crop, inscribe)             nearest gather
//   AFFINE    affine paint of `above` over `below`                    nearest / bilinear
//   PALETTE   palette.frag:21-31                                      coordinate gather
//   INDEX     resize through a nearest index table                    gather
//   BLEND     blend of `above` at an offset over `below`              (new op)
//   RESAMPLE  one separable filter pass (FP64-normalised weights)      (new op)
//   BOX3      3x3 stencil: the derivative operators                   box3.frag:12-53
//   NORMAL2D  normal density generator                                distribution_normal2d.frag
// Gathers whose source and destination formats agree and that carry no fused
// program copy texel bytes verbatim (integer-exact).
#include <atomic>

#include "zs_device.cuh"
#include "zs_kernels.h"

namespace zs {
std::atomic<uint64_t> g_kernel_launches{0};
uint64_t kernel_launch_count() { return g_kernel_launches.load(); }
void add_kernel_launches(uint64_t n) { g_kernel_launches.fetch_add(n); }
}  // namespace zs

// PCG4D hash (Jarzynski and Olano, "Hash Functions for GPU Rendering", JCGT 9(3), 2020),
// as fractal_noise.frag applies it to uvec4(cell, 0, 0).
__device__ __forceinline__ uint4 zs_pcg4d(uint4 v) {
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    v.x ^= v.x >> 16; v.y ^= v.y >> 16; v.z ^= v.z >> 16; v.w ^= v.w >> 16;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    return v;
}

// hash(): the four hashed words as floats divided by float(0xFFFFFFFF) (= 2^32 in f32).
__device__ __forceinline__ float4 zs_noise_hash(uint32_t cx, uint32_t cy) {
    const uint4 h = zs_pcg4d(make_uint4(cx, cy, 0u, 0u));
    const float m = 4294967296.0f;
    return make_float4(__fdiv_rn(__uint2float_rn(h.x), m), __fdiv_rn(__uint2float_rn(h.y), m),
                       __fdiv_rn(__uint2float_rn(h.z), m), __fdiv_rn(__uint2float_rn(h.w), m));
}

// noise() of fractal_noise.frag at grid point (ptx, pty): value noise of the four cell
// corners, smoothstep weights, mix(a, b, u.x) + (c - a) u.y (1 - u.x) + (d - b) u.x u.y.
__device__ __forceinline__ float zs_noise_mix(float a, float b, float c, float d, float ux, float uy) {
    const float m = __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, ux)), __fmul_rn(b, ux));
    const float t1 = __fmul_rn(__fmul_rn(__fsub_rn(c, a), uy), __fsub_rn(1.0f, ux));
    const float t2 = __fmul_rn(__fmul_rn(__fsub_rn(d, b), ux), uy);
    return __fadd_rn(__fadd_rn(m, t1), t2);
}

__device__ __forceinline__ float4 zs_value_noise(float ptx, float pty) {
    const float flx = floorf(ptx), fly = floorf(pty);
    const float fx = __fsub_rn(ptx, flx), fy = __fsub_rn(pty, fly);
    const uint32_t cx = (uint32_t)(int)flx, cy = (uint32_t)(int)fly;
    const float4 A = zs_noise_hash(cx, cy), B = zs_noise_hash(cx + 1u, cy), C = zs_noise_hash(cx, cy + 1u),
                 D = zs_noise_hash(cx + 1u, cy + 1u);
    const float ux = __fmul_rn(__fmul_rn(fx, fx), __fsub_rn(3.0f, __fmul_rn(2.0f, fx)));
    const float uy = __fmul_rn(__fmul_rn(fy, fy), __fsub_rn(3.0f, __fmul_rn(2.0f, fy)));
    return make_float4(zs_noise_mix(A.x, B.x, C.x, D.x, ux, uy), zs_noise_mix(A.y, B.y, C.y, D.y, ux, uy),
                       zs_noise_mix(A.z, B.z, C.z, D.z, ux, uy), zs_noise_mix(A.w, B.w, C.w, D.w, ux, uy));
}

// The gathered image of an AFFINE launch at (x, y): a stored texel, or (virt1) its
// pixel-aligned producer and program evaluated here.
__device__ __forceinline__ float4 zs_src1_px(const ZsRasterArgs &a, int x, int y) {
    if (!a.virt1) return zs_load_px(a.src[1], x, y);
    float4 r = zs_load_px(a.vsrc[0], x, y), r2 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.vproducer == ZS_PR_BLEND) {
        const int ax = x - a.vrect[0], ay = y - a.vrect[1];
        if (ax >= 0 && ay >= 0 && ax < a.vsrc[1].width && ay < a.vsrc[1].height)
            zs_blend_px(r, zs_load_px(a.vsrc[1], ax, ay), a.vmode, a.vstraight);
    } else if (a.vnsrc > 1) {
        r2 = zs_load_px(a.vsrc[1], x, y);
    }
    zs_run_program(a.vprog, a.fmts, r, r2);
    return r;
}

__global__ void __launch_bounds__(256) zs_raster_kernel(const __grid_constant__ ZsRasterArgs a) {
    // Programmatic dependent launch: let the next launch in the stream be scheduled now, and
    // touch no global memory before the previous grid has completed and its writes are visible
    // (griddepcontrol.wait is a no-op for an ordinary launch).
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // Affine gathers walk 32 x 8 pixel tiles (8 x 4 per warp) so that a warp's samples
    // fall into a compact source footprint; everything else walks rows.
    const bool tiled = a.producer == ZS_PR_AFFINE;
    const int tiles_x = (a.width + 31) >> 5;
    const int64_t n = tiled ? (int64_t)tiles_x * ((a.height + 7) >> 3) * 256 : (int64_t)a.width * a.height;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        int x, y;
        if (tiled) {
            zs_tile_pixel(i, tiles_x, x, y);
            if (x >= a.width || y >= a.height) continue;
        } else {
            y = (int)(i / a.width);
            x = (int)(i - (int64_t)y * a.width);
        }
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f), r2 = r;
        uint4 raw = make_uint4(0, 0, 0, 0);
        bool is_raw = false;
        const ZsSource &s0 = a.src[0];
        const ZsSource &s1 = a.src[1];
        switch (a.producer) {
        case ZS_PR_LOAD:
            r = zs_load_px(s0, x, y);
            if (a.nsrc > 1) r2 = zs_load_px(s1, x, y);
            break;
        case ZS_PR_BILINEAR: {
            // Unfused IEEE operations in a fixed order, so that the value (and any
            // truncating quantisation of it) is reproducible on the CPU.
            float u = __fdiv_rn((float)x + 0.5f, (float)a.width), v = __fdiv_rn((float)y + 0.5f, (float)a.height);
            float uv = __fmul_rn(u, v);
            const float *p = a.cons;
            float o[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float fu = __fadd_rn(__fmul_rn(p[k], 1.f - u), __fmul_rn(p[4 + k], u));
                float fv = __fadd_rn(__fmul_rn(p[8 + k], 1.f - v), __fmul_rn(p[12 + k], v));
                float fw = __fadd_rn(__fmul_rn(p[16 + k], 1.f - uv), __fmul_rn(p[20 + k], uv));
                o[k] = __fadd_rn(__fadd_rn(fu, fv), fw);
            }
            r = make_float4(o[0], o[1], o[2], o[3]);
        } break;
        case ZS_PR_SOLID:
            r = make_float4(a.cons[0], a.cons[1], a.cons[2], a.cons[3]);
            break;
        case ZS_PR_QUAD: {
            const bool inside = x >= a.rect[0] && x < a.rect[2] && y >= a.rect[1] && y < a.rect[3];
            if (inside) {
                int sx = zs_clampi(zs_quad_src(x, a.rect[0], a.rect[2], a.sel[0], a.sel[2]), 0, s1.width - 1);
                int sy = zs_clampi(zs_quad_src(y, a.rect[1], a.rect[3], a.sel[1], a.sel[3]), 0, s1.height - 1);
                if (a.raw_copy) {
                    raw = zs_load_raw(s1.ptr + (int64_t)sy * s1.stride + (int64_t)sx * s1.fmt.bpp, s1.fmt.bpp);
                    is_raw = true;
                } else {
                    r = zs_load_px(s1, sx, sy);
                }
            } else if (a.has_below) {
                if (a.raw_copy) {
                    raw = zs_load_raw(s0.ptr + (int64_t)y * s0.stride + (int64_t)x * s0.fmt.bpp, s0.fmt.bpp);
                    is_raw = true;
                } else {
                    r = zs_load_px(s0, x, y);
                }
            } else if (a.raw_copy) {
                is_raw = true;                      // zero canvas: zero bytes
            } else {
                r = make_float4(a.cons[0], a.cons[1], a.cons[2], a.cons[3]);   // constant canvas
            }
        } break;
        case ZS_PR_AFFINE: {
            float qx, qy;
            zs_affine_map(a.aff, x, y, qx, qy);
            const bool inside = qx >= 0.0f && qx < (float)s1.width && qy >= 0.0f && qy < (float)s1.height;
            if (inside && !a.bilinear) {
                int ix = min((int)floorf(qx), s1.width - 1), iy = min((int)floorf(qy), s1.height - 1);
                if (a.raw_copy) {
                    raw = zs_load_raw(s1.ptr + (int64_t)iy * s1.stride + (int64_t)ix * s1.fmt.bpp, s1.fmt.bpp);
                    is_raw = true;
                } else {
                    r = zs_src1_px(a, ix, iy);
                }
            } else if (inside) {
                float tx = qx - 0.5f, ty = qy - 0.5f;
                float fx0 = floorf(tx), fy0 = floorf(ty);
                float fx = tx - fx0, fy = ty - fy0;
                int x0 = (int)fx0, y0 = (int)fy0;
                int xa = zs_clampi(x0, 0, s1.width - 1), xb = zs_clampi(x0 + 1, 0, s1.width - 1);
                int ya = zs_clampi(y0, 0, s1.height - 1), yb = zs_clampi(y0 + 1, 0, s1.height - 1);
                float4 top = zs_lerp4(zs_src1_px(a, xa, ya), zs_src1_px(a, xb, ya), fx);
                float4 bot = zs_lerp4(zs_src1_px(a, xa, yb), zs_src1_px(a, xb, yb), fx);
                r = zs_lerp4(top, bot, fy);
            } else if (a.has_below) {
                if (a.raw_copy) {
                    raw = zs_load_raw(s0.ptr + (int64_t)y * s0.stride + (int64_t)x * s0.fmt.bpp, s0.fmt.bpp);
                    is_raw = true;
                } else {
                    r = zs_load_px(s0, x, y);
                }
            } else if (a.raw_copy) {
                is_raw = true;                      // zero canvas: zero bytes
            } else {
                r = make_float4(a.cons[0], a.cons[1], a.cons[2], a.cons[3]);   // constant canvas
            }
        } break;
        case ZS_PR_PALETTE: {
            // palette.frag:22-31: uv = channels . basis + 0.5 / size(rhs); nearest sample of lhs.
            float4 basis = zs_load_px(s1, x, y);
            const float *c = a.cons;
            float u = c[0] * basis.x + c[1] * basis.y + c[2] * basis.z + c[3] * basis.w;
            float v = c[4] * basis.x + c[5] * basis.y + c[6] * basis.z + c[7] * basis.w;
            float tu = __fadd_rn(u, __fdiv_rn(0.5f, (float)s1.width));
            float tv = __fadd_rn(v, __fdiv_rn(0.5f, (float)s1.height));
            int ix = zs_clampi((int)floorf(__fmul_rn(tu, (float)s0.width)), 0, s0.width - 1);
            int iy = zs_clampi((int)floorf(__fmul_rn(tv, (float)s0.height)), 0, s0.height - 1);
            if (a.raw_copy) {
                raw = zs_load_raw(s0.ptr + (int64_t)iy * s0.stride + (int64_t)ix * s0.fmt.bpp, s0.fmt.bpp);
                is_raw = true;
            } else {
                r = zs_load_px(s0, ix, iy);
            }
        } break;
        case ZS_PR_INDEX: {
            int ix = a.index_x[x], iy = a.index_y[y];
            if (a.raw_copy) {
                raw = zs_load_raw(s0.ptr + (int64_t)iy * s0.stride + (int64_t)ix * s0.fmt.bpp, s0.fmt.bpp);
                is_raw = true;
            } else {
                r = zs_load_px(s0, ix, iy);
            }
        } break;
        case ZS_PR_BLEND: {
            r = zs_load_px(s0, x, y);
            int ax = x - a.rect[0], ay = y - a.rect[1];
            if (ax >= 0 && ay >= 0 && ax < s1.width && ay < s1.height) {
                float4 s = zs_load_px(s1, ax, ay);
                zs_blend_px(r, s, a.blend_mode, a.straight);
            }
        } break;
        case ZS_PR_NORMAL2D: {
            // distribution_normal2d.frag: pos = 2 (uv - 0.5) - mu at the pixel centre; the
            // GLSL mat2 columns are (C+00, C+01) and (C+10, C+11).
            const float *c = a.cons;
            const float u = __fdiv_rn((float)x + 0.5f, (float)a.width), v = __fdiv_rn((float)y + 0.5f, (float)a.height);
            const float px = 2.0f * (u - 0.5f) - c[0], py = 2.0f * (v - 0.5f) - c[1];
            const float q = px * (c[2] * px + c[4] * py) + py * (c[3] * px + c[5] * py);
            const float val = expf(-0.5f * q) / sqrtf(c[6]);
            r = make_float4(val, val, val, 1.0f);
        } break;
        case ZS_PR_FRACTAL: {
            // fractal_noise.frag: fbm(uv) at the pixel centre, every product and sum rounded
            // separately (no contraction), so the result is reproducible on the host.
            const float *c = a.cons;
            float px = __fdiv_rn((float)x + 0.5f, (float)a.width), py = __fdiv_rn((float)y + 0.5f, (float)a.height);
            float amp = c[2];
            const int octaves = (int)c[4];
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int o = 0; o < octaves; ++o) {
                const float4 n = zs_value_noise(__fmul_rn(px, c[0]), __fmul_rn(py, c[1]));
                acc.x = __fadd_rn(acc.x, __fmul_rn(amp, n.x));
                acc.y = __fadd_rn(acc.y, __fmul_rn(amp, n.y));
                acc.z = __fadd_rn(acc.z, __fmul_rn(amp, n.z));
                acc.w = __fadd_rn(acc.w, __fmul_rn(amp, n.w));
                // next_point: (x, y) <- 2 (cos .5 x - sin .5 y, sin .5 x + cos .5 y)
                const float nx = __fadd_rn(__fmul_rn(c[5], px), __fmul_rn(-c[6], py));
                const float ny = __fadd_rn(__fmul_rn(c[6], px), __fmul_rn(c[5], py));
                px = nx;
                py = ny;
                amp = __fmul_rn(amp, c[3]);
            }
            r = acc;
        } break;
        case ZS_PR_BOX3: {
            // box3.frag:12-53: clamp-to-edge nearest taps (the default sampler); each row of
            // the component-wise product is summed, then the three row sums; alpha 1.
            float rows[3][3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int yy = zs_clampi(y + j - 1, 0, s0.height - 1);
                float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const float w = a.cons[3 * j + i];
                    const float4 v = zs_load_px(s0, zs_clampi(x + i - 1, 0, s0.width - 1), yy);
                    acc.x = fmaf(w, v.x, acc.x);
                    acc.y = fmaf(w, v.y, acc.y);
                    acc.z = fmaf(w, v.z, acc.z);
                }
                rows[j][0] = acc.x;
                rows[j][1] = acc.y;
                rows[j][2] = acc.z;
            }
            r = make_float4(rows[0][0] + rows[1][0] + rows[2][0], rows[0][1] + rows[1][1] + rows[2][1],
                            rows[0][2] + rows[1][2] + rows[2][2], 1.0f);
        } break;
        case ZS_PR_RESAMPLE_H: {
            // The tap window is clamped to the source row and the table width, so that no
            // table content (e.g. one rewritten by an overlapping call of the allocation-free
            // entry point) can index outside the source.
            const int first = min(max(a.index_x[x], 0), s0.width - 1);
            const int cnt = min(min(a.index_y[x], a.taps), s0.width - first);
            const float *w = a.weights + (int64_t)x * a.taps;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int t = 0; t < cnt; ++t) {
                float4 s = zs_load_px(s0, first + t, y);
                float wt = w[t];
                acc.x = fmaf(wt, s.x, acc.x); acc.y = fmaf(wt, s.y, acc.y);
                acc.z = fmaf(wt, s.z, acc.z); acc.w = fmaf(wt, s.w, acc.w);
            }
            r = acc;
        } break;
        case ZS_PR_RESAMPLE_V: {
            const int first = min(max(a.index_x[y], 0), s0.height - 1);
            const int cnt = min(min(a.index_y[y], a.taps), s0.height - first);
            const float *w = a.weights + (int64_t)y * a.taps;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int t = 0; t < cnt; ++t) {
                float4 s = zs_load_px(s0, x, first + t);
                float wt = w[t];
                acc.x = fmaf(wt, s.x, acc.x); acc.y = fmaf(wt, s.y, acc.y);
                acc.z = fmaf(wt, s.z, acc.z); acc.w = fmaf(wt, s.w, acc.w);
            }
            r = acc;
        } break;
        default: break;
        }
        uint8_t *dp = a.dst + (int64_t)y * a.dst_stride + (int64_t)x * a.dst_fmt.bpp;
        if (is_raw) {
            zs_store_raw(dp, a.dst_fmt.bpp, raw);
            continue;
        }
        zs_run_program(a.prog, a.fmts, r, r2);
        zs_store_raw(dp, a.dst_fmt.bpp, zs_encode_raw(a.dst_fmt, r));
    }
}

// AFFINE with bilinear sampling of an RGBA16F image under an affine (not projective)
// inverse: the same arithmetic, in the same order, as the generic kernel's AFFINE case
// without the per-tap format dispatch.  Tiles of 32 x 32 pixels (8 x 16 per warp); each
// thread takes four pixels four rows apart (four samples in flight).
#define ZS_AFF_PX 4
__global__ void __launch_bounds__(256) zs_affine_f16_kernel(const __grid_constant__ ZsRasterArgs a) {
    const ZsSource &s0 = a.src[0], &s1 = a.src[1];
    // 32-bit tile arithmetic: the launcher takes this kernel below 2^31 threads' worth of tiles.
    const int tiles_x = (a.width + 31) >> 5;
    const int n = tiles_x * ((a.height + 8 * ZS_AFF_PX - 1) / (8 * ZS_AFF_PX)) * 256;
    const int step = gridDim.x * blockDim.x;
    const float fw = (float)s1.width, fh = (float)s1.height;
    const bool plain = zs_plain_f16_out(a.prog, a.dst_fmt);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        const int tile = i >> 8;
        const int t = i & 255, w = t >> 5, l = t & 31;
        const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
        const int x = (tx << 5) + ((w & 3) << 3) + (l & 7);
        const int y0 = ty * (8 * ZS_AFF_PX) + (w >> 2) * (4 * ZS_AFF_PX) + (l >> 3);
        if (x >= a.width || y0 >= a.height) continue;
        const float cx = (float)x + 0.5f;
        float4 r[ZS_AFF_PX];
#pragma unroll
        for (int p = 0; p < ZS_AFF_PX; ++p) {
            const int y = min(y0 + 4 * p, a.height - 1);
            const float cy = (float)y + 0.5f;
            const float qx = fmaf(a.aff[0], cx, fmaf(a.aff[1], cy, a.aff[2]));
            const float qy = fmaf(a.aff[3], cx, fmaf(a.aff[4], cy, a.aff[5]));
            if (qx >= 0.0f && qx < fw && qy >= 0.0f && qy < fh) {
                const float txf = qx - 0.5f, tyf = qy - 0.5f;
                const float fx0 = floorf(txf), fy0 = floorf(tyf);
                const float fx = txf - fx0, fy = tyf - fy0;
                const int x0 = (int)fx0, y0i = (int)fy0;
                // 0 <= q < size puts the first tap in [-1, size - 1]: one bound per tap is enough.
                const int xa = max(x0, 0), xb = min(x0 + 1, s1.width - 1);
                const int ya = max(y0i, 0), yb = min(y0i + 1, s1.height - 1);
                const uint8_t *ra = s1.ptr + (int64_t)ya * s1.stride, *rb = s1.ptr + (int64_t)yb * s1.stride;
                const float4 t00 = zs_h4(__ldg((const uint2 *)(ra + (int64_t)xa * 8)));
                const float4 t01 = zs_h4(__ldg((const uint2 *)(ra + (int64_t)xb * 8)));
                const float4 t10 = zs_h4(__ldg((const uint2 *)(rb + (int64_t)xa * 8)));
                const float4 t11 = zs_h4(__ldg((const uint2 *)(rb + (int64_t)xb * 8)));
                r[p] = zs_lerp4(zs_lerp4(t00, t01, fx), zs_lerp4(t10, t11, fx), fy);
            } else if (a.has_below) {
                r[p] = zs_load_px(s0, x, y);
            } else {
                r[p] = make_float4(a.cons[0], a.cons[1], a.cons[2], a.cons[3]);
            }
        }
#pragma unroll
        for (int p = 0; p < ZS_AFF_PX; ++p) {
            const int y = y0 + 4 * p;
            if (y >= a.height) break;
            uint8_t *dp = a.dst + (int64_t)y * a.dst_stride + (int64_t)x * a.dst_fmt.bpp;
            if (plain) {
                zs_store_f16x4(dp, r[p]);
                continue;
            }
            float4 v = r[p], r2 = make_float4(0.f, 0.f, 0.f, 0.f);
            zs_run_program(a.prog, a.fmts, v, r2);
            zs_store_raw(dp, a.dst_fmt.bpp, zs_encode_raw(a.dst_fmt, v));
        }
    }
}

namespace zs {

cudaError_t launch_raster(const ZsRasterArgs &args, int sm_count, cudaStream_t stream) {
    const int64_t n = (int64_t)args.width * args.height;
    if (n <= 0) return cudaSuccess;
    if (args.producer == ZS_PR_RESAMPLE_2D) return launch_resample2d(args, sm_count, stream);
    if (args.producer == ZS_PR_AFFINE && args.bilinear && !args.raw_copy && !args.virt1 &&
        args.src[1].fmt.fast == ZS_FAST_F16X4 &&
        args.aff[6] == 0.f && args.aff[7] == 0.f && args.aff[8] == 1.f &&
        (int64_t)((args.width + 31) / 32) * ((args.height + 8 * ZS_AFF_PX - 1) / (8 * ZS_AFF_PX)) * 256 +
                (int64_t)(sm_count > 0 ? sm_count : 148) * 8 * 256 < INT32_MAX) {
        int64_t blocks = (int64_t)((args.width + 31) / 32) * ((args.height + 8 * ZS_AFF_PX - 1) / (8 * ZS_AFF_PX));
        const int64_t cap = (int64_t)(sm_count > 0 ? sm_count : 148) * 8;
        if (blocks > cap) blocks = cap;
        zs_affine_f16_kernel<<<(unsigned)blocks, 256, 0, stream>>>(args);
        g_kernel_launches.fetch_add(1);
        return cudaGetLastError();
    }
    int64_t blocks = (n + 255) / 256;
    const int64_t cap = (int64_t)(sm_count > 0 ? sm_count : 148) * 8;
    if (blocks > cap) blocks = cap;
    // Programmatic stream serialization: this launch's CTAs may be scheduled while the previous
    // kernel drains (they wait for it before any memory access), hiding the launch gap between
    // the short kernels of latency-bound programs.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, zs_raster_kernel, args);
    if (e != cudaSuccess) return e;
    g_kernel_launches.fetch_add(1);
    return cudaGetLastError();
}

}  // namespace zs

ZS_TU_HOOKS(raster)
