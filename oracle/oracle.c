/*
 * oracle.c -- CPU restatement of zosimos' raster-pipeline arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Builds liboracle.so, which holds
 * the FP64 oracle (zo_*) and the plain per-op FP32 CPU pipeline (zo32_*).
 *
 * Sources restated (paths inside the zosimos project):
 *   lib/std/src/stage.frag      transfer functions, texel mux/demux, parts order
 *   lib/std/src/linear.frag     3x3 colour matrix
 *   lib/std/src/oklab.frag      Oklab encode/decode (Ottosson's published M1/M2)
 *   lib/std/src/srlab2.frag     SrLab2 encode/decode (CIECAM02 CAT02 / HPE)
 *   lib/std/src/inject.frag     channel inject
 *   lib/std/src/bilinear.frag   bilinear construct
 *   lib/std/src/copy.frag + box.vert, lib/zosimos/src/program.rs:1897-1935
 *                               quad mapping used by crop / inscribe / affine
 *   lib/std/src/palette.frag + lib/zosimos/src/command.rs:1675-1702   resize
 *   lib/zosimos/src/command.rs:1009-1085, 2527-2548, 3220-3340         matrix folding
 * Third-party arithmetic restated from published definitions (image-canvas 0.5.1
 * primaries, palette 0.7.6 white points and generate_transform_matrix): CIE xy
 * chromaticities of the standards, Lindbloom's white-point XYZ and cone matrices.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants ---------------------------------------------------------- */

/* Oklab (oklab.frag:14-24; the GLSL column-major literals equal these rows). */
static const double zo_oklab_m1[9] = {0.8189330101, 0.3618667424, -0.1288597137,
                                      0.0329845436, 0.9293118715, 0.0361456387,
                                      0.0482003018, 0.2643662691, 0.6338517070};
static const double zo_oklab_m2[9] = {0.2104542553, 0.7936177850, -0.0040720468,
                                      1.9779984951, -2.4285922050, 0.4505937099,
                                      0.0259040371, 0.7827717662, -0.8086757660};
/* SrLab2 (srlab2.frag:14-24), as rows. */
static const double zo_srlab2_cat02[9] = {0.7328, 0.4296, -0.1624, -0.7036, 1.6975, 0.0061,
                                          0.0030, 0.0136, 0.9834};
static const double zo_srlab2_hpe[9] = {0.38971, 0.68898, -0.07868, -0.22981, 1.18340, 0.04641,
                                        0.0, 0.0, 1.0};

/* ---- small FP64 linear algebra ------------------------------------------ */

void zo_mat3_mul(const double a[9], const double b[9], double out[9]) {
    double r[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
    memcpy(out, r, sizeof(r));
}

int zo_mat3_inv(const double m[9], double out[9]) {
    double c00 = m[4] * m[8] - m[5] * m[7];
    double c01 = m[5] * m[6] - m[3] * m[8];
    double c02 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    if (det == 0.0) return -1;
    double r[9] = {c00, m[2] * m[7] - m[1] * m[8], m[1] * m[5] - m[2] * m[4],
                   c01, m[0] * m[8] - m[2] * m[6], m[2] * m[3] - m[0] * m[5],
                   c02, m[1] * m[6] - m[0] * m[7], m[0] * m[4] - m[1] * m[3]};
    for (int i = 0; i < 9; i++) out[i] = r[i] / det;
    return 0;
}

/* White points as XYZ (Y = 1), order A,B,C,D50,D55,D65,D75,E,F2,F7,F11. */
static const double zo_wp[11][3] = {
    {1.09850, 1.0, 0.35585}, {0.99072, 1.0, 0.85223}, {0.98074, 1.0, 1.18232},
    {0.96422, 1.0, 0.82521}, {0.95682, 1.0, 0.92149}, {0.95047, 1.0, 1.08883},
    {0.94972, 1.0, 1.22638}, {1.00000, 1.0, 1.00000}, {0.99186, 1.0, 0.67393},
    {0.95041, 1.0, 1.08747}, {1.00962, 1.0, 0.64350}};

void zo_whitepoint_xyz(int32_t wp, double out[3]) {
    if (wp < 0 || wp > 10) wp = 5;
    memcpy(out, zo_wp[wp], sizeof(double) * 3);
}

/* CIE xy of R, G, B for each primaries code (0 BT601-525, 1 BT601-625, 2 BT709,
 * 3 SMPTE240, 4 BT2020, 5 BT2100, 6 P3, 7 AdobeRGB, 8 XYZ). */
static const double zo_prim[8][6] = {
    {0.630, 0.340, 0.310, 0.595, 0.155, 0.070}, {0.640, 0.330, 0.290, 0.600, 0.150, 0.060},
    {0.640, 0.330, 0.300, 0.600, 0.150, 0.060}, {0.630, 0.340, 0.310, 0.595, 0.155, 0.070},
    {0.708, 0.292, 0.170, 0.797, 0.131, 0.046}, {0.708, 0.292, 0.170, 0.797, 0.131, 0.046},
    {0.680, 0.320, 0.265, 0.690, 0.150, 0.060}, {0.640, 0.330, 0.210, 0.710, 0.150, 0.060}};

void zo_rgb_to_xyz(int32_t primaries, int32_t wp, double out[9]) {
    if (primaries < 0 || primaries > 7) {
        double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        memcpy(out, id, sizeof(id));
        return;
    }
    const double *p = zo_prim[primaries];
    double P[9], Pi[9], W[3], S[3];
    for (int c = 0; c < 3; c++) {
        double x = p[2 * c], y = p[2 * c + 1];
        P[c] = x / y;
        P[3 + c] = 1.0;
        P[6 + c] = (1.0 - x - y) / y;
    }
    zo_whitepoint_xyz(wp, W);
    zo_mat3_inv(P, Pi);
    for (int i = 0; i < 3; i++) S[i] = Pi[3 * i] * W[0] + Pi[3 * i + 1] * W[1] + Pi[3 * i + 2] * W[2];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) out[3 * r + c] = P[3 * r + c] * S[c];
}

/* method: 0 XYZ scaling, 1 von Kries, 2 Bradford (linear); 3 (non-linear Bradford)
 * is NotYetImplemented upstream (command.rs:3328-3332) and returns -1. */
int zo_adaptation(int32_t method, int32_t src_wp, int32_t dst_wp, double out[9]) {
    static const double bradford[9] = {0.8951, 0.2664, -0.1614, -0.7502, 1.7135,
                                       0.0367, 0.0389, -0.0685, 1.0296};
    static const double vonkries[9] = {0.40024, 0.7076, -0.08081, -0.2263, 1.16532,
                                       0.0457, 0.0, 0.0, 0.91822};
    static const double ident[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    const double *m;
    switch (method) {
    case 0: m = ident; break;
    case 1: m = vonkries; break;
    case 2: m = bradford; break;
    default: return -1;
    }
    double ws[3], wd[3], rs[3], rd[3], mi[9], d[9] = {0};
    zo_whitepoint_xyz(src_wp, ws);
    zo_whitepoint_xyz(dst_wp, wd);
    for (int i = 0; i < 3; i++) {
        rs[i] = m[3 * i] * ws[0] + m[3 * i + 1] * ws[1] + m[3 * i + 2] * ws[2];
        rd[i] = m[3 * i] * wd[0] + m[3 * i + 1] * wd[1] + m[3 * i + 2] * wd[2];
        d[4 * i] = rd[i] / rs[i];
    }
    zo_mat3_inv(m, mi);
    double t[9];
    zo_mat3_mul(d, m, t);
    zo_mat3_mul(mi, t, out);
    return 0;
}

/* ---- half precision ----------------------------------------------------- */

uint16_t zo_f32_to_f16(float v) {
    uint32_t x;
    memcpy(&x, &v, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);   /* rounds to >= 65520: inf */
    if (ax < 0x38800000u) {                                      /* half subnormal range */
        if (ax < 0x33000000u) return (uint16_t)sign;             /* below 2^-25: zero */
        uint32_t e = ax >> 23, m = (ax & 0x7fffffu) | 0x800000u;
        uint32_t shift = 126 - e;                                /* value = m * 2^(e-150) */
        uint32_t q = m >> shift, rem = m & ((1u << shift) - 1), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (q & 1))) q++;
        return (uint16_t)(sign | q);
    }
    uint32_t e = (ax >> 23) - 112, m = ax & 0x7fffffu;
    uint32_t q = (e << 10) | (m >> 13), rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1))) q++;
    return (uint16_t)(sign | q);
}

float zo_f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 31, m = h & 1023, x;
    if (e == 0) {
        float f = ldexpf((float)m, -24);
        return sign ? -f : f;
    }
    if (e == 31) x = sign | 0x7f800000u | (m << 13);
    else x = sign | ((e + 112) << 23) | (m << 13);
    float f;
    memcpy(&f, &x, 4);
    return f;
}

int zo_texel_bytes(int32_t bits) {
    static const int b[20] = {1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 4, 4, 6, 8, 4, 4, 4, 4, 8, 16};
    return (bits >= 0 && bits < 20) ? b[bits] : 0;
}

int zo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void zo_set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* Inverse affine map of a pixel centre, f32 with a fixed fmaf order so that the
 * nearest-texel index is reproducible bit for bit. */
static void zo_affine_map(const float inv[9], int32_t x, int32_t y, float *qx, float *qy) {
    float cx = (float)x + 0.5f, cy = (float)y + 0.5f;
    float X = fmaf(inv[0], cx, fmaf(inv[1], cy, inv[2]));
    float Y = fmaf(inv[3], cx, fmaf(inv[4], cy, inv[5]));
    float Z = fmaf(inv[6], cx, fmaf(inv[7], cy, inv[8]));
    if (Z != 1.0f) { X = X / Z; Y = Y / Z; }
    *qx = X;
    *qy = Y;
}

/* ---- FP64 oracle and FP32 per-op pipeline ------------------------------- */

#define REAL double
#define ZO(name) zo_##name
#define RPOW pow
#define RFLOOR floor
#define RSQRT sqrt
#define RATAN2 atan2
#define RCOS cos
#define RSIN sin
#define RRINT nearbyint
#define RCBRT cbrt
#define RFABS fabs
#include "oracle_ops.inc"
#undef REAL
#undef ZO
#undef RPOW
#undef RFLOOR
#undef RSQRT
#undef RATAN2
#undef RCOS
#undef RSIN
#undef RRINT
#undef RCBRT
#undef RFABS
#undef ZO_PQ_M1
#undef ZO_PQ_M2
#undef ZO_PQ_C1
#undef ZO_PQ_C2
#undef ZO_PQ_C3

#define REAL float
#define ZO(name) zo32_##name
#define RPOW powf
#define RFLOOR floorf
#define RSQRT sqrtf
#define RATAN2 atan2f
#define RCOS cosf
#define RSIN sinf
#define RRINT nearbyintf
#define RCBRT cbrtf
#define RFABS fabsf
#include "oracle_ops.inc"

/* ---- integer (byte-exact) gathers ---------------------------------------- */

/* Quad copy used by crop / inscribe (copy.frag through box.vert): the selection
 * [sel0,sel1) of `src` is stretched onto the target [t0,t1) of `dst` with nearest
 * sampling at pixel centres; exact rational form of floor(sel0 + (p-t0+0.5)*S/T). */
void zo_gather_quad2(const uint8_t *src, int64_t sstride, int32_t sw, int32_t sh,
                     const int32_t sel[4], uint8_t *dst, int64_t dstride, int32_t dw, int32_t dh,
                     int32_t bpp, const int32_t tgt[4]) {
    int64_t S = sel[2] - sel[0], T = tgt[2] - tgt[0];
    int64_t Sy = sel[3] - sel[1], Ty = tgt[3] - tgt[1];
    if (S <= 0 || T <= 0 || Sy <= 0 || Ty <= 0) return;
    int32_t y0 = tgt[1] < 0 ? 0 : tgt[1], y1 = tgt[3] > dh ? dh : tgt[3];
    int32_t x0 = tgt[0] < 0 ? 0 : tgt[0], x1 = tgt[2] > dw ? dw : tgt[2];
#pragma omp parallel for schedule(static)
    for (int32_t y = y0; y < y1; y++) {
        int64_t sy = sel[1] + ((2 * (int64_t)(y - tgt[1]) + 1) * Sy) / (2 * Ty);
        if (sy > sh - 1) sy = sh - 1;
        if (sy < 0) sy = 0;
        for (int32_t x = x0; x < x1; x++) {
            int64_t sx = sel[0] + ((2 * (int64_t)(x - tgt[0]) + 1) * S) / (2 * T);
            if (sx > sw - 1) sx = sw - 1;
            if (sx < 0) sx = 0;
            memcpy(dst + y * dstride + (int64_t)x * bpp, src + sy * sstride + sx * bpp, (size_t)bpp);
        }
    }
}

void zo_gather_quad(const uint8_t *src, int64_t src_stride, int32_t sw, int32_t sh, uint8_t *dst,
                    int64_t dst_stride, int32_t dw, int32_t dh, int32_t bpp, int32_t tx0,
                    int32_t ty0, int32_t tx1, int32_t ty1) {
    int32_t sel[4] = {0, 0, sw, sh}, tgt[4] = {tx0, ty0, tx1, ty1};
    zo_gather_quad2(src, src_stride, sw, sh, sel, dst, dst_stride, dw, dh, bpp, tgt);
}

void zo_affine_nearest_bytes(const uint8_t *above, int64_t a_stride, int32_t aw, int32_t ah,
                             uint8_t *dst, int64_t d_stride, int32_t dw, int32_t dh, int32_t bpp,
                             const float inv[9]) {
#pragma omp parallel for schedule(static)
    for (int32_t y = 0; y < dh; y++) {
        for (int32_t x = 0; x < dw; x++) {
            float qx, qy;
            zo_affine_map(inv, x, y, &qx, &qy);
            if (!(qx >= 0.0f && qx < (float)aw && qy >= 0.0f && qy < (float)ah)) continue;
            int32_t ix = (int32_t)floorf(qx), iy = (int32_t)floorf(qy);
            if (ix > aw - 1) ix = aw - 1;
            if (iy > ah - 1) iy = ah - 1;
            memcpy(dst + (int64_t)y * d_stride + (int64_t)x * bpp, above + (int64_t)iy * a_stride + (int64_t)ix * bpp,
                   (size_t)bpp);
        }
    }
}

/* Source index of `resize` (command.rs:1675-1702): the bilinear grid holds u at pixel
 * centres, is stored as 8-bit staged texels (truncating), decoded as q/255 and then
 * used by palette.frag with the 0.5/size bias and nearest sampling.  All f32. */
void zo_resize_ref_index(int32_t src_len, int32_t dst_len, int32_t *index) {
    volatile float fdst = (float)dst_len, fsrc = (float)src_len;
    for (int32_t x = 0; x < dst_len; x++) {
        volatile float u = ((float)x + 0.5f) / fdst;
        volatile float scaled = u * 255.0f;
        uint32_t q = (uint32_t)scaled;
        volatile float basis = (float)q / 255.0f;
        volatile float bias = 0.5f / fdst;
        volatile float t = basis + bias;
        volatile float p = t * fsrc;
        int32_t ix = (int32_t)floorf(p);
        if (ix < 0) ix = 0;
        if (ix > src_len - 1) ix = src_len - 1;
        index[x] = ix;
    }
}

/* General palette.frag index: basis values (f32, already decoded), bias 0.5/size(rhs). */
void zo_palette_index(int32_t src_w, int32_t src_h, const float *basis_u, const float *basis_v,
                      int32_t dw, int32_t dh, int32_t *ix, int32_t *iy) {
    volatile float bu = 0.5f / (float)dw, bv = 0.5f / (float)dh;
    for (int64_t i = 0; i < (int64_t)dw * dh; i++) {
        volatile float tu = basis_u[i] + bu, tv = basis_v[i] + bv;
        volatile float pu = tu * (float)src_w, pv = tv * (float)src_h;
        int32_t a = (int32_t)floorf(pu), b = (int32_t)floorf(pv);
        ix[i] = a < 0 ? 0 : (a > src_w - 1 ? src_w - 1 : a);
        iy[i] = b < 0 ? 0 : (b > src_h - 1 ? src_h - 1 : b);
    }
}

/* ---- resampling weights (FP64, normalised) -------------------------------- */
/* filter: 0 box (area coverage), 1 Lanczos-3, 2 triangle.  Output pixel i has its
 * centre at (i + 0.5) * src/dst in source pixels; the kernel is widened by the
 * downscale factor; taps outside the image are dropped and the rest renormalised. */

static double zo_kernel_radius(int32_t filter) {
    return filter == 1 ? 3.0 : (filter == 2 ? 1.0 : 0.5);
}

int32_t zo_resample_max_taps(int32_t src_len, int32_t dst_len, int32_t filter) {
    double s = (double)src_len / (double)dst_len, f = s > 1.0 ? s : 1.0;
    return (int32_t)ceil(2.0 * zo_kernel_radius(filter) * f) + 2;
}

static double zo_sinc(double x) {
    if (fabs(x) < 1e-12) return 1.0;
    double px = 3.14159265358979323846 * x;
    return sin(px) / px;
}

void zo_resample_weights(int32_t src_len, int32_t dst_len, int32_t filter, int32_t *first,
                         int32_t *count, double *weights, int32_t max_taps) {
    double s = (double)src_len / (double)dst_len, f = s > 1.0 ? s : 1.0;
    double r = zo_kernel_radius(filter) * f;
    for (int32_t i = 0; i < dst_len; i++) {
        double c = ((double)i + 0.5) * s;
        int32_t lo = (int32_t)floor(c - r), hi = (int32_t)ceil(c + r);
        if (lo < 0) lo = 0;
        if (hi > src_len) hi = src_len;
        double *w = weights + (size_t)i * max_taps, sum = 0.0;
        int32_t n = 0, start = -1;
        for (int32_t j = lo; j < hi && n < max_taps; j++) {
            double v;
            if (filter == 0) {
                double a = c - 0.5 * f, b = c + 0.5 * f;
                double ov = fmin(b, (double)j + 1.0) - fmax(a, (double)j);
                v = ov > 0 ? ov : 0.0;
            } else {
                double t = ((double)j + 0.5 - c) / f;
                if (filter == 1) v = fabs(t) < 3.0 ? zo_sinc(t) * zo_sinc(t / 3.0) : 0.0;
                else v = fabs(t) < 1.0 ? 1.0 - fabs(t) : 0.0;
            }
            if (start < 0) {
                if (v == 0.0) continue;
                start = j;
            }
            w[n++] = v;
            sum += v;
        }
        while (n > 0 && w[n - 1] == 0.0) n--;
        if (start < 0 || sum == 0.0) {
            int32_t j = (int32_t)floor(c);
            if (j > src_len - 1) j = src_len - 1;
            start = j;
            n = 1;
            w[0] = 1.0;
            sum = 1.0;
        }
        for (int32_t t = 0; t < n; t++) w[t] /= sum;
        for (int32_t t = n; t < max_taps; t++) w[t] = 0.0;
        first[i] = start;
        count[i] = n;
    }
}
