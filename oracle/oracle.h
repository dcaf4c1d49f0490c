/*
 * oracle.h -- CPU restatement of zosimos' raster-pipeline arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * GB300 executor: tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may call it; the product library never links or calls it.
 *
 * Every function is compiled twice from oracle_ops.inc:
 *   zo_*    with double arithmetic (the FP64 oracle), and
 *   zo32_*  with float arithmetic (the plain per-op CPU pipeline that is
 *           timed as the CPU baseline; OpenMP over rows).
 *
 * Images are "linear buffers": row-major H x W x 4 arrays of REAL holding the
 * value a zosimos fragment shader sees after staging decode (linear colour,
 * Lab for Oklab/SrLab2, raw scalars for Scalars colours).
 *
 * Parity: pinned perceptually against the reference's blockhash256 goldens
 * (lib/zosimos/tests/reference/NAME.crc.png files) and exactly against the byte pins
 * of lib/zosimos/tests/blend.rs:371-372 (transmute) and tests/buffer.rs.
 * Exact primaries / white-point constants come from published standards
 * (image-canvas 0.5.1 and palette 0.7.6 are not available offline).
 */
#ifndef ZOSIMOS_ORACLE_H
#define ZOSIMOS_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Texel format as the oracle sees it (codes follow lib/std/src/stage.frag:102-176). */
typedef struct zo_format {
    int32_t bits;      /* SAMPLE_BITS_* */
    int32_t parts;     /* SAMPLE_PARTS_* */
    int32_t transfer;  /* TRANSFER_* (0x100 = LabLch) */
    int32_t native;    /* 1: hardware unorm format, round-to-nearest; 0: staged, truncating */
} zo_format;

int zo_texel_bytes(int32_t bits);

#define ZO_DECL(P, R)                                                                     \
    void P##decode(const zo_format *f, const uint8_t *src, int64_t row_stride,            \
                   int32_t w, int32_t h, R *out);                                          \
    void P##encode(const zo_format *f, const R *in, int32_t w, int32_t h, uint8_t *dst,    \
                   int64_t row_stride);                                                    \
    void P##mat3(R *img, int64_t n, const double m[9]);                                    \
    void P##clamp01_rgb(R *img, int64_t n);                                                \
    void P##oklab_encode(R *img, int64_t n, const double rgb_to_xyz[9]);                   \
    void P##oklab_decode(R *img, int64_t n, const double xyz_to_rgb[9]);                   \
    void P##srlab2_encode(R *img, int64_t n, const double rgb_to_xyz[9]);                  \
    void P##srlab2_decode(R *img, int64_t n, const double xyz_to_rgb[9],                   \
                          const double wp_xyz[3]);                                         \
    void P##inject(R *bg, const R *fg, int64_t n, const double select[4],                  \
                   const double weights[4]);                                               \
    void P##blend(R *below, const R *above, int32_t bw, int32_t bh, int32_t aw,            \
                  int32_t ah, int32_t ox, int32_t oy, int32_t mode, int32_t straight);     \
    void P##bilinear_construct(R *out, int32_t w, int32_t h, const double p[24]);          \
    void P##affine(R *below, int32_t bw, int32_t bh, const R *above, int32_t aw,           \
                   int32_t ah, const float inv[9], int32_t bilinear);                      \
    void P##resample(const R *src, int32_t sw, int32_t sh, R *dst, int32_t dw,             \
                     int32_t dh, int32_t filter);                                          \
    void P##resample_rows(const R *src, int32_t sw, int32_t sh, R *band, int32_t dw,       \
                          int32_t dh, int32_t y0, int32_t y1, int32_t filter);             \
    void P##affine_rows(R *band, int32_t bw, int32_t y0, int32_t y1, const R *above,       \
                        int32_t aw, int32_t ah, const float inv[9], int32_t bilinear);     \
    void P##transfer(R *img, int64_t n, int32_t transfer, int32_t forward);                 \
    void P##box3(const R *src, int32_t w, int32_t h, R *dst, const double m[9]);

ZO_DECL(zo_, double)
ZO_DECL(zo32_, float)

/* ---- matrices (FP64) ---- */
void zo_rgb_to_xyz(int32_t primaries, int32_t whitepoint, double out[9]);
void zo_whitepoint_xyz(int32_t whitepoint, double out[3]);
int  zo_adaptation(int32_t method, int32_t src_wp, int32_t dst_wp, double out[9]);
void zo_mat3_mul(const double a[9], const double b[9], double out[9]);
int  zo_mat3_inv(const double a[9], double out[9]);

/* ---- byte-exact gathers (integer semantics) ---- */
void zo_gather_quad(const uint8_t *src, int64_t src_stride, int32_t sw, int32_t sh,
                    uint8_t *dst, int64_t dst_stride, int32_t dw, int32_t dh, int32_t bpp,
                    int32_t tx0, int32_t ty0, int32_t tx1, int32_t ty1);
void zo_gather_quad2(const uint8_t *src, int64_t sstride, int32_t sw, int32_t sh,
                     const int32_t sel[4], uint8_t *dst, int64_t dstride, int32_t dw, int32_t dh,
                     int32_t bpp, const int32_t tgt[4]);
void zo_affine_nearest_bytes(const uint8_t *above, int64_t a_stride, int32_t aw, int32_t ah,
                             uint8_t *dst, int64_t d_stride, int32_t dw, int32_t dh,
                             int32_t bpp, const float inv[9]);
void zo_resize_ref_index(int32_t src_len, int32_t dst_len, int32_t *index);
void zo_palette_index(int32_t src_w, int32_t src_h, const float *basis_u, const float *basis_v,
                      int32_t dw, int32_t dh, int32_t *ix, int32_t *iy);
void zo_resample_weights(int32_t src_len, int32_t dst_len, int32_t filter, int32_t *first,
                         int32_t *count, double *weights, int32_t max_taps);
int32_t zo_resample_max_taps(int32_t src_len, int32_t dst_len, int32_t filter);

/* ---- half precision (round to nearest even) ---- */
uint16_t zo_f32_to_f16(float v);
float    zo_f16_to_f32(uint16_t h);

/* ---- OpenMP thread control for the timed CPU baseline ---- */
int  zo_max_threads(void);
void zo_set_threads(int32_t n);

#ifdef __cplusplus
}
#endif
#endif
