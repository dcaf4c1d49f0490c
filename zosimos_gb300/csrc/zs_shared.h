// zs_shared.h -- plain-old-data shared by the C++ host planner and the CUDA kernels.
//
// A compiled zosimos Program is lowered into a list of raster launches.  Each launch
// has a *producer* (how the first value of a pixel is obtained: pixel-aligned loads,
// a construct, a quad/affine/palette gather, a blend or a separable resample pass),
// a *pixel program* (per-pixel ops fused behind the producer: colour matrices, cube
// roots, clamps, declared-texel quantisation, inject, ...) and a *store* in the
// register's storage format.  Everything here is POD so that it can travel as a
// __grid_constant__ kernel parameter.
#pragma once
#include <stdint.h>

#define ZS_MAX_INSTR 48
#define ZS_MAX_PARAMS 320
#define ZS_MAX_FMTS 8
#define ZS_MAX_SRCS 3
// Device ordinals with per-device launcher state (kernel attributes, tables).
#define ZS_MAX_DEVICES 64

// Storage format of one register (what lib/zosimos/src/program.rs:781-946 derives from a
// Descriptor).  `fast` selects a specialised decode/encode path.
enum ZsFast : uint8_t {
    ZS_FAST_GENERIC = 0,
    ZS_FAST_RGBA8_SRGB = 1,    // native Rgba8UnormSrgb: LUT decode, exact round-to-nearest encode
    ZS_FAST_RGBA8_UNORM = 2,   // native Rgba8Unorm
    ZS_FAST_BGRA8_SRGB = 3,
    ZS_FAST_BGRA8_UNORM = 4,
    ZS_FAST_F16X4 = 5,         // Float16x4 RgbA, linear transfer
    ZS_FAST_F32X4 = 6          // Float32x4 RgbA, linear transfer
};

struct ZsFormat {
    uint8_t bits;      // SampleBits code (stage.frag:152-171)
    uint8_t parts;     // SampleParts code (stage.frag:122-142)
    uint8_t native;    // 1: hardware unorm (round to nearest), 0: staged (truncating)
    uint8_t bpp;       // bytes per texel
    uint16_t transfer; // transfer code, 0x100 = LabLch
    uint8_t fast;      // ZsFast
    uint8_t pad;
};

enum ZsPOp : uint8_t {
    ZS_P_NOP = 0,
    ZS_P_MAT3,         // r.rgb = M * r.rgb                   (linear.frag)
    ZS_P_CBRT,         // signed cube root of r.rgb           (oklab.frag:42)
    ZS_P_CUBE,         // r.rgb^3                             (oklab.frag:58)
    ZS_P_CLAMP01,      // clamp r.rgb to [0,1]                (oklab.frag:63, srlab2.frag:84)
    ZS_P_SRL_NL,       // SrLab2 piecewise cube root          (srlab2.frag:87-95)
    ZS_P_SRL_NLINV,    //                                     (srlab2.frag:105-112)
    ZS_P_SRL_ENC_DIFF, // (y, (x-y)*5/1.16, (z-y)*2/1.16)     (srlab2.frag:51-57)
    ZS_P_SRL_DEC_DIFF, //                                     (srlab2.frag:70-74)
    ZS_P_QUANT,        // encode into fmt[a] and decode back (declared intermediate texel)
    ZS_P_TRANSMUTE,    // encode into fmt[a], reinterpret the bytes as fmt[b] and decode
    ZS_P_INJECT,       // r = mix(r, dot(r2, w), select)      (inject.frag:20-25)
    ZS_P_BLEND,        // r = blend(r (below), r2 (above))    (mode in a, straight alpha in b)
    ZS_P_MOV2,         // r2 = r
    ZS_P_SWAP,         // swap r and r2
    ZS_P_PREMUL,       // r.rgb *= r.a
    ZS_P_UNPREMUL      // r.rgb /= r.a (0 where a == 0)
};

struct ZsPInstr {
    uint8_t op;
    uint8_t a, b, c;   // small operands (format ids, modes)
    uint16_t p;        // offset into params
    uint16_t pad;
};

struct ZsPixelProgram {
    int32_t n;
    int32_t pad;
    ZsPInstr ins[ZS_MAX_INSTR];
    float prm[ZS_MAX_PARAMS];
};

enum ZsProducer : uint8_t {
    ZS_PR_LOAD = 0,     // r = src0(x,y), r2 = src1(x,y) (pixel aligned)
    ZS_PR_BILINEAR,     // bilinear.frag construct
    ZS_PR_SOLID,        // solid colour
    ZS_PR_QUAD,         // below(x,y); inside target: src1(nearest map of selection)
    ZS_PR_AFFINE,       // below(x,y); inside transformed quad: sample src1
    ZS_PR_PALETTE,      // src0(coords from src1(x,y))       (palette.frag)
    ZS_PR_INDEX,        // src0(ix[x], iy[y])                (resize via a nearest index table)
    ZS_PR_BLEND,        // below(x,y) blended with src1(x-ox, y-oy)
    ZS_PR_RESAMPLE_H,   // horizontal filter pass over src0 rows
    ZS_PR_RESAMPLE_V,   // vertical filter pass over src0 columns
    ZS_PR_LAYERS,       // planner only: a layer stack, launched by k_layers.cu
    ZS_PR_RESAMPLE_2D,  // both separable passes in one tiled launch (k_resample.cu)
    ZS_PR_BOX3,         // 3x3 stencil of src0, weights in cons[0..8]   (box3.frag)
    ZS_PR_NORMAL2D,     // normal density, params in cons[0..6]          (distribution_normal2d.frag)
    ZS_PR_FRACTAL       // fractal value noise, params in cons[0..6]     (fractal_noise.frag)
};

struct ZsSource {
    const uint8_t *ptr;
    int64_t stride;   // bytes per row
    int32_t width, height;
    ZsFormat fmt;
};

struct ZsRasterArgs {
    // producer
    uint8_t producer;
    uint8_t nsrc;
    uint8_t raw_copy;     // gather producers: copy texel bytes verbatim (same format, no program)
    uint8_t has_below;    // QUAD/AFFINE/BLEND: src0 is the image painted over
    uint8_t bilinear;     // AFFINE: bilinear sampling
    uint8_t blend_mode;
    uint8_t straight;
    uint8_t virt1;        // AFFINE: src1 is evaluated per tap (vsrc / vprog below), not stored
    ZsSource src[ZS_MAX_SRCS];
    int32_t rect[4];      // QUAD target rect / BLEND offset rect
    int32_t sel[4];       // QUAD selection rect in src1
    float aff[9];         // AFFINE inverse matrix (f32, applied with a fixed fmaf order)
    float cons[24];       // BILINEAR params / SOLID colour / PALETTE channel weights (8) / BOX3 weights (9)
    const int32_t *index_x;   // INDEX producer / RESAMPLE first-tap table
    const int32_t *index_y;   // INDEX producer / RESAMPLE tap-count table
    const float *weights;     // RESAMPLE weights [dst][taps]
    int32_t taps;
    int32_t pad1;
    // RESAMPLE_2D: the vertical tables (the horizontal ones are index_x/index_y/weights)
    const int32_t *vfirst;
    const int32_t *vcount;
    const float *vweights;
    int32_t vtaps;
    int32_t max_span;         // widest source column span of one output tile
    int32_t tile_rows;        // output rows per tile: 8, 16 or 32
    int32_t stages;           // staged batches of source rows (set by the launcher)
    // RESAMPLE_2D on the tensor cores (k_resample_tc.cu; tc_tw 0: not planned)
    const uint8_t *vimg;          // vertical band matrices: [chunk][128 rows][64 f16], 128-byte swizzle
    const int32_t *vimg_index;    // per band of 128 output rows: first chunk, chunk count
    int32_t tc_tw;                // output columns per tile
    int32_t tc_atoms;             // 64-element column blocks of source staged per tile (N = 64 * atoms)
    const float *tc_weights;      // horizontal weights [padded width][tc_taps], rows zero-padded
    int32_t tc_taps;              // taps rounded up to a multiple of 4 (16-byte weight rows)
    int32_t tc_pad;
    // destination
    uint8_t *dst;
    int64_t dst_stride;
    int32_t width, height;
    ZsFormat dst_fmt;
    ZsFormat fmts[ZS_MAX_FMTS];   // formats referenced by QUANT / TRANSMUTE (both programs)
    ZsPixelProgram prog;
    // virt1: the pixel-aligned producer of the gathered image -- LOAD of vsrc (r = vsrc[0],
    // r2 = vsrc[1]) or BLEND of vsrc[1] at offset vrect over vsrc[0] -- and its program, run
    // at every tap instead of materialising the image.
    ZsSource vsrc[2];
    int32_t vrect[2];
    uint8_t vproducer, vmode, vstraight, vnsrc;
    int32_t pad3;
    ZsPixelProgram vprog;
};

// RESAMPLE_2D output tile (columns x rows; the rows per launch are 8, 16 or ZS_RS_TH) and
// the source rows staged per batch.  One CTA's shared memory holds `stages` batches of
// raw source rows, two batches of filtered rows and the tile's weight tables.
#define ZS_RS_TW 64
#define ZS_RS_TH 32
#define ZS_RS_RB 8
// Pitch of one staged source row: room for max_span texels plus the 16-byte alignment
// remainder, rounded so that consecutive rows start 16 bytes apart modulo 128.
#define ZS_RS_ROWBYTES(span, bpp) ((((span) * (bpp) + 16 + 127) & ~127) + 16)
#define ZS_RS_MAX_SMEM (200 * 1024)
#define ZS_RS_STAGE_BUDGET (96 * 1024)   // staged source rows of one CTA (2 CTAs per SM)

// Tensor-core resample: bands of 128 output rows (the MMA's M), chunks of 64 source rows
// (the K of one 128-byte swizzle atom), at most 8 atoms of 64 source elements (two MMAs of
// N <= 256 into 512 TMEM columns).
#define ZS_TC_M 128
#define ZS_TC_K 64
#define ZS_TC_MAX_ATOMS 8
#define ZS_TC_CHUNK_BYTES (ZS_TC_M * ZS_TC_K * 2)

// Bits of the device status word.
#define ZS_DEVSTAT_WAIT_TIMEOUT 1u   // an mbarrier wait on a bulk copy exceeded its limit
#define ZS_DEVSTAT_LAYOUT 2u         // a kernel's shared-memory layout did not fit its window; it did nothing

// A stack of layers composited in one pass: for every output pixel, start from the
// base (a constant or a buffer) and for each layer sample it through its inverse affine
// (nearest or bilinear, the layer's canvas colour outside it) and blend the sample onto
// the accumulator, which stays in FP32 registers.
#define ZS_MAX_LAYERS 64

struct ZsLayer {
    const uint8_t *ptr;
    int64_t stride;
    int32_t width, height;
    ZsFormat fmt;
    float inv[9];          // output pixel centre -> layer pixel coordinates (fixed fmaf order)
    float canvas[4];       // value where the layer does not cover the pixel
    uint8_t bilinear;
    uint8_t mode;          // blend mode
    uint8_t straight;      // operands carry straight alpha
    uint8_t quant_sample;  // index+1 into fmts: quantise the sampled layer value (declared texel)
    uint8_t quant_acc;     // index+1 into fmts: quantise the accumulator after the blend
    uint8_t pad[3];
};

struct ZsLayersArgs {
    int32_t nlayers;
    int32_t width, height;
    int32_t has_base;      // 1: base buffer in `base`, 0: constant base_color
    int32_t f16_bilinear;  // 1: every layer RGBA16F, bilinear, affine, premultiplied, no lossy
                           // quantisation (the specialised kernel applies)
    int32_t pad;
    ZsSource base;
    float base_color[4];
    ZsLayer layers[ZS_MAX_LAYERS];
    uint8_t *dst;
    int64_t dst_stride;
    ZsFormat dst_fmt;
    ZsFormat fmts[ZS_MAX_FMTS];
    ZsPixelProgram prog;   // per-pixel ops fused after the stack
};

// Fused colour chain in canonical form (the hot path):
//   decode -> M_a -> [cbrt] -> M_b -> [cube] -> M_c -> [clamp] -> M_d -> encode
struct ZsChainArgs {
    const uint8_t *src;
    uint8_t *dst;
    int64_t npx;          // pixels (flat: the chain is pixel-local)
    float m[4][9];
    int32_t flags;        // ZS_CHAIN_* bits
    int32_t pad;
    float m2[4][9][2];    // the same matrices with every coefficient duplicated (f32x2 operands)
    // ZS_CHAIN_MB_RANK1: M_b = d I + (1,1,1)^T v (an Oklab L/C scaling), applied as
    // s = v . c, c' = d c + s (6 FMAs instead of 9); duplicated for f32x2 operands.
    float mb_v[3][2];
    float mb_d[2];
};

enum {
    ZS_CHAIN_CBRT = 1,
    ZS_CHAIN_CUBE = 2,
    ZS_CHAIN_CLAMP = 4,
    ZS_CHAIN_MA = 8,
    ZS_CHAIN_MB = 16,
    ZS_CHAIN_MC = 32,
    ZS_CHAIN_MD = 64,
    ZS_CHAIN_CBRT_NONNEG = 128,  // M_a maps [0,1]^3 to non-negative values: no sign handling
    ZS_CHAIN_MB_RANK1 = 256      // M_b is d I + (1,1,1)^T v (mb_v, mb_d)
};

// Entry count of the exact sRGB8 encode table: buckets of the float bit pattern
// (bits >> 16) for x in [2^-13, 1], each holding at most one rounding threshold.
#define ZS_ENC_BASE (114u << 7)
#define ZS_ENC_ENTRIES 1665
// The same encode for x' = saturate(x) + 2^-12, which lies in [2^-12, 1 + 2^-12] and
// needs no integer clamp: buckets (bits(x') >> 16) - ZS_ENCS_BASE.
#define ZS_ENCS_BASE (115u << 7)
#define ZS_ENCS_ENTRIES 1537
#define ZS_ENCS_SHIFT 0x39800000u   /* bits of 2^-12 */
