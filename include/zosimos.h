/*
 * zosimos.h -- C ABI of the GB300 executor for zosimos' compiled raster pipeline.
 *
 * Every entry point replaces one call of the reference's Rust API (paths inside
 * the zosimos project, cited per function).  The wgpu backend of the reference
 * is replaced by hand-written CUDA kernels for sm_103a; the API shape (Pool,
 * CommandBuffer, Linker/Program, Executable, Environment, Execution, Retire)
 * is kept so that a thin FFI crate (a Rust -sys crate) can bind it.
 *
 * Conventions
 *  - Every function returns an int status (ZS_OK = 0) unless stated otherwise;
 *    zs_last_error() returns a thread-local description of the last failure.
 *  - Handles are opaque; none is thread-safe, separate handles may be used from
 *    separate threads (an Execution owns one CUDA stream).
 *  - Registers are the SSA value ids of a command buffer (command.rs:32).
 *  - No C++ exception crosses this boundary; no user error aborts the process.
 */
#ifndef ZOSIMOS_GB300_H
#define ZOSIMOS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: CommandError / CompileError / LaunchError / StartError /
 *      StepError / RetireError kinds (command.rs:650-717, program.rs:374-381,
 *      run.rs:369-448). */
enum {
    ZS_OK = 0,
    ZS_ERR_TYPE = 1,            /* CommandError::TYPE_ERR, ConflictingTypes, BadDescriptor */
    ZS_ERR_UNIMPLEMENTED = 2,   /* CommandError::UNIMPLEMENTED, CompileError::NotYetImplemented */
    ZS_ERR_BAD_REGISTER = 3,    /* CommandError::BAD_REGISTER */
    ZS_ERR_OTHER = 4,           /* CommandError::OTHER / INVALID_CALL */
    ZS_ERR_LAUNCH = 5,          /* LaunchError */
    ZS_ERR_MISMATCHED_DESCRIPTOR = 6, /* StartError::MismatchedDescriptor */
    ZS_ERR_MISSING_KEY = 7,     /* StartError::MissingKey / unbound input */
    ZS_ERR_DEVICE = 8,          /* a CUDA runtime error */
    ZS_ERR_TIMEOUT = 9,         /* a bounded device wait gave up */
    ZS_ERR_INVALID_ARG = 10,    /* null handle / pointer / size out of range */
    ZS_ERR_OUT_OF_MEMORY = 11,
    ZS_ERR_STEP_LIMIT = 12      /* StepLimits exhausted (run.rs:3000-3013) */
};

/* ---- descriptor vocabulary (image-canvas 0.5.1 as used by buffer.rs:1-115;
 *      numeric codes of bits/parts/transfer follow lib/std/src/stage.frag:102-176). */
enum { /* SampleBits */
    ZS_BITS_UINT8 = 0, ZS_BITS_UINT332 = 1, ZS_BITS_UINT233 = 2, ZS_BITS_UINT16 = 3,
    ZS_BITS_UINT4X4 = 4, ZS_BITS_UINT_444 = 5, ZS_BITS_UINT444_ = 6, ZS_BITS_UINT565 = 7,
    ZS_BITS_UINT8X2 = 8, ZS_BITS_UINT8X3 = 9, ZS_BITS_UINT8X4 = 10, ZS_BITS_UINT16X2 = 11,
    ZS_BITS_UINT16X3 = 12, ZS_BITS_UINT16X4 = 13, ZS_BITS_UINT1010102 = 14,
    ZS_BITS_UINT2101010 = 15, ZS_BITS_UINT101010_ = 16, ZS_BITS_UINT_101010 = 17,
    ZS_BITS_FLOAT16X4 = 18, ZS_BITS_FLOAT32X4 = 19
};
enum { /* SampleParts */
    ZS_PARTS_A = 0, ZS_PARTS_R = 1, ZS_PARTS_G = 2, ZS_PARTS_B = 3, ZS_PARTS_LUMA = 4,
    ZS_PARTS_LUMAA = 5, ZS_PARTS_RGB = 6, ZS_PARTS_BGR = 7, ZS_PARTS_RGBA = 8,
    ZS_PARTS_RGBX = 9, ZS_PARTS_BGRA = 10, ZS_PARTS_BGRX = 11, ZS_PARTS_ARGB = 12,
    ZS_PARTS_XRGB = 13, ZS_PARTS_ABGR = 14, ZS_PARTS_XBGR = 15, ZS_PARTS_YUV = 16,
    ZS_PARTS_LAB = 17, ZS_PARTS_LABA = 18, ZS_PARTS_LCH = 19, ZS_PARTS_LCHA = 20
};
enum { /* Transfer */
    ZS_TRANSFER_BT709 = 0, ZS_TRANSFER_BT470M = 1, ZS_TRANSFER_BT601 = 2,
    ZS_TRANSFER_SMPTE240 = 3, ZS_TRANSFER_LINEAR = 4, ZS_TRANSFER_SRGB = 5,
    ZS_TRANSFER_BT2020_10BIT = 6, ZS_TRANSFER_BT2020_12BIT = 7, ZS_TRANSFER_SMPTE2084 = 8,
    ZS_TRANSFER_BT2100PQ = 9, ZS_TRANSFER_BT2100HLG = 10, ZS_TRANSFER_LINEAR_SCENE = 11
};
enum { /* Color kind */
    ZS_COLOR_RGB = 0, ZS_COLOR_OKLAB = 1, ZS_COLOR_SRLAB2 = 2, ZS_COLOR_SCALARS = 3
};
enum { /* Primaries */
    ZS_PRIMARIES_BT601_525 = 0, ZS_PRIMARIES_BT601_625 = 1, ZS_PRIMARIES_BT709 = 2,
    ZS_PRIMARIES_SMPTE240 = 3, ZS_PRIMARIES_BT2020 = 4, ZS_PRIMARIES_BT2100 = 5,
    ZS_PRIMARIES_P3 = 6, ZS_PRIMARIES_ADOBE_RGB = 7, ZS_PRIMARIES_XYZ = 8
};
enum { /* Whitepoint */
    ZS_WP_A = 0, ZS_WP_B = 1, ZS_WP_C = 2, ZS_WP_D50 = 3, ZS_WP_D55 = 4, ZS_WP_D65 = 5,
    ZS_WP_D75 = 6, ZS_WP_E = 7, ZS_WP_F2 = 8, ZS_WP_F7 = 9, ZS_WP_F11 = 10
};
enum { ZS_ALPHA_STRAIGHT = 0, ZS_ALPHA_PREMULTIPLIED = 1 };

/* Descriptor (buffer.rs:20-27): layout + colour + texel.  row_stride 0 means
 * tightly packed rows (width * texel bytes). */
typedef struct zs_descriptor {
    uint32_t width, height;
    uint64_t row_stride;
    uint32_t bits, parts;                               /* Texel */
    uint32_t color, primaries, transfer, whitepoint;    /* Color */
    uint32_t alpha;                                     /* ZS_ALPHA_* (extension) */
    uint32_t reserved;
} zs_descriptor;

/* Rectangle (command.rs:3496-3592): [x, max_x) x [y, max_y). */
typedef struct zs_rect { uint32_t x, y, max_x, max_y; } zs_rect;

/* ---- descriptor helpers ------------------------------------------------- */
/* Descriptor::with_srgb_image for an RGBA8 image (buffer.rs). */
int zs_descriptor_srgb_rgba8(uint32_t width, uint32_t height, zs_descriptor *out);
/* Descriptor::is_consistent (buffer.rs) -- 1 when valid, 0 otherwise. */
int zs_descriptor_is_consistent(const zs_descriptor *desc);
/* Bytes of the host (tightly packed or row_stride) layout. */
uint64_t zs_descriptor_byte_len(const zs_descriptor *desc);
/* Bytes of one texel of `bits`. */
uint32_t zs_texel_bytes(uint32_t bits);

/* ---- errors ------------------------------------------------------------- */
const char *zs_last_error(void);
/* Library version string. */
const char *zs_version(void);

/* ---- Pool (pool.rs:180-455) --------------------------------------------- */
typedef struct zs_pool zs_pool;
zs_pool *zs_pool_new(void);                                   /* Pool::new           pool.rs:182 */
void zs_pool_free(zs_pool *pool);
/* Pool::insert (pool.rs:244): copies `bytes` (laid out as `desc`) into pinned host storage. */
int zs_pool_insert(zs_pool *pool, const zs_descriptor *desc, const void *bytes, uint64_t *key);
/* Pool::declare (pool.rs:281): an image slot without contents (e.g. an output). */
int zs_pool_declare(zs_pool *pool, const zs_descriptor *desc, uint64_t *key);
/* PoolImage::descriptor (pool.rs:661). */
int zs_pool_descriptor(zs_pool *pool, uint64_t key, zs_descriptor *out);
/* PoolImage::as_bytes (pool.rs:669): copy the host bytes out (len must match). */
int zs_pool_read(zs_pool *pool, uint64_t key, void *dst, uint64_t len);
/* PoolImageMut::as_bytes_mut (pool.rs:704): overwrite the host bytes in place. */
int zs_pool_write(zs_pool *pool, uint64_t key, const void *src, uint64_t len);
/* Direct pointer to the pinned host storage (valid until the image is removed). */
int zs_pool_host_ptr(zs_pool *pool, uint64_t key, void **ptr, uint64_t *len);
/* PoolImageMut::set_color (pool.rs:719): re-tag the colour of an image. */
int zs_pool_set_descriptor(zs_pool *pool, uint64_t key, const zs_descriptor *desc);
/* Pool::upload (pool.rs:292): make the image device resident (cudaMemcpy). */
int zs_pool_upload(zs_pool *pool, uint64_t key);
/* Device pointer of a device-resident image (GPU-resident IO). */
int zs_pool_device_ptr(zs_pool *pool, uint64_t key, void **ptr);
/* Remove an image. */
int zs_pool_remove(zs_pool *pool, uint64_t key);
/* Pool::clear_cache (pool.rs:450): release cached device buffers. */
int zs_pool_clear_cache(zs_pool *pool);

/* ---- CommandBuffer (command.rs:739-1765) --------------------------------- */
typedef struct zs_cmd zs_cmd;
zs_cmd *zs_cmd_new(void);
void zs_cmd_free(zs_cmd *cmd);
/* CommandBuffer::input (command.rs:743). */
int zs_cmd_input(zs_cmd *cmd, const zs_descriptor *desc, uint32_t *reg);
/* CommandBuffer::crop (command.rs:912). */
int zs_cmd_crop(zs_cmd *cmd, uint32_t src, const zs_rect *rect, uint32_t *reg);
/* CommandBuffer::color_convert (command.rs:986): `target` supplies color/texel fields;
 * its width/height/row_stride are ignored (taken from src). */
int zs_cmd_color_convert(zs_cmd *cmd, uint32_t src, const zs_descriptor *target, uint32_t *reg);
/* CommandBuffer::chromatic_adaptation (command.rs:1112); method: 0 Xyz, 1 VonKries,
 * 2 BradfordVonKries, 3 BradfordNonLinear. */
int zs_cmd_chromatic_adaptation(zs_cmd *cmd, uint32_t src, uint32_t method, uint32_t target_wp,
                                uint32_t *reg);
/* CommandBuffer::inscribe (command.rs:1177).  Keeps the reference semantics exactly,
 * including Rectangle::normalize's max_y = y + width (command.rs:3536-3543). */
int zs_cmd_inscribe(zs_cmd *cmd, uint32_t below, const zs_rect *rect, uint32_t above,
                    uint32_t *reg);
/* Extension: inscribe at any placement inside `below` without the normalize
 * stretch (centred placement needs it; no reference counterpart). */
int zs_cmd_inscribe_placed(zs_cmd *cmd, uint32_t below, const zs_rect *rect, uint32_t above,
                           uint32_t *reg);
/* CommandBuffer::extract (command.rs:1221); channel: 0 R, 1 G, 2 B, 3 Alpha. */
int zs_cmd_extract(zs_cmd *cmd, uint32_t src, uint32_t channel, uint32_t *reg);
/* CommandBuffer::inject (command.rs:1360). */
int zs_cmd_inject(zs_cmd *cmd, uint32_t below, uint32_t channel, uint32_t above, uint32_t *reg);
/* CommandBuffer::transmute (command.rs:1276). */
int zs_cmd_transmute(zs_cmd *cmd, uint32_t src, const zs_descriptor *target, uint32_t *reg);
/* CommandBuffer::palette (command.rs:1442); width/height channel: 0 R, 1 G, 2 B, -1 none. */
int zs_cmd_palette(zs_cmd *cmd, uint32_t palette, int32_t width_channel, int32_t height_channel,
                   uint32_t indices, uint32_t *reg);
/* CommandBuffer::bilinear (command.rs:1615); params = u_min,u_max,v_min,v_max,uv_min,uv_max. */
int zs_cmd_bilinear(zs_cmd *cmd, const zs_descriptor *desc, const float params[24],
                    uint32_t *reg);
/* CommandBuffer::solid_rgba (command.rs:1526). */
int zs_cmd_solid_rgba(zs_cmd *cmd, const zs_descriptor *desc, const float color[4],
                      uint32_t *reg);
/* CommandBuffer::affine (command.rs:1636); matrix row-major homogeneous in pixel units;
 * sampling 0 Nearest, 1 BiLinear (BiLinear is UNIMPLEMENTED upstream, built here). */
int zs_cmd_affine(zs_cmd *cmd, uint32_t below, const float matrix[9], uint32_t sampling,
                  uint32_t above, uint32_t *reg);
/* CommandBuffer::resize (command.rs:1675): the reference's nearest palette resize. */
int zs_cmd_resize(zs_cmd *cmd, uint32_t src, uint32_t width, uint32_t height, uint32_t *reg);
/* Extension of resize with a filter: 0 Box (area), 1 Lanczos-3, 2 Triangle. */
int zs_cmd_resize_filtered(zs_cmd *cmd, uint32_t src, uint32_t width, uint32_t height,
                           uint32_t filter, uint32_t *reg);
/* CommandBuffer::derivative (command.rs:1493): first derivative by a 3x3 operator along the
 * width or height (box3.frag, command.rs:3343-3409); the result keeps the descriptor of
 * `src`, its alpha is 1.  Methods (DerivativeMethod order): 0 Roberts, 1 Prewitt, 2 Sobel,
 * 3 Scharr3, 4 Scharr4, 5 Scharr5, 6 Scharr3To4Bit, 7 Scharr5Tab, 8 Scharr3To8Bit; Roberts,
 * Scharr4, Scharr5 and Scharr5Tab fail in zs_compile with ZS_ERR_UNIMPLEMENTED as in the
 * reference.  direction: 0 Width, 1 Height. */
int zs_cmd_derivative(zs_cmd *cmd, uint32_t src, uint32_t method, uint32_t direction, uint32_t *reg);
/* CommandBuffer::distribution_normal2d (command.rs; shaders/distribution_normal2d.rs,
 * distribution_normal2d.frag): an image of the normal density
 * exp(-0.5 pos.(C+ pos)) / sqrt(pdet), pos = 2 (uv - 0.5) - mu at pixel centres, in all three
 * colour channels, alpha 1.  params = [mu0, mu1, C+00, C+01, C+10, C+11, pdet].  The two
 * constructors of DistributionNormal2d fill `params` as the reference does (f32). */
int zs_cmd_distribution_normal2d(zs_cmd *cmd, const zs_descriptor *desc, const float params[7], uint32_t *reg);
int zs_normal2d_with_diagonal(float var0, float var1, float params[7]);
int zs_normal2d_with_direction(float x, float y, float params[7]);
/* CommandBuffer::buffer_init / buffer_zero (command.rs:1777-1803): a byte buffer register
 * holding a copy of `bytes` (len bytes) or `len` zero bytes.  A buffer register is not an
 * image: image ops given one fail with ZS_ERR_TYPE. */
int zs_cmd_buffer_init(zs_cmd *cmd, const void *bytes, uint64_t len, uint32_t *reg);
int zs_cmd_buffer_zero(zs_cmd *cmd, uint64_t len, uint32_t *reg);
/* CommandBuffer::from_buffer (command.rs:937-968): the buffer's bytes read as an image of
 * `desc` whose rows start every align_up(width * texel bytes, 256) bytes (the GPU row layout of
 * Descriptor::to_aligned, buffer.rs:121-134).  ZS_ERR_TYPE when `buffer` is not a buffer
 * register, ZS_ERR_OTHER (INVALID_CALL) when the buffer holds fewer than height aligned rows. */
int zs_cmd_from_buffer(zs_cmd *cmd, uint32_t buffer, const zs_descriptor *desc, uint32_t *reg);
/* CommandBuffer::distribution_fractal_noise (command.rs:1585-1606; shaders/fractal_noise.rs,
 * fractal_noise.frag): fractal Brownian value noise, uncorrelated in all four channels, from
 * the PCG4D hash of the grid cell corners with smoothstep interpolation, summed over
 * num_octaves octaves (each rotated by 0.5 rad and scaled by 2, amplitude times damping).
 * params = [grid_scale x, grid_scale y, initial_amplitude, amplitude_damping, num_octaves];
 * num_octaves is an integer in [0, 32] (ZS_ERR_INVALID_ARG otherwise).
 * zs_fractal_noise_with_octaves and zs_fractal_noise_set_damping fill `params` as
 * FractalNoise::with_octaves and FractalNoise::set_damping do (shaders/fractal_noise.rs:20-49). */
int zs_cmd_distribution_fractal_noise(zs_cmd *cmd, const zs_descriptor *desc, const float params[5], uint32_t *reg);
int zs_fractal_noise_with_octaves(uint32_t num_octaves, float params[5]);
int zs_fractal_noise_set_damping(float params[5], float damping);
/* CommandBuffer::blend (command.rs:1509, UNIMPLEMENTED upstream, built here):
 * mode 0 Alpha/over, 1 multiply, 2 screen, 3 add; `above` placed at rect.x/rect.y. */
int zs_cmd_blend(zs_cmd *cmd, uint32_t below, const zs_rect *rect, uint32_t above,
                 uint32_t mode, uint32_t *reg);
/* Extension: a 3x3 linear map applied to the colour channels in the image's own
 * colour space (e.g. scaling Oklab L and C); alpha is kept. */
int zs_cmd_color_matrix(zs_cmd *cmd, uint32_t src, const float matrix[9], uint32_t *reg);
/* CommandBuffer::with_knob (command.rs:1740-1742, WithKnob :1865-1961): the next operation's
 * parameter block becomes a knob that a launch may replace without recompiling.  Operations
 * that take one: bilinear (6 x 4 f32), solid_rgba (4 f32), distribution_normal2d (8 f32:
 * mu0, mu1, C+ row major, pseudo-determinant, pad), distribution_fractal_noise (2 f32 grid
 * scale, f32 amplitude, f32 damping, u32 octaves, 4 bytes pad) and buffer_init (the buffer's
 * bytes); any other operation fails with ZS_ERR_UNIMPLEMENTED. */
int zs_cmd_with_knob(zs_cmd *cmd);
/* CommandBuffer::with_buffer (command.rs:1751-1765, WithBuffer :1963-2060): the next
 * operation (bilinear, solid_rgba, distribution_normal2d, distribution_fractal_noise) reads
 * its parameter block from the start of `buffer` (a buffer_init / buffer_zero register), and
 * follows the buffer's knob when it has one.  ZS_ERR_TYPE when `buffer` is not a buffer,
 * ZS_ERR_OTHER (INVALID_CALL) when it is shorter than the parameter block. */
int zs_cmd_with_buffer(zs_cmd *cmd, uint32_t buffer);
/* ---- custom operations (ShaderCommand, command/dynamic.rs:7-51, through
 *      CommandBuffer::construct_dynamic / unary_dynamic / binary_dynamic, command.rs:2933-3048).
 * The reference takes a SPIR-V fragment shader and its uniform bytes; here the compiled GPU
 * program is a PTX or cubin module holding a kernel with this parameter block, launched with
 * 16 x 16 blocks over the result (grid ceil(width / 16) x ceil(height / 16)).  Operands arrive
 * as linear RGBA32F images (the values a shader samples, tightly packed rows), the kernel
 * writes the result as linear RGBA32F, and the executor encodes it to the declared texel. */
typedef struct zs_dyn_args {
    const float *src[2];        /* operands (null where absent), RGBA32F, width * 16 bytes per row */
    int32_t src_width[2], src_height[2];
    float *dst;                 /* result, RGBA32F, width * 16 bytes per row */
    int32_t width, height;
    const void *uniforms;       /* the operation's uniform bytes (device memory), or null */
    uint64_t uniform_len;
} zs_dyn_args;
/* Loads a module (PTX text with its terminating zero, or a cubin / fatbin image) and names its
 * kernel `kernel_name`, whose only parameter is a zs_dyn_args; returns an op id for the
 * *_dynamic commands.  The module is loaded on the current device at registration. */
int zs_register_op(const void *image, uint64_t len, const char *kernel_name, uint32_t *op);
int zs_cmd_construct_dynamic(zs_cmd *cmd, uint32_t op, const void *uniforms, uint64_t len,
                             const zs_descriptor *desc, uint32_t *reg);
int zs_cmd_unary_dynamic(zs_cmd *cmd, uint32_t src, uint32_t op, const void *uniforms, uint64_t len,
                         const zs_descriptor *desc, uint32_t *reg);
int zs_cmd_binary_dynamic(zs_cmd *cmd, uint32_t lhs, uint32_t rhs, uint32_t op, const void *uniforms,
                          uint64_t len, const zs_descriptor *desc, uint32_t *reg);
/* CommandBuffer::output (command.rs:1707). */
int zs_cmd_output(zs_cmd *cmd, uint32_t src, uint32_t *reg, zs_descriptor *outformat);
/* Describe a register (command.rs describe_reg). */
int zs_cmd_describe(const zs_cmd *cmd, uint32_t reg, zs_descriptor *out);

/* ---- generic functions (command.rs:756-922) ------------------------------ */
/* CommandBuffer::generic (command.rs:768): declares a generic descriptor parameter; returns
 * the descriptor variable (DescriptorVar) standing for it. */
int zs_cmd_generic(zs_cmd *cmd, uint32_t *ty);
/* CommandBuffer::input_generic (command.rs:756): an input whose descriptor is the variable's. */
int zs_cmd_input_generic(zs_cmd *cmd, uint32_t ty, uint32_t *reg);
/* CommandBuffer::derive_descriptor (command.rs:786-805): variable `base` with its size replaced
 * by width x height (both 0: kept). */
int zs_cmd_derive_descriptor(zs_cmd *cmd, uint32_t base, uint32_t width, uint32_t height, uint32_t *ty);
/* CommandBuffer::register_descriptor (command.rs:808): a descriptor variable of a register. */
int zs_cmd_register_descriptor(zs_cmd *cmd, uint32_t reg, uint32_t *ty);
/* CommandBuffer::computed_signature (command.rs:821): counts of generics, inputs, outputs. */
int zs_cmd_signature(const zs_cmd *cmd, uint32_t *n_generics, uint32_t *n_inputs, uint32_t *n_outputs);
/* CommandBuffer::function (command.rs:856): declares a function with the signature computed
 * from `signature` (a snapshot is kept); its definition is supplied to zs_link. */
int zs_cmd_function(zs_cmd *cmd, const zs_cmd *signature, uint32_t *function);
/* CommandBuffer::invoke (command.rs:863-922): calls `function` with descriptor variables for its
 * generics and argument registers (checked against its inputs: ZS_ERR_OTHER, INVALID_CALL,
 * on a mismatch); writes the n_results result registers. */
int zs_cmd_invoke(zs_cmd *cmd, uint32_t function, const uint32_t *generics, uint32_t n_generics, const uint32_t *args,
                  uint32_t n_args, uint32_t *results, uint32_t n_results);

/* ---- Linker / Program (command.rs:2063-2185, program.rs:1284-1423) -------- */
typedef struct zs_program zs_program;
/* Linker::compile (command.rs:2069). */
int zs_compile(const zs_cmd *cmd, zs_program **out);
/* Linker::link (command.rs:2083-2185): `main` (its generic parameters given by the n_tys
 * descriptors `tys`) and the function definitions; links[i] (of
 * link_counts[i] entries) names, for each function declared in buffer i (0 = main, i = function
 * i - 1), the buffer defining it.  Every invocation is monomorphised for its generics and
 * inlined, so the program is planned (and fused) as a whole.  Registers of main keep their
 * numbers for binding and retiring; a function's registers are reached with its link index
 * (zs_executable_query_knob). */
int zs_link(const zs_cmd *main, const zs_descriptor *tys, uint32_t n_tys, const zs_cmd *const *functions,
            uint32_t n_functions, const uint32_t *const *links, const uint32_t *link_counts, uint32_t n_links,
            zs_program **out);
void zs_program_free(zs_program *program);

/* Capabilities / lowering options (program.rs:1304 lower_to). */
enum {
    ZS_MODE_FUSED = 0,        /* fused per-pixel chains, FP16 storage at unfusable boundaries */
    ZS_MODE_PER_OP_F32 = 1,   /* one kernel per op, FP32 RGBA intermediates (the plain baseline) */
    ZS_MODE_PER_OP_F16 = 2    /* one kernel per op, FP16 RGBA intermediates */
};
typedef struct zs_capabilities {
    int32_t device;           /* CUDA device ordinal */
    uint32_t mode;            /* ZS_MODE_* */
    uint32_t use_graph;       /* capture a multi-step kernel sequence as a CUDA graph and replay it */
    uint32_t flags;           /* ZS_CAP_* bits */
} zs_capabilities;

enum {
    /* resize_filtered: use the FP32 SIMT resample kernel even where the tensor-core path
     * (f16 band matrices, FP32 accumulation) applies. */
    ZS_CAP_SIMT_RESAMPLE = 1,
    /* zs_run_host: always stage host buffers through device copies, even where the kernel
     * could read and write pinned host memory directly (see zs_run_host). */
    ZS_CAP_NO_ZERO_COPY = 2
};

typedef struct zs_executable zs_executable;
/* Program::lower_to (program.rs:1304). */
int zs_lower(const zs_program *program, const zs_capabilities *caps, zs_executable **out);
void zs_executable_free(zs_executable *exe);
/* Executable::query_knob (run.rs:1012-1014) for RegisterKnob { link_idx, register }: the knob
 * id and the byte length of its parameter block.  link_idx 0 is the linked program's main
 * buffer, i the i-th function buffer given to zs_link (its first instantiation when it is
 * invoked more than once).  ZS_ERR_BAD_REGISTER when the register has no knob. */
int zs_executable_query_knob(const zs_executable *exe, uint32_t link_idx, uint32_t reg, uint32_t *knob,
                             uint64_t *len);
/* Replaces the parameter block of a knob for every later launch of the executable (the
 * one-call paths zs_run_host / zs_run_device / batches included); len must equal the knob's.
 * No counterpart in the reference, whose knob data is per launch (zs_env_knob). */
int zs_executable_set_knob(zs_executable *exe, uint32_t knob, const void *data, uint64_t len);
/* Number of kernel launches one launch of this executable issues. */
int zs_executable_kernel_count(const zs_executable *exe, uint32_t *count);
/* Numbers of input and output registers (either pointer may be null). */
int zs_executable_io_count(const zs_executable *exe, uint32_t *inputs, uint32_t *outputs);
/* Human readable plan (the analogue of Executable::dot, run.rs:491). */
const char *zs_executable_describe(const zs_executable *exe);

/* ---- Environment / Execution / Retire (run.rs:470-2998) ------------------ */
typedef struct zs_environment zs_environment;
typedef struct zs_execution zs_execution;
/* Executable::from_pool (run.rs:471). */
int zs_env_new(zs_executable *exe, zs_pool *pool, zs_environment **out);
void zs_env_free(zs_environment *env);
/* Environment::bind (run.rs:1171). */
int zs_env_bind(zs_environment *env, uint32_t reg, uint64_t key);
/* Environment::knob (run.rs:1292-1306): the parameter block of `knob` for this launch only (len
 * must equal the knob's, else ZS_ERR_INVALID_ARG); launches without one use the static block. */
int zs_env_knob(zs_environment *env, uint32_t knob, const void *data, uint64_t len);
/* Environment::recover_buffers (run.rs:1312-1347): an executable keeps its intermediate device
 * buffers between launches, so there is nothing to take from the pool; *bytes receives the
 * bytes it already holds (RecoveredBufferStats::mem). */
int zs_env_recover_buffers(zs_environment *env, uint64_t *bytes);
/* Environment::bind_output (run.rs:1207): write the output into an existing image. */
int zs_env_bind_output(zs_environment *env, uint32_t reg, uint64_t key);
/* Executable::launch (run.rs:1016): consumes `env` (even on failure). */
int zs_launch(zs_executable *exe, zs_environment *env, zs_execution **out);
/* Execution::is_running (run.rs:1382). */
int zs_exec_is_running(const zs_execution *exec);
/* Execution::step (run.rs:1389): enqueue the next instruction. */
int zs_exec_step(zs_execution *exec);
/* Execution::step_to(StepLimits::new().with_steps(max_steps)) (run.rs:1394, 3000-3013):
 * enqueue up to max_steps instructions (fewer at the end); *steps receives the count. */
int zs_exec_step_to(zs_execution *exec, uint32_t max_steps, uint32_t *steps);
/* SyncPoint::block_on (run.rs:3019): wait for everything enqueued so far. */
int zs_exec_sync(zs_execution *exec);
/* Retire::input (run.rs:2791): the pool key of the image bound to input `reg` (binding does
 * not move the image out of the pool here, so it is the key given to zs_env_bind);
 * ZS_ERR_BAD_REGISTER for a register that is no input (RetireError::NoSuchInput). */
int zs_retire_input(zs_execution *exec, uint32_t reg, uint64_t *key);
/* Retire::output (run.rs:2809): the output moves into the pool; returns its key. */
int zs_retire_output(zs_execution *exec, uint32_t reg, uint64_t *key);
/* Retire::finish (run.rs:2962): release the execution. */
void zs_exec_free(zs_execution *exec);

/* ---- one-call drop-in for host buffers ------------------------------------ */
/* Runs the whole executable once: inputs[i] bound to the i-th input register (in
 * declaration order) from host memory, outputs[j] receive the j-th output (host
 * memory).  Equivalent to insert/bind/launch/step/retire/read.  Host buffers that
 * are pinned (zs_host_alloc) transfer at full link speed.  An executable that is one
 * pixel-local colour chain, given pinned (device-mapped) 16-byte aligned host buffers, runs
 * zero copy: on a Grace host the chain kernel loads its input from and stores its output to
 * host memory over NVLink-C2C, one launch and no staging copies (ZS_CAP_NO_ZERO_COPY
 * turns this off).  Other host buffers of such a chain go through row stripes whose upload,
 * kernel and download overlap on three streams. */
int zs_run_host(zs_executable *exe, const void *const *inputs, uint32_t n_inputs,
                void *const *outputs, uint32_t n_outputs);
/* Same, with device-resident inputs and outputs (no host copies).  Each buffer must start
 * on its texel's natural alignment (the largest power of two dividing the texel size, at
 * most 16 bytes), else ZS_ERR_INVALID_ARG; a colour chain on 16-byte aligned buffers runs
 * on the chain kernel, on others on the generic raster kernel. */
int zs_run_device(zs_executable *exe, const void *const *inputs, uint32_t n_inputs,
                  void *const *outputs, uint32_t n_outputs, void *stream);
/* Pinned host memory helpers. */
void *zs_host_alloc(uint64_t bytes);
void zs_host_free(void *ptr);
/* Device memory helpers (for device-resident IO through zs_run_device). */
void *zs_device_alloc(uint64_t bytes);
void zs_device_free(void *ptr);
int zs_memcpy_h2d(void *dst, const void *src, uint64_t bytes);
int zs_memcpy_d2h(void *dst, const void *src, uint64_t bytes);
int zs_device_synchronize(void);

/* ---- batched uneven images (the reference's batch-reuse case, tests/loop.rs:84-95) ---- */
/* One persistent launch over many RGBA8 sRGB images of different sizes: per image
 * the fused colour chain of `chain` (an executable whose single input and output are
 * RGBA8 images and whose ops are per-pixel), a box fit-resize so the long side is
 * `canvas`, and a centred inscribe on a transparent canvas x canvas image.
 * images: device pointers of tightly packed RGBA8 sources; out: n * canvas^2 * 4 bytes. */
int zs_batch_thumbnails(zs_executable *chain, const void *const *images, const uint32_t *widths,
                        const uint32_t *heights, uint32_t n, uint32_t canvas, void *out,
                        void *stream);

/* ---- batches of runs of one executable (the reference's batch-reuse case: one Executable
 *      launched for many images, tests/loop.rs:80-95, Environment::recover_buffers
 *      run.rs:1312-1347) ---- */
/* Runs `exe` once per set of device buffers: inputs holds n x (number of inputs) pointers,
 * run i's inputs in declaration order at inputs[i * n_inputs ...], outputs likewise.  The n
 * runs are recorded into one CUDA graph -- independent runs on up to 8 parallel branches; an
 * executable that stores intermediates runs them one after another -- which is cached per
 * pointer table and replayed when the same table comes again.  Buffers follow the alignment
 * rule of zs_run_device.  stream may be null (the executable's own stream). */
int zs_batch_run_device(zs_executable *exe, const void *const *inputs, void *const *outputs, uint32_t n,
                        void *stream);
/* The same over pool images: keys holds n x (number of inputs) pool keys, each checked against
 * the input's descriptor (StartError::MismatchedDescriptor) and made device resident
 * (Pool::upload); every run's outputs are retired into new pool images (Retire::output),
 * whose keys are written to out_keys (n x number of outputs).  Synchronous. */
int zs_batch_run(zs_executable *exe, zs_pool *pool, const uint64_t *keys, uint32_t n, uint64_t *out_keys);

/* ---- resample without any device allocation ------------------------------------ */
/* No counterpart in the reference.  For callers that may not allocate device memory
 * while they run (a pre-budgeted host application, a plugin inside someone else's
 * allocator, a latency-critical loop): the separable resample of
 * zs_cmd_resize_filtered for tightly packed RGBA16F linear images, with src/dst
 * supplied by the caller and every temporary (filter tables, FP16 intermediate) kept
 * in one fixed 32 MiB device array per GPU.  Calls that need more than that array
 * (tables + dst_width * src_height * 8 bytes) return ZS_ERR_INVALID_ARG, and so do src or
 * dst pointers that are not 8-byte aligned and sides above 2^24.  All calls on a device
 * share the array: calls that overlap on the GPU race (their results are undefined), so
 * order them on one stream; a non-blocking stream is not ordered against the legacy default
 * stream.  The
 * first call on a device loads the array's module (the driver reserves the 32 MiB then,
 * so that call can fail for lack of memory) and resolves the array's address for the
 * current device: make one warm-up call at start-up, before any stream capture, and do
 * not use this entry point across a device reset.  filter: 0 Box, 1 Lanczos-3,
 * 2 Triangle; stream may be null (the legacy default stream). */
int zs_resample_rgba16f_noalloc(const void *src, uint32_t src_width, uint32_t src_height, void *dst,
                                uint32_t dst_width, uint32_t dst_height, uint32_t filter, void *stream);

/* ---- autotuner (no counterpart in the reference: its render passes have no launch
 *      parameters) ---- */
enum {
    ZS_TUNE_CHAIN_THREADS = 0,   /* colour-chain kernel block size: 1024 (one block per SM) or 512 */
    ZS_TUNE_BATCH_ROWS = 1,      /* batched thumbnails: work-item height, 1..16 (about 16 x value
                                    source rows per item; value output rows for upscaled images) */
    ZS_TUNE_BATCH_THREADS = 2,   /* batched thumbnails: block size, 768 or 640 (one block per SM) */
    ZS_TUNE_RESAMPLE_TILE = 3,   /* tensor-core resample: output columns per tile, 8, 16 or 32 (those
                                    whose source span fits the kernel) */
    ZS_TUNE_CHAIN_VECTORS = 4    /* colour-chain kernel: 16-byte vectors (4 pixels each) per thread
                                    and loop iteration, 2 or 1 */
};
/* Times the candidates of every tunable launch of `exe` (CUDA events, median of `reps`
 * launches each) on the given device buffers -- which receive the result -- and keeps the
 * fastest with the executable and in the process-wide tuning cache, keyed by kernel family,
 * chain specialisation, size class and device; executables lowered later on the same device
 * start from the cached value.  Every candidate computes the same bytes. */
int zs_autotune(zs_executable *exe, const void *const *inputs, uint32_t n_inputs, void *const *outputs,
                uint32_t n_outputs, void *stream, uint32_t reps, int32_t *chain_threads);
/* The same for the work-item height and block size of zs_batch_thumbnails on this batch;
 * returns the height (the block size is read with zs_executable_get_launch). */
int zs_autotune_batch_thumbnails(zs_executable *chain, const void *const *images, const uint32_t *widths,
                                 const uint32_t *heights, uint32_t n, uint32_t canvas, void *out, void *stream,
                                 uint32_t reps, uint32_t *rows);
/* Sets / reads a launch parameter (ZS_TUNE_*) of an executable directly. */
int zs_executable_set_launch(zs_executable *exe, uint32_t param, int32_t value);
int zs_executable_get_launch(const zs_executable *exe, uint32_t param, int32_t *value);
/* The tuning-cache key a parameter of this executable uses (canvas: for the ZS_TUNE_BATCH_*). */
int zs_executable_tune_key(const zs_executable *exe, uint32_t param, uint32_t canvas, char *buf, uint64_t len);
/* The process-wide tuning cache: read / write one value, save to / merge from a text file
 * ("key value" lines).  zs_tune_cache_get fails with ZS_ERR_MISSING_KEY for an unknown key. */
int zs_tune_cache_get(const char *key, int32_t *value);
int zs_tune_cache_put(const char *key, int32_t value);
int zs_tune_cache_save(const char *path);
int zs_tune_cache_load(const char *path);

/* Number of kernels this library has launched since the process started. */
uint64_t zs_kernel_launch_count(void);

/* Device status word of `device` (ZS_DEVSTAT_* bits of zs_shared.h; bit 0: a bounded wait of
 * a kernel on its own bulk copies gave up, and that launch's output is incomplete; bit 1: a
 * kernel found its shared-memory window laid out other than the host checked and wrote
 * nothing), read after synchronising and cleared.  zs_exec_sync reports bit 0 as
 * ZS_ERR_TIMEOUT and bit 1 as ZS_ERR_DEVICE.
 * No counterpart in the reference (wgpu reports device loss through its own callbacks). */
int zs_device_status(int device, uint32_t *flags);

/* Diagnostic for the failure detection above: launches one warp whose mbarrier wait nothing
 * completes, through the same bounded-wait routine as the pipelined kernels but with a limit
 * of `limit_us` microseconds (1..1000000), and synchronises.  The kernel gives up and sets
 * bit 0 of the device status word, which zs_device_status then reports.  No counterpart in
 * the reference. */
int zs_selftest_wait_timeout(int device, uint32_t limit_us);

#ifdef __cplusplus
}
#endif
#endif
