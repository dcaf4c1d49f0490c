// command.cpp -- CommandBuffer: the SSA op builder with the reference's type checks
// (lib/zosimos/src/command.rs:739-1765) and the per-pixel semantics of each colour op
// expressed as a host pixel program (matrices kept in FP64 until lowering).
#include <cmath>
#include <cstring>

#include "zs_host.hpp"

namespace zs {

uint64_t knob_param_bytes(OpKind kind) {
    switch (kind) {
    case OpKind::Bilinear: return 6 * 16;     // shaders/bilinear.rs into_std430
    case OpKind::Solid: return 16;            // shaders/solid_rgb.rs [f32; 4]
    case OpKind::Normal2d: return 32;         // shaders/distribution_normal2d.rs [f32; 8]
    case OpKind::FractalNoise: return 24;     // shaders/fractal_noise.rs, aligned to 8
    default: return 0;
    }
}

std::vector<float> knob_cons(OpKind kind, const uint8_t *data, uint64_t len) {
    const uint64_t need = knob_param_bytes(kind);
    if (!need || len < need) fail(ZS_ERR_INVALID_ARG, "parameter block too short for this operation");
    std::vector<float> f(need / 4);
    std::memcpy(f.data(), data, need);
    if (kind == OpKind::Normal2d) f.resize(7);
    if (kind == OpKind::FractalNoise) {
        uint32_t octaves;
        std::memcpy(&octaves, data + 16, 4);
        if (octaves > 32) fail(ZS_ERR_INVALID_ARG, "fractal noise octaves above 32");
        f.resize(5);
        f[4] = (float)octaves;
    }
    return f;
}

// CommandBuffer::construct_dynamic / unary_dynamic / binary_dynamic (command.rs:2933-3048):
// a registered custom kernel over 0, 1 or 2 image operands, result described by `target`.
uint32_t cmd_dynamic(Command &c, uint32_t nops, uint32_t a, uint32_t b, uint32_t op_id, const void *uniforms,
                     uint64_t len, const Desc &target) {
    if (!dynamic_kernel(op_id)) fail(ZS_ERR_INVALID_ARG, "no custom operation with this id (zs_register_op)");
    if (!is_consistent(target)) fail(ZS_ERR_TYPE, "inconsistent descriptor: " + describe(target));
    // Operands must be images (CommandError::INVALID_CALL otherwise).
    if (nops > 0) c.describe(a);
    if (nops > 1) c.describe(b);
    Op op;
    op.kind = OpKind::Dynamic;
    op.a = a;
    op.b = b;
    op.u0 = nops;
    op.dyn_op = op_id;
    op.desc = target;
    if (len) {
        if (!uniforms) fail(ZS_ERR_INVALID_ARG, "uniform bytes missing");
        op.data.assign((const uint8_t *)uniforms, (const uint8_t *)uniforms + len);
    }
    op.len = len;
    return c.push(op);
}

uint32_t Command::push(Op op) {
    // CommandBuffer::with_knob / with_buffer apply to exactly this op (command.rs:1740-1765).
    const bool knob = pending_knob;
    const int32_t buffer = pending_buffer;
    clear_pending();
    if (knob) {
        if (!knob_param_bytes(op.kind) && op.kind != OpKind::BufferInit)
            fail(ZS_ERR_UNIMPLEMENTED, "this operation takes no knob (bilinear, solid_rgba, distribution_normal2d, "
                                       "distribution_fractal_noise and buffer_init do)");
        op.knob = true;
    }
    if (buffer >= 0) {
        const uint64_t need = knob_param_bytes(op.kind);
        if (!need) fail(ZS_ERR_UNIMPLEMENTED, "this operation takes no parameters from a buffer");
        if (ops[buffer].len < need) fail(ZS_ERR_OTHER, "buffer shorter than the operation's parameters");
        op.param_buffer = buffer;
    }
    ops.push_back(std::move(op));
    return (uint32_t)ops.size() - 1;
}

bool Command::is_value(uint32_t reg) const {
    return reg < ops.size() && ops[reg].kind != OpKind::Output && ops[reg].kind != OpKind::Invoke;
}

const Desc &Command::describe(uint32_t reg) const {
    if (!is_value(reg)) fail(ZS_ERR_BAD_REGISTER, "register does not name an image value");
    if (ops[reg].kind == OpKind::BufferInit) fail(ZS_ERR_TYPE, "register names a buffer, not an image");
    return ops[reg].desc;
}

// CommandBuffer::buffer_init / buffer_zero (command.rs:1777-1803): a byte buffer of `len`
// bytes, the first `n` from `bytes`, the rest zero.
uint32_t cmd_buffer_init(Command &c, const void *bytes, uint64_t n, uint64_t len) {
    if (n > len) fail(ZS_ERR_INVALID_ARG, "buffer initialiser longer than the buffer");
    if (n && !bytes) fail(ZS_ERR_INVALID_ARG, "null buffer initialiser");
    Op op{OpKind::BufferInit};
    op.len = len;
    if (n) op.data.assign((const uint8_t *)bytes, (const uint8_t *)bytes + n);
    return c.push(op);
}

// Rows of an image in a buffer are aligned to 256 bytes, as the GPU copy layout
// (Descriptor::to_aligned, buffer.rs:121-134).
uint64_t aligned_row_bytes(const Desc &d) { return ((uint64_t)d.width * texel_bytes(d.bits) + 255) & ~(uint64_t)255; }

// CommandBuffer::from_buffer (command.rs:937-968): the buffer's bytes read as an image of
// `d` with 256-byte aligned rows; the buffer must hold at least height aligned rows.
uint32_t cmd_from_buffer(Command &c, uint32_t buffer, const Desc &target) {
    if (!c.is_value(buffer) || c.ops[buffer].kind != OpKind::BufferInit)
        fail(ZS_ERR_TYPE, "from_buffer needs a buffer register");
    Desc d = target;
    d.row_stride = 0;
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent descriptor for from_buffer: " + describe(d));
    const uint64_t need = aligned_row_bytes(d) * d.height;
    if (c.ops[buffer].len < need) fail(ZS_ERR_OTHER, "buffer too small for this image descriptor");
    Op op{OpKind::FromBuffer};
    op.a = buffer;
    op.desc = d;
    return c.push(op);
}

static Desc with_size(Desc d, uint32_t w, uint32_t h) {
    d.width = w;
    d.height = h;
    d.row_stride = 0;
    return d;
}

// ---------------------------------------------------------------- colour semantics

// ColorConversion (command.rs:1009-1085 and :3220-3277).  The RGB->RGB case uses
// inv(dst.to_xyz) * src.to_xyz; the reference composes dst.to_xyz * inv(src.to_xyz)
// (command.rs:1022-1025, 3227-3228), which agrees whenever the primaries are equal.
static HProgram color_convert_program(const Desc &src, const Desc &dst) {
    HProgram p;
    const uint32_t sk = src.color, dk = dst.color;
    if (sk == ZS_COLOR_RGB && dk == ZS_COLOR_RGB) {
        if (src.whitepoint != dst.whitepoint) fail(ZS_ERR_TYPE, "color_convert between RGB spaces needs the same whitepoint");
        p.mat(rgb_to_xyz(dst.primaries, dst.whitepoint).inverse() * rgb_to_xyz(src.primaries, src.whitepoint));
    } else if (sk == ZS_COLOR_RGB && dk == ZS_COLOR_OKLAB) {
        p.mat(kOklabM1 * rgb_to_xyz(src.primaries, src.whitepoint));   // oklab.frag:34-47
        p.op(ZS_P_CBRT);
        p.mat(kOklabM2);
    } else if (sk == ZS_COLOR_OKLAB && dk == ZS_COLOR_RGB) {
        p.mat(kOklabM2.inverse());                                       // oklab.frag:50-64
        p.op(ZS_P_CUBE);
        p.mat(rgb_to_xyz(dst.primaries, dst.whitepoint).inverse() * kOklabM1.inverse());
        p.op(ZS_P_CLAMP01);
    } else if (sk == ZS_COLOR_RGB && dk == ZS_COLOR_SRLAB2) {
        // srlab2.frag:36-59: lms = HPE * inv(CAT02) * (CAT02 * xyz) = HPE * xyz.
        p.mat(kHpe * rgb_to_xyz(src.primaries, src.whitepoint));
        p.op(ZS_P_SRL_NL);
        p.mat(kHpe.inverse());
        p.op(ZS_P_SRL_ENC_DIFF);
    } else if (sk == ZS_COLOR_SRLAB2 && dk == ZS_COLOR_RGB) {
        // srlab2.frag:62-85 with the whitepoint of the SrLab2 colour.
        double w[3];
        whitepoint_xyz(src.whitepoint, w);
        double wr[3];
        for (int i = 0; i < 3; ++i) wr[i] = kCat02.m[3 * i] * w[0] + kCat02.m[3 * i + 1] * w[1] + kCat02.m[3 * i + 2] * w[2];
        p.op(ZS_P_SRL_DEC_DIFF);
        p.mat(kHpe);
        p.op(ZS_P_SRL_NLINV);
        Mat3 tail = rgb_to_xyz(dst.primaries, dst.whitepoint).inverse() * kCat02.inverse() *
                    Mat3::diag(wr[0], wr[1], wr[2]) * kCat02 * kHpe.inverse();
        p.mat(tail);
        p.op(ZS_P_CLAMP01);
    } else {
        fail(ZS_ERR_TYPE, "no conversion between these colours");
    }
    return p;
}

}  // namespace zs

using namespace zs;

// The C ABI command-building entry points live here so that they share the checks.
namespace zs {

uint32_t cmd_input(Command &c, const Desc &d) {
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent input declared: " + describe(d));
    Op op{OpKind::Input};
    op.desc = d;
    return c.push(op);
}

uint32_t cmd_crop(Command &c, uint32_t src, const zs_rect &r) {
    // command.rs:912-919: the result keeps the source descriptor; the linker paints the
    // selection over the whole target (command.rs:2507-2526).
    Op op{OpKind::Crop};
    op.a = src;
    op.desc = c.describe(src);
    op.rect = r;
    if (r.max_x <= r.x || r.max_y <= r.y) fail(ZS_ERR_OTHER, "empty crop");
    return c.push(op);
}

uint32_t cmd_color_convert(Command &c, uint32_t src, const Desc &target) {
    const Desc s = c.describe(src);
    Desc d = target;
    d.width = s.width;
    d.height = s.height;
    d.row_stride = 0;
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent conversion target: " + describe(d));
    Op op{OpKind::ColorConvert};
    op.a = src;
    op.desc = d;
    op.prog = color_convert_program(s, d);
    return c.push(op);
}

uint32_t cmd_chromatic_adaptation(Command &c, uint32_t src, uint32_t method, uint32_t target_wp) {
    const Desc s = c.describe(src);
    if (s.color != ZS_COLOR_RGB) fail(ZS_ERR_TYPE, "non-rgb chromatic adaptation");
    if (target_wp > ZS_WP_F11) fail(ZS_ERR_INVALID_ARG, "bad whitepoint");
    Mat3 adapt;
    if (!adaptation_matrix(method, s.whitepoint, target_wp, adapt))
        fail(ZS_ERR_UNIMPLEMENTED, "chromatic adaptation method not implemented");
    Op op{OpKind::ChromaticAdaptation};
    op.a = src;
    op.desc = s;
    op.desc.whitepoint = target_wp;
    op.desc.row_stride = 0;
    // command.rs:2527-2531: from_xyz(target) * adapt * to_xyz(source)
    op.prog.mat(rgb_to_xyz(s.primaries, target_wp).inverse() * adapt * rgb_to_xyz(s.primaries, s.whitepoint));
    op.u0 = method;
    return c.push(op);
}

uint32_t cmd_color_matrix(Command &c, uint32_t src, const float m[9]) {
    Op op{OpKind::ColorMatrix};
    op.a = src;
    op.desc = c.describe(src);
    op.desc.row_stride = 0;
    Mat3 mm{};
    for (int i = 0; i < 9; ++i) mm.m[i] = m[i];
    op.prog.mat(mm);
    return c.push(op);
}

static int channel_index(uint32_t ch) { return ch <= 3 ? (int)ch : -1; }

uint32_t cmd_extract(Command &c, uint32_t src, uint32_t channel) {
    const Desc s = c.describe(src);
    if (channel > 3) fail(ZS_ERR_OTHER, "unsupported channel");
    // command.rs:1221-1268: Texel::channel_texel keeps the bits and selects the part.
    if (channel_count_parts(s.parts) < 3 && !(s.parts == ZS_PARTS_LUMAA && channel == 3))
        fail(ZS_ERR_OTHER, "channel not present in texel");
    static const uint32_t parts[4] = {ZS_PARTS_R, ZS_PARTS_G, ZS_PARTS_B, ZS_PARTS_A};
    Op op{OpKind::Extract};
    op.a = src;
    op.desc = s;
    op.desc.parts = parts[channel];
    op.desc.row_stride = 0;
    op.u0 = channel;
    return c.push(op);
}

uint32_t cmd_inject(Command &c, uint32_t below, uint32_t channel, uint32_t above) {
    const Desc b = c.describe(below), a = c.describe(above);
    if (channel > 2) fail(ZS_ERR_OTHER, "inject supports R, G, B");      // ChannelPosition::new
    if (b.width != a.width || b.height != a.height) fail(ZS_ERR_TYPE, "inject operands differ in size");
    if (channel_count_parts(a.parts) != 1) fail(ZS_ERR_TYPE, "inject needs a single-channel operand");
    Op op{OpKind::Inject};
    op.a = below;
    op.b = above;
    op.u0 = channel;
    op.desc = b;
    op.desc.row_stride = 0;
    HInstr i;
    i.op = ZS_P_INJECT;
    i.v[channel_index(channel)] = 1.0;                 // select
    int w = a.parts == ZS_PARTS_R ? 0 : a.parts == ZS_PARTS_G ? 1 : a.parts == ZS_PARTS_B ? 2 :
            a.parts == ZS_PARTS_A ? 3 : 0;             // channel_weight_vec4 (buffer.rs)
    i.v[4 + w] = 1.0;
    op.prog.ins.push_back(i);
    return c.push(op);
}

uint32_t cmd_transmute(Command &c, uint32_t src, const Desc &target) {
    const Desc s = c.describe(src);
    Desc d = target;
    if (d.width != s.width || d.height != s.height) fail(ZS_ERR_TYPE, "invalid transmute with mismatched size");
    if (texel_bytes(d.bits) != texel_bytes(s.bits)) fail(ZS_ERR_TYPE, "transmute needs texels of equal size");
    d.row_stride = 0;
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "invalid transmute with inconsistent result");
    Op op{OpKind::Transmute};
    op.a = src;
    op.desc = d;
    return c.push(op);
}

static void check_inside(const Desc &below, const zs_rect &r) {
    if (r.x > r.max_x || r.y > r.max_y || r.max_x > below.width || r.max_y > below.height)
        fail(ZS_ERR_OTHER, "placement outside of the image");
}

uint32_t cmd_inscribe(Command &c, uint32_t below, const zs_rect &rect, uint32_t above, bool placed) {
    const Desc b = c.describe(below), a = c.describe(above);
    if (!same_chroma(a, b)) fail(ZS_ERR_TYPE, "inscribe needs equal texel and colour");
    if (!placed) {
        // command.rs:1196-1198: the placement must equal the upper image's rectangle.
        if (!(rect.x == 0 && rect.y == 0 && rect.max_x == a.width && rect.max_y == a.height))
            fail(ZS_ERR_OTHER, "inscribe placement must be the upper image's rectangle");
    } else if (rect.max_x - rect.x != a.width || rect.max_y - rect.y != a.height) {
        fail(ZS_ERR_OTHER, "placement size must equal the upper image size");
    }
    check_inside(b, rect);
    Op op{placed ? OpKind::InscribePlaced : OpKind::Inscribe};
    op.a = below;
    op.b = above;
    op.desc = b;
    op.desc.row_stride = 0;
    op.rect = rect;
    if (!placed) {
        // Rectangle::normalize (command.rs:3536-3543) sets max_y = y + width.
        op.rect.max_y = rect.y + (rect.max_x > rect.x ? rect.max_x - rect.x : 0);
    }
    return c.push(op);
}

uint32_t cmd_palette(Command &c, uint32_t palette, int32_t wch, int32_t hch, uint32_t indices) {
    const Desc lhs = c.describe(palette), rhs = c.describe(indices);
    if (wch > 2 || hch > 2) fail(ZS_ERR_TYPE, "palette coordinate channel must be R, G or B");
    Op op{OpKind::Palette};
    op.a = palette;
    op.b = indices;
    op.desc = with_size(lhs, rhs.width, rhs.height);   // command.rs:1468-1472
    op.i0 = wch;
    op.i1 = hch;
    if (wch >= 0) op.fparams[wch] = 1.0f;
    if (hch >= 0) op.fparams[4 + hch] = 1.0f;
    return c.push(op);
}

uint32_t cmd_bilinear(Command &c, const Desc &d, const float params[24]) {
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent descriptor for bilinear");
    Op op{OpKind::Bilinear};
    op.desc = d;
    op.desc.row_stride = 0;
    std::memcpy(op.fparams, params, sizeof(float) * 24);
    return c.push(op);
}

uint32_t cmd_solid(Command &c, const Desc &d, const float color[4]) {
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent constant color image created");
    Op op{OpKind::Solid};
    op.desc = d;
    op.desc.row_stride = 0;
    std::memcpy(op.fparams, color, sizeof(float) * 4);
    return c.push(op);
}

uint32_t cmd_affine(Command &c, uint32_t below, const float m[9], uint32_t sampling, uint32_t above) {
    const Desc b = c.describe(below), a = c.describe(above);
    if (!same_chroma(a, b)) fail(ZS_ERR_TYPE, "affine needs equal texel and colour");
    // command.rs:1648-1656: |det| must be at least f32::EPSILON.
    double det = (double)m[0] * ((double)m[4] * m[8] - (double)m[5] * m[7]) -
                 (double)m[1] * ((double)m[3] * m[8] - (double)m[5] * m[6]) +
                 (double)m[2] * ((double)m[3] * m[7] - (double)m[4] * m[6]);
    if (!(std::fabs(det) >= 1.1920929e-07)) fail(ZS_ERR_OTHER, "degenerate affine transformation");
    if (sampling > 1) fail(ZS_ERR_INVALID_ARG, "unknown affine sampling");
    Op op{OpKind::Affine};
    op.a = below;
    op.b = above;
    op.desc = b;
    op.desc.row_stride = 0;
    std::memcpy(op.fparams, m, sizeof(float) * 9);
    op.u0 = sampling;
    return c.push(op);
}

// CommandBuffer::distribution_normal2d: a generator with the descriptor given.
uint32_t cmd_normal2d(Command &c, const Desc &d, const float params[7]) {
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent descriptor: " + describe(d));
    Op op{OpKind::Normal2d};
    op.desc = d;
    op.desc.row_stride = 0;
    for (int k = 0; k < 7; ++k) op.fparams[k] = params[k];
    return c.push(op);
}

// CommandBuffer::distribution_fractal_noise (command.rs:1585-1606): a generator with the
// descriptor given; params = [grid_scale x, grid_scale y, initial_amplitude,
// amplitude_damping, num_octaves].  The octave count is capped at 32: past it the grid
// coordinates have grown by 2^32 and carry no fractional bits in f32.
uint32_t cmd_fractal_noise(Command &c, const Desc &d, const float params[5]) {
    if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent descriptor for fractal noise: " + describe(d));
    const float n = params[4];
    if (!(n >= 0.f && n <= 32.f) || n != std::floor(n)) fail(ZS_ERR_INVALID_ARG, "num_octaves must be an integer in [0, 32]");
    Op op{OpKind::FractalNoise};
    op.desc = d;
    op.desc.row_stride = 0;
    for (int k = 0; k < 5; ++k) op.fparams[k] = params[k];
    return c.push(op);
}

// FractalNoise::with_octaves (shaders/fractal_noise.rs:20-31): damping 1, amplitude
// 1 / n (computed in f64, rounded to f32), grid 100 x 100.
void fractal_noise_with_octaves(uint32_t octaves, float p[5]) {
    p[0] = 100.f;
    p[1] = 100.f;
    p[2] = (float)(1.0 / (double)octaves);
    p[3] = 1.f;
    p[4] = (float)octaves;
}

// FractalNoise::set_damping (shaders/fractal_noise.rs:33-49): the initial amplitude is chosen
// so that the amplitudes of all octaves sum to 1, in f32.
void fractal_noise_set_damping(float p[5], float damping) {
    const float n = (float)(double)p[4];
    const float total = 1.0f - std::pow(damping, n);
    p[2] = std::fabs(total) < 1e-7f ? 1.0f : (1.0f - damping) / total;
    p[3] = damping;
}

// DistributionNormal2d::with_diagonal (shaders/distribution_normal2d.rs:24-38), in f32.
void normal2d_with_diagonal(float var0, float var1, float p[7]) {
    const float pi = 3.14159265358979323846f;
    const float d0 = var0 == 0.f ? 0.f : 1.f / var0, d1 = var1 == 0.f ? 0.f : 1.f / var1;
    const float f0 = var0 == 0.f ? 1.f : 2.f * pi * var0, f1 = var1 == 0.f ? 1.f : 2.f * pi * var1;
    const float out[7] = {0.f, 0.f, d0, 0.f, 0.f, d1, f0 * f1};
    for (int k = 0; k < 7; ++k) p[k] = out[k];
}

// DistributionNormal2d::with_direction (shaders/distribution_normal2d.rs:40-94): the pseudo
// inverse dir^T dir / |dir|^4 through the reference's reformulated f32 expressions.
void normal2d_with_direction(float x, float y, float p[7]) {
    const double xt = x, yt = y;
    const float length_sq = (float)(xt * xt + yt * yt);
    if (!std::isfinite(length_sq)) fail(ZS_ERR_INVALID_ARG, "direction length is not finite");
    auto symmetric = [](float a, float b) {
        const float hyp = std::hypot(a, b);
        const float up = (1.0f / hyp) * (a / hyp);
        const float low = a + b * (b / a);
        return up / low;
    };
    auto asymmetric = [](float a, float b) {
        const float lo = std::min(a, b), hi = std::max(a, b);
        const float hyp = std::hypot(lo, hi);
        const float inner = std::fma(lo, lo / hi, hi);
        return ((lo / hyp) / inner) / hyp;
    };
    const float pi = 3.14159265358979323846f;
    const float out[7] = {0.f, 0.f, symmetric(x, x), asymmetric(x, y), asymmetric(y, x), symmetric(y, y),
                          2.0f * pi * length_sq};
    for (int k = 0; k < 7; ++k) p[k] = out[k];
}

// CommandBuffer::derivative (command.rs:1493-1507) with the operator of
// DerivativeMethod::to_shader (command.rs:3343-3409): the f32 outer product of a smoothing
// and the derivative vector [0.5, 0, -0.5], transposed along the height.
uint32_t cmd_derivative(Command &c, uint32_t src, uint32_t method, uint32_t direction) {
    const Desc s = c.describe(src);
    if (method > 8) fail(ZS_ERR_INVALID_ARG, "unknown derivative method");
    if (direction > 1) fail(ZS_ERR_INVALID_ARG, "unknown derivative direction");
    static const float smooth[9][3] = {
        {0.f, 0.f, 0.f},                                    // Roberts (not yet implemented)
        {1.f / 3.f, 1.f / 3.f, 1.f / 3.f},                  // Prewitt
        {1.f / 4.f, 1.f / 2.f, 1.f / 4.f},                  // Sobel
        {46.84f / 256.f, 162.32f / 256.f, 46.84f / 256.f},  // Scharr3
        {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f},                   // Scharr4, Scharr5 (not yet implemented)
        {3.f / 16.f, 10.f / 16.f, 3.f / 16.f},              // Scharr3To4Bit
        {0.f, 0.f, 0.f},                                    // Scharr5Tab (not yet implemented)
        {47.f / 256.f, 162.f / 256.f, 47.f / 256.f},        // Scharr3To8Bit
    };
    const float d[3] = {0.5f, 0.0f, -0.5f};
    Op op{OpKind::Derivative};
    op.a = src;
    op.desc = s;
    op.desc.row_stride = 0;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            const float v = smooth[method][j] * d[i];          // row j, column i
            op.fparams[direction == 0 ? 3 * j + i : 3 * i + j] = v;
        }
    op.u0 = method;
    op.u1 = direction;
    return c.push(op);
}

uint32_t cmd_resize(Command &c, uint32_t src, uint32_t w, uint32_t h, bool filtered, uint32_t filter) {
    const Desc s = c.describe(src);
    if (w == 0 || h == 0) fail(ZS_ERR_OTHER, "empty resize");
    if (filtered && filter > 2) fail(ZS_ERR_INVALID_ARG, "unknown resize filter");
    Op op{filtered ? OpKind::ResizeFiltered : OpKind::Resize};
    op.a = src;
    op.desc = with_size(s, w, h);
    op.u0 = filter;
    return c.push(op);
}

uint32_t cmd_blend(Command &c, uint32_t below, const zs_rect &rect, uint32_t above, uint32_t mode) {
    const Desc b = c.describe(below), a = c.describe(above);
    if (!same_chroma(a, b)) fail(ZS_ERR_TYPE, "blend needs equal texel and colour");
    if (mode > 3) fail(ZS_ERR_INVALID_ARG, "unknown blend mode");
    Op op{OpKind::Blend};
    op.a = below;
    op.b = above;
    op.desc = b;
    op.desc.row_stride = 0;
    op.rect = rect;
    op.u0 = mode;
    return c.push(op);
}

uint32_t cmd_output(Command &c, uint32_t src, Desc *outformat) {
    const Desc s = c.describe(src);
    Op op{OpKind::Output};
    op.a = src;
    op.desc = s;
    op.desc.row_stride = 0;
    if (outformat) *outformat = op.desc;
    return c.push(op);
}

}  // namespace zs
