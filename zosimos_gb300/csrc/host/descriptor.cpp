// descriptor.cpp -- descriptors, storage formats, colour matrices and the host-side
// pixel program (with FP64 matrix folding).
//
// Storage formats follow ImageDescriptor::new (lib/zosimos/src/program.rs:781-946):
// RGBA8/BGRA8 with sRGB or linear transfer are native (round-to-nearest) formats,
// every other texel of an RGB/Scalars colour is "staged" (stage.frag mux/demux with
// truncating quantisation), Oklab/SrLab2 use LchA (LabLch transfer) or LabA.
// Colour matrices follow command.rs:1009-1085, 2527-2548, 3220-3340 with FP64
// arithmetic and the published primaries / white points.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>

#include "zs_host.hpp"

namespace zs {

static thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

[[noreturn]] void fail(int code, const std::string &msg) { throw Error{code, msg}; }

void check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return;
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) fail(ZS_ERR_OUT_OF_MEMORY, std::string(what) + ": out of device memory");
    fail(ZS_ERR_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------- texel vocabulary

uint32_t texel_bytes(uint32_t bits) {
    static const uint32_t b[20] = {1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 4, 4, 6, 8, 4, 4, 4, 4, 8, 16};
    return bits < 20 ? b[bits] : 0;
}

uint32_t channel_count_bits(uint32_t bits) {
    static const uint32_t c[20] = {1, 3, 3, 1, 4, 3, 3, 3, 2, 3, 4, 2, 3, 4, 4, 4, 3, 3, 4, 4};
    return bits < 20 ? c[bits] : 0;
}

uint32_t channel_count_parts(uint32_t parts) {
    static const uint32_t c[21] = {1, 1, 1, 1, 1, 2, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 3, 3, 4, 3, 4};
    return parts < 21 ? c[parts] : 0;
}

bool is_consistent(const Desc &d) {
    if (d.width == 0 || d.height == 0) return false;
    if (d.bits >= 20 || d.parts > 20 || d.color > ZS_COLOR_SCALARS) return false;
    if (d.bits == ZS_BITS_UINT16X3) return false;       // 6-byte texels are not staged anywhere
    uint32_t bpp = texel_bytes(d.bits);
    if (d.row_stride != 0 && d.row_stride < (uint64_t)d.width * bpp) return false;
    // A texel's bit layout has to carry the parts it declares (1 channel in 1..4 slots ok).
    uint32_t pc = channel_count_parts(d.parts), bc = channel_count_bits(d.bits);
    if (pc > bc && !(pc == 1)) return false;
    if (d.color == ZS_COLOR_OKLAB || d.color == ZS_COLOR_SRLAB2) {
        if (d.parts != ZS_PARTS_LCHA && d.parts != ZS_PARTS_LABA) return false;
    }
    if (d.color == ZS_COLOR_RGB && (d.primaries > ZS_PRIMARIES_XYZ || d.whitepoint > ZS_WP_F11)) return false;
    if (d.transfer > ZS_TRANSFER_LINEAR_SCENE) return false;
    return true;
}

uint64_t row_bytes(const Desc &d) { return (uint64_t)d.width * texel_bytes(d.bits); }
uint64_t host_stride(const Desc &d) { return d.row_stride ? d.row_stride : row_bytes(d); }
uint64_t host_len(const Desc &d) { return host_stride(d) * d.height; }

bool same_chroma(const Desc &a, const Desc &b) {
    if (a.bits != b.bits || a.parts != b.parts || a.color != b.color) return false;
    if (a.color == ZS_COLOR_RGB)
        return a.primaries == b.primaries && a.transfer == b.transfer && a.whitepoint == b.whitepoint;
    if (a.color == ZS_COLOR_SRLAB2) return a.whitepoint == b.whitepoint;
    if (a.color == ZS_COLOR_SCALARS) return a.transfer == b.transfer;
    return true;
}

// The stage.frag texel code of a SampleBits value (ShaderData::serialize_bits,
// lib/zosimos/src/shaders/stage.rs:98-118).  It maps UInt1010102 to stage.frag's Int2101010
// layout (three 10-bit samples from bit 0, 2-bit alpha at bits 30-31) and UInt2101010 to
// Int1010102 (2-bit first sample at bit 0): the SampleBits names list samples from bit 0,
// stage.frag's names from the top.  Every other code is the same number.
static uint8_t stage_bits(uint32_t bits) {
    if (bits == ZS_BITS_UINT1010102) return 15;
    if (bits == ZS_BITS_UINT2101010) return 14;
    return (uint8_t)bits;
}

ZsFormat format_of(const Desc &d) {
    ZsFormat f{};
    f.bits = stage_bits(d.bits);
    f.parts = (uint8_t)d.parts;
    f.bpp = (uint8_t)texel_bytes(d.bits);
    f.native = 0;
    f.fast = ZS_FAST_GENERIC;
    if (d.color == ZS_COLOR_OKLAB || d.color == ZS_COLOR_SRLAB2) {
        f.transfer = d.parts == ZS_PARTS_LCHA ? 0x100 : ZS_TRANSFER_LINEAR;
    } else {
        f.transfer = (uint16_t)d.transfer;
    }
    const bool rgba_like = d.parts == ZS_PARTS_RGBA || d.parts == ZS_PARTS_LABA;
    if (d.bits == ZS_BITS_UINT8X4 && d.color == ZS_COLOR_RGB &&
        (d.parts == ZS_PARTS_RGBA || d.parts == ZS_PARTS_BGRA) &&
        (d.transfer == ZS_TRANSFER_SRGB || d.transfer == ZS_TRANSFER_LINEAR)) {
        f.native = 1;
        const bool srgb = d.transfer == ZS_TRANSFER_SRGB;
        if (d.parts == ZS_PARTS_RGBA) f.fast = srgb ? ZS_FAST_RGBA8_SRGB : ZS_FAST_RGBA8_UNORM;
        else f.fast = srgb ? ZS_FAST_BGRA8_SRGB : ZS_FAST_BGRA8_UNORM;
    } else if (d.bits == ZS_BITS_FLOAT16X4 && rgba_like && f.transfer == ZS_TRANSFER_LINEAR) {
        f.fast = ZS_FAST_F16X4;
    } else if (d.bits == ZS_BITS_FLOAT32X4 && rgba_like && f.transfer == ZS_TRANSFER_LINEAR) {
        f.fast = ZS_FAST_F32X4;
    }
    return f;
}

bool format_is_lossless_f32(const ZsFormat &f) { return f.fast == ZS_FAST_F32X4; }

bool format_equal(const ZsFormat &a, const ZsFormat &b) {
    return a.bits == b.bits && a.parts == b.parts && a.native == b.native && a.transfer == b.transfer;
}

ZsFormat linear_f32_format() {
    ZsFormat f{};
    f.bits = ZS_BITS_FLOAT32X4;
    f.parts = ZS_PARTS_RGBA;
    f.bpp = 16;
    f.transfer = ZS_TRANSFER_LINEAR;
    f.fast = ZS_FAST_F32X4;
    return f;
}

ZsFormat linear_f16_format() {
    ZsFormat f{};
    f.bits = ZS_BITS_FLOAT16X4;
    f.parts = ZS_PARTS_RGBA;
    f.bpp = 8;
    f.transfer = ZS_TRANSFER_LINEAR;
    f.fast = ZS_FAST_F16X4;
    return f;
}

std::string describe(const Desc &d) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "%ux%u bits=%u parts=%u color=%u prim=%u transfer=%u wp=%u", d.width, d.height,
                  d.bits, d.parts, d.color, d.primaries, d.transfer, d.whitepoint);
    return buf;
}

// ---------------------------------------------------------------- matrices

Mat3 Mat3::identity() { return Mat3{{1, 0, 0, 0, 1, 0, 0, 0, 1}}; }
Mat3 Mat3::diag(double a, double b, double c) { return Mat3{{a, 0, 0, 0, b, 0, 0, 0, c}}; }

Mat3 Mat3::operator*(const Mat3 &o) const {
    Mat3 r{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = m[3 * i] * o.m[j] + m[3 * i + 1] * o.m[3 + j] + m[3 * i + 2] * o.m[6 + j];
    return r;
}

Mat3 Mat3::inverse() const {
    const double *a = m;
    double c0 = a[4] * a[8] - a[5] * a[7], c1 = a[5] * a[6] - a[3] * a[8], c2 = a[3] * a[7] - a[4] * a[6];
    double det = a[0] * c0 + a[1] * c1 + a[2] * c2;
    if (det == 0.0) fail(ZS_ERR_OTHER, "singular matrix");
    Mat3 r{{c0, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4], c1, a[0] * a[8] - a[2] * a[6],
            a[2] * a[3] - a[0] * a[5], c2, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]}};
    for (double &v : r.m) v /= det;
    return r;
}

bool Mat3::is_identity(double tol) const {
    static const double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < 9; ++i)
        if (std::fabs(m[i] - id[i]) > tol) return false;
    return true;
}

// Ottosson's Oklab matrices (lib/std/src/oklab.frag:14-24), as rows.
const Mat3 kOklabM1{{0.8189330101, 0.3618667424, -0.1288597137, 0.0329845436, 0.9293118715, 0.0361456387,
                     0.0482003018, 0.2643662691, 0.6338517070}};
const Mat3 kOklabM2{{0.2104542553, 0.7936177850, -0.0040720468, 1.9779984951, -2.4285922050, 0.4505937099,
                     0.0259040371, 0.7827717662, -0.8086757660}};
// CIECAM02 CAT02 and Hunt-Pointer-Estevez (lib/std/src/srlab2.frag:14-24), as rows.
const Mat3 kCat02{{0.7328, 0.4296, -0.1624, -0.7036, 1.6975, 0.0061, 0.0030, 0.0136, 0.9834}};
const Mat3 kHpe{{0.38971, 0.68898, -0.07868, -0.22981, 1.18340, 0.04641, 0.0, 0.0, 1.0}};

// White points as XYZ with Y = 1 (order A, B, C, D50, D55, D65, D75, E, F2, F7, F11).
static const double kWhite[11][3] = {
    {1.09850, 1.0, 0.35585}, {0.99072, 1.0, 0.85223}, {0.98074, 1.0, 1.18232}, {0.96422, 1.0, 0.82521},
    {0.95682, 1.0, 0.92149}, {0.95047, 1.0, 1.08883}, {0.94972, 1.0, 1.22638}, {1.00000, 1.0, 1.00000},
    {0.99186, 1.0, 0.67393}, {0.95041, 1.0, 1.08747}, {1.00962, 1.0, 0.64350}};

void whitepoint_xyz(uint32_t wp, double out[3]) {
    if (wp > 10) wp = ZS_WP_D65;
    for (int i = 0; i < 3; ++i) out[i] = kWhite[wp][i];
}

// CIE xy chromaticities of R, G, B per primaries code.
static const double kPrim[8][6] = {
    {0.630, 0.340, 0.310, 0.595, 0.155, 0.070}, {0.640, 0.330, 0.290, 0.600, 0.150, 0.060},
    {0.640, 0.330, 0.300, 0.600, 0.150, 0.060}, {0.630, 0.340, 0.310, 0.595, 0.155, 0.070},
    {0.708, 0.292, 0.170, 0.797, 0.131, 0.046}, {0.708, 0.292, 0.170, 0.797, 0.131, 0.046},
    {0.680, 0.320, 0.265, 0.690, 0.150, 0.060}, {0.640, 0.330, 0.210, 0.710, 0.150, 0.060}};

Mat3 rgb_to_xyz(uint32_t primaries, uint32_t whitepoint) {
    if (primaries >= 8) return Mat3::identity();   // CIE XYZ "primaries"
    const double *p = kPrim[primaries];
    Mat3 P{};
    for (int c = 0; c < 3; ++c) {
        double x = p[2 * c], y = p[2 * c + 1];
        P.m[c] = x / y;
        P.m[3 + c] = 1.0;
        P.m[6 + c] = (1.0 - x - y) / y;
    }
    double w[3];
    whitepoint_xyz(whitepoint, w);
    Mat3 Pi = P.inverse();
    double s[3];
    for (int i = 0; i < 3; ++i) s[i] = Pi.m[3 * i] * w[0] + Pi.m[3 * i + 1] * w[1] + Pi.m[3 * i + 2] * w[2];
    Mat3 r{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[3 * i + j] = P.m[3 * i + j] * s[j];
    return r;
}

// palette 0.7.6 generate_transform_matrix restated: M^-1 diag(M w_dst / M w_src) M.
bool adaptation_matrix(uint32_t method, uint32_t src_wp, uint32_t dst_wp, Mat3 &out) {
    static const Mat3 bradford{{0.8951, 0.2664, -0.1614, -0.7502, 1.7135, 0.0367, 0.0389, -0.0685, 1.0296}};
    static const Mat3 vonkries{{0.40024, 0.7076, -0.08081, -0.2263, 1.16532, 0.0457, 0.0, 0.0, 0.91822}};
    Mat3 cone;
    switch (method) {
    case 0: cone = Mat3::identity(); break;
    case 1: cone = vonkries; break;
    case 2: cone = bradford; break;
    default: return false;       // BradfordNonLinear: NotYetImplemented (command.rs:3328-3332)
    }
    double ws[3], wd[3];
    whitepoint_xyz(src_wp, ws);
    whitepoint_xyz(dst_wp, wd);
    double rs[3], rd[3];
    for (int i = 0; i < 3; ++i) {
        rs[i] = cone.m[3 * i] * ws[0] + cone.m[3 * i + 1] * ws[1] + cone.m[3 * i + 2] * ws[2];
        rd[i] = cone.m[3 * i] * wd[0] + cone.m[3 * i + 1] * wd[1] + cone.m[3 * i + 2] * wd[2];
    }
    out = cone.inverse() * (Mat3::diag(rd[0] / rs[0], rd[1] / rs[1], rd[2] / rs[2]) * cone);
    return true;
}

// ---------------------------------------------------------------- host program

void HProgram::mat(const Mat3 &m) {
    HInstr i;
    i.op = ZS_P_MAT3;
    i.mat = m;
    ins.push_back(i);
}

void HProgram::op(uint8_t o) {
    HInstr i;
    i.op = o;
    ins.push_back(i);
}

void HProgram::quant(const ZsFormat &f) {
    HInstr i;
    i.op = ZS_P_QUANT;
    i.fa = f;
    ins.push_back(i);
}

void HProgram::optimise() {
    std::vector<HInstr> out;
    for (const HInstr &i : ins) {
        if (i.op == ZS_P_QUANT && format_is_lossless_f32(i.fa)) continue;
        // A value just decoded from (or quantised to) format f is representable in f:
        // quantising it again is at best a no-op and, for formats whose decode/encode
        // is not exactly invertible in FP32 (LabLch), would add error.
        if (i.op == ZS_P_QUANT && !out.empty() &&
            ((out.back().op == ZS_P_TRANSMUTE && format_equal(out.back().fb, i.fa)) ||
             (out.back().op == ZS_P_QUANT && format_equal(out.back().fa, i.fa))))
            continue;
        if (i.op == ZS_P_MAT3 && !out.empty() && out.back().op == ZS_P_MAT3) {
            out.back().mat = i.mat * out.back().mat;     // later matrix applied after: M2 * M1
            continue;
        }
        out.push_back(i);
    }
    std::vector<HInstr> res;
    for (const HInstr &i : out)
        if (!(i.op == ZS_P_MAT3 && i.mat.is_identity())) res.push_back(i);
    ins.swap(res);
}

}  // namespace zs
