// capi.cpp -- the extern "C" boundary (include/zosimos.h).  Every entry point catches
// the internal error type and returns a status code; zs_last_error() holds the text.
#include <cstring>
#include <mutex>
#include <exception>
#include <string>

#include "zs_host.hpp"

namespace zs {
const std::string &last_error();
uint32_t cmd_input(Command &c, const Desc &d);
uint32_t cmd_crop(Command &c, uint32_t src, const zs_rect &r);
uint32_t cmd_color_convert(Command &c, uint32_t src, const Desc &target);
uint32_t cmd_chromatic_adaptation(Command &c, uint32_t src, uint32_t method, uint32_t target_wp);
uint32_t cmd_color_matrix(Command &c, uint32_t src, const float m[9]);
uint32_t cmd_extract(Command &c, uint32_t src, uint32_t channel);
uint32_t cmd_inject(Command &c, uint32_t below, uint32_t channel, uint32_t above);
uint32_t cmd_transmute(Command &c, uint32_t src, const Desc &target);
uint32_t cmd_inscribe(Command &c, uint32_t below, const zs_rect &rect, uint32_t above, bool placed);
uint32_t cmd_palette(Command &c, uint32_t palette, int32_t wch, int32_t hch, uint32_t indices);
uint32_t cmd_bilinear(Command &c, const Desc &d, const float params[24]);
uint32_t cmd_solid(Command &c, const Desc &d, const float color[4]);
uint32_t cmd_affine(Command &c, uint32_t below, const float m[9], uint32_t sampling, uint32_t above);
uint32_t cmd_resize(Command &c, uint32_t src, uint32_t w, uint32_t h, bool filtered, uint32_t filter);
uint32_t cmd_blend(Command &c, uint32_t below, const zs_rect &rect, uint32_t above, uint32_t mode);
uint32_t cmd_derivative(Command &c, uint32_t src, uint32_t method, uint32_t direction);
uint32_t cmd_normal2d(Command &c, const Desc &d, const float params[7]);
void normal2d_with_diagonal(float var0, float var1, float p[7]);
void normal2d_with_direction(float x, float y, float p[7]);
uint32_t cmd_fractal_noise(Command &c, const Desc &d, const float params[5]);
uint32_t cmd_buffer_init(Command &c, const void *bytes, uint64_t n, uint64_t len);
uint32_t cmd_from_buffer(Command &c, uint32_t buffer, const Desc &target);
void fractal_noise_with_octaves(uint32_t octaves, float p[5]);
void fractal_noise_set_damping(float p[5], float damping);
uint32_t cmd_output(Command &c, uint32_t src, Desc *outformat);
uint32_t cmd_dynamic(Command &c, uint32_t nops, uint32_t a, uint32_t b, uint32_t op_id, const void *uniforms,
                     uint64_t len, const Desc &target);
int batch_thumbnails(Executable *chain, const void *const *images, const uint32_t *widths, const uint32_t *heights,
                     uint32_t n, uint32_t canvas, void *out, cudaStream_t stream);
}  // namespace zs

using namespace zs;

struct zs_pool { Pool p; };
struct zs_cmd { Command c; };
struct zs_program { Program p; };
#define ZS_BATCH_BRANCHES 8
struct zs_executable {
    std::unique_ptr<Executable> e;
    cudaStream_t stream = nullptr;
    cudaStream_t stripes[3] = {nullptr, nullptr, nullptr};   // striped host round trips
    // zs_batch_run_device: capture streams of the independent runs, fork / join events, and
    // the instantiated graphs per pointer table (bounded, oldest evicted first)
    cudaStream_t branches[ZS_BATCH_BRANCHES] = {};
    cudaEvent_t fork = nullptr, joins[ZS_BATCH_BRANCHES] = {};
    std::map<std::vector<void *>, cudaGraphExec_t> batch_graphs;
    std::vector<std::vector<void *>> batch_order;
    ~zs_executable();
};
struct zs_environment { Environment env; };
struct zs_execution { Execution x; std::vector<int> kinds; std::vector<int> args; };

zs_executable::~zs_executable() {
    for (auto &kv : batch_graphs) cudaGraphExecDestroy(kv.second);
    for (cudaStream_t t : branches)
        if (t) cudaStreamDestroy(t);
    for (cudaEvent_t ev : joins)
        if (ev) cudaEventDestroy(ev);
    if (fork) cudaEventDestroy(fork);
    if (stream) cudaStreamDestroy(stream);
    for (cudaStream_t t : stripes)
        if (t) cudaStreamDestroy(t);
}

// Registered custom operations (zs_register_op): loaded modules and their kernels.
namespace zs {
static std::mutex g_dyn_mutex;
static std::vector<std::pair<cudaLibrary_t, cudaKernel_t>> g_dyn;

void *dynamic_kernel(uint32_t op) {
    std::lock_guard<std::mutex> lock(g_dyn_mutex);
    return op < g_dyn.size() ? (void *)g_dyn[op].second : nullptr;
}
}  // namespace zs

static void note_graph_launch(const Executable &E) {
    uint64_t n = 0;
    for (const Step &st : E.steps)
        if (st.kind != StepKind::Copy) ++n;
    add_kernel_launches(n);
}

template <class F>
static int guarded(F &&f) {
    try {
        f();
        return ZS_OK;
    } catch (const Error &e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("out of host memory");
        return ZS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return ZS_ERR_OTHER;
    } catch (...) {
        set_last_error("unknown error");
        return ZS_ERR_OTHER;
    }
}

#define NEED(ptr)                                                  \
    do {                                                           \
        if (!(ptr)) fail(ZS_ERR_INVALID_ARG, #ptr " is null");     \
    } while (0)

// Command-building calls: a failed call also drops a pending with_knob / with_buffer, so that
// it cannot attach to a later, unrelated operation.
template <class F>
static int cmd_guarded(zs_cmd *cmd, F &&f) {
    const int rc = guarded(std::forward<F>(f));
    if (rc != ZS_OK && cmd) cmd->c.clear_pending();
    return rc;
}

extern "C" {

const char *zs_last_error(void) { return last_error().c_str(); }
const char *zs_version(void) { return "zosimos-gb300 0.1 (sm_103a)"; }

uint32_t zs_texel_bytes(uint32_t bits) { return texel_bytes(bits); }

int zs_descriptor_srgb_rgba8(uint32_t width, uint32_t height, zs_descriptor *out) {
    return guarded([&] {
        NEED(out);
        std::memset(out, 0, sizeof(*out));
        out->width = width;
        out->height = height;
        out->bits = ZS_BITS_UINT8X4;
        out->parts = ZS_PARTS_RGBA;
        out->color = ZS_COLOR_RGB;
        out->primaries = ZS_PRIMARIES_BT709;
        out->transfer = ZS_TRANSFER_SRGB;
        out->whitepoint = ZS_WP_D65;
    });
}

int zs_descriptor_is_consistent(const zs_descriptor *desc) { return desc && is_consistent(*desc) ? 1 : 0; }
uint64_t zs_descriptor_byte_len(const zs_descriptor *desc) { return desc ? host_len(*desc) : 0; }

// ---------------------------------------------------------------- pool

zs_pool *zs_pool_new(void) {
    try {
        return new zs_pool();
    } catch (...) {
        return nullptr;
    }
}
void zs_pool_free(zs_pool *pool) { delete pool; }

static uint64_t pool_add(Pool &p, const Desc &d) {
    auto img = std::make_unique<PoolImage>();
    img->desc = d;
    img->len = host_len(d);
    img->ensure_host();
    uint64_t key = p.next_key++;
    p.images[key] = std::move(img);
    return key;
}

int zs_pool_insert(zs_pool *pool, const zs_descriptor *desc, const void *bytes, uint64_t *key) {
    return guarded([&] {
        NEED(pool); NEED(desc); NEED(bytes); NEED(key);
        if (!is_consistent(*desc)) fail(ZS_ERR_TYPE, "inconsistent descriptor: " + describe(*desc));
        uint64_t k = pool_add(pool->p, *desc);
        PoolImage &img = pool->p.get(k);
        std::memcpy(img.host, bytes, img.len);
        *key = k;
    });
}

int zs_pool_declare(zs_pool *pool, const zs_descriptor *desc, uint64_t *key) {
    return guarded([&] {
        NEED(pool); NEED(desc); NEED(key);
        if (!is_consistent(*desc)) fail(ZS_ERR_TYPE, "inconsistent descriptor: " + describe(*desc));
        uint64_t k = pool_add(pool->p, *desc);
        std::memset(pool->p.get(k).host, 0, pool->p.get(k).len);
        *key = k;
    });
}

int zs_pool_descriptor(zs_pool *pool, uint64_t key, zs_descriptor *out) {
    return guarded([&] {
        NEED(pool); NEED(out);
        *out = pool->p.get(key).desc;
    });
}

static void pool_sync_host(PoolImage &img) {
    if (img.host_valid) return;
    if (!img.dev_valid) fail(ZS_ERR_OTHER, "image has no contents");
    check_cuda(cudaMemcpy2D(img.host, host_stride(img.desc), img.dev, row_bytes(img.desc), row_bytes(img.desc),
                            img.desc.height, cudaMemcpyDeviceToHost),
               "download");
    img.host_valid = true;
}

int zs_pool_read(zs_pool *pool, uint64_t key, void *dst, uint64_t len) {
    return guarded([&] {
        NEED(pool); NEED(dst);
        PoolImage &img = pool->p.get(key);
        if (len != img.len) fail(ZS_ERR_INVALID_ARG, "length mismatch");
        pool_sync_host(img);
        std::memcpy(dst, img.host, len);
    });
}

int zs_pool_write(zs_pool *pool, uint64_t key, const void *src, uint64_t len) {
    return guarded([&] {
        NEED(pool); NEED(src);
        PoolImage &img = pool->p.get(key);
        if (len != img.len) fail(ZS_ERR_INVALID_ARG, "length mismatch");
        std::memcpy(img.host, src, len);
        img.host_valid = true;
        img.dev_valid = false;
    });
}

int zs_pool_host_ptr(zs_pool *pool, uint64_t key, void **ptr, uint64_t *len) {
    return guarded([&] {
        NEED(pool); NEED(ptr);
        PoolImage &img = pool->p.get(key);
        pool_sync_host(img);
        img.dev_valid = false;   // the caller may write through the pointer
        *ptr = img.host;
        if (len) *len = img.len;
    });
}

int zs_pool_set_descriptor(zs_pool *pool, uint64_t key, const zs_descriptor *desc) {
    return guarded([&] {
        NEED(pool); NEED(desc);
        PoolImage &img = pool->p.get(key);
        if (!is_consistent(*desc)) fail(ZS_ERR_TYPE, "inconsistent descriptor");
        if (host_len(*desc) != img.len || desc->width != img.desc.width || desc->height != img.desc.height)
            fail(ZS_ERR_TYPE, "descriptor must keep the byte layout");
        img.desc = *desc;
    });
}

static void pool_upload(PoolImage &img) {
    const uint64_t tight = row_bytes(img.desc) * img.desc.height;
    if (!img.dev) {
        check_cuda(cudaMalloc(&img.dev, tight), "cudaMalloc");
        img.dev_len = tight;
    }
    if (!img.dev_valid) {
        check_cuda(cudaMemcpy2D(img.dev, row_bytes(img.desc), img.host, host_stride(img.desc), row_bytes(img.desc),
                                img.desc.height, cudaMemcpyHostToDevice),
                   "upload");
        img.dev_valid = true;
    }
}

int zs_pool_upload(zs_pool *pool, uint64_t key) {
    return guarded([&] {
        NEED(pool);
        pool_upload(pool->p.get(key));
    });
}

int zs_pool_device_ptr(zs_pool *pool, uint64_t key, void **ptr) {
    return guarded([&] {
        NEED(pool); NEED(ptr);
        PoolImage &img = pool->p.get(key);
        if (!img.dev_valid) fail(ZS_ERR_OTHER, "image is not device resident (zs_pool_upload)");
        *ptr = img.dev;
    });
}

int zs_pool_remove(zs_pool *pool, uint64_t key) {
    return guarded([&] {
        NEED(pool);
        if (!pool->p.images.erase(key)) fail(ZS_ERR_MISSING_KEY, "no image with this key");
    });
}

int zs_pool_clear_cache(zs_pool *pool) {
    return guarded([&] {
        NEED(pool);
        for (auto &kv : pool->p.images) {
            PoolImage &img = *kv.second;
            if (img.dev && img.host_valid) {
                cudaFree(img.dev);
                img.dev = nullptr;
                img.dev_valid = false;
            }
        }
    });
}

// ---------------------------------------------------------------- command buffer

zs_cmd *zs_cmd_new(void) {
    try {
        return new zs_cmd();
    } catch (...) {
        return nullptr;
    }
}
void zs_cmd_free(zs_cmd *cmd) { delete cmd; }

#define CMD_BODY(expr)                 \
    return guarded([&] {               \
        NEED(cmd);                     \
        NEED(reg);                     \
        *reg = (expr);                 \
    })

int zs_cmd_input(zs_cmd *cmd, const zs_descriptor *desc, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(desc); NEED(reg); *reg = cmd_input(cmd->c, *desc); });
}
int zs_cmd_crop(zs_cmd *cmd, uint32_t src, const zs_rect *rect, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(rect); NEED(reg); *reg = cmd_crop(cmd->c, src, *rect); });
}
int zs_cmd_color_convert(zs_cmd *cmd, uint32_t src, const zs_descriptor *target, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(target); NEED(reg); *reg = cmd_color_convert(cmd->c, src, *target); });
}
int zs_cmd_chromatic_adaptation(zs_cmd *cmd, uint32_t src, uint32_t method, uint32_t target_wp, uint32_t *reg) {
    CMD_BODY(cmd_chromatic_adaptation(cmd->c, src, method, target_wp));
}
int zs_cmd_inscribe(zs_cmd *cmd, uint32_t below, const zs_rect *rect, uint32_t above, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(rect); NEED(reg); *reg = cmd_inscribe(cmd->c, below, *rect, above, false); });
}
int zs_cmd_inscribe_placed(zs_cmd *cmd, uint32_t below, const zs_rect *rect, uint32_t above, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(rect); NEED(reg); *reg = cmd_inscribe(cmd->c, below, *rect, above, true); });
}
int zs_cmd_extract(zs_cmd *cmd, uint32_t src, uint32_t channel, uint32_t *reg) {
    CMD_BODY(cmd_extract(cmd->c, src, channel));
}
int zs_cmd_inject(zs_cmd *cmd, uint32_t below, uint32_t channel, uint32_t above, uint32_t *reg) {
    CMD_BODY(cmd_inject(cmd->c, below, channel, above));
}
int zs_cmd_transmute(zs_cmd *cmd, uint32_t src, const zs_descriptor *target, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(target); NEED(reg); *reg = cmd_transmute(cmd->c, src, *target); });
}
int zs_cmd_palette(zs_cmd *cmd, uint32_t palette, int32_t wch, int32_t hch, uint32_t indices, uint32_t *reg) {
    CMD_BODY(cmd_palette(cmd->c, palette, wch, hch, indices));
}
int zs_cmd_bilinear(zs_cmd *cmd, const zs_descriptor *desc, const float params[24], uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(desc); NEED(params); NEED(reg); *reg = cmd_bilinear(cmd->c, *desc, params); });
}
int zs_cmd_solid_rgba(zs_cmd *cmd, const zs_descriptor *desc, const float color[4], uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(desc); NEED(color); NEED(reg); *reg = cmd_solid(cmd->c, *desc, color); });
}
int zs_cmd_affine(zs_cmd *cmd, uint32_t below, const float matrix[9], uint32_t sampling, uint32_t above,
                  uint32_t *reg) {
    return cmd_guarded(cmd, [&] {
        NEED(cmd); NEED(matrix); NEED(reg);
        *reg = cmd_affine(cmd->c, below, matrix, sampling, above);
    });
}
int zs_cmd_resize(zs_cmd *cmd, uint32_t src, uint32_t width, uint32_t height, uint32_t *reg) {
    CMD_BODY(cmd_resize(cmd->c, src, width, height, false, 0));
}
int zs_cmd_resize_filtered(zs_cmd *cmd, uint32_t src, uint32_t width, uint32_t height, uint32_t filter,
                           uint32_t *reg) {
    CMD_BODY(cmd_resize(cmd->c, src, width, height, true, filter));
}
int zs_cmd_distribution_normal2d(zs_cmd *cmd, const zs_descriptor *desc, const float params[7], uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(desc); NEED(params); NEED(reg); *reg = cmd_normal2d(cmd->c, *desc, params); });
}
int zs_normal2d_with_diagonal(float var0, float var1, float params[7]) {
    return guarded([&] { NEED(params); normal2d_with_diagonal(var0, var1, params); });
}
int zs_normal2d_with_direction(float x, float y, float params[7]) {
    return guarded([&] { NEED(params); normal2d_with_direction(x, y, params); });
}
int zs_cmd_distribution_fractal_noise(zs_cmd *cmd, const zs_descriptor *desc, const float params[5], uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(desc); NEED(params); NEED(reg); *reg = cmd_fractal_noise(cmd->c, *desc, params); });
}
int zs_cmd_buffer_init(zs_cmd *cmd, const void *bytes, uint64_t len, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(reg); *reg = cmd_buffer_init(cmd->c, bytes, len, len); });
}
int zs_cmd_buffer_zero(zs_cmd *cmd, uint64_t len, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(reg); *reg = cmd_buffer_init(cmd->c, nullptr, 0, len); });
}
int zs_cmd_from_buffer(zs_cmd *cmd, uint32_t buffer, const zs_descriptor *desc, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(desc); NEED(reg); *reg = cmd_from_buffer(cmd->c, buffer, *desc); });
}
int zs_fractal_noise_with_octaves(uint32_t num_octaves, float params[5]) {
    return guarded([&] { NEED(params); fractal_noise_with_octaves(num_octaves, params); });
}
int zs_fractal_noise_set_damping(float params[5], float damping) {
    return guarded([&] { NEED(params); fractal_noise_set_damping(params, damping); });
}
int zs_cmd_derivative(zs_cmd *cmd, uint32_t src, uint32_t method, uint32_t direction, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(reg); *reg = cmd_derivative(cmd->c, src, method, direction); });
}
int zs_cmd_blend(zs_cmd *cmd, uint32_t below, const zs_rect *rect, uint32_t above, uint32_t mode, uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(rect); NEED(reg); *reg = cmd_blend(cmd->c, below, *rect, above, mode); });
}
int zs_cmd_color_matrix(zs_cmd *cmd, uint32_t src, const float matrix[9], uint32_t *reg) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(matrix); NEED(reg); *reg = cmd_color_matrix(cmd->c, src, matrix); });
}
int zs_cmd_output(zs_cmd *cmd, uint32_t src, uint32_t *reg, zs_descriptor *outformat) {
    return cmd_guarded(cmd, [&] { NEED(cmd); NEED(reg); *reg = cmd_output(cmd->c, src, outformat); });
}
int zs_cmd_with_knob(zs_cmd *cmd) {
    return guarded([&] {
        NEED(cmd);
        cmd->c.pending_knob = true;
    });
}

int zs_cmd_with_buffer(zs_cmd *cmd, uint32_t buffer) {
    return guarded([&] {
        NEED(cmd);
        if (buffer >= cmd->c.ops.size()) fail(ZS_ERR_BAD_REGISTER, "no such register");
        if (cmd->c.ops[buffer].kind != OpKind::BufferInit) fail(ZS_ERR_TYPE, "register is not a buffer");
        cmd->c.pending_buffer = (int32_t)buffer;
    });
}

int zs_cmd_generic(zs_cmd *cmd, uint32_t *ty) {
    return guarded([&] {
        NEED(cmd); NEED(ty);
        TyVar t;
        t.var = cmd->c.nvars++;
        cmd->c.tys.push_back(t);
        *ty = (uint32_t)cmd->c.tys.size() - 1;
    });
}

int zs_cmd_input_generic(zs_cmd *cmd, uint32_t ty, uint32_t *reg) {
    return cmd_guarded(cmd, [&] {
        NEED(cmd); NEED(reg);
        if (ty >= cmd->c.tys.size()) fail(ZS_ERR_BAD_REGISTER, "no such descriptor variable");
        Op op{OpKind::Input};
        op.desc = ty_descriptor(cmd->c, ty);
        op.generic_var = (int32_t)ty;
        *reg = cmd->c.push(op);
    });
}

int zs_cmd_derive_descriptor(zs_cmd *cmd, uint32_t base, uint32_t width, uint32_t height, uint32_t *ty) {
    return guarded([&] {
        NEED(cmd); NEED(ty);
        if (base >= cmd->c.tys.size()) fail(ZS_ERR_BAD_REGISTER, "no such descriptor variable");
        if ((width == 0) != (height == 0)) fail(ZS_ERR_INVALID_ARG, "give both sides of the size or neither");
        TyVar t;
        t.base = (int32_t)base;
        t.width = width;
        t.height = height;
        cmd->c.tys.push_back(t);
        *ty = (uint32_t)cmd->c.tys.size() - 1;
    });
}

int zs_cmd_register_descriptor(zs_cmd *cmd, uint32_t reg, uint32_t *ty) {
    return guarded([&] {
        NEED(cmd); NEED(ty);
        cmd->c.describe(reg);
        TyVar t;
        t.reg = (int32_t)reg;
        cmd->c.tys.push_back(t);
        *ty = (uint32_t)cmd->c.tys.size() - 1;
    });
}

int zs_cmd_signature(const zs_cmd *cmd, uint32_t *n_generics, uint32_t *n_inputs, uint32_t *n_outputs) {
    return guarded([&] {
        NEED(cmd);
        uint32_t ni = 0, no = 0;
        for (const Op &op : cmd->c.ops) {
            ni += op.kind == OpKind::Input;
            no += op.kind == OpKind::Output;
        }
        if (n_generics) *n_generics = (uint32_t)cmd->c.nvars;
        if (n_inputs) *n_inputs = ni;
        if (n_outputs) *n_outputs = no;
    });
}

int zs_cmd_function(zs_cmd *cmd, const zs_cmd *signature, uint32_t *function) {
    return guarded([&] {
        NEED(cmd); NEED(signature); NEED(function);
        if (signature == cmd) fail(ZS_ERR_OTHER, "a command buffer cannot declare itself");
        cmd->c.functions.push_back(std::make_shared<const Command>(signature->c));
        *function = (uint32_t)cmd->c.functions.size() - 1;
    });
}

int zs_cmd_invoke(zs_cmd *cmd, uint32_t function, const uint32_t *generics, uint32_t n_generics, const uint32_t *args,
                  uint32_t n_args, uint32_t *results, uint32_t n_results) {
    return cmd_guarded(cmd, [&] {
        NEED(cmd);
        if (n_generics) NEED(generics);
        if (n_args) NEED(args);
        std::vector<uint32_t> tys(generics, generics + n_generics), as(args, args + n_args);
        // Check the result count before recording the call.
        if (function < cmd->c.functions.size()) {
            uint32_t no = 0;
            for (const Op &op : cmd->c.functions[function]->ops) no += op.kind == OpKind::Output;
            if (no != n_results) fail(ZS_ERR_OTHER, "wrong number of result registers");
            if (no) NEED(results);
        }
        const std::vector<uint32_t> res = cmd_invoke(cmd->c, function, tys, as);
        for (size_t k = 0; k < res.size(); ++k) results[k] = res[k];
    });
}

int zs_register_op(const void *image, uint64_t len, const char *kernel_name, uint32_t *op) {
    return guarded([&] {
        NEED(image); NEED(kernel_name); NEED(op);
        if (len == 0) fail(ZS_ERR_INVALID_ARG, "empty module image");
        cudaLibrary_t lib = nullptr;
        check_cuda(cudaLibraryLoadData(&lib, image, nullptr, nullptr, 0, nullptr, nullptr, 0), "module load");
        cudaKernel_t k = nullptr;
        const cudaError_t e = cudaLibraryGetKernel(&k, lib, kernel_name);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaLibraryUnload(lib);
            fail(ZS_ERR_INVALID_ARG, std::string("no kernel named ") + kernel_name + " in the module");
        }
        std::lock_guard<std::mutex> lock(g_dyn_mutex);
        g_dyn.emplace_back(lib, k);
        *op = (uint32_t)g_dyn.size() - 1;
    });
}

int zs_cmd_construct_dynamic(zs_cmd *cmd, uint32_t op, const void *uniforms, uint64_t len, const zs_descriptor *desc,
                             uint32_t *reg) {
    return cmd_guarded(cmd, [&] {
        NEED(cmd); NEED(desc); NEED(reg);
        *reg = cmd_dynamic(cmd->c, 0, 0, 0, op, uniforms, len, *desc);
    });
}

int zs_cmd_unary_dynamic(zs_cmd *cmd, uint32_t src, uint32_t op, const void *uniforms, uint64_t len,
                         const zs_descriptor *desc, uint32_t *reg) {
    return cmd_guarded(cmd, [&] {
        NEED(cmd); NEED(desc); NEED(reg);
        *reg = cmd_dynamic(cmd->c, 1, src, 0, op, uniforms, len, *desc);
    });
}

int zs_cmd_binary_dynamic(zs_cmd *cmd, uint32_t lhs, uint32_t rhs, uint32_t op, const void *uniforms, uint64_t len,
                          const zs_descriptor *desc, uint32_t *reg) {
    return cmd_guarded(cmd, [&] {
        NEED(cmd); NEED(desc); NEED(reg);
        *reg = cmd_dynamic(cmd->c, 2, lhs, rhs, op, uniforms, len, *desc);
    });
}

int zs_cmd_describe(const zs_cmd *cmd, uint32_t reg, zs_descriptor *out) {
    return guarded([&] { NEED(cmd); NEED(out); *out = cmd->c.describe(reg); });
}

// ---------------------------------------------------------------- compile / lower

int zs_compile(const zs_cmd *cmd, zs_program **out) {
    return guarded([&] {
        NEED(cmd); NEED(out);
        auto prog = std::make_unique<zs_program>();
        prog->p = compile_command(cmd->c);
        *out = prog.release();
    });
}

int zs_link(const zs_cmd *main, const zs_descriptor *tys, uint32_t n_tys, const zs_cmd *const *functions,
            uint32_t n_functions, const uint32_t *const *links, const uint32_t *link_counts, uint32_t n_links,
            zs_program **out) {
    return guarded([&] {
        NEED(main); NEED(out);
        std::vector<Desc> gen;
        for (uint32_t i = 0; i < n_tys; ++i) {
            NEED(tys);
            gen.push_back(tys[i]);
        }
        std::vector<const Command *> buffers{&main->c};
        for (uint32_t i = 0; i < n_functions; ++i) {
            NEED(functions); NEED(functions[i]);
            buffers.push_back(&functions[i]->c);
        }
        std::vector<std::vector<uint32_t>> table(n_links);
        for (uint32_t i = 0; i < n_links; ++i) {
            NEED(link_counts);
            if (link_counts[i]) {
                NEED(links); NEED(links[i]);
                table[i].assign(links[i], links[i] + link_counts[i]);
            }
        }
        auto prog = std::make_unique<zs_program>();
        prog->p = link_commands(buffers, gen, table);
        *out = prog.release();
    });
}
void zs_program_free(zs_program *program) { delete program; }

int zs_lower(const zs_program *program, const zs_capabilities *caps, zs_executable **out) {
    return guarded([&] {
        NEED(program); NEED(out);
        zs_capabilities c{};
        if (caps) c = *caps;
        auto exe = std::make_unique<zs_executable>();
        exe->e = lower(program->p, c);
        exe->e->alias = program->p.alias;
        *out = exe.release();
    });
}
void zs_executable_free(zs_executable *exe) { delete exe; }

int zs_executable_kernel_count(const zs_executable *exe, uint32_t *count) {
    return guarded([&] {
        NEED(exe); NEED(count);
        uint32_t n = 0;
        for (const Step &s : exe->e->steps)
            if (s.kind != StepKind::Copy) ++n;
        *count = n;
    });
}

int zs_executable_io_count(const zs_executable *exe, uint32_t *inputs, uint32_t *outputs) {
    return guarded([&] {
        NEED(exe);
        if (inputs) *inputs = (uint32_t)exe->e->input_regs.size();
        if (outputs) *outputs = (uint32_t)exe->e->output_regs.size();
    });
}

// A register of the linked command buffers (link index 0: the entry point) in the executable.
static uint32_t flat_reg(const Executable &E, uint32_t link_idx, uint32_t reg) {
    auto it = E.alias.find({link_idx, reg});
    if (it != E.alias.end()) return it->second;
    if (link_idx != 0) fail(ZS_ERR_BAD_REGISTER, "register of a linked function that was not instantiated");
    return reg;
}

int zs_executable_query_knob(const zs_executable *exe, uint32_t link_idx, uint32_t reg, uint32_t *knob,
                             uint64_t *len) {
    return guarded([&] {
        NEED(exe); NEED(knob);
        const Executable &E = *exe->e;
        reg = flat_reg(E, link_idx, reg);
        for (size_t i = 0; i < E.knobs.size(); ++i)
            if (E.knobs[i].reg == reg) {
                *knob = (uint32_t)i;
                if (len) *len = E.knobs[i].len;
                return;
            }
        fail(ZS_ERR_BAD_REGISTER, "register has no knob");
    });
}

int zs_executable_set_knob(zs_executable *exe, uint32_t knob, const void *data, uint64_t len) {
    return guarded([&] {
        NEED(exe); NEED(data);
        Executable &E = *exe->e;
        if (knob >= E.knobs.size()) fail(ZS_ERR_INVALID_ARG, "no such knob");
        const KnobInfo &K = E.knobs[knob];
        if (len != K.len) fail(ZS_ERR_INVALID_ARG, "knob data length differs from the knob's parameter block");
        const uint8_t *bytes = (const uint8_t *)data;
        for (const KnobSite &site : K.sites) {
            if (site.step >= 0) {
                const std::vector<float> c = knob_cons(site.kind, bytes, len);
                for (size_t i = 0; i < c.size(); ++i) E.steps[site.step].raster.cons[i] = c[i];
            } else {
                Slot &sl = E.slots[site.slot];
                std::memcpy(sl.table.data(), bytes, std::min<uint64_t>(len, sl.table.size()));
                if (!E.dev_buffers.empty() && E.dev_buffers[site.slot])
                    check_cuda(cudaMemcpy(E.dev_buffers[site.slot], sl.table.data(), sl.bytes, cudaMemcpyHostToDevice),
                               "knob upload");
            }
        }
        // Graphs captured the old parameters.
        for (auto &kv : E.graphs) cudaGraphExecDestroy(kv.second);
        E.graphs.clear();
        E.graph_order.clear();
        for (auto &kv : exe->batch_graphs) cudaGraphExecDestroy(kv.second);
        exe->batch_graphs.clear();
        exe->batch_order.clear();
    });
}

const char *zs_executable_describe(const zs_executable *exe) { return exe ? exe->e->plan_text.c_str() : ""; }

// ---------------------------------------------------------------- environment / execution

int zs_env_new(zs_executable *exe, zs_pool *pool, zs_environment **out) {
    return guarded([&] {
        NEED(exe); NEED(pool); NEED(out);
        auto env = std::make_unique<zs_environment>();
        env->env.exe = exe->e.get();
        env->env.pool = &pool->p;
        *out = env.release();
    });
}
void zs_env_free(zs_environment *env) { delete env; }

static bool desc_matches(const Desc &a, const Desc &b) {
    return a.width == b.width && a.height == b.height && same_chroma(a, b);
}

int zs_env_bind(zs_environment *env, uint32_t reg, uint64_t key) {
    return guarded([&] {
        NEED(env);
        Executable &E = *env->env.exe;
        reg = flat_reg(E, 0, reg);
        size_t i = 0;
        for (; i < E.input_regs.size(); ++i)
            if (E.input_regs[i] == reg) break;
        if (i == E.input_regs.size()) fail(ZS_ERR_BAD_REGISTER, "register is not an input");
        PoolImage &img = env->env.pool->get(key);
        if (!desc_matches(img.desc, E.input_desc[i]))
            fail(ZS_ERR_MISMATCHED_DESCRIPTOR, "bound image " + describe(img.desc) + " does not match input " +
                                                   describe(E.input_desc[i]));
        env->env.binds[reg] = key;
    });
}

int zs_env_knob(zs_environment *env, uint32_t knob, const void *data, uint64_t len) {
    return guarded([&] {
        NEED(env); NEED(data);
        const Executable &E = *env->env.exe;
        if (knob >= E.knobs.size()) fail(ZS_ERR_INVALID_ARG, "no such knob");
        if (len != E.knobs[knob].len) fail(ZS_ERR_INVALID_ARG, "knob data length differs from the knob's parameter block");
        for (const KnobSite &site : E.knobs[knob].sites)
            if (site.step >= 0) (void)knob_cons(site.kind, (const uint8_t *)data, len);   // validate
        env->env.knob_data[knob].assign((const uint8_t *)data, (const uint8_t *)data + len);
    });
}

int zs_env_bind_output(zs_environment *env, uint32_t reg, uint64_t key) {
    return guarded([&] {
        NEED(env);
        Executable &E = *env->env.exe;
        reg = flat_reg(E, 0, reg);
        size_t i = 0;
        for (; i < E.output_regs.size(); ++i)
            if (E.output_regs[i] == reg) break;
        if (i == E.output_regs.size()) fail(ZS_ERR_BAD_REGISTER, "register is not an output");
        PoolImage &img = env->env.pool->get(key);
        if (!desc_matches(img.desc, E.output_desc[i])) fail(ZS_ERR_MISMATCHED_DESCRIPTOR, "output image mismatch");
        env->env.output_binds[reg] = key;
    });
}

// Instruction encoding of an execution: kind 0 = upload input i, kind 1 = run step i.
int zs_launch(zs_executable *exe, zs_environment *env, zs_execution **out) {
    std::unique_ptr<zs_environment> guard(env);
    return guarded([&] {
        NEED(exe); NEED(env); NEED(out);
        Executable &E = *exe->e;
        if (env->env.exe != &E) fail(ZS_ERR_INVALID_ARG, "environment belongs to another executable");
        E.ensure_buffers();
        auto x = std::make_unique<zs_execution>();
        Execution &X = x->x;
        X.exe = &E;
        X.pool = env->env.pool;
        X.output_binds = env->env.output_binds;
        check_cuda(cudaStreamCreateWithFlags(&X.stream, cudaStreamNonBlocking), "stream");
        X.ptrs = E.dev_buffers;
        for (size_t i = 0; i < E.input_regs.size(); ++i) {
            auto it = env->env.binds.find(E.input_regs[i]);
            if (it == env->env.binds.end()) fail(ZS_ERR_MISSING_KEY, "input register is not bound");
            PoolImage &img = X.pool->get(it->second);
            X.input_keys.push_back(it->second);
            if (img.dev_valid) {
                X.ptrs[E.input_slot[i]] = img.dev;     // device resident: no copy
            } else {
                x->kinds.push_back(0);
                x->args.push_back((int)i);
            }
        }
        // Environment::knob (run.rs:1292-1306): this launch's parameter blocks replace the
        // static ones -- producer constants patched at launch, table slots copied into
        // buffers owned by the execution (Low::BufferInit, run.rs:1588-1606).
        for (const auto &kv : env->env.knob_data) {
            const KnobInfo &K = E.knobs[kv.first];
            for (const KnobSite &site : K.sites) {
                if (site.step >= 0) {
                    ConsPatch p;
                    p.step = (size_t)site.step;
                    p.cons = knob_cons(site.kind, kv.second.data(), kv.second.size());
                    X.patches.push_back(p);
                } else {
                    const Slot &sl = E.slots[site.slot];
                    std::vector<uint8_t> bytes(sl.table);
                    std::memcpy(bytes.data(), kv.second.data(), std::min(bytes.size(), kv.second.size()));
                    void *buf = nullptr;
                    check_cuda(cudaMalloc(&buf, sl.bytes), "cudaMalloc");
                    X.owned.push_back(buf);
                    check_cuda(cudaMemcpy(buf, bytes.data(), sl.bytes, cudaMemcpyHostToDevice), "knob upload");
                    X.ptrs[site.slot] = buf;
                }
            }
        }
        for (size_t s = 0; s < E.steps.size(); ++s) {
            x->kinds.push_back(1);
            x->args.push_back((int)s);
        }
        X.total = x->kinds.size();
        *out = x.release();
    });
}

int zs_exec_is_running(const zs_execution *exec) { return exec && exec->x.cursor < exec->x.total ? 1 : 0; }

int zs_exec_step(zs_execution *exec) {
    return guarded([&] {
        NEED(exec);
        Execution &X = exec->x;
        if (X.cursor >= X.total) fail(ZS_ERR_STEP_LIMIT, "execution has no more instructions");
        const int kind = exec->kinds[X.cursor], arg = exec->args[X.cursor];
        Executable &E = *X.exe;
        if (kind == 0) {
            PoolImage &img = X.pool->get(X.input_keys[arg]);
            const int slot = E.input_slot[arg];
            check_cuda(cudaMemcpy2DAsync(X.ptrs[slot], row_bytes(img.desc), img.host, host_stride(img.desc),
                                         row_bytes(img.desc), img.desc.height, cudaMemcpyHostToDevice, X.stream),
                       "input upload");
        } else {
            E.record_range(X.stream, X.ptrs, (size_t)arg, (size_t)arg + 1, &X.patches);
        }
        X.cursor++;
    });
}

int zs_exec_step_to(zs_execution *exec, uint32_t max_steps, uint32_t *steps) {
    return guarded([&] {
        NEED(exec);
        uint32_t n = 0;
        while (n < max_steps && exec->x.cursor < exec->x.total) {
            const int rc = zs_exec_step(exec);
            if (rc != ZS_OK) fail(rc, last_error());
            ++n;
        }
        if (steps) *steps = n;
    });
}

int zs_exec_sync(zs_execution *exec) {
    return guarded([&] {
        NEED(exec);
        check_cuda(cudaStreamSynchronize(exec->x.stream), "synchronize");
        uint32_t flags = 0;
        check_cuda(read_device_status(exec->x.exe->device, &flags, true), "device status");
        if (flags & ZS_DEVSTAT_WAIT_TIMEOUT) fail(ZS_ERR_TIMEOUT, "a kernel's bounded wait on its bulk copies gave up");
        if (flags) fail(ZS_ERR_DEVICE, "a kernel's shared-memory layout did not fit its window");
    });
}

int zs_retire_input(zs_execution *exec, uint32_t reg, uint64_t *key) {
    return guarded([&] {
        NEED(exec); NEED(key);
        Execution &X = exec->x;
        const Executable &E = *X.exe;
        reg = flat_reg(E, 0, reg);
        for (size_t i = 0; i < E.input_regs.size(); ++i)
            if (E.input_regs[i] == reg) {
                if (i >= X.input_keys.size() || !X.input_keys[i]) fail(ZS_ERR_MISSING_KEY, "input was not bound");
                *key = X.input_keys[i];
                return;
            }
        fail(ZS_ERR_BAD_REGISTER, "no such input register (RetireError::NoSuchInput)");
    });
}

int zs_env_recover_buffers(zs_environment *env, uint64_t *bytes) {
    return guarded([&] {
        NEED(env);
        const Executable &E = *env->env.exe;
        uint64_t held = 0;
        for (size_t i = 0; i < E.slots.size() && i < E.dev_buffers.size(); ++i)
            if (E.dev_buffers[i] && E.slots[i].kind == SlotKind::Intermediate) held += E.slots[i].bytes;
        if (bytes) *bytes = held;
    });
}

int zs_retire_output(zs_execution *exec, uint32_t reg, uint64_t *key) {
    return guarded([&] {
        NEED(exec); NEED(key);
        Execution &X = exec->x;
        Executable &E = *X.exe;
        reg = flat_reg(E, 0, reg);
        while (X.cursor < X.total) {
            int rc = zs_exec_step(exec);
            if (rc != ZS_OK) fail(rc, last_error());
        }
        size_t i = 0;
        for (; i < E.output_regs.size(); ++i)
            if (E.output_regs[i] == reg) break;
        if (i == E.output_regs.size()) fail(ZS_ERR_BAD_REGISTER, "register is not an output");
        check_cuda(cudaStreamSynchronize(X.stream), "synchronize");
        const Desc &d = E.output_desc[i];
        uint64_t k;
        auto bound = X.output_binds.find(reg);
        if (bound != X.output_binds.end()) {
            k = bound->second;
        } else {
            k = pool_add(*X.pool, d);
        }
        PoolImage &img = X.pool->get(k);
        const int slot = E.output_slot[i];
        check_cuda(cudaMemcpy2D(img.host, host_stride(img.desc), X.ptrs[slot], row_bytes(d), row_bytes(d), d.height,
                                cudaMemcpyDeviceToHost),
                   "output download");
        img.host_valid = true;
        img.dev_valid = false;
        *key = k;
    });
}

void zs_exec_free(zs_execution *exec) { delete exec; }

// ---------------------------------------------------------------- one-call paths

static cudaStream_t exe_stream(zs_executable *exe) {
    if (!exe->stream) check_cuda(cudaStreamCreateWithFlags(&exe->stream, cudaStreamNonBlocking), "stream");
    return exe->stream;
}

// Device address of a pinned, device-mapped host buffer (cudaMallocHost / cudaHostAlloc /
// cudaHostRegister), or null for any other pointer or one not 16-byte aligned.
static void *mapped_host_pointer(const void *p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer || ((uintptr_t)at.devicePointer & 15u)) return nullptr;
    return at.devicePointer;
}

// A lone fused colour chain on pinned host buffers runs zero copy: the GPU reaches pinned
// host memory through its own address space (over NVLink-C2C on a Grace host), so the chain
// kernel streams the input from and the output to host memory, one launch, no staging.
static bool run_host_zero_copy(zs_executable *exe, const void *const *inputs, void *const *outputs) {
    Executable &E = *exe->e;
    if (E.flags & ZS_CAP_NO_ZERO_COPY) return false;
    if (E.steps.size() != 1 || E.steps[0].kind != StepKind::Chain || E.input_slot.size() != 1 ||
        E.output_slot.size() != 1)
        return false;
    const Step &st = E.steps[0];
    if (st.src_slot[0] != E.input_slot[0] || st.dst_slot != E.output_slot[0]) return false;
    void *din = mapped_host_pointer(inputs[0]), *dout = mapped_host_pointer(outputs[0]);
    if (!din || !dout) return false;
    ZsChainArgs c = st.chain;
    c.src = (const uint8_t *)din;
    c.dst = (uint8_t *)dout;
    cudaStream_t s = exe_stream(exe);
    // Blocks of 256 threads (two per SM, as the tables' shared memory allows), one 16-byte
    // vector per thread in flight: with the link, not the SMs, as the limit, fewer reads in
    // flight keep its two directions busier (one host-to-host copy of 64 MiB each way measured
    // 0.40 ms with 512 threads per SM against 0.46 ms with 1024; this chain 0.418 ms).
    check_cuda(launch_chain(c, st.chain_src_fast, st.chain_dst_fast, E.sm_count, s, 256, 1), st.label.c_str());
    check_cuda(cudaStreamSynchronize(s), "synchronize");
    return true;
}

// A lone fused colour chain is pixel local: its host round trip runs in row stripes on
// three rotating streams, so that the upload of one stripe, the kernel of the previous and
// the download of the one before overlap (both copy directions at once).
static bool run_host_striped(zs_executable *exe, const void *const *inputs, void *const *outputs) {
    Executable &E = *exe->e;
    if (E.steps.size() != 1 || E.steps[0].kind != StepKind::Chain || E.input_slot.size() != 1 ||
        E.output_slot.size() != 1)
        return false;
    const Step &st = E.steps[0];
    if (st.src_slot[0] != E.input_slot[0] || st.dst_slot != E.output_slot[0]) return false;
    const int64_t npx = st.chain.npx;
    const int64_t bytes = npx * 4;
    if (bytes < (int64_t)(16 << 20)) return false;               // small images: one round trip
    const int kStripes = 8;
    const int64_t per = ((npx + kStripes - 1) / kStripes + 1023) & ~(int64_t)1023;   // 4 KiB multiples
    for (cudaStream_t &t : exe->stripes)
        if (!t) check_cuda(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking), "stream");
    uint8_t *din = (uint8_t *)E.dev_buffers[st.src_slot[0]], *dout = (uint8_t *)E.dev_buffers[st.dst_slot];
    const uint8_t *hin = (const uint8_t *)inputs[0];
    uint8_t *hout = (uint8_t *)outputs[0];
    int k = 0;
    for (int64_t p0 = 0; p0 < npx; p0 += per, ++k) {
        const int64_t n = std::min(per, npx - p0);
        cudaStream_t t = exe->stripes[k % 3];
        check_cuda(cudaMemcpyAsync(din + p0 * 4, hin + p0 * 4, n * 4, cudaMemcpyHostToDevice, t), "h2d");
        ZsChainArgs c = st.chain;
        c.src = din + p0 * 4;
        c.dst = dout + p0 * 4;
        c.npx = n;
        check_cuda(launch_chain(c, st.chain_src_fast, st.chain_dst_fast, E.sm_count, t,
                                st.tune_threads ? st.tune_threads : 1024, st.tune_vectors ? st.tune_vectors : 2),
                   st.label.c_str());
        check_cuda(cudaMemcpyAsync(hout + p0 * 4, dout + p0 * 4, n * 4, cudaMemcpyDeviceToHost, t), "d2h");
    }
    for (cudaStream_t t : exe->stripes) check_cuda(cudaStreamSynchronize(t), "synchronize");
    return true;
}

int zs_run_host(zs_executable *exe, const void *const *inputs, uint32_t n_inputs, void *const *outputs,
                uint32_t n_outputs) {
    return guarded([&] {
        NEED(exe);
        Executable &E = *exe->e;
        if (n_inputs != E.input_regs.size() || n_outputs != E.output_regs.size())
            fail(ZS_ERR_INVALID_ARG, "wrong number of inputs or outputs");
        for (uint32_t i = 0; i < n_inputs; ++i) NEED(inputs[i]);
        for (uint32_t j = 0; j < n_outputs; ++j) NEED(outputs[j]);
        E.ensure_buffers();
        if (run_host_zero_copy(exe, inputs, outputs)) return;
        if (run_host_striped(exe, inputs, outputs)) return;
        cudaStream_t s = exe_stream(exe);
        std::vector<void *> ptrs = E.dev_buffers;
        for (uint32_t i = 0; i < n_inputs; ++i) {
            NEED(inputs[i]);
            const Slot &sl = E.slots[E.input_slot[i]];
            check_cuda(cudaMemcpyAsync(ptrs[E.input_slot[i]], inputs[i], sl.bytes, cudaMemcpyHostToDevice, s), "h2d");
        }
        E.record(s, ptrs);
        for (uint32_t j = 0; j < n_outputs; ++j) {
            NEED(outputs[j]);
            const Slot &sl = E.slots[E.output_slot[j]];
            check_cuda(cudaMemcpyAsync(outputs[j], ptrs[E.output_slot[j]], sl.bytes, cudaMemcpyDeviceToHost, s), "d2h");
        }
        check_cuda(cudaStreamSynchronize(s), "synchronize");
    });
}

int zs_run_device(zs_executable *exe, const void *const *inputs, uint32_t n_inputs, void *const *outputs,
                  uint32_t n_outputs, void *stream) {
    return guarded([&] {
        NEED(exe);
        Executable &E = *exe->e;
        if (n_inputs != E.input_regs.size() || n_outputs != E.output_regs.size())
            fail(ZS_ERR_INVALID_ARG, "wrong number of inputs or outputs");
        E.ensure_buffers();
        cudaStream_t s = stream ? (cudaStream_t)stream : exe_stream(exe);
        std::vector<void *> ptrs = E.dev_buffers;
        // Kernels read and write whole texels: a buffer must start on its texel's natural
        // alignment (the largest power of two dividing the texel size, at most 16 bytes).
        auto aligned = [&](const void *p, int slot) {
            const uint32_t bpp = E.slots[slot].fmt.bpp;
            const uintptr_t a = bpp >= 16 ? 16 : (bpp & 7) == 0 ? 8 : (bpp & 3) == 0 ? 4 : (bpp & 1) == 0 ? 2 : 1;
            return ((uintptr_t)p & (a - 1)) == 0;
        };
        for (uint32_t i = 0; i < n_inputs; ++i) {
            NEED(inputs[i]);
            if (!aligned(inputs[i], E.input_slot[i])) fail(ZS_ERR_INVALID_ARG, "input buffer is not texel aligned");
            ptrs[E.input_slot[i]] = const_cast<void *>(inputs[i]);
        }
        for (uint32_t j = 0; j < n_outputs; ++j) {
            NEED(outputs[j]);
            if (!aligned(outputs[j], E.output_slot[j])) fail(ZS_ERR_INVALID_ARG, "output buffer is not texel aligned");
            ptrs[E.output_slot[j]] = outputs[j];
        }
        // A single kernel gains nothing from a graph; launched directly, a colour chain keeps
        // its programmatic dependent launch across consecutive calls (its table staging
        // overlaps the previous kernel's tail), which separate graph launches would not.
        if (!E.use_graph || E.steps.size() == 1) {
            E.record(s, ptrs);
            return;
        }
        auto it = E.graphs.find(ptrs);
        if (it == E.graphs.end()) {
            if (E.graphs.size() >= 16) {          // bounded cache of instantiated graphs
                auto victim = E.graphs.find(E.graph_order.front());
                if (victim != E.graphs.end()) {
                    cudaGraphExecDestroy(victim->second);
                    E.graphs.erase(victim);
                }
                E.graph_order.erase(E.graph_order.begin());
            }
            cudaGraph_t g = nullptr;
            check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
            try {
                E.record(s, ptrs);
            } catch (...) {
                cudaStreamEndCapture(s, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            check_cuda(cudaStreamEndCapture(s, &g), "end capture");
            cudaGraphExec_t ge = nullptr;
            cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            check_cuda(e, "graph instantiate");
            it = E.graphs.emplace(ptrs, ge).first;
            E.graph_order.push_back(ptrs);
        }
        check_cuda(cudaGraphLaunch(it->second, s), "graph launch");
        note_graph_launch(E);
    });
}

void *zs_host_alloc(uint64_t bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
void zs_host_free(void *ptr) {
    if (ptr) cudaFreeHost(ptr);
}
void *zs_device_alloc(uint64_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
void zs_device_free(void *ptr) {
    if (ptr) cudaFree(ptr);
}
int zs_memcpy_h2d(void *dst, const void *src, uint64_t bytes) {
    return guarded([&] { check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "h2d"); });
}
int zs_memcpy_d2h(void *dst, const void *src, uint64_t bytes) {
    return guarded([&] { check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), "d2h"); });
}
int zs_device_synchronize(void) {
    return guarded([&] { check_cuda(cudaDeviceSynchronize(), "synchronize"); });
}

int zs_batch_thumbnails(zs_executable *chain, const void *const *images, const uint32_t *widths,
                        const uint32_t *heights, uint32_t n, uint32_t canvas, void *out, void *stream) {
    return guarded([&] {
        NEED(chain); NEED(images); NEED(widths); NEED(heights); NEED(out);
        cudaStream_t s = stream ? (cudaStream_t)stream : exe_stream(chain);
        int rc = batch_thumbnails(chain->e.get(), images, widths, heights, n, canvas, out, s);
        if (rc != ZS_OK) fail(rc, last_error());
    });
}

// ---------------------------------------------------------------- batches of runs

// The texel alignment a kernel needs of a buffer of this slot (see zs_run_device).
static bool slot_aligned(const Executable &E, int slot, const void *p) {
    const uint32_t bpp = E.slots[slot].fmt.bpp;
    const uintptr_t a = bpp >= 16 ? 16 : (bpp & 7) == 0 ? 8 : (bpp & 3) == 0 ? 4 : (bpp & 1) == 0 ? 2 : 1;
    return ((uintptr_t)p & (a - 1)) == 0;
}

// n runs of one executable recorded into one CUDA graph: run i on capture stream
// i % branches, all forked from and joined back into `s`, so runs on different branches may
// execute at the same time.  An executable that stores intermediates in its own buffers
// records its runs on one branch, one after another.
static cudaGraphExec_t capture_batch(zs_executable *exe, const std::vector<void *> &table, uint32_t n,
                                     cudaStream_t s) {
    Executable &E = *exe->e;
    const size_t ni = E.input_regs.size(), no = E.output_regs.size();
    for (cudaStream_t &t : exe->branches)
        if (!t) check_cuda(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking), "stream");
    for (cudaEvent_t &ev : exe->joins)
        if (!ev) check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
    if (!exe->fork) check_cuda(cudaEventCreateWithFlags(&exe->fork, cudaEventDisableTiming), "event");
    bool shared = false;
    for (const Slot &sl : E.slots) shared = shared || sl.kind == SlotKind::Intermediate;
    const uint32_t nb = shared ? 1u : std::min<uint32_t>(n, ZS_BATCH_BRANCHES);
    check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaGraph_t g = nullptr;
    try {
        check_cuda(cudaEventRecord(exe->fork, s), "fork");
        for (uint32_t b = 0; b < nb; ++b) check_cuda(cudaStreamWaitEvent(exe->branches[b], exe->fork, 0), "fork wait");
        for (uint32_t i = 0; i < n; ++i) {
            std::vector<void *> ptrs = E.dev_buffers;
            for (size_t k = 0; k < ni; ++k) ptrs[E.input_slot[k]] = table[i * (ni + no) + k];
            for (size_t k = 0; k < no; ++k) ptrs[E.output_slot[k]] = table[i * (ni + no) + ni + k];
            E.record(exe->branches[i % nb], ptrs);
        }
        for (uint32_t b = 0; b < nb; ++b) {
            check_cuda(cudaEventRecord(exe->joins[b], exe->branches[b]), "join");
            check_cuda(cudaStreamWaitEvent(s, exe->joins[b], 0), "join wait");
        }
    } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    check_cuda(cudaStreamEndCapture(s, &g), "end capture");
    cudaGraphExec_t ge = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    check_cuda(e, "graph instantiate");
    return ge;
}

static void batch_run_device(zs_executable *exe, const void *const *inputs, void *const *outputs, uint32_t n,
                             cudaStream_t s) {
    Executable &E = *exe->e;
    const size_t ni = E.input_regs.size(), no = E.output_regs.size();
    E.ensure_buffers();
    std::vector<void *> table((ni + no) * n);
    for (uint32_t i = 0; i < n; ++i) {
        for (size_t k = 0; k < ni; ++k) {
            const void *p = inputs[i * ni + k];
            NEED(p);
            if (!slot_aligned(E, E.input_slot[k], p)) fail(ZS_ERR_INVALID_ARG, "input buffer is not texel aligned");
            table[i * (ni + no) + k] = const_cast<void *>(p);
        }
        for (size_t k = 0; k < no; ++k) {
            void *p = outputs[i * no + k];
            NEED(p);
            if (!slot_aligned(E, E.output_slot[k], p)) fail(ZS_ERR_INVALID_ARG, "output buffer is not texel aligned");
            table[i * (ni + no) + ni + k] = p;
        }
    }
    auto it = exe->batch_graphs.find(table);
    if (it == exe->batch_graphs.end()) {
        if (exe->batch_graphs.size() >= 8) {
            auto victim = exe->batch_graphs.find(exe->batch_order.front());
            if (victim != exe->batch_graphs.end()) {
                cudaGraphExecDestroy(victim->second);
                exe->batch_graphs.erase(victim);
            }
            exe->batch_order.erase(exe->batch_order.begin());
        }
        it = exe->batch_graphs.emplace(table, capture_batch(exe, table, n, s)).first;
        exe->batch_order.push_back(table);
    }
    check_cuda(cudaGraphLaunch(it->second, s), "graph launch");
    for (uint32_t i = 0; i < n; ++i) note_graph_launch(E);
}

int zs_batch_run_device(zs_executable *exe, const void *const *inputs, void *const *outputs, uint32_t n,
                        void *stream) {
    return guarded([&] {
        NEED(exe);
        if (n == 0) return;
        NEED(inputs); NEED(outputs);
        cudaStream_t s = stream ? (cudaStream_t)stream : exe_stream(exe);
        batch_run_device(exe, inputs, outputs, n, s);
    });
}

int zs_batch_run(zs_executable *exe, zs_pool *pool, const uint64_t *keys, uint32_t n, uint64_t *out_keys) {
    return guarded([&] {
        NEED(exe); NEED(pool);
        if (n == 0) return;
        NEED(keys); NEED(out_keys);
        Executable &E = *exe->e;
        const size_t ni = E.input_regs.size(), no = E.output_regs.size();
        E.ensure_buffers();
        // Inputs: bound pool images, made device resident (Pool::upload).
        std::vector<const void *> ins(n * ni);
        for (uint32_t i = 0; i < n; ++i)
            for (size_t k = 0; k < ni; ++k) {
                PoolImage &img = pool->p.get(keys[i * ni + k]);
                if (!desc_matches(img.desc, E.input_desc[k]))
                    fail(ZS_ERR_MISMATCHED_DESCRIPTOR, "bound image " + describe(img.desc) + " does not match input " +
                                                           describe(E.input_desc[k]));
                pool_upload(img);
                ins[i * ni + k] = img.dev;
            }
        // Outputs: new pool images with device storage, retired into the pool (Retire::output).
        std::vector<uint64_t> made;
        std::vector<void *> outs(n * no);
        try {
            for (uint32_t i = 0; i < n; ++i)
                for (size_t k = 0; k < no; ++k) {
                    const Desc &d = E.output_desc[k];
                    const uint64_t key = pool_add(pool->p, d);
                    made.push_back(key);
                    PoolImage &img = pool->p.get(key);
                    img.dev_len = row_bytes(d) * d.height;
                    check_cuda(cudaMalloc(&img.dev, img.dev_len), "cudaMalloc");
                    img.host_valid = false;
                    outs[i * no + k] = img.dev;
                }
            cudaStream_t s = exe_stream(exe);
            batch_run_device(exe, ins.data(), outs.data(), n, s);
            check_cuda(cudaStreamSynchronize(s), "synchronize");
        } catch (...) {
            for (uint64_t key : made) pool->p.images.erase(key);
            throw;
        }
        for (size_t j = 0; j < made.size(); ++j) {
            PoolImage &img = pool->p.get(made[j]);
            img.dev_valid = true;
            pool_sync_host(img);
            out_keys[j] = made[j];
        }
    });
}

// ---------------------------------------------------------------- autotuner

int zs_autotune(zs_executable *exe, const void *const *inputs, uint32_t n_inputs, void *const *outputs,
                uint32_t n_outputs, void *stream, uint32_t reps, int32_t *chain_threads) {
    return guarded([&] {
        NEED(exe);
        Executable &E = *exe->e;
        if (n_inputs != E.input_regs.size() || n_outputs != E.output_regs.size())
            fail(ZS_ERR_INVALID_ARG, "wrong number of inputs or outputs");
        if (reps == 0 || reps > 1000) fail(ZS_ERR_INVALID_ARG, "reps out of range (1..1000)");
        E.ensure_buffers();
        std::vector<void *> ptrs = E.dev_buffers;
        for (uint32_t i = 0; i < n_inputs; ++i) {
            NEED(inputs[i]);
            ptrs[E.input_slot[i]] = const_cast<void *>(inputs[i]);
        }
        for (uint32_t j = 0; j < n_outputs; ++j) {
            NEED(outputs[j]);
            ptrs[E.output_slot[j]] = outputs[j];
        }
        const int t = autotune_steps(E, ptrs, stream ? (cudaStream_t)stream : exe_stream(exe), reps);
        for (auto &kv : exe->batch_graphs) cudaGraphExecDestroy(kv.second);
        exe->batch_graphs.clear();
        exe->batch_order.clear();
        if (chain_threads) *chain_threads = t;
    });
}

int zs_autotune_batch_thumbnails(zs_executable *chain, const void *const *images, const uint32_t *widths,
                                 const uint32_t *heights, uint32_t n, uint32_t canvas, void *out, void *stream,
                                 uint32_t reps, uint32_t *rows) {
    return guarded([&] {
        NEED(chain); NEED(images); NEED(widths); NEED(heights); NEED(out);
        if (reps == 0 || reps > 1000) fail(ZS_ERR_INVALID_ARG, "reps out of range (1..1000)");
        cudaStream_t s = stream ? (cudaStream_t)stream : exe_stream(chain);
        const int r = autotune_batch(chain->e.get(), images, widths, heights, n, canvas, out, s, reps);
        if (rows) *rows = (uint32_t)r;
    });
}

int zs_executable_set_launch(zs_executable *exe, uint32_t param, int32_t value) {
    return guarded([&] {
        NEED(exe);
        Executable &E = *exe->e;
        if (param == ZS_TUNE_CHAIN_THREADS) {
            if (value != 1024 && value != 512) fail(ZS_ERR_INVALID_ARG, "chain block size must be 1024 or 512");
            for (Step &st : E.steps)
                if (st.kind == StepKind::Chain) st.tune_threads = value;
            for (auto &kv : E.graphs) cudaGraphExecDestroy(kv.second);
            E.graphs.clear();
            E.graph_order.clear();
        } else if (param == ZS_TUNE_BATCH_ROWS) {
            if (value < 1 || value > 16) fail(ZS_ERR_INVALID_ARG, "rows per batch item must be in 1..16");
            E.batch_rows = value;
        } else if (param == ZS_TUNE_BATCH_THREADS) {
            if (value != 768 && value != 640) fail(ZS_ERR_INVALID_ARG, "batch block size must be 768 or 640");
            E.batch_threads = value;
        } else if (param == ZS_TUNE_CHAIN_VECTORS) {
            if (value != 1 && value != 2) fail(ZS_ERR_INVALID_ARG, "chain vectors per iteration must be 1 or 2");
            for (Step &st : E.steps)
                if (st.kind == StepKind::Chain) st.tune_vectors = value;
            for (auto &kv : E.graphs) cudaGraphExecDestroy(kv.second);
            E.graphs.clear();
            E.graph_order.clear();
        } else if (param == ZS_TUNE_RESAMPLE_TILE) {
            bool any = false;
            for (Step &st : E.steps)
                if (!st.tc_cands.empty()) {
                    if (!set_resample_tile(st, value)) fail(ZS_ERR_INVALID_ARG, "not a tile width this resample fits");
                    any = true;
                }
            if (!any) fail(ZS_ERR_UNIMPLEMENTED, "the executable has no tensor-core resample step");
            for (auto &kv : E.graphs) cudaGraphExecDestroy(kv.second);
            E.graphs.clear();
            E.graph_order.clear();
        } else {
            fail(ZS_ERR_INVALID_ARG, "unknown launch parameter");
        }
    });
}

int zs_executable_get_launch(const zs_executable *exe, uint32_t param, int32_t *value) {
    return guarded([&] {
        NEED(exe); NEED(value);
        const Executable &E = *exe->e;
        if (param == ZS_TUNE_CHAIN_THREADS) {
            *value = 0;
            for (const Step &st : E.steps)
                if (st.kind == StepKind::Chain) *value = st.tune_threads ? st.tune_threads : 1024;
        } else if (param == ZS_TUNE_BATCH_ROWS) {
            *value = E.batch_rows;
        } else if (param == ZS_TUNE_BATCH_THREADS) {
            *value = E.batch_threads;
        } else if (param == ZS_TUNE_CHAIN_VECTORS) {
            *value = 0;
            for (const Step &st : E.steps)
                if (st.kind == StepKind::Chain) *value = st.tune_vectors ? st.tune_vectors : 2;
        } else if (param == ZS_TUNE_RESAMPLE_TILE) {
            *value = 0;
            for (const Step &st : E.steps)
                if (!st.tc_cands.empty()) *value = st.raster.tc_tw;
        } else {
            fail(ZS_ERR_INVALID_ARG, "unknown launch parameter");
        }
    });
}

static void copy_string(const std::string &s, char *buf, uint64_t len) {
    if (!buf || len == 0) fail(ZS_ERR_INVALID_ARG, "no output buffer");
    if (s.size() + 1 > len) fail(ZS_ERR_INVALID_ARG, "output buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
}

int zs_executable_tune_key(const zs_executable *exe, uint32_t param, uint32_t canvas, char *buf, uint64_t len) {
    return guarded([&] {
        NEED(exe);
        const Executable &E = *exe->e;
        if (param == ZS_TUNE_CHAIN_THREADS) {
            for (const Step &st : E.steps)
                if (st.kind == StepKind::Chain) return copy_string(chain_tune_key(st, E.device), buf, len);
            fail(ZS_ERR_UNIMPLEMENTED, "the executable has no chain step");
        } else if (param == ZS_TUNE_BATCH_ROWS) {
            copy_string(batch_tune_key(E, canvas, E.device), buf, len);
        } else if (param == ZS_TUNE_BATCH_THREADS) {
            copy_string(batch_tune_key(E, canvas, E.device, "batch_threads"), buf, len);
        } else if (param == ZS_TUNE_CHAIN_VECTORS) {
            for (const Step &st : E.steps)
                if (st.kind == StepKind::Chain) return copy_string(chain_vectors_key(st, E.device), buf, len);
            fail(ZS_ERR_UNIMPLEMENTED, "the executable has no chain step");
        } else if (param == ZS_TUNE_RESAMPLE_TILE) {
            for (const Step &st : E.steps)
                if (!st.tc_cands.empty()) return copy_string(resample_tune_key(st, E.device), buf, len);
            fail(ZS_ERR_UNIMPLEMENTED, "the executable has no tensor-core resample step");
        } else {
            fail(ZS_ERR_INVALID_ARG, "unknown launch parameter");
        }
    });
}

int zs_tune_cache_get(const char *key, int32_t *value) {
    return guarded([&] {
        NEED(key); NEED(value);
        int v;
        if (!tune_get(key, v)) fail(ZS_ERR_MISSING_KEY, std::string("no tuned value for ") + key);
        *value = v;
    });
}
int zs_tune_cache_put(const char *key, int32_t value) {
    return guarded([&] {
        NEED(key);
        tune_put(key, value);
    });
}
int zs_tune_cache_save(const char *path) {
    return guarded([&] {
        NEED(path);
        tune_save(path);
    });
}
int zs_tune_cache_load(const char *path) {
    return guarded([&] {
        NEED(path);
        tune_load(path);
    });
}

uint64_t zs_kernel_launch_count(void) { return kernel_launch_count(); }

int zs_selftest_wait_timeout(int device, uint32_t limit_us) {
    return guarded([&] {
        if (limit_us == 0 || limit_us > 1000000) fail(ZS_ERR_INVALID_ARG, "limit_us out of range");
        check_cuda(init_device_tables(device), "device tables");
        check_cuda(wait_selftest(device, limit_us), "wait self test");
    });
}

int zs_device_status(int device, uint32_t *flags) {
    return guarded([&] {
        NEED(flags);
        int prev = 0;
        check_cuda(cudaGetDevice(&prev), "get device");
        check_cuda(cudaSetDevice(device), "set device");
        cudaError_t e = cudaDeviceSynchronize();
        cudaSetDevice(prev);
        check_cuda(e, "synchronize");
        check_cuda(read_device_status(device, flags, true), "device status");
    });
}

}  // extern "C"
