// link.cpp -- compiling and linking command buffers (the analogue of lib/zosimos/src/command.rs
// Linker::compile / Linker::link / link_in :2063-2893 and the generic machinery of
// CommandBuffer::generic, input_generic, register_descriptor, function and invoke :756-922).
//
// The reference links each (function, generic instantiation) into a separate function of the
// Program and calls it at run time through a call stack (run.rs:2291-2358).  Here every
// invocation is monomorphised and inlined at link time: the callee's recorded operations are
// replayed through the same builders with the concrete descriptors of the call (which re-runs
// their type checks and recomputes descriptors and colour programs), its inputs bound to the
// call's arguments and its outputs to the call's result registers.  The linked program is one
// flat op list, so the planner fuses across function boundaries exactly as within a function.
#include <cstring>
#include <set>

#include "zs_host.hpp"

namespace zs {

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
uint32_t cmd_fractal_noise(Command &c, const Desc &d, const float params[5]);
uint32_t cmd_buffer_init(Command &c, const void *bytes, uint64_t n, uint64_t len);
uint32_t cmd_from_buffer(Command &c, uint32_t buffer, const Desc &target);
uint32_t cmd_output(Command &c, uint32_t src, Desc *outformat);
uint32_t cmd_dynamic(Command &c, uint32_t nops, uint32_t a, uint32_t b, uint32_t op_id, const void *uniforms,
                     uint64_t len, const Desc &target);

// ---------------------------------------------------------------- compile

Program compile_command(const Command &c) {
    Program p;
    p.ops = c.ops;
    p.uses.assign(p.ops.size(), 0);
    for (uint32_t r = 0; r < p.ops.size(); ++r) {
        const Op &op = p.ops[r];
        switch (op.kind) {
        case OpKind::Input: p.inputs.push_back(r); break;
        case OpKind::Output:
            p.outputs.push_back(op.a);
            p.output_regs.push_back(r);
            p.uses[op.a]++;
            break;
        case OpKind::Bilinear:
        case OpKind::Normal2d:
        case OpKind::FractalNoise:
        case OpKind::BufferInit:
        case OpKind::Solid:
            if (op.param_buffer >= 0) p.uses[op.param_buffer]++;
            break;
        case OpKind::FromBuffer: p.uses[op.a]++; break;
        case OpKind::Derivative:
            // DerivativeMethod::to_shader: Roberts, Scharr4, Scharr5, Scharr5Tab are
            // CompileError::NotYetImplemented (command.rs:3397-3402).
            if (op.u0 == 0 || op.u0 == 4 || op.u0 == 5 || op.u0 == 7)
                fail(ZS_ERR_UNIMPLEMENTED, "derivative method not yet implemented");
            p.uses[op.a]++;
            break;
        case OpKind::Dynamic:
            if (op.u0 > 0) p.uses[op.a]++;
            if (op.u0 > 1) p.uses[op.b]++;
            break;
        case OpKind::Invoke:
        case OpKind::InvokedResult:
            fail(ZS_ERR_UNIMPLEMENTED, "the program invokes functions: link it (zs_link) instead of compiling it");
        case OpKind::Inject:
        case OpKind::Inscribe:
        case OpKind::InscribePlaced:
        case OpKind::Palette:
        case OpKind::Affine:
        case OpKind::Blend:
            p.uses[op.a]++;
            p.uses[op.b]++;
            break;
        default: p.uses[op.a]++; break;
        }
    }
    if (p.output_regs.empty()) fail(ZS_ERR_OTHER, "program has no output");
    return p;
}

// ---------------------------------------------------------------- generics

// The descriptor a generic parameter stands in for while its function is recorded (no bounds
// exist yet: GenericDeclaration { bounds: &[] }); replaced by the concrete one at every call.
static Desc placeholder() {
    Desc d{};
    d.width = d.height = 1;
    d.bits = ZS_BITS_UINT8X4;
    d.parts = ZS_PARTS_RGBA;
    d.color = ZS_COLOR_RGB;
    d.primaries = ZS_PRIMARIES_BT709;
    d.transfer = ZS_TRANSFER_SRGB;
    d.whitepoint = ZS_WP_D65;
    return d;
}

// The descriptor of variable `ty` of `tys`: `generic` gives a generic parameter's, `reg` a
// register's; a derived variable takes its base's with the size replaced.
template <class G, class R>
static Desc resolve_ty(const std::vector<TyVar> &tys, uint32_t ty, G generic, R reg) {
    if (ty >= tys.size()) fail(ZS_ERR_BAD_REGISTER, "no such descriptor variable");
    const TyVar &t = tys[ty];
    if (t.base >= 0) {
        Desc d = resolve_ty(tys, (uint32_t)t.base, generic, reg);
        if (t.width) {
            d.width = t.width;
            d.height = t.height;
        }
        return d;
    }
    if (t.var >= 0) return generic((uint32_t)t.var);
    return reg((uint32_t)t.reg);
}

Desc ty_descriptor(const Command &c, uint32_t ty) {
    return resolve_ty(c.tys, ty, [](uint32_t) { return placeholder(); },
                      [&](uint32_t reg) { return c.describe(reg); });
}

// Replays op `op` of a recorded buffer into `dst` with its operands remapped; returns its
// register there.
static uint32_t replay_op(const Op &op, const std::vector<int64_t> &map, Command &dst) {
    auto m = [&](uint32_t reg) -> uint32_t {
        if (reg >= map.size() || map[reg] < 0) fail(ZS_ERR_BAD_REGISTER, "operand not available after linking");
        return (uint32_t)map[reg];
    };
    dst.pending_knob = op.knob;
    dst.pending_buffer = op.param_buffer >= 0 ? (int32_t)m((uint32_t)op.param_buffer) : -1;
    switch (op.kind) {
    case OpKind::Crop: return cmd_crop(dst, m(op.a), op.rect);
    case OpKind::ColorConvert: return cmd_color_convert(dst, m(op.a), op.desc);
    case OpKind::ChromaticAdaptation: return cmd_chromatic_adaptation(dst, m(op.a), op.u0, op.desc.whitepoint);
    case OpKind::ColorMatrix: {
        float mm[9];
        for (int i = 0; i < 9; ++i) mm[i] = (float)op.prog.ins.at(0).mat.m[i];
        return cmd_color_matrix(dst, m(op.a), mm);
    }
    case OpKind::Extract: return cmd_extract(dst, m(op.a), op.u0);
    case OpKind::Inject: return cmd_inject(dst, m(op.a), op.u0, m(op.b));
    case OpKind::Transmute: return cmd_transmute(dst, m(op.a), op.desc);
    case OpKind::Inscribe: return cmd_inscribe(dst, m(op.a), op.rect, m(op.b), false);
    case OpKind::InscribePlaced: return cmd_inscribe(dst, m(op.a), op.rect, m(op.b), true);
    case OpKind::Palette: return cmd_palette(dst, m(op.a), op.i0, op.i1, m(op.b));
    case OpKind::Bilinear: return cmd_bilinear(dst, op.desc, op.fparams);
    case OpKind::Solid: return cmd_solid(dst, op.desc, op.fparams);
    case OpKind::Affine: return cmd_affine(dst, m(op.a), op.fparams, op.u0, m(op.b));
    case OpKind::Resize: return cmd_resize(dst, m(op.a), op.desc.width, op.desc.height, false, op.u0);
    case OpKind::ResizeFiltered: return cmd_resize(dst, m(op.a), op.desc.width, op.desc.height, true, op.u0);
    case OpKind::Blend: return cmd_blend(dst, m(op.a), op.rect, m(op.b), op.u0);
    case OpKind::Derivative: return cmd_derivative(dst, m(op.a), op.u0, op.u1);
    case OpKind::Normal2d: return cmd_normal2d(dst, op.desc, op.fparams);
    case OpKind::FractalNoise: return cmd_fractal_noise(dst, op.desc, op.fparams);
    case OpKind::BufferInit: return cmd_buffer_init(dst, op.data.data(), op.data.size(), op.len);
    case OpKind::FromBuffer: return cmd_from_buffer(dst, m(op.a), op.desc);
    case OpKind::Dynamic:
        return cmd_dynamic(dst, op.u0, op.u0 > 0 ? m(op.a) : 0, op.u0 > 1 ? m(op.b) : 0, op.dyn_op,
                           op.data.empty() ? nullptr : op.data.data(), op.data.size(), op.desc);
    default: break;
    }
    fail(ZS_ERR_UNIMPLEMENTED, "operation cannot be replayed");
}

// Monomorphises `fn` (a recorded function buffer) with concrete generic descriptors `gen`
// into `dst`: its inputs are `args` (registers of dst), its outputs are returned.  Functions
// it invokes are taken from `resolve`, which maps its function index to a buffer.
struct Linking {
    const std::vector<const Command *> *buffers = nullptr;
    const std::vector<std::vector<uint32_t>> *links = nullptr;
    Program *program = nullptr;
    std::set<uint32_t> active;     // link indices on the current call path (recursion check)
};

static std::vector<uint32_t> instantiate(const Command &fn, uint32_t link_idx, const std::vector<Desc> &gen,
                                         const std::vector<uint32_t> &args, Command &dst, Linking *lk,
                                         std::vector<int64_t> *map_out = nullptr) {
    std::vector<int64_t> map(fn.ops.size(), -1);
    std::vector<uint32_t> outs;
    size_t next_input = 0;
    // Descriptor of a descriptor variable of `fn`, in this instantiation.
    auto ty_desc = [&](uint32_t ty) -> Desc {
        return resolve_ty(
            fn.tys, ty,
            [&](uint32_t var) {
                if (var >= gen.size()) fail(ZS_ERR_OTHER, "generic parameter not given");
                return gen[var];
            },
            [&](uint32_t reg) {
                if (reg >= map.size() || map[reg] < 0) fail(ZS_ERR_BAD_REGISTER, "descriptor of a register not yet available");
                return dst.describe((uint32_t)map[reg]);
            });
    };
    for (uint32_t r = 0; r < fn.ops.size(); ++r) {
        const Op &op = fn.ops[r];
        switch (op.kind) {
        case OpKind::Input: {
            if (lk && link_idx == 0) {                   // the entry point keeps its inputs
                map[r] = cmd_input(dst, op.generic_var >= 0 ? ty_desc((uint32_t)op.generic_var) : op.desc);
                break;
            }
            if (next_input >= args.size()) fail(ZS_ERR_OTHER, "too few arguments for the function's inputs");
            const uint32_t a = args[next_input++];
            const Desc want = op.generic_var >= 0 ? ty_desc((uint32_t)op.generic_var) : op.desc;
            const Desc have = dst.describe(a);
            if (have.width != want.width || have.height != want.height || !same_chroma(have, want))
                fail(ZS_ERR_OTHER, "argument does not match the function's input descriptor");
            map[r] = a;
        } break;
        case OpKind::Output:
            if (lk && link_idx == 0) map[r] = cmd_output(dst, (uint32_t)map[op.a], nullptr);
            else outs.push_back((uint32_t)map[op.a]);
            break;
        case OpKind::Invoke: {
            std::vector<Desc> g;
            for (uint32_t ty : op.tyvars) g.push_back(ty_desc(ty));
            std::vector<uint32_t> a;
            for (uint32_t reg : op.regs) a.push_back((uint32_t)map[reg]);
            std::vector<uint32_t> res;
            if (lk) {
                // Linker::link: the buffer defining this function of buffer `link_idx`.
                const auto &table = link_idx < lk->links->size() ? (*lk->links)[link_idx] : std::vector<uint32_t>{};
                if (op.u0 >= table.size()) fail(ZS_ERR_UNIMPLEMENTED, "function is not linked to a definition");
                const uint32_t def = table[op.u0];
                if (def >= lk->buffers->size()) fail(ZS_ERR_UNIMPLEMENTED, "bad link target");
                if (lk->active.count(def)) fail(ZS_ERR_UNIMPLEMENTED, "recursive function invocation");
                const Command &callee = *(*lk->buffers)[def];
                const Command &declared = *fn.functions.at(op.u0);
                if (callee.nvars != declared.nvars) fail(ZS_ERR_OTHER, "linked function's generics differ from its declaration");
                lk->active.insert(def);
                std::vector<int64_t> inner;
                res = instantiate(callee, def, g, a, dst, lk, &inner);
                lk->active.erase(def);
                // Registers of the callee's knobbed operations, for Executable::query_knob.
                for (uint32_t k = 0; k < callee.ops.size(); ++k)
                    if (inner[k] >= 0 && lk->program->alias.find({def, k}) == lk->program->alias.end())
                        lk->program->alias[{def, k}] = (uint32_t)inner[k];
            } else {
                // Typing only (CommandBuffer::invoke): the declared signature stands in.
                res = instantiate(*fn.functions.at(op.u0), 1, g, a, dst, nullptr);
            }
            // The call's result registers follow the Invoke op in `fn`.
            for (uint32_t k = 0; k < res.size() && r + 1 + k < fn.ops.size(); ++k) map[r + 1 + k] = res[k];
        } break;
        case OpKind::InvokedResult:
            if (map[r] < 0) fail(ZS_ERR_OTHER, "invoked function returned fewer results than declared");
            break;
        default:
            map[r] = replay_op(op, map, dst);
            break;
        }
    }
    if (map_out) *map_out = std::move(map);
    return outs;
}

std::vector<uint32_t> cmd_invoke(Command &c, uint32_t function, const std::vector<uint32_t> &tyvars,
                                 const std::vector<uint32_t> &args) {
    if (function >= c.functions.size()) fail(ZS_ERR_BAD_REGISTER, "no such function");
    const Command &sig = *c.functions[function];
    size_t ninputs = 0, noutputs = 0;
    for (const Op &op : sig.ops) {
        ninputs += op.kind == OpKind::Input;
        noutputs += op.kind == OpKind::Output;
    }
    if (args.size() != ninputs || tyvars.size() != (size_t)sig.nvars) fail(ZS_ERR_OTHER, "wrong number of arguments");
    std::vector<Desc> gen;
    for (uint32_t ty : tyvars) gen.push_back(ty_descriptor(c, ty));
    for (uint32_t a : args) c.describe(a);
    // The result descriptors: the signature monomorphised on a scratch buffer holding
    // stand-ins with the arguments' descriptors.
    Command scratch;
    std::vector<uint32_t> stand_ins;
    for (uint32_t a : args) stand_ins.push_back(cmd_input(scratch, c.describe(a)));
    const std::vector<uint32_t> res = instantiate(sig, 1, gen, stand_ins, scratch, nullptr);
    if (res.size() != noutputs) fail(ZS_ERR_OTHER, "function outputs differ from its signature");
    Op call{OpKind::Invoke};
    call.u0 = function;
    call.regs = args;
    call.tyvars = tyvars;
    const uint32_t at = c.push(call);
    std::vector<uint32_t> out;
    for (uint32_t k = 0; k < res.size(); ++k) {
        Op r{OpKind::InvokedResult};
        r.a = at;
        r.u0 = k;
        r.desc = scratch.describe(res[k]);
        out.push_back(c.push(r));
    }
    return out;
}

Program link_commands(const std::vector<const Command *> &buffers, const std::vector<Desc> &tys,
                      const std::vector<std::vector<uint32_t>> &links) {
    if (buffers.empty() || !buffers[0]) fail(ZS_ERR_INVALID_ARG, "no main command buffer");
    if (links.size() > buffers.size()) fail(ZS_ERR_UNIMPLEMENTED, "more link lists than command buffers");
    const Command &main = *buffers[0];
    if (tys.size() != (size_t)main.nvars) fail(ZS_ERR_OTHER, "the entry point's generics are not all given");
    for (const Desc &d : tys)
        if (!is_consistent(d)) fail(ZS_ERR_TYPE, "inconsistent descriptor for a generic parameter");
    Program tmp;
    Linking lk;
    lk.buffers = &buffers;
    lk.links = &links;
    lk.program = &tmp;
    lk.active.insert(0);
    Command flat;
    std::vector<int64_t> map;
    instantiate(main, 0, tys, {}, flat, &lk, &map);
    Program p = compile_command(flat);
    p.alias = tmp.alias;
    for (uint32_t r = 0; r < map.size(); ++r)
        if (map[r] >= 0 && map[r] != (int64_t)r) p.alias[{0u, r}] = (uint32_t)map[r];
    return p;
}

}  // namespace zs
