// lower.cpp -- Program::lower_to for CUDA (the analogue of program.rs:1304-1651 and the
// Encoder of program/encoder.rs): turns the SSA op list into raster launches.
//
// The reference emits, per op, one render pass plus a staging encode pass after it and
// a decode pass before the next op (program.rs:1486-1533).  Here each register is
// either *materialised* (a device buffer in a storage format) or *pending* (a launch
// under construction: producer + fused pixel program).  Per-pixel colour ops extend
// the pending program of their operand, so a chain of them becomes one HBM pass; a
// gather/construct/blend/resample op starts a new launch whose sources are
// materialised.  Lossy declared intermediate texels are honoured by quantising in
// registers (QUANT), so results equal the per-op semantics without the round trips.
//
// Modes: FUSED (default; FP32 intermediates that must be materialised are stored as
// FP16), PER_OP_F32 / PER_OP_F16 (one launch per op, linear RGBA intermediates: the
// plain baseline the fused executor is measured against).
#include <cmath>
#include <algorithm>
#include <cstring>
#include <sstream>

#include "zs_host.hpp"

namespace zs {

struct Pending {
    ZsRasterArgs a;
    int src_slot[ZS_MAX_SRCS] = {-1, -1, -1};
    int idx_x_slot = -1, idx_y_slot = -1, weight_slot = -1;
    int vfirst_slot = -1, vcount_slot = -1, vweight_slot = -1;
    int vimg_slot = -1, vimg_index_slot = -1, tc_weight_slot = -1;
    std::vector<std::pair<int, int>> tc_cands;   // tensor-core tiles that fit: (tile width, atoms)
    HProgram prog;
    // virt1: the gathered image's producer sources and program (evaluated per tap)
    int vsrc_slot[2] = {-1, -1};
    HProgram vprog;
    std::string label;
    // ZS_PR_LAYERS: base (src_slot[0] when has_below, else a.cons[0..3]) and the layers.
    std::vector<LayerRef> layers;
    // A knob whose parameter block feeds this launch's producer constants (or -1), and the
    // construct whose layout those constants follow.
    int knob = -1;
    OpKind knob_kind = OpKind::BufferInit;
};

struct Val {
    bool materialized = false;
    int slot = -1;
    ZsFormat fmt{};
    std::unique_ptr<Pending> pend;
};

struct Planner {
    const Program &P;
    Executable &E;
    std::vector<Val> vals;
    std::vector<int> out_slot_of;     // value register -> output slot (or -1)
    std::vector<uint32_t> remaining;  // remaining uses

    Planner(const Program &p, Executable &e) : P(p), E(e) {}

    const Desc &desc(uint32_t r) const { return P.ops[r].desc; }

    // The knob declared on register `reg` (parameter block of `len` bytes), created on first use.
    int knob_of(uint32_t reg, uint64_t len) {
        for (size_t i = 0; i < E.knobs.size(); ++i)
            if (E.knobs[i].reg == reg) return (int)i;
        KnobInfo k;
        k.reg = reg;
        k.len = len;
        E.knobs.push_back(k);
        return (int)E.knobs.size() - 1;
    }

    // Producer constants of a parameterised construct: its own parameters, or those read from a
    // buffer (CommandBuffer::with_buffer); registers the knob the constants answer to.
    void construct_params(uint32_t r, const Op &op, Pending &p, float *cons, int n) {
        if (op.param_buffer >= 0) {
            const Op &b = P.ops[op.param_buffer];
            std::vector<uint8_t> bytes(b.data);
            bytes.resize(std::max<uint64_t>(b.len, knob_param_bytes(op.kind)), 0);
            const std::vector<float> f = knob_cons(op.kind, bytes.data(), bytes.size());
            for (int k = 0; k < n && k < (int)f.size(); ++k) cons[k] = f[k];
            if (b.knob) p.knob = knob_of((uint32_t)op.param_buffer, b.len);
        } else {
            for (int k = 0; k < n; ++k) cons[k] = op.fparams[k];
            if (op.knob) p.knob = knob_of(r, knob_param_bytes(op.kind));
        }
    }

    int new_slot(SlotKind k, int w, int h, const ZsFormat &f, uint32_t reg = 0) {
        Slot s;
        s.kind = k;
        s.width = w;
        s.height = h;
        s.fmt = f;
        s.stride = (int64_t)w * f.bpp;
        s.bytes = (uint64_t)s.stride * h;
        s.reg = reg;
        E.slots.push_back(std::move(s));
        return (int)E.slots.size() - 1;
    }

    int table_slot(const void *data, size_t bytes) {
        Slot s;
        s.kind = SlotKind::Table;
        s.bytes = bytes;
        s.table.assign((const uint8_t *)data, (const uint8_t *)data + bytes);
        E.slots.push_back(std::move(s));
        return (int)E.slots.size() - 1;
    }

    ZsFormat storage_format(uint32_t reg) const {
        ZsFormat declared = format_of(desc(reg));
        if (E.mode == ZS_MODE_PER_OP_F32) return linear_f32_format();
        if (E.mode == ZS_MODE_PER_OP_F16) return linear_f16_format();
        if (declared.fast == ZS_FAST_F32X4) return linear_f16_format();   // FP16 storage
        return declared;
    }

    std::unique_ptr<Pending> new_pending(uint8_t producer, int w, int h, const std::string &label) {
        auto p = std::make_unique<Pending>();
        std::memset(&p->a, 0, sizeof(p->a));
        p->a.producer = producer;
        p->a.width = w;
        p->a.height = h;
        p->label = label;
        return p;
    }

    void set_src(Pending &p, int i, uint32_t reg) {
        Val &v = vals[reg];
        set_src_slot(p, i, v.slot);
        p.a.src[i].fmt = v.fmt;
    }

    void set_src_slot(Pending &p, int i, int slot) {
        p.src_slot[i] = slot;
        Slot &s = E.slots[slot];
        p.a.src[i].fmt = s.fmt;
        p.a.src[i].width = s.width;
        p.a.src[i].height = s.height;
        p.a.src[i].stride = s.stride;
        if (i + 1 > p.a.nsrc) p.a.nsrc = (uint8_t)(i + 1);
    }

    void emit_layers(Pending &p, int dst_slot) {
        Slot &d = E.slots[dst_slot];
        p.prog.optimise();
        while (!p.prog.ins.empty() && p.prog.ins.back().op == ZS_P_QUANT && format_equal(p.prog.ins.back().fa, d.fmt))
            p.prog.ins.pop_back();
        Step st;
        st.kind = StepKind::Layers;
        st.label = p.label;
        st.dst_slot = dst_slot;
        auto L = std::make_shared<ZsLayersArgs>();
        std::memset(L.get(), 0, sizeof(ZsLayersArgs));
        L->width = p.a.width;
        L->height = p.a.height;
        L->has_base = p.a.has_below;
        if (p.a.has_below) {
            st.base_slot = p.src_slot[0];
            L->base = p.a.src[0];
        } else {
            for (int k = 0; k < 4; ++k) L->base_color[k] = p.a.cons[k];
        }
        L->dst_stride = d.stride;
        L->dst_fmt = d.fmt;
        int nf = 0;
        auto fmt_id = [&](const ZsFormat &f) -> uint8_t {
            for (int i = 0; i < nf; ++i)
                if (format_equal(L->fmts[i], f)) return (uint8_t)i;
            if (nf >= ZS_MAX_FMTS) fail(ZS_ERR_UNIMPLEMENTED, "too many formats in one layer stack");
            L->fmts[nf] = f;
            return (uint8_t)nf++;
        };
        L->nlayers = (int32_t)p.layers.size();
        for (size_t i = 0; i < p.layers.size(); ++i) {
            const LayerRef &lr = p.layers[i];
            L->layers[i] = lr.proto;
            if (lr.quant_sample) L->layers[i].quant_sample = (uint8_t)(fmt_id(lr.sample_fmt) + 1);
            if (lr.quant_acc) L->layers[i].quant_acc = (uint8_t)(fmt_id(lr.acc_fmt) + 1);
            st.layer_slots.push_back(lr.slot);
        }
        int np = 0;
        for (const HInstr &hi : p.prog.ins) {
            if (L->prog.n >= ZS_MAX_INSTR) fail(ZS_ERR_UNIMPLEMENTED, "fused program too long");
            ZsPInstr &o = L->prog.ins[L->prog.n++];
            o.op = hi.op;
            o.a = hi.a;
            o.b = hi.b;
            o.p = (uint16_t)np;
            if (hi.op == ZS_P_MAT3) {
                for (int k = 0; k < 9; ++k) L->prog.prm[np++] = (float)hi.mat.m[k];
            } else if (hi.op == ZS_P_QUANT) {
                o.a = fmt_id(hi.fa);
            } else if (hi.op == ZS_P_TRANSMUTE) {
                o.a = fmt_id(hi.fa);
                o.b = fmt_id(hi.fb);
            } else if (hi.op == ZS_P_INJECT || hi.op == ZS_P_BLEND) {
                fail(ZS_ERR_UNIMPLEMENTED, "binary op after a layer stack");
            }
        }
        // The specialised kernel: RGBA16F bilinear layers under affine (not projective)
        // inverses, premultiplied operands, and only lossless FP32 quantisation.
        bool fast = true;
        for (int i = 0; i < L->nlayers; ++i) {
            const ZsLayer &ly = L->layers[i];
            const bool lossless_s = !ly.quant_sample || L->fmts[ly.quant_sample - 1].fast == ZS_FAST_F32X4;
            const bool lossless_a = !ly.quant_acc || L->fmts[ly.quant_acc - 1].fast == ZS_FAST_F32X4;
            fast = fast && ly.fmt.fast == ZS_FAST_F16X4 && ly.bilinear && !ly.straight && lossless_s && lossless_a &&
                   ly.inv[6] == 0.f && ly.inv[7] == 0.f && ly.inv[8] == 1.f;
        }
        L->f16_bilinear = fast ? 1 : 0;
        st.layers = L;
        st.label += " [fused layer stack, " + std::to_string(p.layers.size()) + " layers" +
                    (fast ? ", RGBA16F bilinear kernel]" : "]");
        E.steps.push_back(st);
    }

    void emit_step(Pending &p, int dst_slot) {
        if (p.a.producer == ZS_PR_LAYERS) {
            emit_layers(p, dst_slot);
            return;
        }
        Slot &d = E.slots[dst_slot];
        p.prog.optimise();
        // A trailing quantisation to the very format being stored is implied by the store.
        while (!p.prog.ins.empty() && p.prog.ins.back().op == ZS_P_QUANT && format_equal(p.prog.ins.back().fa, d.fmt))
            p.prog.ins.pop_back();
        Step st;
        st.kind = StepKind::Raster;
        st.label = p.label;
        if (p.knob >= 0) {
            KnobSite site;
            site.step = (int)E.steps.size();
            site.kind = p.knob_kind;
            E.knobs[p.knob].sites.push_back(site);
            st.label += " [knob]";
        }
        st.raster = p.a;
        st.raster.dst_stride = d.stride;
        st.raster.dst_fmt = d.fmt;
        st.dst_slot = dst_slot;
        for (int i = 0; i < ZS_MAX_SRCS; ++i) st.src_slot[i] = p.src_slot[i];
        st.idx_x_slot = p.idx_x_slot;
        st.idx_y_slot = p.idx_y_slot;
        st.weight_slot = p.weight_slot;
        st.vfirst_slot = p.vfirst_slot;
        st.vcount_slot = p.vcount_slot;
        st.vweight_slot = p.vweight_slot;
        st.vimg_slot = p.vimg_slot;
        st.vimg_index_slot = p.vimg_index_slot;
        st.tc_weight_slot = p.tc_weight_slot;
        st.tc_cands = p.tc_cands;
        // Pixel program: FP64 host program -> FP32 parameters.
        ZsPixelProgram &pp = st.raster.prog;
        std::memset(&pp, 0, sizeof(pp));
        int nf = 0;
        auto fmt_id = [&](const ZsFormat &f) -> uint8_t {
            for (int i = 0; i < nf; ++i)
                if (format_equal(st.raster.fmts[i], f)) return (uint8_t)i;
            if (nf >= ZS_MAX_FMTS) fail(ZS_ERR_UNIMPLEMENTED, "too many formats in one fused program");
            st.raster.fmts[nf] = f;
            return (uint8_t)nf++;
        };
        auto compile = [&](const HProgram &hp, ZsPixelProgram &out) {
            int np = 0;
            for (const HInstr &hi : hp.ins) {
                if (out.n >= ZS_MAX_INSTR) fail(ZS_ERR_UNIMPLEMENTED, "fused program too long");
                ZsPInstr &o = out.ins[out.n++];
                o.op = hi.op;
                o.a = hi.a;
                o.b = hi.b;
                o.p = (uint16_t)np;
                if (hi.op == ZS_P_MAT3) {
                    if (np + 9 > ZS_MAX_PARAMS) fail(ZS_ERR_UNIMPLEMENTED, "too many parameters");
                    for (int k = 0; k < 9; ++k) out.prm[np++] = (float)hi.mat.m[k];
                } else if (hi.op == ZS_P_INJECT) {
                    if (np + 8 > ZS_MAX_PARAMS) fail(ZS_ERR_UNIMPLEMENTED, "too many parameters");
                    for (int k = 0; k < 8; ++k) out.prm[np++] = (float)hi.v[k];
                } else if (hi.op == ZS_P_QUANT) {
                    o.a = fmt_id(hi.fa);
                } else if (hi.op == ZS_P_TRANSMUTE) {
                    o.a = fmt_id(hi.fa);
                    o.b = fmt_id(hi.fb);
                }
            }
        };
        compile(p.prog, pp);
        if (p.a.virt1) {
            HProgram vp = p.vprog;
            vp.optimise();
            std::memset(&st.raster.vprog, 0, sizeof(st.raster.vprog));
            compile(vp, st.raster.vprog);
            st.vsrc_slot[0] = p.vsrc_slot[0];
            st.vsrc_slot[1] = p.vsrc_slot[1];
        }
        // Gathers with no program between equal formats copy texel bytes verbatim.
        const uint8_t pr = p.a.producer;
        if (pp.n == 0 && !p.a.virt1 &&
            (pr == ZS_PR_QUAD || (pr == ZS_PR_AFFINE && !p.a.bilinear) || pr == ZS_PR_PALETTE || pr == ZS_PR_INDEX)) {
            bool same = true;
            const int gather_src = (pr == ZS_PR_QUAD || pr == ZS_PR_AFFINE) ? 1 : 0;
            same = format_equal(p.a.src[gather_src].fmt, d.fmt) && p.a.src[gather_src].fmt.bpp == d.fmt.bpp;
            if (p.a.has_below) same = same && format_equal(p.a.src[0].fmt, d.fmt);
            if ((pr == ZS_PR_QUAD || pr == ZS_PR_AFFINE) && !p.a.has_below) {
                // Uncovered pixels take the constant canvas colour: zero bytes only when
                // the colour is zero and the format stores zero as zero bytes.
                const bool zero = p.a.cons[0] == 0.f && p.a.cons[1] == 0.f && p.a.cons[2] == 0.f && p.a.cons[3] == 0.f;
                const bool plain = d.fmt.fast != ZS_FAST_GENERIC;
                same = same && zero && plain;
            }
            st.raster.raw_copy = same ? 1 : 0;
        }
        try_chain(st, p.prog);
        E.steps.push_back(st);
    }

    // M == d I + (1,1,1)^T v (every row of M - d I equal), the middle matrix of an Oklab L/C
    // scaling: M2^-1 diag(sL, sC, sC) M2 = sC I + (sL - sC) M2^-1 e1 (row 0 of M2), and
    // M2^-1 e1 = (1, 1, 1).  Checked in FP64: the rows may differ by less than 2^-24 of the
    // matrix's scale, below the rounding of the coefficients to f32 (Oklab's published M2
    // has 10 digits, so its inverse's first column is (1, 1 + 1e-8, 1 + 5e-8)).
    static bool rank1_middle(const Mat3 &m, double &d, double v[3]) {
        double scale = 0.0;
        for (double x : m.m) scale = std::max(scale, std::fabs(x));
        if (scale == 0.0) return false;
        d = m.m[0] - m.m[3];
        for (int j = 0; j < 3; ++j) {
            double col[3];
            for (int i = 0; i < 3; ++i) col[i] = m.m[3 * i + j] - (i == j ? d : 0.0);
            const double tol = scale * 0x1p-24;
            if (std::fabs(col[0] - col[1]) > tol || std::fabs(col[0] - col[2]) > tol) return false;
            v[j] = (col[0] + col[1] + col[2]) / 3.0;
        }
        return true;
    }

    // The canonical colour chain: [M] [cbrt [M]] [cube [M]] [clamp [M]], RGBA8 sRGB in/out.
    // `hp` is the FP64 form of the launch's pixel program (the matrices before rounding).
    void try_chain(Step &st, const HProgram &hp) {
        if (E.mode != ZS_MODE_FUSED) return;
        const ZsRasterArgs &a = st.raster;
        if (a.producer != ZS_PR_LOAD || a.nsrc != 1) return;
        if (a.src[0].fmt.fast != ZS_FAST_RGBA8_SRGB || a.dst_fmt.fast != ZS_FAST_RGBA8_SRGB) return;
        ZsChainArgs c;
        std::memset(&c, 0, sizeof(c));
        Mat3 mats[4] = {Mat3::identity(), Mat3::identity(), Mat3::identity(), Mat3::identity()};
        int stage = 0;   // 0: before cbrt (M_a), 1: M_b, 2: M_c, 3: M_d
        for (const HInstr &o : hp.ins) {
            if (o.op == ZS_P_MAT3) {
                // two matrices in one stage cannot happen after optimise(); guard anyway
                if (c.flags & (ZS_CHAIN_MA << stage)) return;
                mats[stage] = o.mat;
                c.flags |= ZS_CHAIN_MA << stage;
            } else if (o.op == ZS_P_CBRT && stage < 1) {
                stage = 1;
                c.flags |= ZS_CHAIN_CBRT;
            } else if (o.op == ZS_P_CUBE && stage < 2) {
                stage = 2;
                c.flags |= ZS_CHAIN_CUBE;
            } else if (o.op == ZS_P_CLAMP01 && stage < 3) {
                stage = 3;
                c.flags |= ZS_CHAIN_CLAMP;
            } else {
                return;
            }
        }
        if (a.src[0].width != a.width || a.src[0].height != a.height) return;
        for (int s = 0; s < 4; ++s)
            for (int k = 0; k < 9; ++k) c.m[s][k] = (float)mats[s].m[k];
        c.npx = (int64_t)a.width * a.height;
        // Decoded sRGB8 values are in [0, 1]; a non-negative M_a keeps the cube-root
        // arguments non-negative, so the kernel may skip the sign handling.
        bool nonneg = true;
        for (int k = 0; k < 9; ++k) nonneg = nonneg && c.m[0][k] >= 0.0f;
        if (nonneg) c.flags |= ZS_CHAIN_CBRT_NONNEG;
        double d, v[3];
        if ((c.flags & ZS_CHAIN_CBRT) && (c.flags & ZS_CHAIN_CUBE) && rank1_middle(mats[1], d, v)) {
            c.flags |= ZS_CHAIN_MB_RANK1;
            for (int j = 0; j < 3; ++j) c.mb_v[j][0] = c.mb_v[j][1] = (float)v[j];
            c.mb_d[0] = c.mb_d[1] = (float)d;
        }
        for (int s = 0; s < 4; ++s)
            for (int k = 0; k < 9; ++k) c.m2[s][k][0] = c.m2[s][k][1] = c.m[s][k];
        st.kind = StepKind::Chain;
        st.chain = c;
        st.chain_src_fast = ZS_FAST_RGBA8_SRGB;
        st.chain_dst_fast = ZS_FAST_RGBA8_SRGB;
        st.label += (c.flags & ZS_CHAIN_MB_RANK1) ? " [fused chain kernel, rank-1 L/C scaling]" : " [fused chain kernel]";
    }

    void materialize(uint32_t reg) {
        Val &v = vals[reg];
        if (v.materialized) return;
        const Desc &d = desc(reg);
        int slot;
        ZsFormat f;
        if (out_slot_of[reg] >= 0) {
            slot = out_slot_of[reg];
            f = E.slots[slot].fmt;
        } else {
            f = storage_format(reg);
            slot = new_slot(SlotKind::Intermediate, d.width, d.height, f);
        }
        emit_step(*v.pend, slot);
        v.pend.reset();
        v.materialized = true;
        v.slot = slot;
        v.fmt = f;
    }

    // Take the pending launch of `reg` to extend it, or start a LOAD launch from its buffer.
    std::unique_ptr<Pending> take(uint32_t reg, const std::string &label) {
        Val &v = vals[reg];
        if (!v.materialized && v.pend && remaining[reg] == 0 && out_slot_of[reg] < 0) {
            auto p = std::move(v.pend);
            v.materialized = true;    // consumed: nothing else may read it
            v.slot = -1;
            p->label += " + " + label;
            return p;
        }
        need(reg);
        const Desc &d = desc(reg);
        auto p = new_pending(ZS_PR_LOAD, d.width, d.height, label);
        set_src(*p, 0, reg);
        return p;
    }

    // A pixel-aligned pending value (LOAD or BLEND producer and its program) that only this
    // gather reads is not stored: the gather evaluates it at every tap (fused mode).  Plain
    // decodes of one buffer are left to need(), which forwards the buffer itself.
    bool attach_virtual(Pending &p, uint32_t reg) {
        if (E.mode != ZS_MODE_FUSED) return false;
        Val &v = vals[reg];
        if (v.materialized || !v.pend || remaining[reg] != 0 || out_slot_of[reg] >= 0) return false;
        const Pending &q = *v.pend;
        if ((q.a.producer != ZS_PR_LOAD && q.a.producer != ZS_PR_BLEND) || q.a.nsrc < 1 || q.a.nsrc > 2) return false;
        if (q.a.producer == ZS_PR_LOAD && q.a.nsrc == 1) {
            HProgram t = q.prog;
            t.optimise();
            if (t.ins.empty()) return false;
        }
        p.a.virt1 = 1;
        p.a.vproducer = q.a.producer;
        p.a.vmode = q.a.blend_mode;
        p.a.vstraight = q.a.straight;
        p.a.vnsrc = q.a.nsrc;
        p.a.vrect[0] = q.a.rect[0];
        p.a.vrect[1] = q.a.rect[1];
        for (int i = 0; i < 2; ++i) {
            p.a.vsrc[i] = q.a.src[i];
            p.vsrc_slot[i] = q.src_slot[i];
        }
        p.vprog = q.prog;
        const Desc &d = desc(reg);
        p.a.src[1].width = (int)d.width;
        p.a.src[1].height = (int)d.height;
        p.a.src[1].fmt = format_of(d);
        p.a.src[1].stride = 0;
        p.src_slot[1] = -1;
        if (p.a.nsrc < 2) p.a.nsrc = 2;
        p.label += " [evaluates " + q.label + " per tap]";
        v.pend.reset();
        v.materialized = true;     // consumed by the gather
        v.slot = -1;
        return true;
    }

    // A source operand must be readable from a buffer.  A pending value that is just the
    // decode of one buffer (LOAD with an empty program, e.g. sRGB8 -> linear FP32 whose
    // matrix folded to the identity) is forwarded to that buffer instead of being stored.
    void need(uint32_t reg) {
        Val &v = vals[reg];
        if (!v.materialized && v.pend && out_slot_of[reg] < 0 && v.pend->a.producer == ZS_PR_LOAD &&
            v.pend->a.nsrc == 1) {
            HProgram p = v.pend->prog;
            p.optimise();
            if (p.ins.empty()) {
                v.materialized = true;
                v.slot = v.pend->src_slot[0];
                v.fmt = v.pend->a.src[0].fmt;
                v.pend.reset();
                return;
            }
        }
        materialize(reg);
    }

    // A buffer holding `reg` as linear RGBA32F with tight rows (the layout custom kernels
    // read): its own buffer when it is stored that way, else a conversion launch into one.
    int f32_operand(uint32_t reg) {
        need(reg);
        const Val &v = vals[reg];
        const Slot &s = E.slots[v.slot];
        if (format_equal(v.fmt, linear_f32_format()) && s.stride == (int64_t)s.width * 16) return v.slot;
        const Desc &d = desc(reg);
        auto p = new_pending(ZS_PR_LOAD, d.width, d.height, "operand to RGBA32F");
        set_src(*p, 0, reg);
        const int slot = new_slot(SlotKind::Intermediate, d.width, d.height, linear_f32_format());
        emit_step(*p, slot);
        return slot;
    }

    // A register that is a still-pending solid colour whose program is empty (its
    // declared texel does not quantise it): its value is the constant itself.
    bool solid_value(uint32_t reg, float out[4]) {
        Val &v = vals[reg];
        if (E.mode != ZS_MODE_FUSED || v.materialized || !v.pend || v.pend->a.producer != ZS_PR_SOLID ||
            out_slot_of[reg] >= 0 || v.pend->knob >= 0)
            return false;
        HProgram p = v.pend->prog;
        p.optimise();
        // Quantising to the declared texel leaves 0 and 1 unchanged in every format.
        bool exact = true;
        for (int k = 0; k < 4; ++k) exact = exact && (v.pend->a.cons[k] == 0.0f || v.pend->a.cons[k] == 1.0f);
        for (const HInstr &i : p.ins)
            if (!(i.op == ZS_P_QUANT && exact && i.fa.fast != ZS_FAST_GENERIC)) return false;
        for (int k = 0; k < 4; ++k) out[k] = v.pend->a.cons[k];
        return true;
    }

    // blend(acc, affine(constant canvas, A, layer)) at offset 0: append the layer to a
    // layer stack instead of storing the transformed layer and the blended image.
    bool try_layer(uint32_t r, const Op &op) {
        if (E.mode != ZS_MODE_FUSED || op.rect.x != 0 || op.rect.y != 0) return false;
        Val &tv = vals[op.b];
        if (tv.materialized || !tv.pend || tv.pend->a.producer != ZS_PR_AFFINE || tv.pend->a.has_below || tv.pend->a.virt1 ||
            remaining[op.b] != 0 || out_slot_of[op.b] >= 0)
            return false;
        const Desc &d = P.ops[r].desc;
        if (desc(op.b).width != d.width || desc(op.b).height != d.height) return false;
        HProgram tp = tv.pend->prog;
        tp.optimise();
        if (tp.ins.size() > 1 || (tp.ins.size() == 1 && !(tp.ins[0].op == ZS_P_QUANT && tp.ins[0].fa.fast != ZS_FAST_GENERIC)))
            return false;
        // The accumulator side: extend its stack, start from a constant, or start from a buffer.
        std::unique_ptr<Pending> p;
        Val &av = vals[op.a];
        float solid[4];
        if (!av.materialized && av.pend && av.pend->a.producer == ZS_PR_LAYERS && remaining[op.a] == 0 &&
            out_slot_of[op.a] < 0 && av.pend->prog.ins.empty() && av.pend->layers.size() < ZS_MAX_LAYERS) {
            p = std::move(av.pend);
            av.materialized = true;
            av.slot = -1;
        } else {
            p = new_pending(ZS_PR_LAYERS, d.width, d.height, "layer stack");
            if (solid_value(op.a, solid)) {
                p->a.has_below = 0;
                for (int k = 0; k < 4; ++k) p->a.cons[k] = solid[k];
            } else {
                need(op.a);
                set_src(*p, 0, op.a);
                p->a.has_below = 1;
            }
        }
        const Pending &t = *tv.pend;
        LayerRef lr;
        lr.slot = t.src_slot[1];
        lr.proto.stride = t.a.src[1].stride;
        lr.proto.width = t.a.src[1].width;
        lr.proto.height = t.a.src[1].height;
        lr.proto.fmt = t.a.src[1].fmt;
        for (int k = 0; k < 9; ++k) lr.proto.inv[k] = t.a.aff[k];
        for (int k = 0; k < 4; ++k) lr.proto.canvas[k] = t.a.cons[k];
        lr.proto.bilinear = t.a.bilinear;
        lr.proto.mode = (uint8_t)op.u0;
        lr.proto.straight = d.alpha == ZS_ALPHA_PREMULTIPLIED ? 0 : 1;
        if (tp.ins.size() == 1) {
            lr.quant_sample = true;
            lr.sample_fmt = tp.ins[0].fa;
        }
        p->layers.push_back(lr);
        tv.pend.reset();
        tv.materialized = true;     // consumed by the stack
        tv.slot = -1;
        set_pending(r, std::move(p));
        return true;
    }

    void set_pending(uint32_t reg, std::unique_ptr<Pending> p) {
        Val &v = vals[reg];
        if (p->a.producer == ZS_PR_LAYERS && p->prog.ins.empty() && !p->layers.empty()) {
            // The declared texel of the blended result quantises the accumulator.
            ZsFormat declared = format_of(desc(reg));
            if (!format_is_lossless_f32(declared)) {
                if (declared.fast == ZS_FAST_GENERIC) {
                    p->prog.quant(declared);          // rare: ends the stack
                } else {
                    p->layers.back().quant_acc = true;
                    p->layers.back().acc_fmt = declared;
                }
            }
            v.pend = std::move(p);
            v.materialized = false;
            return;
        }
        // The declared texel of the op's result bounds its precision (faithful semantics).
        ZsFormat declared = format_of(desc(reg));
        if (!format_is_lossless_f32(declared)) p->prog.quant(declared);
        v.pend = std::move(p);
        v.materialized = false;
        if (E.mode != ZS_MODE_FUSED) materialize(reg);
    }

    void use(uint32_t reg) {
        if (remaining[reg] > 0) remaining[reg]--;
    }

    void run() {
        const size_t n = P.ops.size();
        vals.resize(n);
        out_slot_of.assign(n, -1);
        remaining = P.uses;
        // Output slots first (declaration order).
        for (size_t k = 0; k < P.output_regs.size(); ++k) {
            uint32_t oreg = P.output_regs[k];
            uint32_t src = P.ops[oreg].a;
            const Desc &d = desc(src);
            int s = new_slot(SlotKind::Output, d.width, d.height, format_of(d), oreg);
            E.output_slot.push_back(s);
            E.output_regs.push_back(oreg);
            E.output_desc.push_back(d);
            if (out_slot_of[src] < 0 && P.ops[src].kind != OpKind::Input) out_slot_of[src] = s;
        }
        for (uint32_t r = 0; r < n; ++r) {
            const Op &op = P.ops[r];
            const Desc &d = op.desc;
            switch (op.kind) {
            case OpKind::Input: {
                int s = new_slot(SlotKind::Input, d.width, d.height, format_of(d), r);
                E.input_slot.push_back(s);
                E.input_regs.push_back(r);
                E.input_desc.push_back(d);
                vals[r].materialized = true;
                vals[r].slot = s;
                vals[r].fmt = format_of(d);
            } break;
            case OpKind::Output: {
                uint32_t src = op.a;
                int slot = out_slot_of[src];
                use(src);
                if (slot >= 0 && !vals[src].materialized) {
                    materialize(src);
                    break;
                }
                // The value lives elsewhere (an input or a shared buffer): copy / convert.
                need(src);
                int os = -1;
                for (size_t k = 0; k < E.output_regs.size(); ++k)
                    if (E.output_regs[k] == r) os = E.output_slot[k];
                if (os == vals[src].slot) break;
                if (format_equal(vals[src].fmt, E.slots[os].fmt)) {
                    // The same texels: a byte copy (row by row when the strides differ, as for
                    // a from_buffer image with 256-byte aligned rows).
                    Step st;
                    st.kind = StepKind::Copy;
                    st.src_slot[0] = vals[src].slot;
                    st.dst_slot = os;
                    const Slot &ss = E.slots[vals[src].slot], &ds = E.slots[os];
                    st.copy_bytes = ds.bytes;
                    if (ss.stride != ds.stride) {
                        st.copy_bytes = (uint64_t)ds.width * ds.fmt.bpp;
                        st.copy_rows = (uint64_t)ds.height;
                        st.copy_src_pitch = ss.stride;
                        st.copy_dst_pitch = ds.stride;
                    }
                    st.label = "copy to output";
                    E.steps.push_back(st);
                } else {
                    auto p = new_pending(ZS_PR_LOAD, d.width, d.height, "store output");
                    set_src(*p, 0, src);
                    emit_step(*p, os);
                }
            } break;
            case OpKind::ColorConvert:
            case OpKind::ChromaticAdaptation:
            case OpKind::ColorMatrix: {
                use(op.a);
                auto p = take(op.a, op.kind == OpKind::ColorConvert ? "color_convert"
                                    : op.kind == OpKind::ColorMatrix ? "color_matrix" : "chromatic_adaptation");
                for (const HInstr &i : op.prog.ins) p->prog.ins.push_back(i);
                set_pending(r, std::move(p));
            } break;
            case OpKind::Extract: {
                use(op.a);
                auto p = take(op.a, "extract");
                set_pending(r, std::move(p));
            } break;
            case OpKind::Transmute: {
                use(op.a);
                Val &sv = vals[op.a];
                ZsFormat from = format_of(desc(op.a)), to = format_of(d);
                if (sv.materialized && sv.slot >= 0 && format_equal(sv.fmt, from)) {
                    // Pure reinterpretation of a buffer in its declared format: no work.
                    vals[r].materialized = true;
                    vals[r].slot = sv.slot;
                    vals[r].fmt = to;
                    break;
                }
                auto p = take(op.a, "transmute");
                HInstr t;
                t.op = ZS_P_TRANSMUTE;
                t.fa = from;
                t.fb = to;
                p->prog.ins.push_back(t);
                set_pending(r, std::move(p));
            } break;
            case OpKind::Inject: {
                use(op.a);
                use(op.b);
                need(op.b);
                auto p = take(op.a, "inject");
                if (p->a.producer != ZS_PR_LOAD || p->a.nsrc != 1) {
                    // A second pixel-aligned operand cannot join a gather: store it first.
                    const Desc &bd = desc(op.a);
                    ZsFormat f = storage_format(op.a);
                    int slot = new_slot(SlotKind::Intermediate, bd.width, bd.height, f);
                    emit_step(*p, slot);
                    p = new_pending(ZS_PR_LOAD, d.width, d.height, "inject");
                    set_src_slot(*p, 0, slot);
                }
                set_src(*p, 1, op.b);
                for (const HInstr &i : op.prog.ins) p->prog.ins.push_back(i);
                set_pending(r, std::move(p));
            } break;
            case OpKind::Crop:
            case OpKind::Inscribe:
            case OpKind::InscribePlaced: {
                const bool crop = op.kind == OpKind::Crop;
                if (!crop) { use(op.a); need(op.a); }
                uint32_t above = crop ? op.a : op.b;
                use(above);
                need(above);
                auto p = new_pending(ZS_PR_QUAD, d.width, d.height, crop ? "crop" : "inscribe");
                if (!crop) {
                    set_src(*p, 0, op.a);
                    p->a.has_below = 1;
                }
                set_src(*p, 1, above);
                const Desc &ad = desc(above);
                if (crop) {
                    p->a.rect[0] = 0; p->a.rect[1] = 0; p->a.rect[2] = (int)d.width; p->a.rect[3] = (int)d.height;
                    p->a.sel[0] = (int)op.rect.x; p->a.sel[1] = (int)op.rect.y;
                    p->a.sel[2] = (int)op.rect.max_x; p->a.sel[3] = (int)op.rect.max_y;
                } else {
                    p->a.rect[0] = (int)op.rect.x; p->a.rect[1] = (int)op.rect.y;
                    p->a.rect[2] = (int)op.rect.max_x; p->a.rect[3] = (int)op.rect.max_y;
                    p->a.sel[0] = 0; p->a.sel[1] = 0; p->a.sel[2] = (int)ad.width; p->a.sel[3] = (int)ad.height;
                }
                set_pending(r, std::move(p));
            } break;
            case OpKind::Affine: {
                use(op.a);
                use(op.b);
                auto p = new_pending(ZS_PR_AFFINE, d.width, d.height, op.u0 ? "affine bilinear" : "affine nearest");
                const bool virt = attach_virtual(*p, op.b);
                if (!virt) need(op.b);
                float solid[4];
                if (solid_value(op.a, solid)) {
                    // Painting onto a constant canvas: the canvas is never stored.
                    p->a.has_below = 0;
                    for (int k = 0; k < 4; ++k) p->a.cons[k] = solid[k];
                    p->label = "solid canvas + " + p->label;
                    p->a.nsrc = 2;
                } else {
                    need(op.a);
                    set_src(*p, 0, op.a);
                    p->a.has_below = 1;
                }
                if (!virt) set_src(*p, 1, op.b);
                p->a.bilinear = (uint8_t)op.u0;
                Mat3 fwd{};
                for (int k = 0; k < 9; ++k) fwd.m[k] = op.fparams[k];
                Mat3 inv = fwd.inverse();
                for (int k = 0; k < 9; ++k) p->a.aff[k] = (float)inv.m[k];
                set_pending(r, std::move(p));
            } break;
            case OpKind::Palette: {
                use(op.a);
                use(op.b);
                need(op.a);
                need(op.b);
                auto p = new_pending(ZS_PR_PALETTE, d.width, d.height, "palette");
                set_src(*p, 0, op.a);
                set_src(*p, 1, op.b);
                for (int k = 0; k < 8; ++k) p->a.cons[k] = op.fparams[k];
                set_pending(r, std::move(p));
            } break;
            case OpKind::Bilinear: {
                auto p = new_pending(ZS_PR_BILINEAR, d.width, d.height, "bilinear");
                p->knob_kind = OpKind::Bilinear;
                construct_params(r, op, *p, p->a.cons, 24);
                set_pending(r, std::move(p));
            } break;
            case OpKind::Solid: {
                auto p = new_pending(ZS_PR_SOLID, d.width, d.height, "solid");
                p->knob_kind = OpKind::Solid;
                construct_params(r, op, *p, p->a.cons, 4);
                set_pending(r, std::move(p));
            } break;
            case OpKind::Resize: {
                use(op.a);
                need(op.a);
                const Desc &sd = desc(op.a);
                auto p = new_pending(ZS_PR_INDEX, d.width, d.height, "resize");
                set_src(*p, 0, op.a);
                std::vector<int32_t> ix(d.width), iy(d.height);
                resize_index(sd.width, d.width, ix.data());
                resize_index(sd.height, d.height, iy.data());
                p->idx_x_slot = table_slot(ix.data(), ix.size() * 4);
                p->idx_y_slot = table_slot(iy.data(), iy.size() * 4);
                set_pending(r, std::move(p));
            } break;
            case OpKind::ResizeFiltered: {
                use(op.a);
                need(op.a);
                const Desc &sd = desc(op.a);
                if (E.mode == ZS_MODE_FUSED && try_resample_2d(r, op, sd, d)) break;
                // Pass 1: horizontal, into an intermediate (dst width x src height).
                auto h = new_pending(ZS_PR_RESAMPLE_H, d.width, sd.height, "resample horizontal");
                set_src(*h, 0, op.a);
                add_weights(*h, sd.width, d.width, op.u0);
                ZsFormat mid = E.mode == ZS_MODE_PER_OP_F32 ? linear_f32_format() : linear_f16_format();
                int ms = new_slot(SlotKind::Intermediate, d.width, sd.height, mid);
                emit_step(*h, ms);
                // Pass 2: vertical, pending so that following per-pixel ops fuse into it.
                auto v = new_pending(ZS_PR_RESAMPLE_V, d.width, d.height, "resample vertical");
                v->src_slot[0] = ms;
                v->a.src[0].fmt = mid;
                v->a.src[0].width = (int)d.width;
                v->a.src[0].height = (int)sd.height;
                v->a.src[0].stride = (int64_t)d.width * mid.bpp;
                v->a.nsrc = 1;
                add_weights(*v, sd.height, d.height, op.u0);
                set_pending(r, std::move(v));
            } break;
            case OpKind::Normal2d: {
                auto p = new_pending(ZS_PR_NORMAL2D, d.width, d.height, "distribution normal2d");
                p->knob_kind = OpKind::Normal2d;
                construct_params(r, op, *p, p->a.cons, 7);
                set_pending(r, std::move(p));
            } break;
            case OpKind::BufferInit:
                break;   // bytes only: every from_buffer view of it becomes a constant image
            case OpKind::FromBuffer: {
                // CommandBuffer::from_buffer (command.rs:937-968): the buffer's bytes as an image
                // with 256-byte aligned rows, uploaded once with the executable's tables.
                use(op.a);
                const Op &b = P.ops[op.a];
                const ZsFormat f = format_of(d);
                const int64_t stride = (int64_t)((((uint64_t)d.width * f.bpp) + 255) & ~(uint64_t)255);
                std::vector<uint8_t> bytes((size_t)stride * d.height, 0);
                if (!b.data.empty()) std::memcpy(bytes.data(), b.data.data(), std::min(bytes.size(), b.data.size()));
                const int s = table_slot(bytes.data(), bytes.size());
                if (b.knob) {
                    KnobSite site;
                    site.slot = s;
                    site.kind = OpKind::BufferInit;
                    E.knobs[knob_of(op.a, b.len)].sites.push_back(site);
                }
                Slot &sl = E.slots[s];
                sl.width = d.width;
                sl.height = d.height;
                sl.fmt = f;
                sl.stride = stride;
                vals[r].materialized = true;
                vals[r].slot = s;
                vals[r].fmt = f;
            } break;
            case OpKind::FractalNoise: {
                auto p = new_pending(ZS_PR_FRACTAL, d.width, d.height, "distribution fractal noise");
                p->knob_kind = OpKind::FractalNoise;
                construct_params(r, op, *p, p->a.cons, 5);
                // The rotation between octaves, 2 mat3(cos .5, sin .5, 1, -sin .5, cos .5, 1, 0, 0, 1)
                // (fractal_noise.frag), its constants rounded to f32 before the doubling.
                p->a.cons[5] = 2.0f * (float)std::cos(0.5);
                p->a.cons[6] = 2.0f * (float)std::sin(0.5);
                set_pending(r, std::move(p));
            } break;
            case OpKind::Derivative: {
                use(op.a);
                need(op.a);
                auto p = new_pending(ZS_PR_BOX3, d.width, d.height, "derivative");
                set_src(*p, 0, op.a);
                for (int k = 0; k < 9; ++k) p->a.cons[k] = op.fparams[k];
                set_pending(r, std::move(p));
            } break;
            case OpKind::Dynamic: {
                // A custom kernel: operands as linear RGBA32F buffers, result into an RGBA32F
                // buffer, then read back like any stored value (its declared texel quantises it).
                int srcs[2] = {-1, -1};
                for (uint32_t i = 0; i < op.u0; ++i) {
                    const uint32_t reg = i == 0 ? op.a : op.b;
                    use(reg);
                    srcs[i] = f32_operand(reg);
                }
                const int out = new_slot(SlotKind::Intermediate, d.width, d.height, linear_f32_format());
                Step st;
                st.kind = StepKind::Dynamic;
                st.dyn_op = op.dyn_op;
                st.src_slot[0] = srcs[0];
                st.src_slot[1] = srcs[1];
                st.dst_slot = out;
                if (!op.data.empty()) st.dyn_uniform_slot = table_slot(op.data.data(), op.data.size());
                st.label = "custom op " + std::to_string(op.dyn_op);
                E.steps.push_back(st);
                auto p = new_pending(ZS_PR_LOAD, d.width, d.height, "custom op result");
                set_src_slot(*p, 0, out);
                set_pending(r, std::move(p));
            } break;
            case OpKind::Blend: {
                use(op.a);
                use(op.b);
                if (try_layer(r, op)) break;
                need(op.a);
                need(op.b);
                auto p = new_pending(ZS_PR_BLEND, d.width, d.height, "blend");
                set_src(*p, 0, op.a);
                set_src(*p, 1, op.b);
                p->a.rect[0] = (int)op.rect.x;
                p->a.rect[1] = (int)op.rect.y;
                p->a.blend_mode = (uint8_t)op.u0;
                p->a.straight = d.alpha == ZS_ALPHA_PREMULTIPLIED ? 0 : 1;
                set_pending(r, std::move(p));
            } break;
            }
        }
        // Anything still pending with an output slot (defensive).
        for (uint32_t r = 0; r < n; ++r)
            if (!vals[r].materialized && vals[r].pend && out_slot_of[r] >= 0) materialize(r);
    }

    // The reference's resize (command.rs:1675-1702): a bilinear grid holding u at pixel
    // centres, stored as truncated 8-bit staged texels, decoded as q/255, then palette.frag
    // with the 0.5/size bias and nearest sampling -- all f32.
    static void resize_index(uint32_t src_len, uint32_t dst_len, int32_t *index) {
        volatile float fdst = (float)dst_len, fsrc = (float)src_len;
        for (uint32_t x = 0; x < dst_len; ++x) {
            volatile float u = ((float)x + 0.5f) / fdst;
            volatile float scaled = u * 255.0f;
            uint32_t q = (uint32_t)scaled;
            volatile float basis = (float)q / 255.0f;
            volatile float bias = 0.5f / fdst;
            volatile float t = basis + bias;
            volatile float pos = t * fsrc;
            int32_t ix = (int32_t)std::floor((float)pos);
            if (ix < 0) ix = 0;
            if (ix > (int32_t)src_len - 1) ix = (int32_t)src_len - 1;
            index[x] = ix;
        }
    }

    // Widest source span (first tap of the tile's first output .. last tap of its last)
    // over the tiles of one axis, or -1 when the windows are not monotone (a tile's span
    // would then not cover every window inside it).
    static int tile_span(const std::vector<int32_t> &first, const std::vector<int32_t> &count, int tile) {
        const int n = (int)first.size();
        for (int i = 1; i < n; ++i)
            if (first[i] < first[i - 1] || first[i] + count[i] < first[i - 1] + count[i - 1]) return -1;
        int span = 0;
        for (int t0 = 0; t0 < n; t0 += tile) {
            const int t1 = std::min(t0 + tile, n) - 1;
            span = std::max(span, first[t1] + count[t1] - first[t0]);
        }
        return span;
    }

    // resize_filtered as one tiled launch (k_resample.cu): the horizontally filtered rows
    // stay in shared memory, so no intermediate image is stored.
    bool try_resample_2d(uint32_t r, const Op &op, const Desc &sd, const Desc &d) {
        std::vector<int32_t> hf, hc, vf, vc;
        std::vector<float> hw, vw;
        const int htaps = resample_weights(sd.width, d.width, op.u0, hf, hc, hw);
        const int vtaps = resample_weights(sd.height, d.height, op.u0, vf, vc, vw);
        const int span = tile_span(hf, hc, ZS_RS_TW);
        if (span < 0 || tile_span(vf, vc, ZS_RS_TH) < 0) return false;
        // Two staged batches of rows, the filtered-row buffers and the tile's weights
        // (at the tallest tile) must fit one CTA.
        const size_t bpp = vals[op.a].fmt.bpp;
        const size_t rowbytes = (size_t)ZS_RS_ROWBYTES((size_t)span, bpp);
        const size_t weights = 4 * (ZS_RS_TW * (size_t)(htaps | 1) + ZS_RS_TH * (size_t)vtaps) + 32;
        if (2 * ZS_RS_RB * rowbytes + 2 * ZS_RS_RB * (ZS_RS_TW + 1) * 16 + weights + 16 > ZS_RS_MAX_SMEM) return false;
        // Tile height: the tallest that still leaves several tiles per CTA slot (fewer
        // source rows are then re-read as the vertical filter halo of the next tile).
        const int tiles_x = ((int)d.width + ZS_RS_TW - 1) / ZS_RS_TW;
        int th = 8;
        for (int cand : {32, 16})
            if ((int64_t)tiles_x * (((int)d.height + cand - 1) / cand) >= 6 * 152) {
                th = cand;
                break;
            }
        auto p = new_pending(ZS_PR_RESAMPLE_2D, d.width, d.height, "resample 2d");
        set_src(*p, 0, op.a);
        p->a.tile_rows = th;
        // Horizontal tables padded with zero rows to a multiple of 32 output columns: the
        // tensor-core kernel copies whole tiles of them into shared memory.
        const size_t padded = (d.width + 31) / 32 * 32;
        std::vector<int32_t> hfp(hf), hcp(hc);
        std::vector<float> hwp(hw);
        hfp.resize(padded, 0);
        hcp.resize(padded, 0);
        hwp.resize(padded * (size_t)htaps, 0.f);
        p->idx_x_slot = table_slot(hfp.data(), hfp.size() * 4);
        p->idx_y_slot = table_slot(hcp.data(), hcp.size() * 4);
        p->weight_slot = table_slot(hwp.data(), hwp.size() * 4);
        p->vfirst_slot = table_slot(vf.data(), vf.size() * 4);
        p->vcount_slot = table_slot(vc.data(), vc.size() * 4);
        p->vweight_slot = table_slot(vw.data(), vw.size() * 4);
        p->a.taps = htaps;
        p->a.vtaps = vtaps;
        p->a.max_span = span;
        const Slot &ss = E.slots[vals[op.a].slot];
        if (!(E.flags & ZS_CAP_SIMT_RESAMPLE) && vals[op.a].fmt.fast == ZS_FAST_F16X4 && ss.stride % 16 == 0 &&
            htaps <= 64)
            plan_resample_tc(*p, hf, hc, hw, htaps, vf, vc, vw, vtaps, d);
        set_pending(r, std::move(p));
        return true;
    }

    // IEEE binary16 bits of `f`, round to nearest even (subnormals kept).
    static uint16_t f32_to_f16_bits(float f) {
        uint32_t x;
        std::memcpy(&x, &f, 4);
        const uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7FFFFFFFu;
        if (ax >= 0x7F800000u) return (uint16_t)(sign | 0x7C00u | (ax > 0x7F800000u ? 0x200u : 0u));
        const int e = (int)(ax >> 23) - 127 + 15;
        uint32_t mant = ax & 0x7FFFFFu;
        if (e >= 31) return (uint16_t)(sign | 0x7C00u);
        if (e <= 0) {
            if (e < -10) return (uint16_t)sign;
            mant |= 0x800000u;
            const int shift = 14 - e;
            uint32_t h = mant >> shift;
            const uint32_t rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
            if (rem > half || (rem == half && (h & 1u))) ++h;
            return (uint16_t)(sign | h);
        }
        uint32_t h = ((uint32_t)e << 10) | (mant >> 13);
        const uint32_t rem = mant & 0x1FFFu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }

    // Tensor-core plan of a resample (k_resample_tc.cu): the widest tile of output columns
    // whose staged source columns (from an even column, 4 f16 values each) fit N <= 256,
    // and per band of 128 output rows the vertical weights as f16 band matrices, one
    // 128 x 64 chunk per 64 source rows, laid out as the MMA reads them (K-major rows of
    // 128 bytes, 16-byte chunk c of row m stored at chunk c ^ (m % 8)).
    void plan_resample_tc(Pending &p, const std::vector<int32_t> &hf, const std::vector<int32_t> &hc,
                          const std::vector<float> &hw, int htaps, const std::vector<int32_t> &vf,
                          const std::vector<int32_t> &vc, const std::vector<float> &vw, int vtaps, const Desc &d) {
        const int dw = (int)d.width, dh = (int)d.height;
        // Prefer tiles whose span fits 4 atoms (two accumulators: the epilogue of one tile
        // overlaps the MMAs of the next), else up to 8 atoms (one 512-column accumulator).
        int tw = 0, span = 0;
        std::vector<std::pair<int, int>> cands;      // every tile width that fits 8 atoms
        for (int cand : {32, 16, 8}) {
            int sp = 0;
            for (int x0 = 0; x0 < dw; x0 += cand) {
                const int x1 = std::min(x0 + cand, dw) - 1;
                sp = std::max(sp, hf[x1] + hc[x1] - (hf[x0] & ~1));
            }
            if (sp * 4 <= 64 * ZS_TC_MAX_ATOMS) cands.push_back({cand, (sp * 4 + 63) / 64});
        }
        for (int max_atoms : {4, ZS_TC_MAX_ATOMS}) {
            for (const auto &c : cands)
                if (c.second <= max_atoms) {
                    tw = c.first;
                    span = c.second * 64 / 4;
                    break;
                }
            if (tw) break;
        }
        if (!tw) return;
        p.tc_cands = cands;
        const int bands = (dh + ZS_TC_M - 1) / ZS_TC_M;
        std::vector<int32_t> index(2 * (size_t)bands);
        std::vector<uint16_t> img;
        for (int b = 0; b < bands; ++b) {
            const int oy0 = b * ZS_TC_M, y1 = std::min(oy0 + ZS_TC_M, dh) - 1;
            const int rbase = vf[oy0], rend = vf[y1] + vc[y1];
            const int nk = (rend - rbase + ZS_TC_K - 1) / ZS_TC_K;
            index[2 * b] = (int32_t)(img.size() / (ZS_TC_M * ZS_TC_K));
            index[2 * b + 1] = nk;
            for (int kc = 0; kc < nk; ++kc) {
                const size_t base = img.size();
                img.resize(base + (size_t)ZS_TC_M * ZS_TC_K, 0);
                for (int m = 0; m < ZS_TC_M && oy0 + m <= y1; ++m) {
                    const int oy = oy0 + m;
                    for (int k = 0; k < ZS_TC_K; ++k) {
                        const int t = rbase + ZS_TC_K * kc + k - vf[oy];
                        if (t < 0 || t >= vc[oy]) continue;
                        const size_t e = (size_t)m * ZS_TC_K + (size_t)((((k >> 3) ^ (m & 7)) << 3) | (k & 7));
                        img[base + e] = f32_to_f16_bits(vw[(size_t)oy * vtaps + t]);
                    }
                }
            }
        }
        p.vimg_slot = table_slot(img.data(), img.size() * 2);
        p.vimg_index_slot = table_slot(index.data(), index.size() * 4);
        // Horizontal weights with rows of a multiple of 4 taps (zeros after each output's
        // count), so that the epilogue reads four weights per 16-byte shared load; padded with
        // zero rows to a multiple of 32 output columns like the tap windows.
        const int taps4 = (htaps + 3) & ~3;
        const size_t padded = ((size_t)dw + 31) / 32 * 32;
        std::vector<float> hw4(padded * (size_t)taps4, 0.f);
        for (int x = 0; x < dw; ++x)
            for (int t = 0; t < htaps; ++t) hw4[(size_t)x * taps4 + t] = hw[(size_t)x * htaps + t];
        p.tc_weight_slot = table_slot(hw4.data(), hw4.size() * 4);
        p.a.tc_taps = taps4;
        p.a.tc_tw = tw;
        p.a.tc_atoms = (span * 4 + 63) / 64;   // the candidate's atoms (span rounded to atoms above)
        p.label = "resample 2d [tensor cores: f16 band matrices, FP32 accumulation]";
    }

    void add_weights(Pending &p, uint32_t src_len, uint32_t dst_len, uint32_t filter) {
        std::vector<int32_t> first, count;
        std::vector<float> w;
        int taps = resample_weights(src_len, dst_len, filter, first, count, w);
        p.idx_x_slot = table_slot(first.data(), first.size() * 4);
        p.idx_y_slot = table_slot(count.data(), count.size() * 4);
        p.weight_slot = table_slot(w.data(), w.size() * 4);
        p.a.taps = taps;
    }

    // Separable filter weights, FP64-normalised (box = area coverage, Lanczos-3, triangle);
    // output pixel i is centred at (i + 0.5) * src/dst; the kernel widens by the downscale
    // factor; taps outside the image are dropped and the rest renormalised.
    static int resample_weights(uint32_t src_len, uint32_t dst_len, uint32_t filter, std::vector<int32_t> &first,
                                std::vector<int32_t> &count, std::vector<float> &weights) {
        const double s = (double)src_len / (double)dst_len, f = s > 1.0 ? s : 1.0;
        const double R = filter == 1 ? 3.0 : (filter == 2 ? 1.0 : 0.5);
        const double r = R * f;
        const int taps = (int)std::ceil(2.0 * R * f) + 2;
        first.assign(dst_len, 0);
        count.assign(dst_len, 0);
        weights.assign((size_t)dst_len * taps, 0.0f);
        std::vector<double> w(taps);
        for (uint32_t i = 0; i < dst_len; ++i) {
            const double c = ((double)i + 0.5) * s;
            int lo = (int)std::floor(c - r), hi = (int)std::ceil(c + r);
            if (lo < 0) lo = 0;
            if (hi > (int)src_len) hi = (int)src_len;
            int n = 0, start = -1;
            double sum = 0.0;
            for (int j = lo; j < hi && n < taps; ++j) {
                double v;
                if (filter == 0) {
                    double a = c - 0.5 * f, b = c + 0.5 * f;
                    double ov = std::fmin(b, j + 1.0) - std::fmax(a, (double)j);
                    v = ov > 0 ? ov : 0.0;
                } else {
                    double t = (j + 0.5 - c) / f;
                    if (filter == 1) {
                        auto sinc = [](double x) {
                            if (std::fabs(x) < 1e-12) return 1.0;
                            double px = 3.14159265358979323846 * x;
                            return std::sin(px) / px;
                        };
                        v = std::fabs(t) < 3.0 ? sinc(t) * sinc(t / 3.0) : 0.0;
                    } else {
                        v = std::fabs(t) < 1.0 ? 1.0 - std::fabs(t) : 0.0;
                    }
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
                int j = (int)std::floor(c);
                if (j > (int)src_len - 1) j = (int)src_len - 1;
                start = j;
                n = 1;
                w[0] = 1.0;
                sum = 1.0;
            }
            for (int t = 0; t < n; ++t) weights[(size_t)i * taps + t] = (float)(w[t] / sum);
            first[i] = start;
            count[i] = n;
        }
        return taps;
    }
};

std::unique_ptr<Executable> lower(const Program &prog, const zs_capabilities &caps) {
    auto E = std::make_unique<Executable>();
    E->device = caps.device;
    E->mode = caps.mode;
    E->use_graph = caps.use_graph != 0;
    E->flags = caps.flags;
    if (caps.mode > ZS_MODE_PER_OP_F16) fail(ZS_ERR_INVALID_ARG, "unknown lowering mode");
    Planner pl(prog, *E);
    pl.run();
    std::ostringstream os;
    os << "executable: " << E->steps.size() << " launches, mode " << E->mode << "\n";
    for (size_t i = 0; i < E->steps.size(); ++i) {
        const Step &s = E->steps[i];
        os << "  [" << i << "] "
           << (s.kind == StepKind::Chain ? "chain" : s.kind == StepKind::Copy ? "copy"
               : s.kind == StepKind::Layers ? "layers" : s.kind == StepKind::Dynamic ? "custom" : "raster")
           << " " << s.label << " -> slot " << s.dst_slot;
        if (s.kind == StepKind::Raster) os << " (" << s.raster.width << "x" << s.raster.height << ", " << s.raster.prog.n
                                           << " ops" << (s.raster.raw_copy ? ", raw" : "") << ")";
        os << "\n";
    }
    E->plan_text = os.str();
    return E;
}

}  // namespace zs
