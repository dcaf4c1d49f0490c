// zs_host.hpp -- host-side model of the executor: descriptors, command buffer,
// program, lowered executable and runtime objects behind the C ABI.
//
// Mirrors the reference's Rust API shape (lib/zosimos/src/command.rs CommandBuffer,
// Linker; program.rs Program::lower_to; run.rs Executable / Environment /
// Execution / Retire; pool.rs Pool) with a CUDA runtime underneath.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../../include/zosimos.h"
#include "../zs_kernels.h"
#include "../zs_shared.h"

namespace zs {

// ---------------------------------------------------------------- errors

struct Error {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string &msg);
void check_cuda(cudaError_t e, const char *what);
void set_last_error(const std::string &msg);

// ---------------------------------------------------------------- descriptors

using Desc = zs_descriptor;

uint32_t texel_bytes(uint32_t bits);
uint32_t channel_count_bits(uint32_t bits);
uint32_t channel_count_parts(uint32_t parts);
bool is_consistent(const Desc &d);
uint64_t row_bytes(const Desc &d);      // width * texel bytes
uint64_t host_stride(const Desc &d);    // row_stride or tight
uint64_t host_len(const Desc &d);
bool same_chroma(const Desc &a, const Desc &b);   // texel + colour equal (descriptor_chroma)
ZsFormat format_of(const Desc &d);
bool format_is_lossless_f32(const ZsFormat &f);
bool format_equal(const ZsFormat &a, const ZsFormat &b);
ZsFormat linear_f32_format();
ZsFormat linear_f16_format();
std::string describe(const Desc &d);

// ---------------------------------------------------------------- colour matrices (FP64)

struct Mat3 {
    double m[9];
    static Mat3 identity();
    static Mat3 diag(double a, double b, double c);
    Mat3 operator*(const Mat3 &o) const;
    Mat3 inverse() const;
    bool is_identity(double tol = 1e-14) const;
};

Mat3 rgb_to_xyz(uint32_t primaries, uint32_t whitepoint);
void whitepoint_xyz(uint32_t whitepoint, double out[3]);
bool adaptation_matrix(uint32_t method, uint32_t src_wp, uint32_t dst_wp, Mat3 &out);
extern const Mat3 kOklabM1, kOklabM2, kCat02, kHpe;

// ---------------------------------------------------------------- host pixel program

struct HInstr {
    uint8_t op = ZS_P_NOP;
    uint8_t a = 0, b = 0;
    Mat3 mat{};                 // MAT3
    double v[8] = {0};          // INJECT select/weights
    ZsFormat fa{}, fb{};        // QUANT / TRANSMUTE formats
};

struct HProgram {
    std::vector<HInstr> ins;
    void mat(const Mat3 &m);
    void op(uint8_t o);
    void quant(const ZsFormat &f);
    void optimise();            // fold matrices (FP64), drop identities and no-op quantisation
};

// ---------------------------------------------------------------- command buffer

enum class OpKind {
    Input, Output, Crop, ColorConvert, ChromaticAdaptation, ColorMatrix, Extract, Inject,
    Transmute, Inscribe, InscribePlaced, Palette, Bilinear, Solid, Affine, Resize,
    ResizeFiltered, Blend, Derivative, Normal2d, FractalNoise, BufferInit, FromBuffer, Dynamic,
    Invoke, InvokedResult
};

struct Op {
    OpKind kind;
    uint32_t a = 0, b = 0;       // operand registers
    Desc desc{};                 // result descriptor
    zs_rect rect{};
    float fparams[24] = {0};
    uint32_t u0 = 0, u1 = 0;     // sampling / filter / mode / channels
    int32_t i0 = -1, i1 = -1;
    HProgram prog;               // per-pixel semantics of colour ops
    std::vector<uint8_t> data;   // BufferInit: initial bytes (zero-extended to `len`)
    uint64_t len = 0;            // BufferInit: buffer size in bytes
    uint32_t dyn_op = 0;         // Dynamic: registered op id; u0 = number of operands (0, 1, 2)
    int32_t generic_var = -1;    // Input: the descriptor variable it is declared with (input_generic)
    std::vector<uint32_t> regs;  // Invoke: argument registers
    std::vector<uint32_t> tyvars;// Invoke: descriptor variables given for the callee's generics
    bool knob = false;           // WithKnob: the parameters can be replaced at run time
    int32_t param_buffer = -1;   // WithBuffer: parameters read from this buffer register
};

// Bytes of the parameter block of a knob-capable op (the reference's uniform layouts):
// bilinear 6 vec4, solid_rgba vec4, distribution_normal2d 8 f32, fractal noise
// (vec2, f32, f32, u32) aligned to 8; 0 for ops that take no knob.
uint64_t knob_param_bytes(OpKind kind);
// Producer constants (ZsRasterArgs::cons) of a parameter block; throws on a bad block.
std::vector<float> knob_cons(OpKind kind, const uint8_t *data, uint64_t len);

// A descriptor variable of a command buffer (command.rs DescriptorVar): a generic parameter
// (var >= 0, its descriptor a placeholder until instantiation) or the descriptor of a register.
struct TyVar {
    int32_t var = -1;
    int32_t reg = -1;
    int32_t base = -1;           // derive_descriptor: the variable this one modifies
    uint32_t width = 0, height = 0;   // derive_descriptor: the replaced size (0: kept)
};

struct Command;
// CommandBuffer::computed_signature (command.rs:821-853): the declared function, kept as a
// snapshot of the command buffer it was computed from.
using Signature = std::shared_ptr<const Command>;

struct Command {
    std::vector<Op> ops;
    std::vector<TyVar> tys;              // descriptor variables
    int32_t nvars = 0;                   // generic parameters declared
    std::vector<Signature> functions;    // CommandBuffer::function declarations
    bool pending_knob = false;       // CommandBuffer::with_knob: applies to the next op
    int32_t pending_buffer = -1;     // CommandBuffer::with_buffer: applies to the next op
    void clear_pending() {
        pending_knob = false;
        pending_buffer = -1;
    }
    uint32_t push(Op op);
    const Desc &describe(uint32_t reg) const;
    bool is_value(uint32_t reg) const;
};

// ---------------------------------------------------------------- program

struct Program {
    // Registers of the linked command buffers (link index, register) -> register of `ops`
    // (only where they differ: after inlining of invoked functions).
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> alias;
    std::vector<Op> ops;
    std::vector<uint32_t> inputs, outputs;   // registers (outputs: the value registers)
    std::vector<uint32_t> output_regs;       // the Output op registers
    std::vector<uint32_t> uses;              // use counts of every register
};

// ---------------------------------------------------------------- executable

enum class SlotKind { Input, Intermediate, Output, Table };

struct Slot {
    SlotKind kind;
    uint64_t bytes = 0;
    int64_t stride = 0;
    int32_t width = 0, height = 0;
    ZsFormat fmt{};
    uint32_t reg = 0;            // Input: input register; Output: output register
    std::vector<uint8_t> table;  // Table contents (weights / indices), uploaded at lowering
};

struct SrcRef {
    int slot = -1;
    ZsFormat fmt{};
    int32_t width = 0, height = 0;
    int64_t stride = 0;
};

enum class StepKind { Raster, Chain, Copy, Layers, Dynamic };

// A registered custom operation: its loaded module's kernel (cudaKernel_t) per registration.
void *dynamic_kernel(uint32_t op);

// One layer of a fused layer stack: its source buffer and the sampling/blend setup.
struct LayerRef {
    int slot = -1;
    ZsLayer proto{};
    bool quant_sample = false, quant_acc = false;
    ZsFormat sample_fmt{}, acc_fmt{};
};

struct Step {
    StepKind kind;
    std::shared_ptr<ZsLayersArgs> layers;   // Layers: template (pointers filled at launch)
    std::vector<int> layer_slots;
    int base_slot = -1;
    ZsRasterArgs raster;         // pointers filled at launch from slots
    ZsChainArgs chain;
    uint8_t chain_src_fast = 0, chain_dst_fast = 0;
    int src_slot[ZS_MAX_SRCS] = {-1, -1, -1};
    int dst_slot = -1;
    int idx_x_slot = -1, idx_y_slot = -1, weight_slot = -1;
    int vfirst_slot = -1, vcount_slot = -1, vweight_slot = -1;   // RESAMPLE_2D vertical tables
    int vimg_slot = -1, vimg_index_slot = -1;                   // RESAMPLE_2D tensor-core band images
    int tc_weight_slot = -1;                                    // and its 16-byte-row horizontal weights
    int vsrc_slot[2] = {-1, -1};                                // AFFINE virt1: the gathered producer's sources
    uint64_t copy_bytes = 0;
    // Copy of rows between different row strides (copy_rows > 0): copy_bytes per row.
    uint64_t copy_rows = 0;
    int64_t copy_src_pitch = 0, copy_dst_pitch = 0;
    int tune_threads = 0;        // Chain: block size chosen by the autotuner (0: default)
    int tune_vectors = 0;        // Chain: 16-byte vectors per thread and iteration (0: default 2)
    // RESAMPLE_2D on the tensor cores: the tile widths that fit, with their atoms; the
    // autotuner picks among them (raster.tc_tw / tc_atoms hold the choice).
    std::vector<std::pair<int, int>> tc_cands;
    uint32_t dyn_op = 0;         // Dynamic: registered op; src_slot[0..1] RGBA32F operands,
    int dyn_uniform_slot = -1;   //   dst_slot an RGBA32F result, uniforms in this table slot
    std::string label;
};

// Where the bytes of a knob land: the constants of a raster step's producer (step >= 0,
// interpreted for `kind`) or a constant table slot holding the bytes (slot >= 0).
struct KnobSite {
    int step = -1;
    int slot = -1;
    OpKind kind = OpKind::BufferInit;
};

struct KnobInfo {
    uint32_t reg = 0;            // the register the knob was declared on (RegisterKnob)
    uint64_t len = 0;            // bytes of its parameter block
    std::vector<KnobSite> sites;
};

// A knob value applied to one launch: new producer constants of a step.
struct ConsPatch {
    size_t step = 0;
    std::vector<float> cons;
};

struct Executable {
    int device = 0;
    uint32_t mode = ZS_MODE_FUSED;
    bool use_graph = false;
    uint32_t flags = 0;                                // ZS_CAP_* bits
    int sm_count = 148;
    std::vector<Slot> slots;
    std::vector<Step> steps;
    std::vector<uint32_t> input_regs, output_regs;     // value registers in declaration order
    std::vector<Desc> input_desc, output_desc;
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> alias;   // Program::alias
    std::vector<int> input_slot, output_slot;
    std::vector<void *> dev_buffers;                   // device allocation per slot (owned ones)
    // zs_batch_thumbnails: two sets (alternate batches) of device image/prefix tables, their
    // pinned staging copy, the event of the batch that last used them, and that set's captured
    // graph with its key, so that the tables of one batch are built while the previous runs.
    struct BatchSet {
        void *scratch = nullptr;
        void *staging = nullptr;
        size_t bytes = 0;
        cudaEvent_t done = nullptr;
        cudaGraphExec_t graph = nullptr;
        std::vector<uint64_t> key;
    };
    BatchSet batch_sets[2];
    int batch_next = 0;
    int batch_rows = 0;                                // batch work-item height (0: tuned or default)
    int batch_threads = 0;                             // batch kernel block size (0: tuned or default)
    std::string plan_text;
    std::vector<KnobInfo> knobs;                      // Executable::query_knob
    // CUDA graphs of the launch sequence for zs_run_device, keyed by the bound pointers
    std::map<std::vector<void *>, cudaGraphExec_t> graphs;
    std::vector<std::vector<void *>> graph_order;     // insertion order for eviction
    cudaStream_t graph_stream = nullptr;
    ~Executable();
    void ensure_buffers();
    void record(cudaStream_t stream, const std::vector<void *> &ptrs);
    void record_range(cudaStream_t stream, const std::vector<void *> &ptrs, size_t begin, size_t end,
                      const std::vector<ConsPatch> *patches = nullptr);
};

std::unique_ptr<Executable> lower(const Program &prog, const zs_capabilities &caps);

// ---------------------------------------------------------------- linking (link.cpp)

// Linker::compile (command.rs:2069): use counts, inputs and outputs of a flat command buffer.
Program compile_command(const Command &c);
// Linker::link (command.rs:2083-2893): `buffers` = main then the function definitions, `tys`
// the descriptors of main's generic parameters,
// links[i][f] = the buffer defining function f of buffer i; invoked functions are
// monomorphised and inlined, so the whole program is one op list for the planner.
Program link_commands(const std::vector<const Command *> &buffers, const std::vector<Desc> &tys,
                      const std::vector<std::vector<uint32_t>> &links);
// CommandBuffer::invoke (command.rs:863-922): checks the arguments and records the call;
// returns the result registers.
std::vector<uint32_t> cmd_invoke(Command &c, uint32_t function, const std::vector<uint32_t> &tyvars,
                                 const std::vector<uint32_t> &args);
// Descriptor of descriptor variable `ty` of `c` (a placeholder for a generic parameter).
Desc ty_descriptor(const Command &c, uint32_t ty);

// ---------------------------------------------------------------- autotuner (autotune.cpp)

const std::string &last_error();
bool tune_get(const std::string &key, int &value);
void tune_put(const std::string &key, int value);
void tune_save(const std::string &path);
void tune_load(const std::string &path);
std::string device_key(int device);
std::string chain_tune_key(const Step &st, int device);
// `family`: "batch" (work-item height) or "batch_threads" (block size).
std::string batch_tune_key(const Executable &E, uint32_t canvas, int device, const char *family = "batch");
// Chain steps: the key of the vectors-per-iteration choice.
std::string chain_vectors_key(const Step &st, int device);
// Tensor-core resample steps: filter taps, source and output size classes.
std::string resample_tune_key(const Step &st, int device);
// Sets the tile width of a tensor-core resample step to one of its candidates; false when
// the width is not one.
bool set_resample_tile(Step &st, int tw);
// Tuned values of the executable's steps from the process-wide cache.
void apply_tuned(Executable &E);
// Times the candidates of every tunable step on these buffers and keeps the fastest.
int autotune_steps(Executable &E, const std::vector<void *> &ptrs, cudaStream_t s, uint32_t reps);
int autotune_batch(Executable *chain, const void *const *images, const uint32_t *widths, const uint32_t *heights,
                   uint32_t n, uint32_t canvas, void *out, cudaStream_t s, uint32_t reps);

// ---------------------------------------------------------------- pool / runtime

struct PoolImage {
    Desc desc{};
    uint8_t *host = nullptr;     // pinned (or malloc'd when no device)
    bool host_pinned = false;
    uint64_t len = 0;
    void *dev = nullptr;         // device copy (tight rows)
    uint64_t dev_len = 0;
    bool dev_valid = false;      // device holds the current contents
    bool host_valid = true;
    ~PoolImage();
    void ensure_host();
};

struct Pool {
    std::map<uint64_t, std::unique_ptr<PoolImage>> images;
    uint64_t next_key = 1;
    PoolImage &get(uint64_t key);
};

struct Environment {
    Executable *exe = nullptr;
    Pool *pool = nullptr;
    std::map<uint32_t, uint64_t> binds;          // input register -> key
    std::map<uint32_t, uint64_t> output_binds;   // output register -> key
    std::map<uint32_t, std::vector<uint8_t>> knob_data;   // Environment::knob: knob -> bytes
};

struct Execution {
    Executable *exe = nullptr;
    Pool *pool = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<void *> ptrs;                    // per slot
    std::vector<void *> owned;                   // temporary device buffers of this execution
    std::map<uint32_t, uint64_t> output_binds;
    size_t cursor = 0;                           // next instruction
    size_t total = 0;
    std::vector<uint64_t> input_keys;
    std::vector<ConsPatch> patches;              // knob values of this launch
    ~Execution();
};

}  // namespace zs
