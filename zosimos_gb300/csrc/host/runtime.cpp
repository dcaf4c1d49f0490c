// runtime.cpp -- Pool, device buffers, launch recording, CUDA-graph replay and the
// step-wise Execution (the analogue of lib/zosimos/src/run.rs: Executable::launch
// :1016-1048, Execution::step :1389-1464, Retire :2786-2998, pool.rs).
//
// The reference interprets a stream of GL-like `Low` instructions against wgpu, with
// one queue submit and host row copies per op.  Here an Execution owns one CUDA
// stream; its instructions are the host->device copies of bound inputs followed by the
// executable's kernel launches; results stay device resident until retired.
#include <cstdlib>
#include <cstring>

#include "zs_host.hpp"

namespace zs {

static bool have_device() {
    int n = 0;
    return cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
}

static void *host_alloc(uint64_t bytes, bool &pinned) {
    void *p = nullptr;
    pinned = false;
    if (bytes == 0) bytes = 1;
    if (have_device() && cudaMallocHost(&p, bytes) == cudaSuccess) {
        pinned = true;
        return p;
    }
    cudaGetLastError();
    p = std::malloc(bytes);
    if (!p) fail(ZS_ERR_OUT_OF_MEMORY, "host allocation failed");
    return p;
}

static void host_release(void *p, bool pinned) {
    if (!p) return;
    if (pinned) cudaFreeHost(p);
    else std::free(p);
}

// ---------------------------------------------------------------- pool

PoolImage::~PoolImage() {
    host_release(host, host_pinned);
    if (dev) cudaFree(dev);
}

void PoolImage::ensure_host() {
    if (!host) host = (uint8_t *)host_alloc(len, host_pinned);
}

PoolImage &Pool::get(uint64_t key) {
    auto it = images.find(key);
    if (it == images.end()) fail(ZS_ERR_MISSING_KEY, "no image with this key in the pool");
    return *it->second;
}

// ---------------------------------------------------------------- executable

Executable::~Executable() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    for (BatchSet &b : batch_sets) {
        if (b.graph) cudaGraphExecDestroy(b.graph);
        if (b.done) {
            cudaEventSynchronize(b.done);
            cudaEventDestroy(b.done);
        }
        if (b.scratch) cudaFree(b.scratch);
        if (b.staging) cudaFreeHost(b.staging);
    }
    if (graph_stream) cudaStreamDestroy(graph_stream);
    for (void *p : dev_buffers)
        if (p) cudaFree(p);
}

void Executable::ensure_buffers() {
    if (!dev_buffers.empty()) return;
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    check_cuda(init_device_tables(device), "sRGB tables");
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0) sm_count = sms;
    apply_tuned(*this);
    dev_buffers.assign(slots.size(), nullptr);
    for (size_t i = 0; i < slots.size(); ++i) {
        const Slot &s = slots[i];
        if (s.bytes == 0) continue;
        void *p = nullptr;
        check_cuda(cudaMalloc(&p, s.bytes), "cudaMalloc");
        dev_buffers[i] = p;
        if (s.kind == SlotKind::Table)
            check_cuda(cudaMemcpy(p, s.table.data(), s.bytes, cudaMemcpyHostToDevice), "table upload");
    }
}

void Executable::record(cudaStream_t stream, const std::vector<void *> &ptrs) {
    record_range(stream, ptrs, 0, steps.size());
}

// The raster arguments of a step with this launch's buffer pointers filled in.
static ZsRasterArgs raster_args(const Step &st, const std::vector<void *> &ptrs) {
    ZsRasterArgs a = st.raster;
    for (int i = 0; i < ZS_MAX_SRCS; ++i)
        a.src[i].ptr = st.src_slot[i] >= 0 ? (const uint8_t *)ptrs[st.src_slot[i]] : nullptr;
    a.dst = (uint8_t *)ptrs[st.dst_slot];
    a.index_x = st.idx_x_slot >= 0 ? (const int32_t *)ptrs[st.idx_x_slot] : nullptr;
    a.index_y = st.idx_y_slot >= 0 ? (const int32_t *)ptrs[st.idx_y_slot] : nullptr;
    a.weights = st.weight_slot >= 0 ? (const float *)ptrs[st.weight_slot] : nullptr;
    a.vfirst = st.vfirst_slot >= 0 ? (const int32_t *)ptrs[st.vfirst_slot] : nullptr;
    a.vcount = st.vcount_slot >= 0 ? (const int32_t *)ptrs[st.vcount_slot] : nullptr;
    a.vweights = st.vweight_slot >= 0 ? (const float *)ptrs[st.vweight_slot] : nullptr;
    a.vimg = st.vimg_slot >= 0 ? (const uint8_t *)ptrs[st.vimg_slot] : nullptr;
    a.vimg_index = st.vimg_index_slot >= 0 ? (const int32_t *)ptrs[st.vimg_index_slot] : nullptr;
    a.tc_weights = st.tc_weight_slot >= 0 ? (const float *)ptrs[st.tc_weight_slot] : nullptr;
    for (int i = 0; i < 2; ++i)
        a.vsrc[i].ptr = st.vsrc_slot[i] >= 0 ? (const uint8_t *)ptrs[st.vsrc_slot[i]] : nullptr;
    return a;
}

// Launches go to the executable's device whatever device the caller has current; the
// caller's current device is restored afterwards.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        if (prev != device) check_cuda(cudaSetDevice(device), "cudaSetDevice");
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

void Executable::record_range(cudaStream_t stream, const std::vector<void *> &ptrs, size_t begin, size_t end,
                              const std::vector<ConsPatch> *patches) {
    DeviceScope scope(device);
    for (size_t k = begin; k < end && k < steps.size(); ++k) {
        const Step &st = steps[k];
        switch (st.kind) {
        case StepKind::Copy:
            if (st.copy_rows > 0)
                check_cuda(cudaMemcpy2DAsync(ptrs[st.dst_slot], (size_t)st.copy_dst_pitch, ptrs[st.src_slot[0]],
                                             (size_t)st.copy_src_pitch, st.copy_bytes, st.copy_rows,
                                             cudaMemcpyDeviceToDevice, stream),
                           "device row copy");
            else
                check_cuda(cudaMemcpyAsync(ptrs[st.dst_slot], ptrs[st.src_slot[0]], st.copy_bytes,
                                           cudaMemcpyDeviceToDevice, stream),
                           "device copy");
            break;
        case StepKind::Layers: {
            ZsLayersArgs &L = *st.layers;      // pointers change per launch: patch a copy
            ZsLayersArgs a = L;
            if (st.base_slot >= 0) a.base.ptr = (const uint8_t *)ptrs[st.base_slot];
            for (size_t i = 0; i < st.layer_slots.size(); ++i) a.layers[i].ptr = (const uint8_t *)ptrs[st.layer_slots[i]];
            a.dst = (uint8_t *)ptrs[st.dst_slot];
            check_cuda(launch_layers(a, sm_count, stream), st.label.c_str());
        } break;
        case StepKind::Chain: {
            ZsChainArgs c = st.chain;
            c.src = (const uint8_t *)ptrs[st.src_slot[0]];
            c.dst = (uint8_t *)ptrs[st.dst_slot];
            const cudaError_t e =
                launch_chain(c, st.chain_src_fast, st.chain_dst_fast, sm_count, stream, st.tune_threads ? st.tune_threads : 1024,
                             st.tune_vectors ? st.tune_vectors : 2);
            if (e != cudaErrorNotSupported) {
                check_cuda(e, st.label.c_str());
                break;
            }
            // Buffers the chain kernel cannot stream (not 16-byte aligned): the same fused
            // program on the generic raster kernel.
            cudaGetLastError();
            check_cuda(launch_raster(raster_args(st, ptrs), sm_count, stream), st.label.c_str());
        } break;
        case StepKind::Dynamic: {
            void *kernel = dynamic_kernel(st.dyn_op);
            if (!kernel) fail(ZS_ERR_INVALID_ARG, "custom operation is no longer registered");
            zs_dyn_args a{};
            for (int i = 0; i < 2; ++i)
                if (st.src_slot[i] >= 0) {
                    a.src[i] = (const float *)ptrs[st.src_slot[i]];
                    a.src_width[i] = slots[st.src_slot[i]].width;
                    a.src_height[i] = slots[st.src_slot[i]].height;
                }
            const Slot &d = slots[st.dst_slot];
            a.dst = (float *)ptrs[st.dst_slot];
            a.width = d.width;
            a.height = d.height;
            if (st.dyn_uniform_slot >= 0) {
                a.uniforms = ptrs[st.dyn_uniform_slot];
                a.uniform_len = slots[st.dyn_uniform_slot].bytes;
            }
            void *params[] = {&a};
            const dim3 block(16, 16), grid((unsigned)(d.width + 15) / 16, (unsigned)(d.height + 15) / 16);
            check_cuda(cudaLaunchKernel(kernel, grid, block, params, 0, stream), st.label.c_str());
            add_kernel_launches(1);
        } break;
        case StepKind::Raster: {
            ZsRasterArgs a = raster_args(st, ptrs);
            if (patches)
                for (const ConsPatch &p : *patches)
                    if (p.step == k)
                        for (size_t i = 0; i < p.cons.size() && i < 24; ++i) a.cons[i] = p.cons[i];
            check_cuda(launch_raster(a, sm_count, stream), st.label.c_str());
        } break;
        }
    }
}

// ---------------------------------------------------------------- execution

Execution::~Execution() {
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    for (void *p : owned)
        if (p) cudaFree(p);
}

}  // namespace zs
