// autotune.cpp -- the launch-parameter autotuner: candidates timed with CUDA events on the
// caller's own buffers, the winner kept with the executable and in a process-wide cache keyed
// by (kernel family, chain flags, shape class, device), which can be saved to and loaded from
// a text file so that later processes start tuned.
//
// Tunables (every candidate runs the same arithmetic per pixel, so results are byte-identical):
//  * the colour-chain kernel's block size, 1024 threads (one block per SM) or 512, and its
//    16-byte vectors per thread and loop iteration, 2 or 1;
//  * the tensor-core resample's tile width (8, 16 or 32 output columns, each with the atoms its
//    source span needs; the same MMAs and taps per output pixel, so the same bytes);
//  * the batched-thumbnail kernel's work-item height, 1, 2, 4, 8 or 16 (a streaming item covers
//    about 16 x that many source rows: taller items share fewer boundary rows between items,
//    shorter ones balance the warps better), and its block size, 768 or 640 threads (one block
//    per SM either way: 24 warps with a few registers spilled, or 20 warps without).
//
// The reference has no autotuner (its render passes have no launch parameters).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <mutex>
#include <sstream>

#include "zs_host.hpp"

namespace zs {

const std::string &last_error();
int batch_thumbnails(Executable *chain, const void *const *images, const uint32_t *widths, const uint32_t *heights,
                     uint32_t n, uint32_t canvas, void *out, cudaStream_t stream);

namespace {

std::mutex g_tune_mutex;
std::map<std::string, int> g_tune;

}  // namespace

bool tune_get(const std::string &key, int &value) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune.find(key);
    if (it == g_tune.end()) return false;
    value = it->second;
    return true;
}

void tune_put(const std::string &key, int value) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune[key] = value;
}

void tune_save(const std::string &path) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    std::ofstream f(path, std::ios::trunc);
    if (!f) fail(ZS_ERR_INVALID_ARG, "cannot write the tuning cache " + path);
    f << "# zosimos-gb300 tuning cache: key value\n";
    for (const auto &kv : g_tune) f << kv.first << ' ' << kv.second << '\n';
}

void tune_load(const std::string &path) {
    std::ifstream f(path);
    if (!f) fail(ZS_ERR_INVALID_ARG, "cannot read the tuning cache " + path);
    std::map<std::string, int> read;
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        std::string key;
        int value;
        if (!(is >> key >> value)) fail(ZS_ERR_INVALID_ARG, "malformed tuning cache line: " + line);
        read[key] = value;
    }
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    for (const auto &kv : read) g_tune[kv.first] = kv.second;
}

// "<name>/sm<count>/cc<major>.<minor>" of a device, or "nodevice" without one.
std::string device_key(int device) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) {
        cudaGetLastError();
        return "nodevice";
    }
    std::string name(p.name);
    std::replace(name.begin(), name.end(), ' ', '_');
    std::ostringstream os;
    os << name << "/sm" << p.multiProcessorCount << "/cc" << p.major << '.' << p.minor;
    return os.str();
}

// Chain steps: the specialisation (flags) and the image size class (log2 of the pixels).
std::string chain_tune_key(const Step &st, int device) {
    std::ostringstream os;
    const int64_t npx = std::max<int64_t>(st.chain.npx, 1);
    os << "chain/flags" << st.chain.flags << "/px2^" << (int)std::floor(std::log2((double)npx)) << '/'
       << device_key(device);
    return os.str();
}

std::string chain_vectors_key(const Step &st, int device) { return "chain_vectors/" + chain_tune_key(st, device).substr(6); }

std::string batch_tune_key(const Executable &E, uint32_t canvas, int device, const char *family) {
    int flags = 0;
    for (const Step &st : E.steps)
        if (st.kind == StepKind::Chain) flags = st.chain.flags;
    std::ostringstream os;
    os << family << "/flags" << flags << "/canvas" << canvas << '/' << device_key(device);
    return os.str();
}

// Tensor-core resample steps: the horizontal tap count, log2 size classes of the source and
// output widths, and the device.
std::string resample_tune_key(const Step &st, int device) {
    std::ostringstream os;
    const ZsRasterArgs &a = st.raster;
    os << "resample_tc/taps" << a.taps << "/src2^" << (int)std::floor(std::log2((double)std::max(a.src[0].width, 1)))
       << "/dst2^" << (int)std::floor(std::log2((double)std::max(a.width, 1))) << '/' << device_key(device);
    return os.str();
}

bool set_resample_tile(Step &st, int tw) {
    for (const auto &c : st.tc_cands)
        if (c.first == tw) {
            st.raster.tc_tw = c.first;
            st.raster.tc_atoms = c.second;
            return true;
        }
    return false;
}

static bool is_tc_resample(const Step &st) {
    return st.kind == StepKind::Raster && st.raster.producer == ZS_PR_RESAMPLE_2D && st.raster.tc_tw > 0 &&
           !st.tc_cands.empty();
}

// Tuned values of an executable's steps from the cache (called once its device is known).
void apply_tuned(Executable &E) {
    for (Step &st : E.steps) {
        int v;
        if (st.kind == StepKind::Chain && !st.tune_threads && tune_get(chain_tune_key(st, E.device), v)) st.tune_threads = v;
        if (st.kind == StepKind::Chain && !st.tune_vectors && tune_get(chain_vectors_key(st, E.device), v) &&
            (v == 1 || v == 2))
            st.tune_vectors = v;
        if (is_tc_resample(st) && tune_get(resample_tune_key(st, E.device), v)) set_resample_tile(st, v);
    }
}

// Device time of one recorded step (median of `reps` launches after a warm-up).
static float time_step(Executable &E, const std::vector<void *> &ptrs, size_t k, cudaStream_t s, uint32_t reps) {
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    std::vector<float> ms;
    try {
        E.record_range(s, ptrs, k, k + 1);
        for (uint32_t r = 0; r < reps; ++r) {
            check_cuda(cudaEventRecord(e0, s), "event");
            E.record_range(s, ptrs, k, k + 1);
            check_cuda(cudaEventRecord(e1, s), "event");
            check_cuda(cudaEventSynchronize(e1), "synchronize");
            float t = 0.f;
            check_cuda(cudaEventElapsedTime(&t, e0, e1), "elapsed");
            ms.push_back(t);
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::nth_element(ms.begin(), ms.begin() + ms.size() / 2, ms.end());
    return ms[ms.size() / 2];
}

// Tunes every chain step (block size) and tensor-core resample step (tile width) of E on the
// given buffers; returns the chosen block size of the last chain step (0 when E has none).
int autotune_steps(Executable &E, const std::vector<void *> &ptrs, cudaStream_t s, uint32_t reps) {
    int chosen = 0;
    for (size_t k = 0; k < E.steps.size(); ++k) {
        Step &st = E.steps[k];
        if (is_tc_resample(st) && st.tc_cands.size() > 1) {
            int best = st.raster.tc_tw;
            float best_ms = 0.f;
            bool first = true;
            const std::vector<std::pair<int, int>> cands = st.tc_cands;
            for (const auto &c : cands) {
                set_resample_tile(st, c.first);
                const float t = time_step(E, ptrs, k, s, reps);
                if (first || t < best_ms) {
                    best = c.first;
                    best_ms = t;
                    first = false;
                }
            }
            set_resample_tile(st, best);
            tune_put(resample_tune_key(st, E.device), best);
            continue;
        }
        if (st.kind != StepKind::Chain) continue;
        int best = 1024, best_vec = 2;
        float best_ms = 0.f;
        bool first = true;
        for (int cand : {1024, 512})
            for (int vec : {2, 1}) {
                st.tune_threads = cand;
                st.tune_vectors = vec;
                const float t = time_step(E, ptrs, k, s, reps);
                if (first || t < best_ms) {
                    best = cand;
                    best_vec = vec;
                    best_ms = t;
                    first = false;
                }
            }
        st.tune_threads = best;
        st.tune_vectors = best_vec;
        tune_put(chain_tune_key(st, E.device), best);
        tune_put(chain_vectors_key(st, E.device), best_vec);
        chosen = best;
    }
    // Captured graphs hold the old launch parameters.
    for (auto &kv : E.graphs) cudaGraphExecDestroy(kv.second);
    E.graphs.clear();
    E.graph_order.clear();
    return chosen;
}

int autotune_batch(Executable *chain, const void *const *images, const uint32_t *widths, const uint32_t *heights,
                   uint32_t n, uint32_t canvas, void *out, cudaStream_t s, uint32_t reps) {
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    int best = 0, best_threads = 0;
    float best_ms = 0.f;
    int rc = ZS_OK;
    for (int threads : {768, 640}) {
        for (int cand : {1, 2, 4, 8, 16}) {
            chain->batch_threads = threads;
            chain->batch_rows = cand;
            std::vector<float> ms;
            for (uint32_t r = 0; r <= reps && rc == ZS_OK; ++r) {
                cudaEventRecord(e0, s);
                rc = batch_thumbnails(chain, images, widths, heights, n, canvas, out, s);
                cudaEventRecord(e1, s);
                if (rc != ZS_OK) break;
                check_cuda(cudaEventSynchronize(e1), "synchronize");
                float t = 0.f;
                check_cuda(cudaEventElapsedTime(&t, e0, e1), "elapsed");
                if (r > 0) ms.push_back(t);      // the first batch of a candidate captures its graph
            }
            if (rc != ZS_OK) break;
            std::nth_element(ms.begin(), ms.begin() + ms.size() / 2, ms.end());
            const float t = ms[ms.size() / 2];
            if (!best || t < best_ms) {
                best = cand;
                best_threads = threads;
                best_ms = t;
            }
        }
        if (rc != ZS_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != ZS_OK) {
        chain->batch_rows = 0;
        chain->batch_threads = 0;
        fail(rc, "autotune of the batched thumbnails: " + last_error());
    }
    chain->batch_rows = best;
    chain->batch_threads = best_threads;
    tune_put(batch_tune_key(*chain, canvas, chain->device), best);
    tune_put(batch_tune_key(*chain, canvas, chain->device, "batch_threads"), best_threads);
    return best;
}

}  // namespace zs
