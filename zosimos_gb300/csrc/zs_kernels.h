// zs_kernels.h -- host-callable launchers of the CUDA kernels (no torch types).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "zs_shared.h"

namespace zs {

// Kernel launches issued since process start (defined in k_raster.cu).
extern std::atomic<uint64_t> g_kernel_launches;

// Exact sRGB8 tables (zs_tables.cu).
void build_srgb_tables(float *decode, uint32_t *encode, uint32_t *encode_shifted);
cudaError_t init_device_tables(int device);

// Generic raster launch: producer + fused pixel program + store (k_raster.cu).
cudaError_t launch_raster(const ZsRasterArgs &args, int sm_count, cudaStream_t stream);
// Both passes of a separable resample in one tiled launch (k_resample.cu); launch_raster
// dispatches ZS_PR_RESAMPLE_2D here.
cudaError_t launch_resample2d(const ZsRasterArgs &args, int sm_count, cudaStream_t stream);
// The tensor-core form of RESAMPLE_2D (k_resample_tc.cu), usable when planned (tc_tw > 0),
// the source is RGBA16F with 16-byte aligned rows and the TMA encoder is available.
bool resample_tc_usable(const ZsRasterArgs &args);
cudaError_t launch_resample_tc(const ZsRasterArgs &args, int sm_count, cudaStream_t stream);

// Fused colour chain in canonical form, RGBA8 in / RGBA8 out (k_chain.cu).
// Returns cudaErrorNotSupported when no specialisation exists for the formats or the buffers
// are not 16-byte aligned.  threads: 1024 (default, one block per SM), 512 or 256; vectors:
// 16-byte vectors per thread and loop iteration, 2 (default) or 1.
cudaError_t launch_chain(const ZsChainArgs &args, uint8_t src_fast, uint8_t dst_fast, int sm_count,
                         cudaStream_t stream, int threads = 1024, int vectors = 2);

// A stack of affine-transformed layers blended in one pass (k_layers.cu).
cudaError_t launch_layers(const ZsLayersArgs &args, int sm_count, cudaStream_t stream);

// Runs the bounded-wait self test on `device` (k_selftest.cu): a wait that nothing
// completes gives up after `limit_us` and sets ZS_DEVSTAT_WAIT_TIMEOUT.
cudaError_t wait_selftest(int device, uint32_t limit_us);
// Device status word (ZS_DEVSTAT_* bits) of `device`, optionally cleared after reading.
cudaError_t read_device_status(int device, uint32_t *flags, bool clear);
// Number of kernel launches issued since process start (instrumentation for the bench).
uint64_t kernel_launch_count();
// Kernels launched through a replayed CUDA graph (counted on the host at replay).
void add_kernel_launches(uint64_t n);

}  // namespace zs
