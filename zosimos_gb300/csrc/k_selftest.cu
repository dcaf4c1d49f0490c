// k_selftest.cu -- failure detection of the bounded device waits, exercised without a fault.
//
// One warp initialises an mbarrier that nothing ever arrives on and waits for it through
// zs_mbar_wait, the routine every pipelined kernel uses, with a short limit.  The wait gives
// up, the kernel sets ZS_DEVSTAT_WAIT_TIMEOUT in the device status word exactly as a real
// timeout does, and returns; the context stays usable.
#include "zs_device.cuh"
#include "zs_kernels.h"
#include "zs_ptx.cuh"

__global__ void zs_wait_selftest_kernel(uint64_t limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        zs_mbar_init(zs_smem_addr(&bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !zs_mbar_wait(zs_smem_addr(&bar), 0, limit_ns))
        atomicOr(&zs_device_status_word, ZS_DEVSTAT_WAIT_TIMEOUT);
}

namespace zs {

cudaError_t wait_selftest(int device, uint32_t limit_us) {
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return e;
    if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
    zs_wait_selftest_kernel<<<1, 32>>>((uint64_t)limit_us * 1000ull);
    g_kernel_launches.fetch_add(1);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (prev != device) cudaSetDevice(prev);
    return e;
}

}  // namespace zs

ZS_TU_HOOKS(selftest)
