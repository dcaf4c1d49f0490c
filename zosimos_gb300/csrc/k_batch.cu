// k_batch.cu -- batched uneven thumbnails (one persistent launch over many images).
#include "zs_device.cuh"
#include "zs_kernels.h"
#include "host/zs_host.hpp"

namespace zs {

int batch_thumbnails(Executable *, const void *const *, const uint32_t *, const uint32_t *, uint32_t, uint32_t, void *,
                     cudaStream_t) {
    set_last_error("batched thumbnails are not built yet");
    return ZS_ERR_UNIMPLEMENTED;
}

}  // namespace zs
