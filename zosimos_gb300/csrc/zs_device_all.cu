// zs_device_all.cu -- single translation unit for all device code, so that the
// __device__ tables of zs_tables.cu are one object shared by every kernel without
// relocatable device code.
#include "zs_tables.cu"
#include "k_raster.cu"
#include "k_resample.cu"
#include "k_resample_tc.cu"
#include "k_chain.cu"
#include "k_layers.cu"
#include "k_batch.cu"
#include "k_noalloc.cu"
#include "k_selftest.cu"
