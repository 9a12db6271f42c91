// device.cuh -- per-device facts the launchers need: the SM count (grids
// are sized in resident waves) and the dynamic shared-memory limit of the
// kernels that stage more than 48 KB.  Both are kept per device, so a
// process with contexts on several GPUs launches correctly on each.
#pragma once

#include <cuda_runtime.h>

namespace g3m3 {

// Multiprocessors of the current device (cached per device; 148 if the
// query fails, which only sizes grids and never affects results).
int sm_count();

// Allow `func` `bytes` of dynamic shared memory on the current device.  The
// attribute is per device: the first call on a device sets it, later calls
// return the first call's result.  Not a stream operation, so it is legal
// during a stream capture; contexts still call it at creation so that no
// capture is the first to set it.
cudaError_t prepare_smem(const void* func, int bytes);

// Every kernel of the library that needs prepare_smem, on the current
// device (called by g3m3_ctx_create with the context's device current).
cudaError_t prepare_device_kernels();

}  // namespace g3m3
