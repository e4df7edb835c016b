// Error reporting and device helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>

namespace cipc {

// Records a formatted message for cipc_last_error() and returns `status`.
int set_error(int status, const char* fmt, ...);
// Records a CUDA error for cipc_last_error() and returns CIPC_ERR_CUDA.
int set_cuda_error(cudaError_t e, const char* where);
// Checks that a CUDA device is usable on this thread; CIPC_ERR_NO_DEVICE otherwise.
int ensure_device();
// Streaming multiprocessor count of the current device (cached per device).
int num_sms();

}  // namespace cipc
