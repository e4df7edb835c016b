// Library identification, error strings and device helpers (include/cipc.h).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/cipc.h"
#include "cipc_util.h"

namespace cipc {

static thread_local char g_last_error[512] = "";

int set_error(int status, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

int set_cuda_error(cudaError_t e, const char* where)
{
    cudaGetLastError();  // clear a sticky launch error if there is one
    return set_error(CIPC_ERR_CUDA, "%s: CUDA error %d (%s)", where, (int)e, cudaGetErrorString(e));
}

int ensure_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return set_error(CIPC_ERR_NO_DEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
    // Host-buffer calls stage their inputs in stream-ordered allocations; the
    // default pool would hand that memory back to the driver at every
    // synchronisation and map it again on the next call (milliseconds for the
    // ~2 GB of a 10M-pair pass), so up to 8 GiB of freed blocks stay reserved.
    static bool pool_set[64] = {false};
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && !pool_set[dev]) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = 8ull << 30;
            if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess)
                pool_set[dev] = true;
        }
        cudaGetLastError();
    }
    return CIPC_OK;
}

int num_sms()
{
    static int cache[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cache[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

}  // namespace cipc

extern "C" const char* cipc_version(void) { return "cipc-gb300 0.1 (sm_103a)"; }

extern "C" const char* cipc_last_error(void) { return cipc::g_last_error; }

extern "C" const char* cipc_status_string(int status)
{
    switch (status) {
        case CIPC_OK: return "ok";
        case CIPC_ERR_INVALID_ARG: return "invalid argument";
        case CIPC_ERR_CUDA: return "CUDA error";
        case CIPC_ERR_ITER_CAP: return "iteration cap reached";
        case CIPC_ERR_NONPOSITIVE_DISTANCE: return "non-positive distance";
        case CIPC_ERR_NOT_CONVERGED: return "not converged";
        case CIPC_ERR_NAN: return "NaN encountered";
        case CIPC_ERR_NO_DEVICE: return "no CUDA device";
        case CIPC_ERR_INDEX_RANGE: return "index out of range";
        case CIPC_ERR_TIMEOUT: return "device-side wait timed out";
    }
    return "unknown status";
}

extern "C" int cipc_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}
