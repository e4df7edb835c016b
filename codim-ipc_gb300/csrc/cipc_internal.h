// Internal declarations shared by the CUDA translation units and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cipc {

struct CcdArgs;

cudaError_t launch_accd_exact(const CcdArgs& a, int grid, cudaStream_t s);
// two-pass form (ccd_core.cuh): state holds a.n AccdState records (128 bytes each)
struct AccdState;
cudaError_t launch_accd_exact_split(const CcdArgs& a, AccdState* state, int grid, cudaStream_t s);
int accd_exact_steps_blocks_per_sm();
cudaError_t launch_accd_mixed(const CcdArgs& a, int grid, cudaStream_t s);
int accd_exact_blocks_per_sm();
int accd_mixed_blocks_per_sm();

struct BarrierLaunch {
    int64_t n;
    const uint8_t* type;
    const int32_t* idx;
    const double* x;
    const double* x_rest;
    double xi2, shat, kappa;
    int project;
    int fp64_hessian;
    int64_t nv;
    double* E;
    double* grad;
    void* hess;
    unsigned long long* bad;
};
cudaError_t launch_barrier(const BarrierLaunch& L, cudaStream_t s);

}  // namespace cipc
