// Per-pair contact barrier: energy, gradient and PSD-projected Hessian.
//
// Restates the per-constraint bodies of Compute_Barrier / _Gradient / _Hessian
// (Library/FEM/IPC.h:742-1731, weight 1, multiplicity 1) for the four classified
// pair types:  s = d^2 - xi^2,  shat = dHat^2 + 2 dHat xi,
//   E = b(s),  grad = b'(s) grad d^2,  H = PSD(b'' grad d^2 grad d^2^T + b' hess d^2)
// with the EE mollifier product rule (IPC.h:1472-1478) when |ea x eb|^2 is below
// 1e-3 |ea_rest|^2 |eb_rest|^2.
//
// Precision: d^2, s, the activity test and b, b', b'' are FP64 in both variants,
// and so is the gradient (it is the Newton residual).  The Hessian and its
// eigen-decomposition are FP64 in the exact variant and FP32 in the mixed one.
#include <cuda_runtime.h>

#include "barrier_pair.cuh"
#include "cipc_internal.h"

namespace cipc {

template <typename HT>
__global__ void __launch_bounds__(128) k_barrier(BarrierArgs a)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = barrier_one<HT>(a, i);
        if (r) atomicAdd(a.bad + (r - 1), 1ull);
    }
}

cudaError_t launch_barrier(const BarrierLaunch& L, cudaStream_t s)
{
    BarrierArgs a;
    a.n = L.n;
    a.type = L.type;
    a.idx = reinterpret_cast<const int4*>(L.idx);
    a.x = L.x;
    a.x_rest = L.x_rest;
    a.xi2 = L.xi2;
    a.shat = L.shat;
    a.kappa = L.kappa;
    a.project = L.project;
    a.nv = L.nv;
    a.E = L.E;
    a.grad = L.grad;
    a.hess = L.hess;
    a.bad = L.bad;
    const int threads = 128;
    int64_t blocks = (L.n + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (blocks > (1 << 30)) blocks = 1 << 30;
    if (L.fp64_hessian)
        k_barrier<double><<<(unsigned)blocks, threads, 0, s>>>(a);
    else
        k_barrier<float><<<(unsigned)blocks, threads, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace cipc
