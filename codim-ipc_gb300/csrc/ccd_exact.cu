// ACCD, exact FP64 variant.  Compiled with -fmad=false: the only fused
// multiply-adds are the explicit fma() calls of geom.cuh, so times of impact and
// hit/miss decisions are reproducible bit for bit on the CPU.
//
// The distance types and the gap test of each step are decided by the certified
// FP32 evaluations of cert.cuh, which return the FP64 decision or "undecided"
// (then the FP64 code decides); every value that reaches a result (squared
// distances, square roots, steps, times) is the FP64 arithmetic of geom.cuh.
#include <cuda_runtime.h>

#include "ccd_core.cuh"
#include "cert.cuh"
#include "cipc_internal.h"

namespace cipc {

struct ExactPol {
    // distance function f = d^2 - xi^2 with the EE fallback of CCD.h:339-345
    static __device__ __forceinline__ double dfunc(int tp, const d3 (&v)[4], double th2, double& d2)
    {
        switch (tp) {
            case kPP: d2 = pp_d2(v[0], v[1]); return d2 - th2;
            case kPE: d2 = pe_d2_any(v[0], v[1], v[2]); return d2 - th2;
            case kPT: d2 = pt_d2_cert(v[0], v[1], v[2], v[3]); return d2 - th2;
            default: {
                d2 = ee_d2_cert(v[0], v[1], v[2], v[3]);
                double f = d2 - th2;
                if (f <= 0) {
                    const double p0 = pp_d2(v[0], v[2]), p1 = pp_d2(v[0], v[3]);
                    const double p2 = pp_d2(v[1], v[2]), p3 = pp_d2(v[1], v[3]);
                    d2 = dmin(dmin(dmin(p0, p1), p2), p3);
                    f = d2 - th2;
                }
                return f;
            }
        }
    }
    static __device__ __forceinline__ double sqrt_(double v) { return sqrt(v); }
    static __device__ __forceinline__ double div_(double a, double b) { return a / b; }
    // RN(f / den) < gap
    static __device__ __forceinline__ bool gap_less(double f, double den, double gap)
    {
        const int c = gap_less_cert(f, den, gap);
        return c >= 0 ? c == 1 : f / den < gap;
    }
};

cudaError_t launch_accd_exact(const CcdArgs& a, int grid, cudaStream_t s)
{
    k_accd<ExactPol><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_accd_exact_split(const CcdArgs& a, AccdState* state, int grid, cudaStream_t s)
{
    if (a.max_iter < 1) return cudaErrorInvalidValue;
    const int64_t need = (a.n + 255) / 256;
    const int sgrid = (int)(need < 4096 ? need : 4096);
    k_accd_setup<ExactPol><<<sgrid > 0 ? sgrid : 1, 256, 0, s>>>(a, state);
    k_accd_steps<ExactPol><<<grid, 256, 0, s>>>(a, state);
    return cudaGetLastError();
}

int accd_exact_steps_blocks_per_sm()
{
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_accd_steps<ExactPol>, 256, 0);
    return b > 0 ? b : 1;
}

int accd_exact_blocks_per_sm()
{
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_accd<ExactPol>, 256, 0);
    return b > 0 ? b : 1;
}

}  // namespace cipc
