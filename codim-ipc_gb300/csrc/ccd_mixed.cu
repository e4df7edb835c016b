// ACCD, mixed-precision variant.  The distance-type classification (which of the
// 7 point-triangle / 9 edge-edge / 3 point-edge regions is closest) runs in FP32 on
// FP64 difference vectors; the squared distance of the chosen region, the
// distance function d^2 - xi^2, the position updates and the accumulated time of
// impact stay FP64.  Reciprocals and square roots start from the FP32 hardware
// approximations and are refined by Newton steps in FP64 (relative error ~1e-15),
// which avoids the FP64 divide and square-root sequences on this part's reduced
// FP64 pipe.  Results differ from the exact variant only where a pair lies within
// FP32 rounding of a region boundary, where the distance is continuous.
#include <cuda_runtime.h>

#include "ccd_core.cuh"
#include "cipc_internal.h"

namespace cipc {

__device__ __forceinline__ double fast_rcp(double b)
{
    const double ab = fabs(b);
    if (!(ab > 1e-36 && ab < 1e36)) return 1.0 / b;
    double r = (double)__frcp_rn((float)b);
    r = r * fma(-b, r, 2.0);
    r = r * fma(-b, r, 2.0);
    return r;
}
__device__ __forceinline__ double fast_div(double a, double b)
{
    const double r = fast_rcp(b);
    const double q = a * r;
    return fma(r, fma(-b, q, a), q);
}
__device__ __forceinline__ double fast_sqrt(double v)
{
    if (!(v > 1e-36 && v < 1e36)) return sqrt(v);
    double y = (double)rsqrtf((float)v);
    y = y * fma(-0.5 * v, y * y, 1.5);
    y = y * fma(-0.5 * v, y * y, 1.5);
    return v * y;
}

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 tf(d3 v) { return f3{(float)v.x, (float)v.y, (float)v.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 fneg(f3 a) { return f3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 fcross(f3 a, f3 b)
{
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// edge parameter s along r0 and the sign of the in-plane normal coordinate q
// (the basis r0, r0 x n is orthogonal, so the 2x2 solve decouples)
__device__ __forceinline__ void pt_param_f(f3 r0, f3 n, f3 v, float& s, float& q)
{
    s = fdot(r0, v) / fdot(r0, r0);
    q = fdot(fcross(r0, n), v);
}

// point-triangle region from a = p - t0, e1 = t1 - t0, e2 = t2 - t0
__device__ __forceinline__ int pt_type_f(f3 a, f3 e1, f3 e2)
{
    const f3 n = fcross(e1, e2);
    float s0, q0, s1, q1, s2, q2;
    pt_param_f(e1, n, a, s0, q0);
    if (s0 > 0.f && s0 < 1.f && q0 >= 0.f) return 3;
    pt_param_f(e2 - e1, n, a - e1, s1, q1);
    if (s1 > 0.f && s1 < 1.f && q1 >= 0.f) return 4;
    pt_param_f(fneg(e2), n, a - e2, s2, q2);
    if (s2 > 0.f && s2 < 1.f && q2 >= 0.f) return 5;
    if (s0 <= 0.f && s2 >= 1.f) return 0;
    if (s1 <= 0.f && s0 >= 1.f) return 1;
    if (s2 <= 0.f && s1 >= 1.f) return 2;
    return 6;
}

// edge-edge region from u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0
__device__ __forceinline__ int ee_type_f(f3 u, f3 v, f3 w)
{
    const float a = fdot(u, u), b = fdot(u, v), c = fdot(v, v), d = fdot(u, w), e = fdot(v, w);
    const float D = a * c - b * b;
    float tD = D, tN;
    int dc = 8;
    const float sN = b * e - c * d;
    if (sN <= 0.f) {
        tN = e;
        tD = c;
        dc = 2;
    } else if (sN >= D) {
        tN = e + b;
        tD = c;
        dc = 5;
    } else {
        tN = a * e - b * d;
        if (tN > 0.f && tN < tD) {
            const f3 uxv = fcross(u, v);
            if (fdot(uxv, w) == 0.f || fdot(uxv, uxv) < 1.0e-20f * a * c) {
                if (sN < D / 2) {
                    tN = e;
                    tD = c;
                    dc = 2;
                } else {
                    tN = e + b;
                    tD = c;
                    dc = 5;
                }
            }
        }
    }
    if (tN <= 0.f) {
        if (-d <= 0.f) return 0;
        if (-d >= a) return 3;
        return 6;
    } else if (tN >= tD) {
        if ((-d + b) <= 0.f) return 1;
        if ((-d + b) >= a) return 4;
        return 7;
    }
    return dc;
}

// squared distance from point (relative vector w = p - e0) to the line of edge e
__device__ __forceinline__ double line_d2(d3 w, d3 e) { return fast_div(n2(cross(w, e)), n2(e)); }

struct MixedPol {
    static __device__ __forceinline__ double dfunc(int tp, const d3 (&v)[4], double th2, double& d2)
    {
        switch (tp) {
            case kPP: d2 = pp_d2(v[0], v[1]); return d2 - th2;
            case kPE: {
                const d3 w = v[0] - v[1], e = v[2] - v[1];
                const f3 wf = tf(w), ef = tf(e);
                const float c1 = fdot(wf, ef), c2 = fdot(ef, ef);
                if (c1 <= 0.f) d2 = n2(w);
                else if (c2 <= c1) d2 = n2(v[0] - v[2]);
                else d2 = line_d2(w, e);
                return d2 - th2;
            }
            case kPT: {
                const d3 a = v[0] - v[1], e1 = v[2] - v[1], e2 = v[3] - v[1];
                switch (pt_type_f(tf(a), tf(e1), tf(e2))) {
                    case 0: d2 = n2(a); break;
                    case 1: d2 = n2(a - e1); break;
                    case 2: d2 = n2(a - e2); break;
                    case 3: d2 = line_d2(a, e1); break;
                    case 4: d2 = line_d2(a - e1, e2 - e1); break;
                    case 5: d2 = line_d2(a - e2, e2); break;
                    default: {
                        const d3 nn = cross(e1, e2);
                        const double aTb = dot(a, nn);
                        d2 = fast_div(aTb * aTb, n2(nn));
                    }
                }
                return d2 - th2;
            }
            default: {
                const d3 u = v[1] - v[0], vv = v[3] - v[2], w = v[0] - v[2];
                switch (ee_type_f(tf(u), tf(vv), tf(w))) {
                    case 0: d2 = n2(w); break;
                    case 1: d2 = n2(w - vv); break;
                    case 2: d2 = line_d2(w, vv); break;
                    case 3: d2 = n2(w + u); break;
                    case 4: d2 = n2((w + u) - vv); break;
                    case 5: d2 = line_d2(w + u, vv); break;
                    case 6: d2 = line_d2(w, u); break;
                    case 7: d2 = line_d2(vv - w, u); break;
                    default: {
                        const d3 b = cross(u, vv);
                        const double aTb = dot(w, b);
                        d2 = fast_div(aTb * aTb, n2(b));
                    }
                }
                double f = d2 - th2;
                if (f <= 0) {
                    const double p0 = n2(w), p1 = n2(w - vv), p2 = n2(w + u), p3 = n2((w + u) - vv);
                    d2 = dmin(dmin(dmin(p0, p1), p2), p3);
                    f = d2 - th2;
                }
                return f;
            }
        }
    }
    static __device__ __forceinline__ double sqrt_(double v) { return fast_sqrt(v); }
    static __device__ __forceinline__ double div_(double a, double b) { return fast_div(a, b); }
};

cudaError_t launch_accd_mixed(const CcdArgs& a, int grid, cudaStream_t s)
{
    k_accd<MixedPol><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

int accd_mixed_blocks_per_sm()
{
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_accd<MixedPol>, 256, 0);
    return b > 0 ? b : 1;
}

}  // namespace cipc
