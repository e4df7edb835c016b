// ACCD, mixed-precision variant (CIPC_PRECISION_MIXED).
//
// Same algorithm and lane-refill loop as the FP64 variant (ccd_core.cuh), with the
// arithmetic split by what needs FP64 on a part whose FP64 pipe is 1/64 of FP32:
//   * A pair is carried by its translation-free difference vectors, which are
//     affine in time: r(s) = r(0) + s dr, evaluated with one FP64 fma per
//     component from the t = 0 values (no accumulated position updates).
//   * Region classification (which of the 7 point-triangle / 9 edge-edge / 3
//     point-edge closest-feature regions) runs in FP32 on FP32 copies of r(s).
//   * The distance function f = d^2 - xi^2 of the chosen region is formed in FP64
//     as a numerator/denominator pair (num = u^2 - xi^2 w with u a triple
//     product, or |w x e|^2 - xi^2 |e|^2), because the triple product cancels
//     when the separation is tiny against the primitive size; only the final
//     ratio is taken in FP32.
//   * The conservative step (1-eta) f / ((d + xi) maxDispMag), the stopping test
//     and d = sqrt(d^2) are FP32 (relative error ~1e-7 against the eta = 0.1
//     slack of the bound); the accumulated time of impact is FP64.
// Results differ from the FP64 variant when a pair sits within FP32 rounding of a
// region boundary or of the stopping threshold (then ACCD may stop one
// conservative step earlier or later); both answers are conservative.
#include <cuda_runtime.h>

#include "ccd_core.cuh"
#include "cipc_internal.h"

namespace cipc {

struct f3 {
    float x, y, z;
};
CIPC_HD f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
CIPC_HD f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
CIPC_HD f3 fneg(f3 a) { return f3{-a.x, -a.y, -a.z}; }
CIPC_HD float fdot(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
CIPC_HD f3 fcross(f3 a, f3 b)
{
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
CIPC_HD f3 tf(d3 v) { return f3{(float)v.x, (float)v.y, (float)v.z}; }
CIPC_HD f3 faxpy(float s, f3 d, f3 x) { return f3{fmaf(s, d.x, x.x), fmaf(s, d.y, x.y), fmaf(s, d.z, x.z)}; }

// point-triangle region from a = p - t0, e1 = t1 - t0, e2 = t2 - t0 (the basis
// (r0, r0 x n) is orthogonal, so the edge parameter and the side decouple)
CIPC_HD int pt_region_f(f3 a, f3 e1, f3 e2)
{
    const f3 n = fcross(e1, e2);
    const float s0 = fdot(e1, a) / fdot(e1, e1), q0 = fdot(fcross(e1, n), a);
    if (s0 > 0.f && s0 < 1.f && q0 >= 0.f) return 3;
    const f3 r1 = e2 - e1, v1 = a - e1;
    const float s1 = fdot(r1, v1) / fdot(r1, r1), q1 = fdot(fcross(r1, n), v1);
    if (s1 > 0.f && s1 < 1.f && q1 >= 0.f) return 4;
    const f3 r2 = fneg(e2), v2 = a - e2;
    const float s2 = fdot(r2, v2) / fdot(r2, r2), q2 = fdot(fcross(r2, n), v2);
    if (s2 > 0.f && s2 < 1.f && q2 >= 0.f) return 5;
    if (s0 <= 0.f && s2 >= 1.f) return 0;
    if (s1 <= 0.f && s0 >= 1.f) return 1;
    if (s2 <= 0.f && s1 >= 1.f) return 2;
    return 6;
}

// edge-edge region from u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0
CIPC_HD int ee_region_f(f3 u, f3 v, f3 w)
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

// (num, den) with f = num / den, d^2 = sq / den
struct Frac {
    double num, sq, den;
};
CIPC_HD Frac pp_frac(d3 d, double th2)
{
    const double q = n2(d);
    return Frac{q - th2, q, 1.0};
}
// point at w (relative to an edge endpoint) against the line of edge e
CIPC_HD Frac line_frac(d3 w, d3 e, double th2)
{
    const double N = n2(cross(w, e)), D = n2(e);
    return Frac{fma(-th2, D, N), N, D};
}
// point at a (relative to t0) against the plane of (e1, e2) / line-line for EE
CIPC_HD Frac plane_frac(d3 a, d3 e1, d3 e2, double th2)
{
    const d3 nn = cross(e1, e2);
    const double u = dot(a, nn), w = n2(nn);
    const double uu = u * u;
    return Frac{fma(-th2, w, uu), uu, w};
}

struct MixedLane {
    d3 r0[3], dr[3];   // FP64 difference vectors at t = 0 and their rates
    f3 q0[3], dq[3];   // FP32 copies for classification
};

// distance function at time s for the lane's pair: returns f as (num, sq, den)
CIPC_HD Frac mixed_eval(int tp, const MixedLane& L, double s, float sf, double th2)
{
    switch (tp) {
        case kPP: return pp_frac(axpy(s, L.dr[0], L.r0[0]), th2);
        case kPE: {
            // r[0] = w = p - e0, r[1] = e = e1 - e0
            const d3 w = axpy(s, L.dr[0], L.r0[0]), e = axpy(s, L.dr[1], L.r0[1]);
            const f3 wf = faxpy(sf, L.dq[0], L.q0[0]), ef = faxpy(sf, L.dq[1], L.q0[1]);
            const float c1 = fdot(wf, ef), c2 = fdot(ef, ef);
            if (c1 <= 0.f) return pp_frac(w, th2);
            if (c2 <= c1) return pp_frac(w - e, th2);
            return line_frac(w, e, th2);
        }
        case kPT: {
            // r[0] = a = p - t0, r[1] = e1 = t1 - t0, r[2] = e2 = t2 - t0
            const d3 a = axpy(s, L.dr[0], L.r0[0]), e1 = axpy(s, L.dr[1], L.r0[1]), e2 = axpy(s, L.dr[2], L.r0[2]);
            const f3 af = faxpy(sf, L.dq[0], L.q0[0]), e1f = faxpy(sf, L.dq[1], L.q0[1]),
                     e2f = faxpy(sf, L.dq[2], L.q0[2]);
            switch (pt_region_f(af, e1f, e2f)) {
                case 0: return pp_frac(a, th2);
                case 1: return pp_frac(a - e1, th2);
                case 2: return pp_frac(a - e2, th2);
                case 3: return line_frac(a, e1, th2);
                case 4: return line_frac(a - e1, e2 - e1, th2);
                case 5: return line_frac(a - e2, e2, th2);
                default: return plane_frac(a, e1, e2, th2);
            }
        }
        default: {
            // r[0] = u = ea1 - ea0, r[1] = v = eb1 - eb0, r[2] = w = ea0 - eb0
            const d3 u = axpy(s, L.dr[0], L.r0[0]), v = axpy(s, L.dr[1], L.r0[1]), w = axpy(s, L.dr[2], L.r0[2]);
            const f3 uf = faxpy(sf, L.dq[0], L.q0[0]), vf = faxpy(sf, L.dq[1], L.q0[1]),
                     wf = faxpy(sf, L.dq[2], L.q0[2]);
            Frac F;
            switch (ee_region_f(uf, vf, wf)) {
                case 0: F = pp_frac(w, th2); break;
                case 1: F = pp_frac(w - v, th2); break;
                case 2: F = line_frac(w, v, th2); break;
                case 3: F = pp_frac(w + u, th2); break;
                case 4: F = pp_frac((w + u) - v, th2); break;
                case 5: F = line_frac(w + u, v, th2); break;
                case 6: F = line_frac(w, u, th2); break;
                case 7: F = line_frac(v - w, u, th2); break;
                default: F = plane_frac(w, u, v, th2); break;
            }
            if (!(F.num > 0) || !(F.den > 0)) {  // CCD.h:339-345 fallback (nearly parallel edges)
                const double p0 = n2(w), p1 = n2(w - v), p2 = n2(w + u), p3 = n2((w + u) - v);
                const double m = dmin(dmin(dmin(p0, p1), p2), p3);
                F = Frac{m - th2, m, 1.0};
            }
            return F;
        }
    }
}

// Per-lane ACCD state and its two operations, shared by the kernel's lane-refill
// loop and host-side checks.
struct MixedState {
    MixedLane L;
    int tp, phase;
    float maxDisp, gap;
    double t, s, tlb;
    int64_t adv;
};

// Loads pair pid.  Returns 0 when the pair needs stepping, otherwise writes the
// pair's result and returns 1 (no motion) or 2 (invalid pair).
CIPC_HD int mixed_init(const CcdArgs& a, int64_t pid, MixedState& S)
{
    S.tp = a.type[pid];
    const int4 id = a.idx[pid];
    const int tp = S.tp;
    const int nv = tp == kPP ? 2 : (tp == kPE ? 3 : 4);
    const int ids[4] = {id.x, id.y, id.z, id.w};
    bool ok = tp <= kEE;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k < nv) ok = ok && ids[k] >= 0 && ids[k] < a.nv;
    if (!ok) {
        a.toc_out[pid] = a.toc_in;
        a.hit[pid] = 0;
        if (a.iters) a.iters[pid] = 0;
        return 2;
    }
    d3 v[4], dv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k < nv) {
            v[k] = ld(a.x, ids[k]);
            dv[k] = ld(a.dx, ids[k]);
        } else {
            v[k] = mk(0, 0, 0);
            dv[k] = mk(0, 0, 0);
        }
    }
    MixedLane& L = S.L;
    // difference vectors and their rates (differences of displacements are
    // unaffected by removing the mean displacement)
    switch (tp) {
        case kPP:
            L.r0[0] = v[0] - v[1];
            L.dr[0] = dv[0] - dv[1];
            L.r0[1] = L.r0[2] = L.dr[1] = L.dr[2] = mk(0, 0, 0);
            break;
        case kPE:
            L.r0[0] = v[0] - v[1];
            L.dr[0] = dv[0] - dv[1];
            L.r0[1] = v[2] - v[1];
            L.dr[1] = dv[2] - dv[1];
            L.r0[2] = L.dr[2] = mk(0, 0, 0);
            break;
        case kPT:
            L.r0[0] = v[0] - v[1];
            L.dr[0] = dv[0] - dv[1];
            L.r0[1] = v[2] - v[1];
            L.dr[1] = dv[2] - dv[1];
            L.r0[2] = v[3] - v[1];
            L.dr[2] = dv[3] - dv[1];
            break;
        default:
            L.r0[0] = v[1] - v[0];
            L.dr[0] = dv[1] - dv[0];
            L.r0[1] = v[3] - v[2];
            L.dr[1] = dv[3] - dv[2];
            L.r0[2] = v[0] - v[2];
            L.dr[2] = dv[0] - dv[2];
            break;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        L.q0[k] = tf(L.r0[k]);
        L.dq[k] = tf(L.dr[k]);
    }
    S.maxDisp = (float)ccd_prepare(tp, dv);
    S.adv = 0;
    S.phase = 0;
    S.s = 0;
    S.t = 0;
    S.tlb = 0;
    if (S.maxDisp == 0.f) {
        a.toc_out[pid] = a.toc_in;
        a.hit[pid] = 0;
        if (a.iters) a.iters[pid] = 0;
        return 1;
    }
    return 0;
}

// One ACCD step.  Returns 0 to continue, 1 when the pair finished (result
// written), 3 when it reached the iteration cap (reported as no hit).
CIPC_HD int mixed_step(const CcdArgs& a, int64_t pid, MixedState& S)
{
    const double th2 = a.th * a.th, toc_prev = a.toc_in;
    const float thf = (float)a.th, etaf = (float)a.eta, oneme = 1.0f - (float)a.eta;
    const Frac F = mixed_eval(S.tp, S.L, S.s, (float)S.s, th2);
    const float den = (float)F.den;
    const float ff = (float)F.num / den;          // f = d^2 - xi^2
    const float dist = sqrtf((float)F.sq / den);  // d
    const float ratio = ff / (dist + thf);         // (d^2 - xi^2) / (d + xi)
    if (S.phase == 0) {
        S.gap = etaf * ratio;
        S.t = 0;
        S.phase = 1;
    } else {
        if (S.t != 0 && ratio < S.gap) {
            a.toc_out[pid] = S.t;
            a.hit[pid] = 1;
            if (a.iters) a.iters[pid] = (int32_t)S.adv;
            return 1;
        }
        S.t += S.tlb;
        if (S.t > toc_prev) {
            a.toc_out[pid] = toc_prev;
            a.hit[pid] = 0;
            if (a.iters) a.iters[pid] = (int32_t)S.adv;
            return 1;
        }
    }
    if (S.adv >= a.max_iter) {
        a.toc_out[pid] = toc_prev;
        a.hit[pid] = 0;
        if (a.iters) a.iters[pid] = (int32_t)S.adv;
        return 3;
    }
    S.tlb = (double)(oneme * ratio / S.maxDisp);
    S.s = S.t + S.tlb;
    ++S.adv;
    return 0;
}

#ifdef __CUDACC__
__global__ void __launch_bounds__(256) k_accd_mixed(CcdArgs a)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int64_t pid = -1;
    bool exhausted = false;
    bool fresh = false;
    MixedState S;
    while (true) {
        const bool need = (pid < 0) && !exhausted;
        const unsigned m = __ballot_sync(FULL, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(m));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const unsigned long long my = base + __popc(m & ((1u << lane) - 1u));
                if (my < (unsigned long long)a.n) {
                    pid = (int64_t)my;
                    fresh = true;
                } else {
                    exhausted = true;
                }
            }
        }
        const bool active = pid >= 0;
        if (!__any_sync(FULL, active)) break;
        if (!active) continue;
        if (fresh) {
            fresh = false;
            const int r = mixed_init(a, pid, S);
            if (r) {
                if (r == 2) atomicAdd(a.counter + 2, 1ull);
                pid = -1;
                continue;
            }
        }
        const int r = mixed_step(a, pid, S);
        if (r) {
            if (r == 3) atomicAdd(a.counter + 1, 1ull);
            pid = -1;
        }
    }
}
#endif

cudaError_t launch_accd_mixed(const CcdArgs& a, int grid, cudaStream_t s)
{
    k_accd_mixed<<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

int accd_mixed_blocks_per_sm()
{
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_accd_mixed, 256, 0);
    return b > 0 ? b : 1;
}

}  // namespace cipc
