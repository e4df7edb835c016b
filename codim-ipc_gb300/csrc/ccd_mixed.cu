// ACCD, mixed-precision variant (CIPC_PRECISION_MIXED).
//
// Same algorithm and lane-refill loop as the FP64 variant (ccd_core.cuh), with no
// FP64 arithmetic in the loop, on a part whose FP64 pipe issues 1/64 of the FP32
// rate (the previous form of this kernel, FP64 distance numerators, kept the FP64
// pipe 87% busy with the FP32 pipe at 1.5%):
//   * A pair is carried by its translation-free difference vectors r(s) = r(0) +
//     s dr, affine in time.  The 18 differences (positions and displacements) are
//     the only FP64 operations: one subtraction each, exact for nearby vertices
//     (Sterbenz), so precision does not depend on where the scene sits; they are
//     then split into float-float values (ff.cuh) by integer operations on their
//     bit patterns, and r(s) is evaluated in float-float from the t = 0 values (no
//     accumulated position updates).
//   * Each pair is rescaled by a power of two (exact) so that its largest
//     difference component is ~1: ACCD's step and stopping test are invariant under
//     a common scaling of positions, displacements and xi, and the FP32 ratios
//     below then neither underflow nor overflow whatever the scene's units.
//   * Region classification (which of the 7 point-triangle / 9 edge-edge / 3
//     point-edge closest-feature regions) runs in FP32 on the high parts of r(s).
//   * The distance function f = d^2 - xi^2 of the chosen region is formed in
//     float-float as a numerator/denominator pair (num = u^2 - xi^2 w with u a
//     triple product, or |w x e|^2 - xi^2 |e|^2), because the triple product
//     cancels when the separation is tiny against the primitive size (~48
//     significant bits against FP64's 53); only the final ratio is taken in FP32.
//   * The conservative step (1-eta) f / ((d + xi) maxDispMag), the stopping test,
//     d = sqrt(d^2) and maxDispMag (from the difference rates) are FP32 (relative
//     error ~1e-7 against the eta = 0.1 slack of the bound); the accumulated time
//     of impact is float-float.
// Results differ from the FP64 variant when a pair sits within FP32 rounding of a
// region boundary or of the stopping threshold (then ACCD may stop one
// conservative step earlier or later); both answers are conservative.
#include <cuda_runtime.h>

#include "ccd_core.cuh"
#include "ff.cuh"
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

// Edge parameter s = num / den (den = |r|^2 >= 0) compared with 0 and 1 without
// the division; at den == 0 the tests give what the division's infinity / NaN
// would (num > 0: +inf, num < 0: -inf, num == 0: NaN, every test false).
struct EdgeParam {
    float num, den;
};
CIPC_HD bool ep_in01(EdgeParam p) { return p.num > 0.f && p.num < p.den; }
CIPC_HD bool ep_le0(EdgeParam p) { return p.num <= 0.f && (p.num != 0.f || p.den != 0.f); }
CIPC_HD bool ep_ge1(EdgeParam p) { return p.num >= p.den && p.num > 0.f; }

// point-triangle region from a = p - t0, e1 = t1 - t0, e2 = t2 - t0 (the basis
// (r0, r0 x n) is orthogonal, so the edge parameter and the side decouple)
CIPC_HD int pt_region_f(f3 a, f3 e1, f3 e2)
{
    const f3 n = fcross(e1, e2);
    const EdgeParam s0{fdot(e1, a), fdot(e1, e1)};
    const float q0 = fdot(fcross(e1, n), a);
    if (ep_in01(s0) && q0 >= 0.f) return 3;
    const f3 r1 = e2 - e1, v1 = a - e1;
    const EdgeParam s1{fdot(r1, v1), fdot(r1, r1)};
    const float q1 = fdot(fcross(r1, n), v1);
    if (ep_in01(s1) && q1 >= 0.f) return 4;
    const f3 r2 = fneg(e2), v2 = a - e2;
    const EdgeParam s2{fdot(r2, v2), fdot(r2, r2)};
    const float q2 = fdot(fcross(r2, n), v2);
    if (ep_in01(s2) && q2 >= 0.f) return 5;
    if (ep_le0(s0) && ep_ge1(s2)) return 0;
    if (ep_le0(s1) && ep_ge1(s0)) return 1;
    if (ep_le0(s2) && ep_ge1(s1)) return 2;
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

// f = num / den, d^2 = sq / den
struct Frac {
    ff num;
    float sq, den;
};
__device__ __forceinline__ Frac pp_frac(const ff3& d, const ff& th2)
{
    const ff q = ff3_n2(d);
    return Frac{ff_sub(q, th2), q.hi, 1.f};
}
// point at w (relative to an edge endpoint) against the line of edge e
__device__ __forceinline__ Frac line_frac(const ff3& w, const ff3& e, const ff& th2)
{
    const ff N = ff3_n2(ff3_cross(w, e)), D = ff3_n2(e);
    return Frac{ff_fma(ff_neg(th2), D, N), N.hi, D.hi};
}
// point at a (relative to t0) against the plane of (e1, e2) / line-line for EE
__device__ __forceinline__ Frac plane_frac(const ff3& a, const ff3& e1, const ff3& e2, const ff& th2)
{
    const ff3 nn = ff3_cross(e1, e2);
    const ff u = ff3_dot(a, nn), w = ff3_n2(nn);
    const ff uu = ff_mul(u, u);
    return Frac{ff_fma(ff_neg(th2), w, uu), uu.hi, w.hi};
}

__device__ __forceinline__ f3 hi3(const ff3& v) { return f3{v.x.hi, v.y.hi, v.z.hi}; }

struct MixedLane {
    ff3 r0[3], dr[3];  // scaled difference vectors at t = 0 and their rates
};

// distance function at time s for the lane's pair
__device__ __forceinline__ Frac mixed_eval(int tp, const MixedLane& L, ff s, const ff& th2)
{
    switch (tp) {
        case kPP: return pp_frac(ff3_axpy(s, L.dr[0], L.r0[0]), th2);
        case kPE: {
            // r[0] = w = p - e0, r[1] = e = e1 - e0
            const ff3 w = ff3_axpy(s, L.dr[0], L.r0[0]), e = ff3_axpy(s, L.dr[1], L.r0[1]);
            const f3 wf = hi3(w), ef = hi3(e);
            const float c1 = fdot(wf, ef), c2 = fdot(ef, ef);
            if (c1 <= 0.f) return pp_frac(w, th2);
            if (c2 <= c1) return pp_frac(ff3_sub(w, e), th2);
            return line_frac(w, e, th2);
        }
        case kPT: {
            // r[0] = a = p - t0, r[1] = e1 = t1 - t0, r[2] = e2 = t2 - t0
            const ff3 a = ff3_axpy(s, L.dr[0], L.r0[0]), e1 = ff3_axpy(s, L.dr[1], L.r0[1]),
                      e2 = ff3_axpy(s, L.dr[2], L.r0[2]);
            switch (pt_region_f(hi3(a), hi3(e1), hi3(e2))) {
                case 0: return pp_frac(a, th2);
                case 1: return pp_frac(ff3_sub(a, e1), th2);
                case 2: return pp_frac(ff3_sub(a, e2), th2);
                case 3: return line_frac(a, e1, th2);
                case 4: return line_frac(ff3_sub(a, e1), ff3_sub(e2, e1), th2);
                case 5: return line_frac(ff3_sub(a, e2), e2, th2);
                default: return plane_frac(a, e1, e2, th2);
            }
        }
        default: {
            // r[0] = u = ea1 - ea0, r[1] = v = eb1 - eb0, r[2] = w = ea0 - eb0
            const ff3 u = ff3_axpy(s, L.dr[0], L.r0[0]), v = ff3_axpy(s, L.dr[1], L.r0[1]),
                      w = ff3_axpy(s, L.dr[2], L.r0[2]);
            Frac F;
            switch (ee_region_f(hi3(u), hi3(v), hi3(w))) {
                case 0: F = pp_frac(w, th2); break;
                case 1: F = pp_frac(ff3_sub(w, v), th2); break;
                case 2: F = line_frac(w, v, th2); break;
                case 3: F = pp_frac(ff3_add(w, u), th2); break;
                case 4: F = pp_frac(ff3_sub(ff3_add(w, u), v), th2); break;
                case 5: F = line_frac(ff3_add(w, u), v, th2); break;
                case 6: F = line_frac(w, u, th2); break;
                case 7: F = line_frac(ff3_sub(v, w), u, th2); break;
                default: F = plane_frac(w, u, v, th2); break;
            }
            if (!(F.num.hi > 0.f) || !(F.den > 0.f)) {  // CCD.h:339-345 fallback (nearly parallel edges)
                const ff wu = ff3_n2(ff3_add(w, u));
                ff m = ff3_n2(w);
                const ff p1 = ff3_n2(ff3_sub(w, v)), p3 = ff3_n2(ff3_sub(ff3_add(w, u), v));
                if (ff_gt(m, p1)) m = p1;
                if (ff_gt(m, wu)) m = wu;
                if (ff_gt(m, p3)) m = p3;
                F = Frac{ff_sub(m, th2), m.hi, 1.f};
            }
            return F;
        }
    }
}

// Per-lane ACCD state and its two operations, used by the kernel's lane-refill loop.
struct MixedState {
    MixedLane L;
    ff th2;        // (scaled xi)^2
    ff t, s;       // accumulated time of impact and the time of the next evaluation
    float thf;     // scaled xi
    float rmd;     // (1 - eta) / maxDispMag (scaled)
    float gap, tlb;
    int tp, phase;
    int64_t adv;
};

__device__ __forceinline__ ff3 ffd(d3 a) { return ff3{ff_from_double(a.x), ff_from_double(a.y), ff_from_double(a.z)}; }
__device__ __forceinline__ float f3_norm(f3 a) { return sqrtf(fdot(a, a)); }
__device__ __forceinline__ float amax3(const ff3& v)
{
    return fmaxf(fmaxf(fabsf(v.x.hi), fabsf(v.y.hi)), fabsf(v.z.hi));
}

// Sets up pair pid from its vertices (positions v, displacements dv).  Returns 0 when the pair needs stepping, otherwise writes the
// pair's result and returns 1 (no motion).
__device__ __forceinline__ int mixed_init(const CcdArgs& a, const ff& th_ff, float oneme, int64_t pid, int tp,
                                          const d3 (&v)[4], const d3 (&dv)[4], MixedState& S)
{
    S.tp = tp;
    const ff3 z3 = ff3{ffv(0.f), ffv(0.f), ffv(0.f)};
    MixedLane& L = S.L;
    // difference vectors and their rates, and maxDispMag from the rates: the
    // reference removes the mean displacement (CCD.h:290-299, 320-329, 395-401,
    // 445-450); relative to vertex b, with D_k = dv_k - dv_b and M the mean of the
    // D_k, vertex k moves by D_k - M
    float maxDisp;
    switch (tp) {
        case kPP: {
            L.r0[0] = ffd(v[0] - v[1]);
            L.dr[0] = ffd(dv[0] - dv[1]);
            L.r0[1] = L.r0[2] = L.dr[1] = L.dr[2] = z3;
            maxDisp = f3_norm(hi3(L.dr[0]));
            break;
        }
        case kPE: {
            L.r0[0] = ffd(v[0] - v[1]);
            L.dr[0] = ffd(dv[0] - dv[1]);
            L.r0[1] = ffd(v[2] - v[1]);
            L.dr[1] = ffd(dv[2] - dv[1]);
            L.r0[2] = L.dr[2] = z3;
            const f3 B0 = hi3(L.dr[0]), B2 = hi3(L.dr[1]);
            const float third = 1.f / 3.f;
            const f3 M = f3{(B0.x + B2.x) * third, (B0.y + B2.y) * third, (B0.z + B2.z) * third};
            maxDisp = f3_norm(B0 - M) + fmaxf(f3_norm(M), f3_norm(B2 - M));
            break;
        }
        case kPT: {
            L.r0[0] = ffd(v[0] - v[1]);
            L.dr[0] = ffd(dv[0] - dv[1]);
            L.r0[1] = ffd(v[2] - v[1]);
            L.dr[1] = ffd(dv[2] - dv[1]);
            L.r0[2] = ffd(v[3] - v[1]);
            L.dr[2] = ffd(dv[3] - dv[1]);
            const f3 D0 = hi3(L.dr[0]), D2 = hi3(L.dr[1]), D3 = hi3(L.dr[2]);
            const f3 M = f3{0.25f * (D0.x + D2.x + D3.x), 0.25f * (D0.y + D2.y + D3.y), 0.25f * (D0.z + D2.z + D3.z)};
            maxDisp = f3_norm(D0 - M) + fmaxf(fmaxf(f3_norm(M), f3_norm(D2 - M)), f3_norm(D3 - M));
            break;
        }
        default: {
            L.r0[0] = ffd(v[1] - v[0]);
            L.dr[0] = ffd(dv[1] - dv[0]);
            L.r0[1] = ffd(v[3] - v[2]);
            L.dr[1] = ffd(dv[3] - dv[2]);
            L.r0[2] = ffd(v[0] - v[2]);
            L.dr[2] = ffd(dv[0] - dv[2]);
            // relative to eb0: ea0 moves by A0 = w rate, ea1 by A0 + u rate, eb1 by v rate
            const f3 A0 = hi3(L.dr[2]), A1 = hi3(L.dr[2]) + hi3(L.dr[0]), A3 = hi3(L.dr[1]);
            const f3 M = f3{0.25f * (A0.x + A1.x + A3.x), 0.25f * (A0.y + A1.y + A3.y), 0.25f * (A0.z + A1.z + A3.z)};
            maxDisp = fmaxf(f3_norm(A0 - M), f3_norm(A1 - M)) + fmaxf(f3_norm(M), f3_norm(A3 - M));
            break;
        }
    }
    S.adv = 0;
    S.phase = 0;
    S.t = ffv(0.f);
    S.s = ffv(0.f);
    S.tlb = 0.f;
    if (maxDisp == 0.f) {
        a.toc_out[pid] = a.toc_in;
        a.hit[pid] = 0;
        if (a.iters) a.iters[pid] = 0;
        return 1;
    }
    // power-of-two rescaling: largest difference component to [1, 2)
    float m = fmaxf(fmaxf(amax3(L.r0[0]), amax3(L.r0[1])), amax3(L.r0[2]));
    if (m == 0.f) m = maxDisp;
    const int em = (int)((__float_as_uint(m) >> 23) & 0xffu);
    const int k = min(max(127 - em, -100), 100);
    const float sc = __uint_as_float((unsigned)(127 + k) << 23);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        L.r0[j] = ff3_scale(L.r0[j], sc);
        L.dr[j] = ff3_scale(L.dr[j], sc);
    }
    S.rmd = oneme / (maxDisp * sc);
    const ff ths = ff_scale(th_ff, sc);
    S.thf = ths.hi;
    S.th2 = ff_mul(ths, ths);
    return 0;
}

// One ACCD step.  Returns 0 to continue, 1 when the pair finished (result
// written), 3 when it reached the iteration cap (reported as no hit).
__device__ __forceinline__ int mixed_step(const CcdArgs& a, const ff& tocp, float etaf, int64_t pid, MixedState& S)
{
    const Frac F = mixed_eval(S.tp, S.L, S.s, S.th2);
    const float rden = __frcp_rn(F.den);
    const float ffv_ = F.num.hi * rden;                  // f = d^2 - xi^2
    const float dist = sqrtf(F.sq * rden);               // d
    const float ratio = __fdividef(ffv_, dist + S.thf);  // (d^2 - xi^2) / (d + xi); d + xi ~ 1 after scaling
    if (S.phase == 0) {
        S.gap = etaf * ratio;
        S.phase = 1;
    } else {
        if (S.t.hi != 0.f && ratio < S.gap) {
            a.toc_out[pid] = ff_to_double(S.t);
            a.hit[pid] = 1;
            if (a.iters) a.iters[pid] = (int32_t)S.adv;
            return 1;
        }
        S.t = S.s;  // t += tlb
        if (ff_gt(S.t, tocp)) {
            a.toc_out[pid] = a.toc_in;
            a.hit[pid] = 0;
            if (a.iters) a.iters[pid] = (int32_t)S.adv;
            return 1;
        }
    }
    if (S.adv >= a.max_iter) {
        a.toc_out[pid] = a.toc_in;
        a.hit[pid] = 0;
        if (a.iters) a.iters[pid] = (int32_t)S.adv;
        return 3;
    }
    S.tlb = ratio * S.rmd;
    S.s = ff_add_f(S.t, S.tlb);
    ++S.adv;
    return 0;
}

#ifdef __CUDACC__
// Refills are prefetched in two stages per lane, so that a lane taking a new pair
// does not hold its warp for two dependent global round trips (pair record, then
// vertices).  Stage A: a claimed pair with its type and vertex ids in registers.
// Stage B: the next pair, its vertices' positions and displacements copied into
// the lane's shared-memory slot by cp.async; each lane has two slots used in
// turn, so a copy never targets the slot that was read last.  A lane whose pair
// finishes takes B (its copies were issued one refill earlier), moves A to B and
// claims a new A.
constexpr int kAccdThreads = 256;
constexpr int kSlotDoubles = 24;  // 4 vertices x (position, displacement) x 3
constexpr int kAccdSmem = 2 * kSlotDoubles * kAccdThreads * (int)sizeof(double);

__device__ __forceinline__ void cp_async8(double* dst, const double* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ int pair_nv(int tp) { return tp == kPP ? 2 : (tp == kPE ? 3 : 4); }

__global__ void __launch_bounds__(kAccdThreads) k_accd_mixed(CcdArgs a)
{
    extern __shared__ double sbuf[];  // [slot][k][thread], k = 3 v + c (positions), 12 + 3 v + c (displacements)
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, tid = threadIdx.x;
    const ff tocp0 = ff_from_double(a.toc_in), th_ff = ff_from_double(a.th);
    const ff tocp = fast_two_sum(tocp0.hi, tocp0.lo);  // normalised for ff_gt
    const float etaf = (float)a.eta, oneme = 1.0f - etaf;
    int64_t pid = -1;                 // pair being stepped
    int64_t bp = -1;                  // stage B pair
    int btp = 0, bslot = 0;           // its type (-1: invalid record, nothing copied) and slot
    int64_t ap = -1;                  // stage A pair
    int atp = 0;
    int4 aid = make_int4(0, 0, 0, 0);
    bool exhausted = false;
    MixedState S;
    while (true) {
        // claim stage A
        const bool want = ap < 0 && !exhausted;
        const unsigned m = __ballot_sync(FULL, want);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(m));
            base = __shfl_sync(FULL, base, leader);
            if (want) {
                const unsigned long long my = base + __popc(m & ((1u << lane) - 1u));
                if (my < (unsigned long long)a.n) {
                    ap = (int64_t)my;
                    atp = a.type[ap];
                    aid = a.idx[ap];
                } else {
                    exhausted = true;
                }
            }
        }
        // take stage B
        if (pid < 0 && bp >= 0) {
            const int64_t q = bp;
            const int tq = btp;
            const double* slot = sbuf + bslot * (kSlotDoubles * kAccdThreads);
            bp = -1;
            bslot ^= 1;
            if (tq < 0) {  // invalid record: reported, never dereferenced
                a.toc_out[q] = a.toc_in;
                a.hit[q] = 0;
                if (a.iters) a.iters[q] = 0;
                atomicAdd(a.counter + 2, 1ull);
            } else {
                cp_async_wait_all();
                const int nv = pair_nv(tq);
                d3 v[4], dv[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (k < nv) {
                        const double* px = slot + (3 * k) * kAccdThreads + tid;
                        const double* pd = slot + (12 + 3 * k) * kAccdThreads + tid;
                        v[k] = d3{px[0], px[kAccdThreads], px[2 * kAccdThreads]};
                        dv[k] = d3{pd[0], pd[kAccdThreads], pd[2 * kAccdThreads]};
                    } else {
                        v[k] = mk(0, 0, 0);
                        dv[k] = mk(0, 0, 0);
                    }
                }
                if (mixed_init(a, th_ff, oneme, q, tq, v, dv, S) == 0) pid = q;
            }
        }
        // move stage A to B: validate the record, then copy its vertices
        if (bp < 0 && ap >= 0) {
            const int nv = pair_nv(atp);
            const int ids[4] = {aid.x, aid.y, aid.z, aid.w};
            bool ok = atp <= kEE;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < nv) ok = ok && ids[k] >= 0 && ids[k] < a.nv;
            if (ok) {
                double* slot = sbuf + bslot * (kSlotDoubles * kAccdThreads);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (k < nv) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            cp_async8(slot + (3 * k + c) * kAccdThreads + tid, a.x + 3 * (int64_t)ids[k] + c);
                            cp_async8(slot + (12 + 3 * k + c) * kAccdThreads + tid, a.dx + 3 * (int64_t)ids[k] + c);
                        }
                    }
                }
                cp_async_commit();
                btp = atp;
            } else {
                btp = -1;
            }
            bp = ap;
            ap = -1;
        }
        const bool busy = pid >= 0 || bp >= 0 || ap >= 0;
        if (!__any_sync(FULL, busy)) break;
        if (pid < 0) continue;
        const int r = mixed_step(a, tocp, etaf, pid, S);
        if (r) {
            if (r == 3) atomicAdd(a.counter + 1, 1ull);
            pid = -1;
        }
    }
    cp_async_wait_all();
}
#endif

cudaError_t launch_accd_mixed(const CcdArgs& a, int grid, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(k_accd_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, kAccdSmem);
    if (e != cudaSuccess) return e;
    k_accd_mixed<<<grid, kAccdThreads, kAccdSmem, s>>>(a);
    return cudaGetLastError();
}

int accd_mixed_blocks_per_sm()
{
    int b = 0;
    if (cudaFuncSetAttribute(k_accd_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, kAccdSmem) == cudaSuccess)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_accd_mixed, kAccdThreads, kAccdSmem);
    return b > 0 ? b : 1;
}

}  // namespace cipc
