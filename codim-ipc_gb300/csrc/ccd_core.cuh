// Additive CCD (ACCD) over a list of contact pairs, one lane per pair.
//
// Restates the reference's Point_Triangle_CCD / Edge_Edge_CCD / Point_Edge_CCD /
// Point_Point_CCD (Library/Math/Distance/CCD.h:279-483): remove the mean
// displacement, bound the relative motion by maxDispMag, and advance the time of
// impact by the conservative step (1-eta)(d^2 - xi^2) / ((d + xi) maxDispMag)
// until the distance function falls below eta times its initial value (hit) or
// the accumulated time passes the step fraction (no hit).
//
// GPU structure.  The iteration count differs per pair (one to thousands), so a
// pair-per-thread loop would leave most lanes of a warp idle behind the slowest
// pair.  Instead every lane runs one flat loop whose body is a single ACCD step:
// a lane whose pair has finished writes its result and takes the next pair from a
// global work counter (one atomicAdd per warp, ballot-aggregated).  Lanes stay
// busy until the list is drained; warps see pairs of one type as long as the list
// is grouped by type.  The loop is capped (max_iter steps per pair): a pair that
// reaches the cap is reported as an overflow instead of spinning.
#pragma once
#include "geom.cuh"

namespace cipc {

struct CcdArgs {
    int64_t n;
    const uint8_t* type;
    const int4* idx;
    const double* x;
    const double* dx;
    double eta, th, toc_in;
    int64_t max_iter;
    int64_t nv;                        // vertex count, for index validation
    double* toc_out;
    uint8_t* hit;
    int32_t* iters;                    // optional
    unsigned long long* counter;       // [0] work counter, [1] overflow count, [2] invalid pairs
    // Optional running minimum (bits of a non-negative double, initialised to
    // toc_in by the caller).  When set, a pair stops as soon as its time passes
    // the smallest time of impact found so far, and every hit lowers it: the
    // final minimum is the one the reference's sequential loop finds, where each
    // narrow-phase call is bounded by the step size found so far
    // (IPC.h:1959-2242), and pairs beyond it do no further work.  A pair that
    // reaches the iteration cap lowers it to the time it has safely advanced to.
    unsigned long long* toc_min = nullptr;
};

CIPC_HD double dmax(double a, double b) { return (a < b) ? b : a; }
CIPC_HD double dmin(double a, double b) { return (b < a) ? b : a; }

// Removes the mean displacement and returns maxDispMag (CCD.h:290-299, 320-329,
// 395-401, 445-450); v/dv hold (p,t0,t1,t2) / (ea0,ea1,eb0,eb1) / (p,e0,e1) / (p0,p1).
CIPC_HD double ccd_prepare(int tp, d3 (&dv)[4])
{
    switch (tp) {
        case kPP: {
            const d3 mov = scl(dv[0] + dv[1], 0.5);
            dv[1] = dv[1] - mov;
            dv[0] = dv[0] - mov;
            return sqrt(n2(dv[0])) + sqrt(n2(dv[1]));
        }
        case kPE: {
            const d3 mov = dvs((dv[0] + dv[1]) + dv[2], 3.0);
            dv[1] = dv[1] - mov;
            dv[2] = dv[2] - mov;
            dv[0] = dv[0] - mov;
            return sqrt(n2(dv[0])) + sqrt(dmax(n2(dv[1]), n2(dv[2])));
        }
        case kPT: {
            const d3 mov = scl(((dv[1] + dv[2]) + dv[3]) + dv[0], 0.25);
            dv[1] = dv[1] - mov;
            dv[2] = dv[2] - mov;
            dv[3] = dv[3] - mov;
            dv[0] = dv[0] - mov;
            const double m2 = dmax(dmax(n2(dv[1]), n2(dv[2])), n2(dv[3]));
            return sqrt(n2(dv[0])) + sqrt(m2);
        }
        default: {
            const d3 mov = scl(((dv[0] + dv[1]) + dv[2]) + dv[3], 0.25);
            dv[0] = dv[0] - mov;
            dv[1] = dv[1] - mov;
            dv[2] = dv[2] - mov;
            dv[3] = dv[3] - mov;
            return sqrt(dmax(n2(dv[0]), n2(dv[1]))) + sqrt(dmax(n2(dv[2]), n2(dv[3])));
        }
    }
}

__device__ __forceinline__ double load_min(const unsigned long long* p)
{
    return __longlong_as_double((long long)*(const volatile unsigned long long*)p);
}

template <class Pol>
__global__ void __launch_bounds__(256) k_accd(CcdArgs a)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double th = a.th, th2 = a.th * a.th, eta = a.eta, toc_prev = a.toc_in;
    int64_t pid = -1;
    bool exhausted = false;
    int tp = 0, phase = 0;
    d3 v[4], dv[4];
    double maxDisp = 0, gap = 0, t = 0, tlb = 0, lim = toc_prev;
    int64_t adv = 0;
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
                    phase = 0;
                } else {
                    exhausted = true;
                }
            }
        }
        const bool active = pid >= 0;
        if (!__any_sync(FULL, active)) break;
        if (!active) continue;
        if (phase == 0) {
            tp = a.type[pid];
            const int4 id = a.idx[pid];
            const int nv = tp == kPP ? 2 : (tp == kPE ? 3 : 4);
            const int ids[4] = {id.x, id.y, id.z, id.w};
            bool ok = tp <= kEE;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < nv) ok = ok && ids[k] >= 0 && ids[k] < a.nv;
            if (!ok) {  // invalid pair: reported, never dereferenced
                a.toc_out[pid] = toc_prev;
                a.hit[pid] = 0;
                if (a.iters) a.iters[pid] = 0;
                atomicAdd(a.counter + 2, 1ull);
                pid = -1;
                continue;
            }
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
            maxDisp = ccd_prepare(tp, dv);
            adv = 0;
            lim = a.toc_min ? dmin(toc_prev, load_min(a.toc_min)) : toc_prev;
            if (maxDisp == 0) {
                a.toc_out[pid] = toc_prev;
                a.hit[pid] = 0;
                if (a.iters) a.iters[pid] = 0;
                pid = -1;
                continue;
            }
        }
        double d2;
        const double f = Pol::dfunc(tp, v, th2, d2);
        const double dist = Pol::sqrt_(d2);
        if (phase == 0) {
            gap = eta * f / (dist + th);
            t = 0;
            phase = 1;
        } else {
            if (t != 0 && Pol::gap_less(f, dist + th, gap)) {
                a.toc_out[pid] = t;
                a.hit[pid] = 1;
                if (a.toc_min) atomicMin(a.toc_min, (unsigned long long)__double_as_longlong(t));
                if (a.iters) a.iters[pid] = (int32_t)adv;
                pid = -1;
                continue;
            }
            t += tlb;
            if (a.toc_min && (adv & 15) == 0) lim = dmin(lim, load_min(a.toc_min));
            if (t > lim) {
                a.toc_out[pid] = toc_prev;
                a.hit[pid] = 0;
                if (a.iters) a.iters[pid] = (int32_t)adv;
                pid = -1;
                continue;
            }
        }
        if (adv >= a.max_iter) {
            a.toc_out[pid] = toc_prev;
            a.hit[pid] = 0;
            if (a.toc_min) atomicMin(a.toc_min, (unsigned long long)__double_as_longlong(t));
            if (a.iters) a.iters[pid] = (int32_t)adv;
            atomicAdd(a.counter + 1, 1ull);
            pid = -1;
            continue;
        }
        tlb = Pol::div_((1 - eta) * f, (dist + th) * maxDisp);
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = axpy(tlb, dv[k], v[k]);
        ++adv;
    }
}

}  // namespace cipc

namespace cipc {

// ---------------------------------------------------------------------------
// Two-pass form of k_accd, same results bit for bit.
//
// In k_accd a lane that takes a new pair runs the set-up (mean removal, the
// displacement bound with its two square roots, the first distance and step)
// while the other lanes of its warp step their pairs; on GB300's narrow FP64 pipe
// that divergence idles ~40% of the FP64 issue slots (19 of 32 lanes active per
// instruction).  Here k_accd_setup does the set-up for every pair with converged
// warps (one thread per pair) and leaves each pair's state in memory
// (AccdState, 128 bytes); k_accd_steps then runs the lane-refill loop whose
// refill only loads that state, so every FP64 operation in the loop is the same
// step for all active lanes.  The operation sequence per pair is exactly k_accd's:
// setup computes f and dist at x0, the gap, and the first step tlb; the loop
// applies x1 = x0 + tlb dv (the same fma), starts with t = 0 and one step taken.
// ---------------------------------------------------------------------------
struct AccdState {
    double dv[12];         // displacements with the mean motion removed
    double maxDisp, gap, tlb;
    int32_t tp;            // pair type, or -1 when the set-up already wrote the result
    int32_t pad;
};
static_assert(sizeof(AccdState) == 128, "one 128-byte line per pair");

template <class Pol>
__global__ void __launch_bounds__(256) k_accd_setup(CcdArgs a, AccdState* __restrict__ st)
{
    const double th = a.th, th2 = a.th * a.th, eta = a.eta, toc_prev = a.toc_in;
    for (int64_t pid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pid < a.n;
         pid += (int64_t)gridDim.x * blockDim.x) {
        const int tp = a.type[pid];
        const int4 id = a.idx[pid];
        const int nv = tp == kPP ? 2 : (tp == kPE ? 3 : 4);
        const int ids[4] = {id.x, id.y, id.z, id.w};
        bool ok = tp <= kEE;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < nv) ok = ok && ids[k] >= 0 && ids[k] < a.nv;
        AccdState& S = st[pid];
        if (!ok) {  // invalid pair: reported, never dereferenced
            a.toc_out[pid] = toc_prev;
            a.hit[pid] = 0;
            if (a.iters) a.iters[pid] = 0;
            atomicAdd(a.counter + 2, 1ull);
            S.tp = -1;
            continue;
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
        const double maxDisp = ccd_prepare(tp, dv);
        if (maxDisp == 0) {
            a.toc_out[pid] = toc_prev;
            a.hit[pid] = 0;
            if (a.iters) a.iters[pid] = 0;
            S.tp = -1;
            continue;
        }
        double d2;
        const double f = Pol::dfunc(tp, v, th2, d2);
        const double dist = Pol::sqrt_(d2);
        S.gap = eta * f / (dist + th);
        S.tlb = Pol::div_((1 - eta) * f, (dist + th) * maxDisp);
        S.maxDisp = maxDisp;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            S.dv[3 * k] = dv[k].x;
            S.dv[3 * k + 1] = dv[k].y;
            S.dv[3 * k + 2] = dv[k].z;
        }
        S.tp = tp;
    }
}

// a.max_iter must be at least 1 (the set-up took the first step)
template <class Pol>
__global__ void __launch_bounds__(256) k_accd_steps(CcdArgs a, const AccdState* __restrict__ st)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double th = a.th, th2 = a.th * a.th, eta = a.eta, toc_prev = a.toc_in;
    int64_t pid = -1;
    bool exhausted = false;
    int tp = 0;
    d3 v[4], dv[4];
    double maxDisp = 0, gap = 0, t = 0, tlb = 0, lim = toc_prev;
    int64_t adv = 0;
    while (true) {
        // refill: pairs whose set-up wrote the result are skipped here
        bool need = (pid < 0) && !exhausted;
        while (__any_sync(FULL, need)) {
            const unsigned m = __ballot_sync(FULL, need);
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(m));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const unsigned long long my = base + __popc(m & ((1u << lane) - 1u));
                if (my >= (unsigned long long)a.n) {
                    exhausted = true;
                    need = false;
                } else {
                    const AccdState& S = st[my];
                    tp = S.tp;
                    if (tp >= 0) {
                        pid = (int64_t)my;
                        need = false;
                        const int4 id = a.idx[pid];
                        const int nv = tp == kPP ? 2 : (tp == kPE ? 3 : 4);
                        const int ids[4] = {id.x, id.y, id.z, id.w};
                        maxDisp = S.maxDisp;
                        gap = S.gap;
                        tlb = S.tlb;
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            dv[k] = mk(S.dv[3 * k], S.dv[3 * k + 1], S.dv[3 * k + 2]);
                            v[k] = axpy(tlb, dv[k], k < nv ? ld(a.x, ids[k]) : mk(0, 0, 0));
                        }
                        t = 0;
                        adv = 1;
                        lim = a.toc_min ? dmin(toc_prev, load_min(a.toc_min)) : toc_prev;
                    }
                }
            }
        }
        const bool active = pid >= 0;
        if (!__any_sync(FULL, active)) break;
        if (!active) continue;
        double d2;
        const double f = Pol::dfunc(tp, v, th2, d2);
        const double dist = Pol::sqrt_(d2);
        if (t != 0 && Pol::gap_less(f, dist + th, gap)) {
            a.toc_out[pid] = t;
            a.hit[pid] = 1;
            if (a.toc_min) atomicMin(a.toc_min, (unsigned long long)__double_as_longlong(t));
            if (a.iters) a.iters[pid] = (int32_t)adv;
            pid = -1;
            continue;
        }
        t += tlb;
        if (a.toc_min && (adv & 15) == 0) lim = dmin(lim, load_min(a.toc_min));
        if (t > lim) {
            a.toc_out[pid] = toc_prev;
            a.hit[pid] = 0;
            if (a.iters) a.iters[pid] = (int32_t)adv;
            pid = -1;
            continue;
        }
        if (adv >= a.max_iter) {
            a.toc_out[pid] = toc_prev;
            a.hit[pid] = 0;
            if (a.toc_min) atomicMin(a.toc_min, (unsigned long long)__double_as_longlong(t));
            if (a.iters) a.iters[pid] = (int32_t)adv;
            atomicAdd(a.counter + 1, 1ull);
            pid = -1;
            continue;
        }
        tlb = Pol::div_((1 - eta) * f, (dist + th) * maxDisp);
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = axpy(tlb, dv[k], v[k]);
        ++adv;
    }
}

}  // namespace cipc
