// Preconditioned conjugate gradients on the Newton system as one persistent
// cooperative kernel per solve, every scalar kept on the device (replaces the
// reference's per-iteration CHOLMOD factorization and solve,
// Library/Math/DIRECT_SOLVER.h:13-88).
//
// Operator H = (elastic + mass, 3x3 block CSR) + sum over contact constraints of
// their stored PSD blocks (packed upper triangle, 78 per constraint) + sum over
// friction constraints of w_a w_b T M T^T (applied from the 2x2 inner matrix).
// Constraints whose blocks were folded into the rows (sim_fold.cu) are left out of
// the two constraint sums, which then run over the listed rest.
// The preconditioner is a 3x3 block per vertex (block Jacobi, or any other
// block-diagonal M^-1 written into the same array), or the inverses of the
// aggregates' diagonal blocks (aggregate block Jacobi, sim_aggregate.cu).
//
// Iteration k (standard PCG arithmetic, p_k = z_k + beta_k p_{k-1}), two phases
// separated by grid barriers:
//   apply    p_k is formed on the fly from z and p_{k-1} wherever it is
//            gathered; q_e = H_rows p_k one scalar row per thread (plain
//            stores), the matrix-free contact and friction parts are accumulated
//            into q_c with atomics, and p_k^T H p_k is summed element by element.
//   update   alpha = (r,z)/(p,Hp); x += alpha p; r -= alpha (q_e + q_c); q_c = 0;
//            z = M^-1 r (per vertex, or per aggregate by the block's warps); (r,z), (r,r).
// Each phase ends with a grid-wide sum (grid_allreduce): per-block partials, a
// release/acquire arrival counter, and a fixed-order sum of the partials read by
// every block, so every block takes the same stop decision.  The atomics of the
// matrix-free constraint part add in arrival order, so the last bits of q_c (and
// of the iterates) can differ from run to run.  Data written by other blocks
// during the solve is read through L2 (ld.global.cg), never from a stale L1 line.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/cipc.h"
#include "agg_rounds.h"
#include "cipc_util.h"
#include "constraint_eval.cuh"
#include "sim.h"
#include "sim_kernels.h"
#include "sim_pcg.h"

namespace cipc {

// results of one solve, and the grid reduction's state (zeroed before each solve)
struct PcgScalars {
    double rr;      // (r, r) at exit
    double bb;      // (b, b)
    double pq;      // last (p, Hp)
    int it;         // completed iterations
    int done;       // 1 converged, 2 NaN, 3 (p, Hp) <= 0, 4 iteration cap, 5 barrier wait gave up
    int err;
    int pad;
    // arrivals (monotone: gridDim.x per reduction), on its own 128-byte line
    alignas(128) unsigned int arrive;
    // with tracing on: block 0's time (ns) in apply, reduction 1, the aggregate
    // rows (part of update), update, reduction 2, the aggregate items (part of
    // update), summed over iterations
    unsigned long long tphase[6];
};

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// (z, p) pairs: iteration k reads z_k and p_{k-1} of a scalar row with one load
template <typename XT>
struct Pair;
template <>
struct Pair<float> {
    using T = float2;
};
template <>
struct Pair<double> {
    using T = double2;
};

template <typename VT, typename XT, typename PT>
struct PcgArgs {
    using XT2 = typename Pair<XT>::T;
    int nv, ell_k;
    const int* col;
    const int* rowlen;  // real blocks of each row (a row's later slots are zero padding)
    const VT* val;
    const int* ckind;
    const int4* cverts;
    const VT* chess;  // entry h of constraint c at chess[h * hs + c]
    size_t hs;
    const int* fkind;
    const int4* fverts;
    const double* fw;
    const double* fT;
    const double* fM;
    const uint8_t* proj;
    const PT* pinv;
    // aggregate block Jacobi (nagg > 0): vertices of aggregate g at
    // averts[avoff[g] .. avoff[g + 1]), its symmetric inverse block at ainv + aboff[g];
    // the blocks' rounds of aggregates (agg_phase)
    int nagg;
    const int* avoff;
    const int* averts;
    const long long* aboff;
    const PT* ainv;
    const int* abround;
    const int* arstart;
    const XT* b;
    XT* x;
    XT* r;
    XT2* zp[2];  // iteration k reads zp[k % 2] = (z_k, p_{k-1}); writes p_k and z_{k+1} into zp[(k + 1) % 2]
    XT* qe;
    XT* qc;
    PcgScalars* d;
    double tol;
    int maxit;
    int ncon, nfric;
    // matrix-free constraints: clist[j] / flist[j] (j < nlist[0] / nlist[1]) when
    // the operator's rows hold the folded constraints, else all ncon / nfric
    const int* clist;
    const int* flist;
    const int* nlist;
    int trace;
    unsigned int wait_polls;  // polls of the arrival counter before a grid wait gives up
    double* part;             // 2 x gridDim.x x 4 block partial sums (reduction e uses half e % 2)
};

// 256-thread blocks: a grid-wide reduction costs ~2.5 us with 152 blocks, ~3.7
// with 304 and ~6 with 608 (arrivals on one counter), against ~3.5 / ~5 with
// 512-thread blocks (the block-level sum grows)
constexpr int kPcgThreads = 256;
// default polls of the arrival counter before a wait gives up: each poll is an L2
// round trip (>= ~0.3 us), and past kBarrierBackoff polls a 64 ns sleep is added,
// so the limit is over a second (cipc_step_params.pcg_wait_polls overrides it)
constexpr unsigned int kBarrierSpinLimit = 1u << 22;
constexpr unsigned int kBarrierBackoff = 4096;

template <typename T>
__device__ __forceinline__ T ldcg(const T* p)
{
    return __ldcg(p);
}

__device__ __forceinline__ void red_release_add_u32(unsigned int* p, unsigned int v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide sum of v (N <= 4 values per thread, summed over all threads of all
// blocks), returned in v to every thread; also a grid barrier.  epoch counts the
// reductions this thread has taken part in (the same in every thread).  Thread 0
// of each block stores the block's sums into its slot of part[epoch % 2], arrives
// on a monotone counter with release semantics and polls it (acquire) until every
// block of reduction `epoch` has arrived; then warp 0 of every block adds all
// blocks' partials in one fixed order (lane l takes blocks l, l + 32, ...; then a
// fixed shuffle tree), so the totals are identical in every block and do not
// depend on the order in which blocks arrive.  part[epoch % 2] is rewritten only by
// reduction epoch + 2, which no block can reach before every block has passed
// reduction epoch + 1, i.e. finished reading it.  Returns false if the wait gave
// up (err set; the kernel returns).  Warp-level sums of the thread values run in
// the solver's precision AT (FP32 shuffles and adds in the FP32 solver: this
// part's FP64 work otherwise competes for GB300's narrow FP64 pipe); block and
// grid sums are FP64.  The totals land in out.
template <int N, typename AT>
__device__ __forceinline__ bool grid_allreduce(const AT (&v)[N], double (&out)[N], PcgScalars* d, unsigned int& epoch,
                                               unsigned int limit, double* part)
{
    static_assert(N >= 1 && N <= 4, "reduction width");
    __shared__ double sh[N][kPcgThreads / 32];
    __shared__ double res[N];
    __shared__ int ok;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        AT a = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[k][wid] = (double)a;
    }
    __syncthreads();
    double* half = part + (size_t)(epoch & 1u) * gridDim.x * 4;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double a = 0;
#pragma unroll
            for (int w = 0; w < kPcgThreads / 32; ++w) a += sh[k][w];
            __stcg(half + 4 * (size_t)blockIdx.x + k, a);
        }
        red_release_add_u32(&d->arrive, 1u);
        const unsigned int target = (epoch + 1) * gridDim.x;
        int good = 1;
        unsigned int spins = 0;
        while ((int)(ld_acquire_u32(&d->arrive) - target) < 0) {
            ++spins;
            if (spins > limit || ((spins & 255) == 0 && *(volatile int*)&d->err)) {
                atomicExch(&d->err, 1);
                good = 0;
                break;
            }
            if (spins > kBarrierBackoff) __nanosleep(64);
        }
        ok = good;
    }
    __syncthreads();
    ++epoch;
    if (!ok) return false;
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double a = 0;
            for (int b = lane; b < (int)gridDim.x; b += 32) a += __ldcg(half + 4 * (size_t)b + k);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if (lane == 0) res[k] = a;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = res[k];
    return true;
}

// Aggregate block Jacobi inside a phase.  Every block owns a contiguous range of
// aggregates of about equal cost (the phase's column items and rows: agg_partition
// in agg_rounds.h), cut on the host into rounds of at most AggTile::kStage scalar
// rows and kAggRoundMax aggregates (rounds [abround[b], abround[b + 1]) of block
// b, round q = aggregates [arstart[q], arstart[q + 1])).  Per round:
//  (1) warp 0 tabulates the round's aggregates while all threads perform the
//      phase's update of the round's scalar rows (rfun(j0, j1, two, r0, r1)
//      updates row j0 and, if two, row j1, and returns their r) and stage r in
//      shared memory;
//  (2) the product of each dense inverse B (symmetric, so a column's entries are
//      consecutive) with r is cut into items of C columns x all rows, lane = row
//      (up to three row groups; C = kLoads / row groups, so every lane has kLoads
//      loads in flight), dealt round-robin to the warps; item c of an aggregate
//      stores its partial sums in shared slot c;
//  (3) one thread per row sums its aggregate's slots in slot order (or, in a pack
//      of isolated vertices, applies the vertex's own 3x3 block) and writes z_j to
//      zout[j].x.
// The lanes' shares of (r, z) and (r, r) are added into rz and rr.  The sums do
// not depend on which warp takes an item, so z is the same in every run.
template <typename XT>
struct AggTile;
template <>
struct AggTile<float> {
    static constexpr int kLoads = 48, kStage = 768, kSlots = 8;
};
template <>
struct AggTile<double> {
    static constexpr int kLoads = 18, kStage = 384, kSlots = 16;
};
constexpr int kAggRoundMax = 64;
constexpr int kAggMaxRows = 96;  // 32 vertices
// slots an aggregate of up to kAggMaxRows rows needs (its items)
constexpr int agg_slots(int L)
{
    const int s3 = (kAggMaxRows + L / 3 - 1) / (L / 3), s2 = (64 + L / 2 - 1) / (L / 2), s1 = (32 + L - 1) / L;
    return s3 > s2 ? (s3 > s1 ? s3 : s1) : (s2 > s1 ? s2 : s1);
}
static_assert(agg_slots(AggTile<float>::kLoads) <= AggTile<float>::kSlots, "FP32 item slots");
static_assert(agg_slots(AggTile<double>::kLoads) <= AggTile<double>::kSlots, "FP64 item slots");
static_assert(kAggMaxRows <= AggTile<float>::kStage && kAggMaxRows <= AggTile<double>::kStage, "round staging");
// the item widths agg_phase dispatches on (L / row groups) are agg_cols's
static_assert(AggTile<float>::kLoads >= 3 && AggTile<double>::kLoads >= 3, "item width");

struct AggEnt {
    int m;        // scalar rows
    int bo;       // offset of the inverse block
    int rowbase;  // first row in the round's staging
    int ibeg;     // first item (items of aggregate e: [ibeg(e), ibeg(e + 1)))
    int pk;       // pack of isolated vertices (3x3 blocks)
};

template <typename XT>
struct AggSmem {
    XT rs[AggTile<XT>::kStage];
    XT part[AggTile<XT>::kSlots][AggTile<XT>::kStage];
    int jrow[AggTile<XT>::kStage];             // scalar row of each staged row
    unsigned char rent[AggTile<XT>::kStage];   // its aggregate's table entry
    AggEnt ent[kAggRoundMax + 1];
    int nitems;
    // the block's rounds [q0, q1); a block with one round keeps its table, rows
    // and entries from one phase to the next (cached = that round, else -1)
    int q0, q1, cached, ne, nrows;
};

// item: columns c0 .. c0 + C - 1 of B (m x m) times rsb, rows lane + 32 k; the
// loads are all issued before the multiply-adds
template <int RG, int C, typename XT, typename PT>
__device__ __forceinline__ void agg_item(const PT* __restrict__ B, int m, int c0, int lane, const XT* rsb, XT* out)
{
    // one pointer walks the columns (m apart); the row groups are fixed offsets
    PT b[RG][C];
    const PT* p = B + (size_t)c0 * m + lane;
#pragma unroll
    for (int u = 0; u < C; ++u) {
        const bool cu = c0 + u < m;
#pragma unroll
        for (int k = 0; k < RG; ++k) b[k][u] = (cu && lane + 32 * k < m) ? __ldg(p + 32 * k) : PT(0);
        p += cu ? m : 0;
    }
    XT acc[RG];
#pragma unroll
    for (int k = 0; k < RG; ++k) acc[k] = 0;
#pragma unroll
    for (int u = 0; u < C; ++u) {
        const XT rv = c0 + u < m ? rsb[c0 + u] : XT(0);
#pragma unroll
        for (int k = 0; k < RG; ++k) acc[k] += (XT)b[k][u] * rv;
    }
#pragma unroll
    for (int k = 0; k < RG; ++k)
        if (lane + 32 * k < m) out[lane + 32 * k] = acc[k];
}

// (tp: block 0's lap accumulators with tracing on, else null: [2] += time to the
// end of step (1), [5] += time in step (2))
template <typename VT, typename XT, typename PT, typename XT2, typename RF>
__device__ __forceinline__ void agg_phase(const PcgArgs<VT, XT, PT>& a, AggSmem<XT>& sm, XT2* zout, const RF& rfun,
                                          XT& rz, XT& rr, unsigned long long* tp)
{
    unsigned long long mark = tp && threadIdx.x == 0 ? gtimer() : 0;
    auto lap = [&](int k) {
        if (tp && threadIdx.x == 0) {
            const unsigned long long t = gtimer();
            tp[k] += t - mark;
            mark = t;
        }
    };
    using Tile = AggTile<XT>;
    constexpr int L = Tile::kLoads;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int q0 = sm.q0, q1 = sm.q1;
    for (int q = q0; q < q1; ++q) {
        const bool reuse = sm.cached == q;
        int ne, vb = 0, nrows;
        if (reuse) {
            ne = sm.ne;
            nrows = sm.nrows;
        } else {
            const int ga = __ldg(a.arstart + q);
            ne = __ldg(a.arstart + q + 1) - ga;
            vb = __ldg(a.avoff + ga);
            nrows = 3 * (__ldg(a.avoff + ga + ne) - vb);
        }
        if (!reuse && wib == 0) {
            const int ga = __ldg(a.arstart + q);
            int carry = 0;
            for (int base = 0; base < ne; base += 32) {
                const int e = base + lane;
                int nc = 0;
                if (e < ne) {
                    const int g = ga + e;
                    const int v0 = __ldg(a.avoff + g), sv = __ldg(a.avoff + g + 1) - v0, m = 3 * sv;
                    const long long bo = __ldg(a.aboff + g), bsz = __ldg(a.aboff + g + 1) - bo;
                    const int pk = sv > 1 && bsz == 9LL * sv;
                    nc = agg_items(m, pk, L);
                    sm.ent[e].m = m;
                    sm.ent[e].bo = (int)bo;
                    sm.ent[e].rowbase = 3 * (v0 - vb);
                    sm.ent[e].pk = pk;
                }
                int incl = nc;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                if (e < ne) sm.ent[e].ibeg = carry + incl - nc;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (lane == 0) {
                sm.ent[ne].ibeg = carry;
                sm.ent[ne].rowbase = nrows;
                sm.nitems = carry;
            }
        }
        // two rows per thread and step, both rows' loads issued before the stores
        for (int lr = threadIdx.x; lr < nrows; lr += 2 * blockDim.x) {
            const int lr1 = lr + blockDim.x;
            const bool two = lr1 < nrows;
            const int j0 = reuse ? sm.jrow[lr] : 3 * __ldg(a.averts + vb + lr / 3) + lr % 3;
            const int j1 = !two ? j0 : (reuse ? sm.jrow[lr1] : 3 * __ldg(a.averts + vb + lr1 / 3) + lr1 % 3);
            XT r0, r1;
            rfun(j0, j1, two, r0, r1);
            sm.rs[lr] = r0;
            if (!reuse) sm.jrow[lr] = j0;
            rr += r0 * r0;
            if (two) {
                sm.rs[lr1] = r1;
                if (!reuse) sm.jrow[lr1] = j1;
                rr += r1 * r1;
            }
        }
        __syncthreads();
        lap(2);
        {
            const int nit = sm.nitems;
            int e = 0;
            for (int it = wib; it < nit; it += nwarp) {
                while (sm.ent[e + 1].ibeg <= it) ++e;
                const AggEnt E = sm.ent[e];
                const int c = it - E.ibeg, rg = (E.m + 31) >> 5;
                const PT* B = a.ainv + E.bo;
                const XT* rsb = sm.rs + E.rowbase;
                XT* out = sm.part[c] + E.rowbase;
                if (rg == 3) agg_item<3, L / 3>(B, E.m, c * (L / 3), lane, rsb, out);
                else if (rg == 2) agg_item<2, L / 2>(B, E.m, c * (L / 2), lane, rsb, out);
                else agg_item<1, L>(B, E.m, c * L, lane, rsb, out);
            }
        }
        __syncthreads();
        lap(5);
        for (int lr = threadIdx.x; lr < nrows; lr += blockDim.x) {
            // the row's aggregate: the last entry with rowbase <= lr
            int lo = 0;
            if (reuse) {
                lo = sm.rent[lr];
            } else {
                int hi = ne - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (sm.ent[mid].rowbase <= lr) lo = mid;
                    else hi = mid - 1;
                }
                sm.rent[lr] = (unsigned char)lo;
            }
            const AggEnt E = sm.ent[lo];
            XT z;
            if (E.pk) {
                const int t = lr - E.rowbase, v = t / 3, c = t - 3 * v;
                const PT* Bc = a.ainv + E.bo + 9 * v + 3 * c;
                const XT* rv = sm.rs + E.rowbase + 3 * v;
                z = (XT)__ldg(Bc) * rv[0] + (XT)__ldg(Bc + 1) * rv[1] + (XT)__ldg(Bc + 2) * rv[2];
            } else {
                const int nc = sm.ent[lo + 1].ibeg - E.ibeg;
                z = 0;
                for (int c = 0; c < nc; ++c) z += sm.part[c][lr];
            }
            zout[sm.jrow[lr]].x = z;
            rz += sm.rs[lr] * z;
        }
        if (!reuse && q1 - q0 == 1 && threadIdx.x == 0) {
            sm.cached = q;
            sm.ne = ne;
            sm.nrows = nrows;
        }
        __syncthreads();  // the next round rewrites the staging
    }
}

// z = M^-1 r for vertex i
template <typename XT, typename PT>
__device__ __forceinline__ void precond_vertex(const PT* __restrict__ pinv, int i, const XT (&r)[3], XT (&z)[3])
{
    const PT* P = pinv + 9 * (size_t)i;
    z[0] = (XT)__ldg(P + 0) * r[0] + (XT)__ldg(P + 1) * r[1] + (XT)__ldg(P + 2) * r[2];
    z[1] = (XT)__ldg(P + 3) * r[0] + (XT)__ldg(P + 4) * r[1] + (XT)__ldg(P + 5) * r[2];
    z[2] = (XT)__ldg(P + 6) * r[0] + (XT)__ldg(P + 7) * r[1] + (XT)__ldg(P + 8) * r[2];
}

// y = H_c x_c for one contact constraint of NV vertices by a group of 4 lanes
// (lane k of the group owns vertex k; lanes k >= NV only pass values along).
// The packed upper triangle is stored row by row, entry h at H[h * hs], so
// consecutive constraints are adjacent and loads of one entry by several groups
// share cache lines.  Each owning lane gathers its vertex's 3 values, the group
// exchanges them by shuffles, and the lane forms its 3 rows of H_c x_c and adds
// them into q; returns the lane's share of x_c . H_c x_c.  All 4 lanes of the
// group must call this together (gmask = the group's lanes, gbase = its first).
template <int NV, typename VT, typename XT, typename G>
__device__ __forceinline__ XT con_apply_lane(const VT* __restrict__ H, size_t hs, int4 iv, int k, unsigned gmask,
                                                 int gbase, const G& pget, XT* q)
{
    constexpr int M = 3 * NV;
    const bool own = k < NV;
    const int me = k == 0 ? iv.x : (k == 1 ? iv.y : (k == 2 ? iv.z : iv.w));
    XT xk[3];
#pragma unroll
    for (int t = 0; t < 3; ++t) xk[t] = own ? pget(3 * me + t) : XT(0);
    XT xs[M];
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
        for (int t = 0; t < 3; ++t) xs[3 * j + t] = __shfl_sync(gmask, xk[t], gbase + j);
    if (!own) return XT(0);
    XT s = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int p = 3 * k + r;
        XT y = 0;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const int i = min(p, m), j = max(p, m);
            const int h = i * M - (i * (i - 1)) / 2 + (j - i);
            y += (XT)__ldg(H + (size_t)h * hs) * xs[m];
        }
        s += xk[r] * y;
        if (y != XT(0)) atomicAdd(q + 3 * me + r, y);
    }
    return s;
}

// apply phase: q_e, q_c = H p_k (p_k formed on the fly and stored for the owned
// rows); returns this thread's share of (p_k, H p_k)
template <typename VT, typename XT, typename PT>
__device__ __forceinline__ XT apply_phase(const PcgArgs<VT, XT, PT>& a, XT beta,
                                              const typename PcgArgs<VT, XT, PT>::XT2* zp,
                                              typename PcgArgs<VT, XT, PT>::XT2* zp_next, int ncon, int nfric)
{
    // p_k = z_k + beta p_{k-1} (beta = 0 in the first iteration, where p_{-1} is
    // never written: the pair's second half is ignored then)
    auto pget = [&](int j) -> XT {
        const auto v = ldcg(zp + j);
        return beta == XT(0) ? v.x : v.x + beta * v.y;
    };
    // work items: the scalar rows of the 3x3 block rows, two per thread and step in
    // the FP32 solver (both rows' loads in flight: on large systems a thread has
    // several rows and the loop is latency-bound otherwise), then 4 lanes per matrix-free contact
    // constraint (starting 4-aligned, so a constraint's lanes are 4 aligned lanes of
    // one warp: the grid stride is a multiple of 32), then friction constraints
    const int nrow = 3 * a.nv;
    const int cbeg = (nrow + 3) & ~3, cend = cbeg + 4 * ncon;
    const int total = cend + nfric;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    XT v = 0;  // this thread's share, in the solver's precision; block sums are FP64
    {
        const int nv = a.nv;
        // (the FP64 solver keeps one row per step: its doubled registers spill)
        constexpr int RS = sizeof(XT) == 4 ? 2 : 1;
        for (int w = gtid; w < nrow; w += RS * gstride) {
            const int wb = w + gstride;
            const bool two = RS == 2 && wb < nrow;
            const int i0 = w / 3, r0 = w - 3 * i0;
            const int i1 = two ? wb / 3 : i0, r1 = two ? wb - 3 * i1 : r0;
            XT acc0 = 0, acc1 = 0;
            auto blk = [&](int k, int i, int r) -> XT {
                const size_t e = (size_t)k * nv + i;
                const int j = __ldg(a.col + e);
                const VT* B = a.val + 9 * e + 3 * r;
                return (XT)__ldg(B) * pget(3 * j) + (XT)__ldg(B + 1) * pget(3 * j + 1) +
                       (XT)__ldg(B + 2) * pget(3 * j + 2);
            };
            if (!a.rowlen) {
                // every row has the full length (uniform meshes): no per-row test in
                // the loop (it costs time there); the second row repeats the first at
                // the tail
                const int K = a.ell_k;
#pragma unroll 4
                for (int k = 0; k < K; ++k) {
                    acc0 += blk(k, i0, r0);
                    acc1 += blk(k, i1, r1);
                }
            } else {
                // only the real blocks of each row (on meshes that mix cloth, rods and
                // particles most slots of the widest row's length are padding)
                const int L0 = __ldg(a.rowlen + i0), L1 = two ? __ldg(a.rowlen + i1) : 0;
#pragma unroll 4
                for (int k = 0; k < max(L0, L1); ++k) {
                    if (k < L0) acc0 += blk(k, i0, r0);
                    if (k < L1) acc1 += blk(k, i1, r1);
                }
            }
            const XT pw0 = pget(w);
            zp_next[w].y = pw0;
            a.qe[w] = acc0;
            v += pw0 * acc0;
            if (two) {
                const XT pw1 = pget(wb);
                zp_next[wb].y = pw1;
                a.qe[wb] = acc1;
                v += pw1 * acc1;
            }
        }
    }
    for (int w = cbeg + gtid; w < total; w += gstride) {
        if (w < cend) {
            // contact constraint c, lane k of its group of 4
            const int j = (w - cbeg) >> 2, k = (w - cbeg) & 3;
            const int c = a.clist ? __ldg(a.clist + j) : j;
            const int lane = threadIdx.x & 31, gbase = lane & ~3;
            const unsigned gmask = 0xFu << gbase;
            const int cnv = con_nv(__ldg(a.ckind + c));
            const int4 iv = a.cverts[c];
            const VT* H = a.chess + c;
            if (cnv == 2) v += con_apply_lane<2>(H, a.hs, iv, k, gmask, gbase, pget, a.qc);
            else if (cnv == 3) v += con_apply_lane<3>(H, a.hs, iv, k, gmask, gbase, pget, a.qc);
            else v += con_apply_lane<4>(H, a.hs, iv, k, gmask, gbase, pget, a.qc);
        } else {
            // friction constraint: w_a T M T^T sum_b w_b p_b over non-projected vertices
            const int c = a.flist ? __ldg(a.flist + (w - cend)) : w - cend;
            if (a.fkind[c] >= kc_EEM) continue;
            const int cnv = con_nv(a.fkind[c]);
            const int4 iv = a.fverts[c];
            const int id[4] = {iv.x, iv.y, iv.z, iv.w};
            XT s0 = 0, s1 = 0, s2 = 0;
            for (int q = 0; q < cnv; ++q) {
                if (a.proj[id[q]]) continue;
                const XT wq = (XT)a.fw[4 * c + q];
                s0 += wq * pget(3 * id[q]);
                s1 += wq * pget(3 * id[q] + 1);
                s2 += wq * pget(3 * id[q] + 2);
            }
            const double* Td = a.fT + 6 * (size_t)c;
            const XT T[6] = {(XT)Td[0], (XT)Td[1], (XT)Td[2], (XT)Td[3], (XT)Td[4], (XT)Td[5]};
            const XT t0 = T[0] * s0 + T[1] * s1 + T[2] * s2, t1 = T[3] * s0 + T[4] * s1 + T[5] * s2;
            const XT m00 = (XT)a.fM[3 * c], m01 = (XT)a.fM[3 * c + 1], m11 = (XT)a.fM[3 * c + 2];
            const XT u0 = m00 * t0 + m01 * t1, u1 = m01 * t0 + m11 * t1;
            v += t0 * u0 + t1 * u1;
            const XT o0 = T[0] * u0 + T[3] * u1, o1 = T[1] * u0 + T[4] * u1, o2 = T[2] * u0 + T[5] * u1;
            for (int q = 0; q < cnv; ++q) {
                if (a.proj[id[q]]) continue;
                const XT wq = (XT)a.fw[4 * c + q];
                atomicAdd(a.qc + 3 * id[q], (XT)(wq * o0));
                atomicAdd(a.qc + 3 * id[q] + 1, (XT)(wq * o1));
                atomicAdd(a.qc + 3 * id[q] + 2, (XT)(wq * o2));
            }
        }
    }
    return v;
}

// two blocks per SM (the grid's size, coresident_grid): 128 registers a thread,
// which the aggregate phase's loads in flight use (against 80 at three blocks)
template <typename VT, typename XT, typename PT>
__global__ void __launch_bounds__(kPcgThreads, 2) k_pcg_solve(PcgArgs<VT, XT, PT> a)
{
    PcgScalars* d = a.d;
    unsigned int epoch = 0;
    const int ncon = a.nlist ? min(__ldg(a.nlist), a.ncon) : a.ncon;
    const int nfric = a.nlist ? min(__ldg(a.nlist + 1), a.nfric) : a.nfric;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    // the aggregate phase's staging (dynamic: launched with it only when nagg > 0)
    extern __shared__ __align__(16) unsigned char pcg_dyn_smem[];
    AggSmem<XT>& agg_sm = *reinterpret_cast<AggSmem<XT>*>(pcg_dyn_smem);
    // r = b, x = 0, q_c = 0, z = M^-1 r
    double tot[2];
    if (a.nagg > 0) {
        if (threadIdx.x == 0) {
            agg_sm.q0 = __ldg(a.abround + blockIdx.x);
            agg_sm.q1 = __ldg(a.abround + blockIdx.x + 1);
            agg_sm.cached = -1;
        }
        __syncthreads();
        XT rz0 = 0, rr0 = 0;
        agg_phase(
            a, agg_sm, a.zp[0],
            [&](int j0, int j1, bool two, XT& r0, XT& r1) {
                r0 = a.b[j0];
                r1 = a.b[j1];
                a.r[j0] = r0;
                a.x[j0] = 0;
                a.qc[j0] = 0;
                if (two) {
                    a.r[j1] = r1;
                    a.x[j1] = 0;
                    a.qc[j1] = 0;
                }
            },
            rz0, rr0, nullptr);
        const XT v0[2] = {rz0, rr0};
        double v[2];
        if (!grid_allreduce<2>(v0, v, d, epoch, a.wait_polls, a.part)) return;
        tot[0] = v[0];
        tot[1] = v[1];
    } else {
        double v[2] = {0, 0};
        for (int i = gtid; i < a.nv; i += gstride) {
            XT r[3], z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                r[c] = a.b[3 * i + c];
                a.r[3 * i + c] = r[c];
                a.x[3 * i + c] = 0;
                a.qc[3 * i + c] = 0;
            }
            precond_vertex<XT, PT>(a.pinv, i, r, z);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                a.zp[0][3 * i + c].x = z[c];
                v[0] += (double)r[c] * (double)z[c];
                v[1] += (double)r[c] * (double)r[c];
            }
        }
        if (!grid_allreduce<2>(v, v, d, epoch, a.wait_polls, a.part)) return;
        tot[0] = v[0];
        tot[1] = v[1];
    }
    double rz = tot[0], rz_prev = 1, rr = tot[1], pq = 0;
    const double bb = tot[1], thr = a.tol * a.tol * bb;
    int done = 0, k = 0;
    if (!(bb == bb) || !(rz == rz)) done = 2;
    else if (!(bb > 0)) done = 1;
    const bool tr = a.trace && blockIdx.x == 0 && threadIdx.x == 0;
    // phase laps of block 0 (kept in shared memory: registers are the scarce
    // resource of this kernel, and a spilled loop-carried value costs an L2 round
    // trip per iteration once the streamed operands have evicted it from L1)
    __shared__ unsigned long long tp[7];
    if (tr) {
        for (int q = 0; q < 6; ++q) tp[q] = 0;
        tp[6] = gtimer();
    }
    auto lap = [&](int k) {
        if (tr) {
            const unsigned long long t = gtimer();
            tp[k] += t - tp[6];
            tp[6] = t;
        }
    };
    while (!done) {
        if (k >= a.maxit) {
            done = 4;
            break;
        }
        const bool first = (k == 0);
        const XT beta = first ? XT(0) : (XT)(rz / rz_prev);
        const auto* zp = a.zp[k & 1];
        auto* zp_next = a.zp[(k + 1) & 1];
        const XT va[1] = {apply_phase<VT, XT, PT>(a, beta, zp, zp_next, ncon, nfric)};
        double vd[1];
        lap(0);
        if (!grid_allreduce<1>(va, vd, d, epoch, a.wait_polls, a.part)) return;
        lap(1);
        pq = vd[0];
        if (!(pq > 0 && pq < INFINITY)) {
            done = (pq == pq) ? 3 : 2;
            break;
        }
        const XT alpha = (XT)(rz / pq);
        XT rz_t = 0, rr_t = 0;
        if (a.nagg > 0)
            agg_phase(
                a, agg_sm, zp_next,
                [&](int j0, int j1, bool two, XT& r0, XT& r1) {
                    const XT x0 = ldcg(a.x + j0), p0 = ldcg(&zp_next[j0].y), s0 = ldcg(a.r + j0),
                             e0 = ldcg(a.qe + j0), c0 = ldcg(a.qc + j0);
                    const XT x1 = ldcg(a.x + j1), p1 = ldcg(&zp_next[j1].y), s1 = ldcg(a.r + j1),
                             e1 = ldcg(a.qe + j1), c1 = ldcg(a.qc + j1);
                    a.x[j0] = x0 + alpha * p0;
                    r0 = s0 - alpha * (e0 + c0);
                    a.r[j0] = r0;
                    a.qc[j0] = 0;
                    r1 = s1 - alpha * (e1 + c1);
                    if (two) {
                        a.x[j1] = x1 + alpha * p1;
                        a.r[j1] = r1;
                        a.qc[j1] = 0;
                    }
                },
                rz_t, rr_t, tr ? tp : nullptr);
        else
        for (int i = gtid; i < a.nv; i += gstride) {
            // all loads of the vertex's three rows before its stores (the stores
            // could alias them, so the loads would otherwise wait for each row)
            XT r[3], z[3], xv[3], pv[3], rv[3], ev[3], cv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int j = 3 * i + c;
                xv[c] = ldcg(a.x + j);
                pv[c] = ldcg(&zp_next[j].y);
                rv[c] = ldcg(a.r + j);
                ev[c] = ldcg(a.qe + j);
                cv[c] = ldcg(a.qc + j);
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int j = 3 * i + c;
                a.x[j] = xv[c] + alpha * pv[c];
                r[c] = rv[c] - alpha * (ev[c] + cv[c]);
                a.r[j] = r[c];
                a.qc[j] = 0;
            }
            precond_vertex<XT, PT>(a.pinv, i, r, z);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                zp_next[3 * i + c].x = z[c];
                rz_t += r[c] * z[c];
                rr_t += r[c] * r[c];
            }
        }
        const XT vb_t[2] = {rz_t, rr_t};
        double vb[2];
        lap(3);
        if (!grid_allreduce<2>(vb_t, vb, d, epoch, a.wait_polls, a.part)) return;
        lap(4);
        tot[0] = vb[0];
        tot[1] = vb[1];
        rz_prev = rz;
        rz = tot[0];
        rr = tot[1];
        ++k;
        if (!(rz == rz) || !(rr == rr)) done = 2;
        else if (rr <= thr) done = 1;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        d->rr = rr;
        d->bb = bb;
        d->pq = pq;
        d->it = k;
        d->done = done;
        for (int q = 0; q < 6; ++q) d->tphase[q] = tp[q];
    }
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
namespace {

constexpr int kVecs = 9;  // r, (z, p) pairs x 2 (two vectors each), q_e, q_c, and b, x of the FP32 inner solve

struct PcgState {
    DBuf<char> vec;              // kVecs vectors of 3 nv entries
    DBuf<PcgScalars> dsc;        // device scalars
    DBuf<double> part;           // block partial sums of the grid reductions
    PcgScalars* host = nullptr;  // pinned copy of the results
    cudaEvent_t ev[2] = {nullptr, nullptr};  // around each launch: the solve's device time
    int grid[2] = {0, 0};        // co-resident grid per precision (0 FP64, 1 FP32)
    ~PcgState()
    {
        if (host) cudaFreeHost(host);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        vec.release();
        dsc.release();
        part.release();
    }
};

template <typename VT, typename XT, typename PT>
int coresident_grid(int nv)
{
    int per_sm = 0;
    // (with the aggregate phase's shared staging, so both launches fit; the FP64
    // staging is above the default 48 KB of dynamic shared memory)
    cudaError_t e = cudaFuncSetAttribute(k_pcg_solve<VT, XT, PT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(AggSmem<XT>));
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_solve<VT, XT, PT>, kPcgThreads,
                                                          sizeof(AggSmem<XT>));
    if (e != cudaSuccess || per_sm < 1) return 0;
    // blocks per SM trade apply-phase parallelism against the cost of the grid
    // reductions, which grows with the number of blocks: two per SM measured best
    // on the 200x200 cloth (FP32: 26 us per iteration against 30 with four and 35
    // with one, before the kernel's launch bounds fixed two);
    // CIPC_PCG_BLOCKS_PER_SM (1..occupancy) overrides
    int want = 2;
    if (const char* env = std::getenv("CIPC_PCG_BLOCKS_PER_SM")) {
        const int b = std::atoi(env);
        if (b >= 1) want = b;
    }
    per_sm = std::min(per_sm, want);
    // the apply phase has one work item per scalar row plus one per contact and
    // friction constraint, so every co-resident block has work
    (void)nv;
    return per_sm * num_sms();
}

int state(Sim* s, PcgState** out)
{
    if (!s->pcg) {
        PcgState* st = new PcgState();
        if (st->dsc.alloc(1) != cudaSuccess || cudaMemset(st->dsc.p, 0, sizeof(PcgScalars)) != cudaSuccess ||
            cudaMallocHost((void**)&st->host, sizeof(PcgScalars)) != cudaSuccess ||
            cudaEventCreate(&st->ev[0]) != cudaSuccess || cudaEventCreate(&st->ev[1]) != cudaSuccess) {
            delete st;
            return set_error(CIPC_ERR_CUDA, "PCG state allocation");
        }
        st->grid[0] = coresident_grid<double, double, double>(s->nv);
        st->grid[1] = coresident_grid<float, float, float>(s->nv);
        if (std::min(st->grid[0], st->grid[1]) < 1) {
            delete st;
            return set_error(CIPC_ERR_CUDA, "PCG: no co-resident grid");
        }
        s->pcg = st;
    }
    *out = static_cast<PcgState*>(s->pcg);
    return CIPC_OK;
}

int ensure_vectors(Sim* s, PcgState* st, size_t elem)
{
    const size_t vbytes = ((3 * (size_t)s->nv * elem + 255) & ~(size_t)255);
    if (st->vec.n < kVecs * vbytes) {
        cudaStreamSynchronize(s->stream);
        if (st->vec.alloc(kVecs * vbytes) != cudaSuccess) return set_error(CIPC_ERR_CUDA, "PCG vectors");
    }
    return CIPC_OK;
}

template <typename VT, typename XT, typename PT>
int solve(Sim* s, const XT* b, XT* x, double tol, int maxit, int* iters, double* rel)
{
    PcgState* st = nullptr;
    int rc = state(s, &st);
    if (rc || (rc = ensure_vectors(s, st, sizeof(XT)))) return rc;
    cudaStream_t str = s->stream;
    const size_t vbytes = ((3 * (size_t)s->nv * sizeof(XT) + 255) & ~(size_t)255);
    auto vecp = [&](int k) { return reinterpret_cast<XT*>(st->vec.p + k * vbytes); };
    const int g = st->grid[sizeof(XT) == 4 ? 1 : 0];
    PcgArgs<VT, XT, PT> a;
    std::memset(&a, 0, sizeof(a));
    a.nv = s->nv;
    a.ell_k = s->ell_k;
    a.col = s->col.p;
    a.rowlen = s->rows_uniform ? nullptr : s->rowlen.p;
    a.val = reinterpret_cast<const VT*>(s->folded ? s->hval_op.p : s->hval.p);
    a.ckind = s->ckind.p;
    a.cverts = s->cverts.p;
    a.chess = reinterpret_cast<const VT*>(s->chess.p);
    a.hs = (size_t)s->cap_con;
    a.fkind = s->fkind.p;
    a.fverts = s->fverts.p;
    a.fw = s->fw.p;
    a.fT = s->fT.p;
    a.fM = reinterpret_cast<const double*>(s->fhess.p);
    a.proj = s->proj.p;
    a.pinv = reinterpret_cast<const PT*>(s->pinv.p);
    a.b = b;
    a.x = x;
    a.r = vecp(0);
    a.zp[0] = reinterpret_cast<typename PcgArgs<VT, XT, PT>::XT2*>(vecp(1));  // pairs span vectors 1-2
    a.zp[1] = reinterpret_cast<typename PcgArgs<VT, XT, PT>::XT2*>(vecp(3));  // and 3-4
    a.qe = vecp(5);
    a.qc = vecp(6);
    a.d = st->dsc.p;
    a.tol = tol;
    a.maxit = maxit;
    a.ncon = s->prm.withCollision ? s->ncon : 0;
    a.nfric = (s->prm.withCollision && s->prm.mu > 0) ? s->nfric : 0;
    if (s->prm.precond == 2 && s->agg_ready) {
        const AggView av = agg_view(s);
        a.nagg = av.nagg;
        a.avoff = av.voff;
        a.averts = av.verts;
        a.aboff = av.boff;
        a.ainv = reinterpret_cast<const PT*>(av.inv);
        rc = agg_rounds(s, g, AggTile<XT>::kStage, kAggRoundMax, AggTile<XT>::kLoads, &a.abround, &a.arstart);
        if (rc) return rc;
    }
    if (s->folded) {
        a.clist = s->crest.p;
        a.flist = s->frest.p;
        a.nlist = s->fold_cnt.p;
    }
    a.trace = s->trace;
    a.wait_polls = s->prm.pcg_wait_polls > 0 ? (unsigned int)s->prm.pcg_wait_polls : kBarrierSpinLimit;
    if ((int)st->part.n < 8 * g && st->part.alloc(8 * (size_t)g) != cudaSuccess)
        return set_error(CIPC_ERR_CUDA, "PCG partial sums");
    a.part = st->part.p;
    // barrier state starts clear (a previous solve may have given up mid-way)
    cudaError_t e = cudaMemsetAsync(st->dsc.p, 0, sizeof(PcgScalars), str);
    void* args[] = {&a};
    if (e == cudaSuccess) e = cudaEventRecord(st->ev[0], str);
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((const void*)k_pcg_solve<VT, XT, PT>, dim3(g), dim3(kPcgThreads), args,
                                        a.nagg > 0 ? sizeof(AggSmem<XT>) : 0, str);
    if (e == cudaSuccess) e = cudaEventRecord(st->ev[1], str);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st->host, st->dsc.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, str);
    if (e == cudaSuccess) e = cudaStreamSynchronize(str);
    if (e != cudaSuccess) return set_cuda_error(e, "PCG");
    float ms = 0;
    if (cudaEventElapsedTime(&ms, st->ev[0], st->ev[1]) == cudaSuccess) s->solve_ms += ms;
    const PcgScalars* h = st->host;
    *iters = h->it;
    *rel = h->bb > 0 ? std::sqrt(h->rr / h->bb) : 0.0;
    if (s->trace) {
        const double it = std::max(1, h->it);
        std::fprintf(stderr,
                     "cipc pcg: rel %.3e iters %d stop %d grid %d  us/iter: apply %.2f reduce %.2f update %.2f "
                     "reduce %.2f (aggregate rows %.2f items %.2f)\n",
                     *rel, h->it, h->done, g, h->tphase[0] * 1e-3 / it, h->tphase[1] * 1e-3 / it,
                     h->tphase[3] * 1e-3 / it, h->tphase[4] * 1e-3 / it, h->tphase[2] * 1e-3 / it,
                     h->tphase[5] * 1e-3 / it);
    }
    if (h->err) return set_error(CIPC_ERR_TIMEOUT, "PCG: a grid-wide wait gave up after %u polls", a.wait_polls);
    if (h->done == 2) return set_error(CIPC_ERR_NAN, "PCG produced NaN");
    if (h->done == 3) return set_error(CIPC_ERR_NOT_CONVERGED, "PCG: non-positive curvature (p, Hp) = %g", h->pq);
    if (h->done == 4) return set_error(CIPC_ERR_NOT_CONVERGED, "PCG stopped at relative residual %g", *rel);
    return CIPC_OK;
}

}  // namespace

int pcg_solve_fp64(Sim* s, const double* b, double* x, double tol, int maxit, int* iters, double* rel)
{
    return solve<double, double, double>(s, b, x, tol, maxit, iters, rel);
}

int pcg_solve_fp32(Sim* s, const float* b, float* x, double tol, int maxit, int* iters, double* rel)
{
    return solve<float, float, float>(s, b, x, tol, maxit, iters, rel);
}

int pcg_fp32_io(Sim* s, float** b, float** x)
{
    PcgState* st = nullptr;
    int rc = state(s, &st);
    if (rc || (rc = ensure_vectors(s, st, sizeof(float)))) return rc;
    const size_t vbytes = ((3 * (size_t)s->nv * sizeof(float) + 255) & ~(size_t)255);
    *b = reinterpret_cast<float*>(st->vec.p + 7 * vbytes);
    *x = reinterpret_cast<float*>(st->vec.p + 8 * vbytes);
    return CIPC_OK;
}

void pcg_release(Sim* s)
{
    if (s->pcg) delete static_cast<PcgState*>(s->pcg);
    s->pcg = nullptr;
}

}  // namespace cipc
