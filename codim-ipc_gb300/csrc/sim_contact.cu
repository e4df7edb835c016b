// Contact terms of the time step on the GPU.
//
// Broad phase: a uniform hash grid built by a counting sort on the cell hash
// (one "digit" radix sort).  Items (triangles or edges) are inserted into every
// cell their box overlaps; a query visits the cells of its padded box and takes
// a candidate only in the first cell of the intersection of the two cell ranges,
// so each pair is tested exactly once and hash collisions are filtered by range.
// The grid only generates candidates: membership is decided by the reference's
// own predicates (the AABB test of CCD.h:149-185, the distance classification of
// DISTANCE_TYPE.h, activation d^2 < (dhat + xi)^2 of IPC.h:53-54).
//
// Constraint set (IPC.h:19-740): per boundary node against triangles, per edge
// against edges of higher index, emitting PT / EE / mollified EE-PE-PP directly
// and PP / PE through a device hash table keyed by the reference's code, which
// merges duplicates into a multiplicity (IPC.h:571-661).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/cipc.h"
#include "ccd_core.cuh"
#include "cert.cuh"
#include "cipc_internal.h"
#include "cipc_util.h"
#include "constraint_eval.cuh"
#include "sim.h"
#include "sim_kernels.h"

namespace cipc {

static inline int nblk(long long n, int bs) { return n > 0 ? (int)((n + bs - 1) / bs) : 1; }

__global__ void k_set_u64(unsigned long long* p, unsigned long long v) { *p = v; }

// internal status: the scratch buffer was too small; Sim::scratch_bytes holds the need
static const int kNeedScratch = 1000;
// a grid would hold more than kMaxGridEntries (item, cell) entries: boxes swept by
// an enormous step (the step-size search then halves its trial step) or
// primitives far larger than the cells
static const int kSpanTooLarge = 1001;
static const unsigned long long kMaxGridEntries = 1ull << 25;

// ---------------------------------------------------------------------------
// exclusive scan of int counts (three-phase block scan, recursive over blocks)
// ---------------------------------------------------------------------------
__global__ void k_scan_block(const int* in, int* out, int n, int* bsum)
{
    __shared__ int sh[1024];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sh[threadIdx.x] - v;
    if (threadIdx.x == 1023) bsum[blockIdx.x] = sh[1023];
}
__global__ void k_scan_add(int* out, int n, const int* boff)
{
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += boff[blockIdx.x];
}

// out[0..n) = exclusive scan of in; out[n] = total.  tmp needs >= 2 * (n/1024 + 2) ints.
static void scan_exclusive(const int* in, int* out, int n, int* tmp, cudaStream_t s)
{
    const int nb = (n + 1023) / 1024;
    int* bsum = tmp;
    int* boff = tmp + nb + 1;
    k_scan_block<<<nb, 1024, 0, s>>>(in, out, n, bsum);
    if (nb > 1) {
        scan_exclusive(bsum, boff, nb, boff + nb + 1, s);
        k_scan_add<<<nb, 1024, 0, s>>>(out, n, boff);
        // total = boff[nb]
        cudaMemcpyAsync(out + n, boff + nb, sizeof(int), cudaMemcpyDeviceToDevice, s);
    } else {
        cudaMemcpyAsync(out + n, bsum, sizeof(int), cudaMemcpyDeviceToDevice, s);
    }
}

// ---------------------------------------------------------------------------
// hash grid
// ---------------------------------------------------------------------------
// One (cell, item) entry of the grid, sorted by bucket: everything a query needs
// to test the item is in this 64-byte record (one cache line, read with four
// 16-byte loads and no dependent gather): the item id, its cell range (for the
// once-per-pair test) and its FP32 box (for the prefilter; zero when the grid
// was built without boxes)
struct __align__(16) GridEntry {
    int4 a;    // item, lo x, lo y, lo z
    int4 b;    // hi x, hi y, hi z, -
    float4 c;  // box lo x, lo y, lo z, hi x
    float4 d;  // box hi y, hi z, -, -
};

struct Grid {
    double inv;              // 1 / cell size
    unsigned mask;           // bucket count - 1
    const int* bstart;       // bucket start (mask + 2 entries)
    const GridEntry* ent;    // entries sorted by bucket
};

__device__ __forceinline__ unsigned cell_hash(int i, int j, int k, unsigned mask)
{
    return ((unsigned)i * 73856093u ^ (unsigned)j * 19349663u ^ (unsigned)k * 83492791u) & mask;
}
__device__ __forceinline__ int cellc(double v, double inv) { return (int)floor(v * inv); }

// item boxes: kind 0 = triangle (3 verts), 1 = edge (2 verts); swept with dir*alpha if dir
struct ItemArgs {
    int n, nvi;
    const int* verts;
    const double* x;
    const double* dir;
    double alpha;
    double inv;
    int* lo;
    int* hi;
    int* count;
    unsigned long long* total;  // sum over items of the uncapped cell counts
};

__global__ void __launch_bounds__(256) k_item_cells(ItemArgs a)
{
    __shared__ unsigned long long part[8];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long want = 0;
    if (t < a.n) {
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < a.nvi; ++k) {
        const int v = a.verts[a.nvi * t + k];
        for (int d = 0; d < 3; ++d) {
            double p = a.x[3 * v + d];
            mn[d] = fmin(mn[d], p);
            mx[d] = fmax(mx[d], p);
            if (a.dir) {
                p = p + a.alpha * a.dir[3 * v + d];
                mn[d] = fmin(mn[d], p);
                mx[d] = fmax(mx[d], p);
            }
        }
    }
    long long c = 1;
    for (int d = 0; d < 3; ++d) {
        const int l = cellc(mn[d], a.inv), h = cellc(mx[d], a.inv);
        a.lo[3 * t + d] = l;
        a.hi[3 * t + d] = h;
        c = min(c * max((long long)h - (long long)l + 1, 1ll), (long long)kMaxGridEntries + 1);
    }
    a.count[t] = (int)min(c, (long long)(1 << 28));
    want = (unsigned long long)c;
    }
    // block sum, one atomic per block (each term <= 2^27 + 1, so no overflow)
    for (int o = 16; o > 0; o >>= 1) want += __shfl_down_sync(0xffffffffu, want, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = want;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += part[w];
        atomicAdd(a.total, b);
    }
}

__global__ void k_item_emit(int n, const int* lo, const int* hi, const int* off, unsigned mask, unsigned* ebucket,
                            int* eitem, int* bcount)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int o = off[t];
    const int cnt = off[t + 1] - o;
    int k = 0;
    for (int i = lo[3 * t]; i <= hi[3 * t] && k < cnt; ++i)
        for (int j = lo[3 * t + 1]; j <= hi[3 * t + 1] && k < cnt; ++j)
            for (int l = lo[3 * t + 2]; l <= hi[3 * t + 2] && k < cnt; ++l, ++k) {
                const unsigned b = cell_hash(i, j, l, mask);
                ebucket[o + k] = b;
                eitem[o + k] = t;
                atomicAdd(bcount + b, 1);
            }
}

__global__ void k_bucket_scatter(int ne, const unsigned* ebucket, const int* eitem, const int* bstart, int* cursor,
                                 const int* lo, const int* hi, const float* box, GridEntry* ent)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const unsigned b = ebucket[e];
    const int t = eitem[e];
    GridEntry g;
    g.a = make_int4(t, lo[3 * t], lo[3 * t + 1], lo[3 * t + 2]);
    g.b = make_int4(hi[3 * t], hi[3 * t + 1], hi[3 * t + 2], 0);
    if (box) {
        const float* q = box + 6 * (size_t)t;
        g.c = make_float4(q[0], q[1], q[2], q[3]);
        g.d = make_float4(q[4], q[5], 0.f, 0.f);
    } else {
        g.c = make_float4(0.f, 0.f, 0.f, 0.f);
        g.d = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    ent[bstart[b] + atomicAdd(cursor + b, 1)] = g;
}

// simple bump allocator over the sim scratch buffer
struct Arena {
    char* base;
    size_t cap, used = 0;
    template <typename T>
    T* take(size_t n)
    {
        size_t off = (used + 255) & ~(size_t)255;
        used = off + n * sizeof(T);
        return (T*)(base + off);
    }
};

static int ensure_scratch(Sim* s, size_t bytes)
{
    if (s->scratch.n >= bytes) return CIPC_OK;
    cudaStreamSynchronize(s->stream);
    if (s->scratch.alloc(bytes + bytes / 2) != cudaSuccess) return set_error(CIPC_ERR_CUDA, "scratch allocation");
    return CIPC_OK;
}

static size_t grid_bytes(int n, int cells_per_item);

// Builds a grid over n items (box: their FP32 boxes, 6 per item, copied into the
// entries; may be null); returns the Grid view (valid until the arena is reused)
static int build_grid(Sim* s, Arena& ar, int n, int nvi, const int* verts, const double* x, const double* dir,
                      double alpha, const float* box, Grid& G)
{
    cudaStream_t st = s->stream;
    const double inv = 1.0 / s->cell;
    int* lo = ar.take<int>(3 * (size_t)n + 3);
    int* hi = ar.take<int>(3 * (size_t)n + 3);
    int* cnt = ar.take<int>((size_t)n + 1);
    int* off = ar.take<int>((size_t)n + 2);
    int* tmp = ar.take<int>(2 * ((size_t)n / 1024 + 8) + 64);
    unsigned long long* want = ar.take<unsigned long long>(1);
    if (ar.used > ar.cap) {  // checked before any kernel writes into the arena
        s->scratch_bytes = 2 * ar.used + grid_bytes(n, 64);
        return kNeedScratch;
    }
    cudaMemsetAsync(want, 0, sizeof(unsigned long long), st);
    ItemArgs a{n, nvi, verts, x, dir, alpha, inv, lo, hi, cnt, want};
    if (n > 0) k_item_cells<<<nblk(n, 256), 256, 0, st>>>(a);
    else cudaMemsetAsync(cnt, 0, sizeof(int), st);
    unsigned long long hw = 0;
    cudaMemcpyAsync(&hw, want, sizeof(hw), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (hw > kMaxGridEntries) return kSpanTooLarge;  // before the int scan could overflow
    scan_exclusive(cnt, off, std::max(n, 1), tmp, st);
    // every item's count is below the cap here, so the scanned total is hw
    const int total = (int)hw;
    unsigned nb = 1024;
    while (nb < 2u * (unsigned)std::max(total, 1)) nb <<= 1;
    unsigned* eb = ar.take<unsigned>((size_t)total + 1);
    int* ei = ar.take<int>((size_t)total + 1);
    int* bcount = ar.take<int>((size_t)nb + 1);
    int* bstart = ar.take<int>((size_t)nb + 2);
    int* cursor = ar.take<int>((size_t)nb + 1);
    GridEntry* ent = ar.take<GridEntry>((size_t)total + 1);
    int* tmp2 = ar.take<int>(2 * ((size_t)nb / 1024 + 8) + 64);
    if (ar.used > ar.cap) {
        s->scratch_bytes = ar.used + ar.used / 2;
        return kNeedScratch;
    }
    cudaMemsetAsync(bcount, 0, sizeof(int) * (nb + 1), st);
    cudaMemsetAsync(cursor, 0, sizeof(int) * (nb + 1), st);
    if (n > 0) k_item_emit<<<nblk(n, 256), 256, 0, st>>>(n, lo, hi, off, nb - 1, eb, ei, bcount);
    scan_exclusive(bcount, bstart, (int)nb, tmp2, st);
    if (total > 0)
        k_bucket_scatter<<<nblk(total, 256), 256, 0, st>>>(total, eb, ei, bstart, cursor, lo, hi, box, ent);
    G.inv = inv;
    G.mask = nb - 1;
    G.bstart = bstart;
    G.ent = ent;
    return CIPC_OK;
}

// constraint-set grids have no step to shrink: an oversized grid is an error
static int static_grid(int rc)
{
    if (rc == kSpanTooLarge)
        return set_error(CIPC_ERR_INVALID_ARG, "spatial grid: primitives span more than %llu cells",
                         (unsigned long long)kMaxGridEntries);
    return rc;
}

// upper bound of scratch bytes for a grid over n items with ~c cells per item
static size_t grid_bytes(int n, int cells_per_item)
{
    size_t total = (size_t)n * cells_per_item + 16;
    size_t nb = 1024;
    while (nb < 2 * total) nb <<= 1;
    return 4 * (size_t)(10 * n + 4 * total + 4 * nb) + sizeof(GridEntry) * (total + 1) + (1 << 16);
}

// ---------------------------------------------------------------------------
// constraint set
// ---------------------------------------------------------------------------
struct ConSink {
    int* kind;
    int4* verts;
    int* mult;
    int cap;
    unsigned long long* counter;  // [0] list count, [1] overflow flag, [2] table overflow
    unsigned long long* tkeys;    // merge table
    int* tcount;
    unsigned tmask;
};

__device__ __forceinline__ void emit(const ConSink& S, int k, int a, int b, int c, int d)
{
    const unsigned long long i = atomicAdd(S.counter, 1ull);
    if (i < (unsigned long long)S.cap) {
        S.kind[i] = k;
        S.verts[i] = make_int4(a, b, c, d);
        S.mult[i] = 1;
    } else {
        S.counter[1] = 1;
    }
}

// PP (v2 = -1) or PE merged by code
__device__ __forceinline__ void emit_merge(const ConSink& S, int k, int a, int b, int c)
{
    const unsigned long long key = ((unsigned long long)(k == kc_PE) << 63) | ((unsigned long long)a << 42) |
                                   ((unsigned long long)b << 21) | (unsigned long long)(c < 0 ? 0x1FFFFF : c);
    unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 32) & S.tmask;
    for (unsigned probe = 0; probe <= S.tmask; ++probe) {
        const unsigned long long prev = atomicCAS(S.tkeys + h, ~0ull, key);
        if (prev == ~0ull || prev == key) {
            atomicAdd(S.tcount + h, 1);
            return;
        }
        h = (h + 1) & S.tmask;
    }
    S.counter[2] = 1;
}

struct CsArgs {
    int nbn, nbe;
    const int* bnode;
    const int* bedge;
    const int* btri;
    const double* x;
    const double* X0;
    const uint8_t* dbc;
    double dHat, dh2;
    Grid G;
    ConSink S;
    // FP32 boxes (lo xyz, hi xyz) of the boundary triangles and edges, rounded
    // outward, and dHat rounded up: a conservative prefilter in front of the
    // FP64 box test (see box_apart)
    const float* tbox;
    const float* ebox;
    float dHat_f;
};

// FP32 boxes of n items of nvi vertices: lo rounded down, hi rounded up, so each
// box contains the FP64 box of the item
__global__ void k_item_boxes(int n, int nvi, const int* verts, const double* x, float* box)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < nvi; ++k) {
        const int v = verts[nvi * t + k];
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], x[3 * v + d]);
            mx[d] = fmax(mx[d], x[3 * v + d]);
        }
    }
    for (int d = 0; d < 3; ++d) {
        box[6 * t + d] = __double2float_rd(mn[d]);
        box[6 * t + 3 + d] = __double2float_ru(mx[d]);
    }
}

// True only if the FP64 box test (any coordinate gap between the two boxes above
// dHat) rejects the pair too: a, b contain the FP64 boxes, the rounded-down
// difference bounds the real gap from below, and a gap above dHat rounded up to
// float exceeds dHat by at least one float ulp, far more than the FP64 rounding of
// the gap.  Candidates it keeps go through the unchanged FP64 tests, so the
// constraint set is the same.
__device__ __forceinline__ bool box_apart(const float* a, const float* b, float dh)
{
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (__fsub_rd(a[k], b[3 + k]) > dh || __fsub_rd(b[k], a[3 + k]) > dh) return true;
    return false;
}

__device__ __forceinline__ bool any_gt3(d3 a, double d) { return a.x > d || a.y > d || a.z > d; }
__device__ __forceinline__ d3 vmin3(d3 a, d3 b) { return mk(fmin(a.x, b.x), fmin(a.y, b.y), fmin(a.z, b.z)); }
__device__ __forceinline__ d3 vmax3(d3 a, d3 b) { return mk(fmax(a.x, b.x), fmax(a.y, b.y), fmax(a.z, b.z)); }

// iterate the candidates of a query cell range [ql, qh]; calls f(item, box) once
// per pair, box = the item's FP32 box from its grid entry
template <typename F>
__device__ __forceinline__ void grid_query(const Grid& G, const int (&ql)[3], const int (&qh)[3], F&& f)
{
    for (int i = ql[0]; i <= qh[0]; ++i)
        for (int j = ql[1]; j <= qh[1]; ++j)
            for (int k = ql[2]; k <= qh[2]; ++k) {
                const unsigned b = cell_hash(i, j, k, G.mask);
                const int e1 = __ldg(G.bstart + b + 1);
                for (int e = __ldg(G.bstart + b); e < e1; ++e) {
                    const GridEntry* g = G.ent + e;
                    const int4 A = __ldg(&g->a), B = __ldg(&g->b);
                    const float4 C = __ldg(&g->c), D = __ldg(&g->d);
                    if (i < A.y || j < A.z || k < A.w) continue;
                    if (i > B.x || j > B.y || k > B.z) continue;
                    // first cell of the intersection of both ranges
                    if (i != max(ql[0], A.y) || j != max(ql[1], A.z) || k != max(ql[2], A.w)) continue;
                    const float bx[6] = {C.x, C.y, C.z, C.w, D.x, D.y};
                    f(A.x, bx);
                }
            }
}

// The same query with the whole warp on one query range: lane l takes cells l,
// l + 32, ... of the range, the warp scans their entry counts, and then every lane
// takes one entry of the concatenated lists per round (its cell found by a binary
// search over the lanes' prefix sums), so the lanes stay busy however the entries
// are spread over the cells.  All 32 lanes of the warp must call it with the same
// range; f(item, box) runs on the lanes that hold a candidate.
template <typename F>
__device__ __forceinline__ void grid_query_warp(const Grid& G, const int (&ql)[3], const int (&qh)[3], F&& f)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int nx = qh[0] - ql[0] + 1, ny = qh[1] - ql[1] + 1, nz = qh[2] - ql[2] + 1;
    const long long ncell = (long long)nx * ny * nz;
    for (long long c0 = 0; c0 < ncell; c0 += 32) {
        const long long c = c0 + lane;
        int ci = 0, cj = 0, ck = 0, st = 0, n = 0;
        if (c < ncell) {
            ck = ql[2] + (int)(c % nz);
            cj = ql[1] + (int)((c / nz) % ny);
            ci = ql[0] + (int)(c / ((long long)nz * ny));
            const unsigned b = cell_hash(ci, cj, ck, G.mask);
            st = __ldg(G.bstart + b);
            n = __ldg(G.bstart + b + 1) - st;
        }
        int incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        for (int t0 = 0; t0 < total; t0 += 32) {
            const int t = t0 + lane;
            // owner = the first lane whose inclusive count exceeds t
            int owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int v = __shfl_sync(FULL, incl, owner + step - 1);
                if (t >= v) owner += step;
            }
            owner = min(owner, 31);
            const int o_incl = __shfl_sync(FULL, incl, owner), o_n = __shfl_sync(FULL, n, owner);
            const int o_st = __shfl_sync(FULL, st, owner);
            const int i = __shfl_sync(FULL, ci, owner), j = __shfl_sync(FULL, cj, owner),
                      k = __shfl_sync(FULL, ck, owner);
            if (t >= total) continue;
            const GridEntry* g = G.ent + o_st + (t - (o_incl - o_n));
            const int4 A = __ldg(&g->a), B = __ldg(&g->b);
            const float4 C = __ldg(&g->c), D = __ldg(&g->d);
            if (i < A.y || j < A.z || k < A.w) continue;
            if (i > B.x || j > B.y || k > B.z) continue;
            // first cell of the intersection of both ranges
            if (i != max(ql[0], A.y) || j != max(ql[1], A.z) || k != max(ql[2], A.w)) continue;
            const float bx[6] = {C.x, C.y, C.z, C.w, D.x, D.y};
            f(A.x, bx);
        }
    }
}

// Query set-up values of lane k, broadcast to the warp: the set-up (cell range,
// FP32 box, ids) is computed one query per lane for kQueryChunk queries, so its
// FP64 work is shared by that many queries, and the warp then runs the queries
// one after another (a warp per query paid it 32 times over: the FP64 pipe was
// 80% busy; a chunk of 32 left too few warps in flight)
constexpr int kQueryChunk = 8;
struct QuerySetup {
    int ql[3], qh[3];
    float box[6];
    int id[3];
};

__device__ __forceinline__ QuerySetup bcast_setup(const QuerySetup& q, int k)
{
    const unsigned FULL = 0xffffffffu;
    QuerySetup r;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        r.ql[d] = __shfl_sync(FULL, q.ql[d], k);
        r.qh[d] = __shfl_sync(FULL, q.qh[d], k);
        r.id[d] = __shfl_sync(FULL, q.id[d], k);
    }
#pragma unroll
    for (int d = 0; d < 6; ++d) r.box[d] = __shfl_sync(FULL, q.box[d], k);
    return r;
}

// Candidate lists between the grid traversal and the FP64 tests.  The traversal
// kernels (one warp per query primitive, grid_query_warp) keep only the cheap
// integer and FP32 tests and append the surviving pairs here; the evaluation kernels then run the
// FP64 box test, the classification and the distance one thread per pair, with
// every lane of a warp busy (in the traversal the candidate counts differ from
// lane to lane: 3-5 of 32 lanes were active, and the FP64 pipe, which counts warp
// instructions, was 70-82% busy).  Appends are aggregated over the lanes that
// arrive together; a list that overflows its capacity is counted and the caller
// reruns with a larger one.
struct CandList {
    int2* v;
    unsigned long long* n;
    int cap;
};

__device__ __forceinline__ void push_cand(const CandList& L, int x, int y)
{
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(L.n, (unsigned long long)g.size());
    base = g.shfl(base, 0);
    const unsigned long long i = base + g.thread_rank();
    if (i < (unsigned long long)L.cap) L.v[i] = make_int2(x, y);
}

__device__ __forceinline__ int cand_count(const CandList& L)
{
    const unsigned long long n = *L.n;
    return (int)(n < (unsigned long long)L.cap ? n : (unsigned long long)L.cap);
}

__global__ void k_cs_pt(CsArgs a, CandList L)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kQueryChunk; base < a.nbn;
         base += nw * kQueryChunk) {
        QuerySetup mine{};
        const int sv = base + lane;
        if (lane < kQueryChunk && sv < a.nbn) {
            const int vI = a.bnode[sv];
            const d3 p = ld(a.x, vI);
            mine.ql[0] = cellc(p.x - a.dHat, a.G.inv);
            mine.ql[1] = cellc(p.y - a.dHat, a.G.inv);
            mine.ql[2] = cellc(p.z - a.dHat, a.G.inv);
            mine.qh[0] = cellc(p.x + a.dHat, a.G.inv);
            mine.qh[1] = cellc(p.y + a.dHat, a.G.inv);
            mine.qh[2] = cellc(p.z + a.dHat, a.G.inv);
            const float pb[6] = {__double2float_rd(p.x), __double2float_rd(p.y), __double2float_rd(p.z),
                                 __double2float_ru(p.x), __double2float_ru(p.y), __double2float_ru(p.z)};
#pragma unroll
            for (int d = 0; d < 6; ++d) mine.box[d] = pb[d];
            mine.id[0] = vI;
        }
        const int nq = min(kQueryChunk, a.nbn - base);
        for (int k = 0; k < nq; ++k) {
            const QuerySetup q = bcast_setup(mine, k);
            const int vI = q.id[0];
            grid_query_warp(a.G, q.ql, q.qh, [&](int t, const float (&bx)[6]) {
                if (box_apart(q.box, bx, a.dHat_f)) return;
                const int t0i = a.btri[3 * t], t1i = a.btri[3 * t + 1], t2i = a.btri[3 * t + 2];
                if (vI == t0i || vI == t1i || vI == t2i) return;
                if (a.dbc[vI] && a.dbc[t0i] && a.dbc[t1i] && a.dbc[t2i]) return;
                push_cand(L, vI, t);
            });
        }
    }
}

// point-triangle candidates (point vI, boundary triangle t): FP64 box test,
// classification and distance (IPC.h:19-740)
__global__ void __launch_bounds__(128) k_cs_pt_eval(CsArgs a, CandList L)
{
    const int n = cand_count(L);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int2 q = L.v[c];
        const int vI = q.x, t = q.y;
        const d3 p = ld(a.x, vI);
        const int t0i = a.btri[3 * t], t1i = a.btri[3 * t + 1], t2i = a.btri[3 * t + 2];
        const d3 t0 = ld(a.x, t0i), t1 = ld(a.x, t1i), t2 = ld(a.x, t2i);
        const d3 mx = vmax3(vmax3(t0, t1), t2), mn = vmin3(vmin3(t0, t1), t2);
        if (any_gt3(p - mx, a.dHat) || any_gt3(mn - p, a.dHat)) continue;
        const d3 e1 = t1 - t0, e2 = t2 - t0, w = p - t0;
        switch (pt_type_fast(p, t0, t1, t2, w, e1, e2)) {
            case 0: if (n2(w) < a.dh2) emit_merge(a.S, kc_PP, vI, t0i, -1); break;
            case 1: if (pp_d2(p, t1) < a.dh2) emit_merge(a.S, kc_PP, vI, t1i, -1); break;
            case 2: if (pp_d2(p, t2) < a.dh2) emit_merge(a.S, kc_PP, vI, t2i, -1); break;
            case 3: if (pe_d2(p, t0, t1) < a.dh2) emit_merge(a.S, kc_PE, vI, t0i, t1i); break;
            case 4: if (pe_d2(p, t1, t2) < a.dh2) emit_merge(a.S, kc_PE, vI, t1i, t2i); break;
            case 5: if (pe_d2(p, t2, t0) < a.dh2) emit_merge(a.S, kc_PE, vI, t2i, t0i); break;
            default: if (pt_d2_w(w, e1, e2) < a.dh2) emit(a.S, kc_PT, vI, t0i, t1i, t2i); break;
        }
    }
}

__global__ void k_cs_ee(CsArgs a, CandList L)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kQueryChunk; base < a.nbe;
         base += nw * kQueryChunk) {
        QuerySetup mine{};
        const int e = base + lane;
        if (lane < kQueryChunk && e < a.nbe) {
            const int a0 = a.bedge[2 * e], a1 = a.bedge[2 * e + 1];
            const d3 ea0 = ld(a.x, a0), ea1 = ld(a.x, a1);
            const d3 mna = vmin3(ea0, ea1), mxa = vmax3(ea0, ea1);
            mine.ql[0] = cellc(mna.x - a.dHat, a.G.inv);
            mine.ql[1] = cellc(mna.y - a.dHat, a.G.inv);
            mine.ql[2] = cellc(mna.z - a.dHat, a.G.inv);
            mine.qh[0] = cellc(mxa.x + a.dHat, a.G.inv);
            mine.qh[1] = cellc(mxa.y + a.dHat, a.G.inv);
            mine.qh[2] = cellc(mxa.z + a.dHat, a.G.inv);
#pragma unroll
            for (int d = 0; d < 6; ++d) mine.box[d] = a.ebox[6 * (size_t)e + d];
            mine.id[0] = e;
            mine.id[1] = a0;
            mine.id[2] = a1;
        }
        const int nq = min(kQueryChunk, a.nbe - base);
        for (int k = 0; k < nq; ++k) {
            const QuerySetup q = bcast_setup(mine, k);
            const int eI = q.id[0], a0 = q.id[1], a1 = q.id[2];
            grid_query_warp(a.G, q.ql, q.qh, [&](int eJ, const float (&bx)[6]) {
                if (eJ <= eI) return;
                if (box_apart(q.box, bx, a.dHat_f)) return;
                const int b0 = a.bedge[2 * eJ], b1 = a.bedge[2 * eJ + 1];
                if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) return;
                if (a.dbc[a0] && a.dbc[a1] && a.dbc[b0] && a.dbc[b1]) return;
                push_cand(L, eI, eJ);
            });
        }
    }
}

// edge-edge candidates (boundary edges eI < eJ): FP64 box test, classification,
// distance and the mollifier test (IPC.h:19-740); the mollifier threshold is
// formed only for pairs within dHat
__global__ void __launch_bounds__(128) k_cs_ee_eval(CsArgs a, CandList L)
{
    const int n = cand_count(L);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int2 q = L.v[c];
        const int eI = q.x, eJ = q.y;
        const int a0 = a.bedge[2 * eI], a1 = a.bedge[2 * eI + 1];
        const int b0 = a.bedge[2 * eJ], b1 = a.bedge[2 * eJ + 1];
        const d3 ea0 = ld(a.x, a0), ea1 = ld(a.x, a1);
        const d3 mna = vmin3(ea0, ea1), mxa = vmax3(ea0, ea1);
        const d3 eb0 = ld(a.x, b0), eb1 = ld(a.x, b1);
        const d3 mnb = vmin3(eb0, eb1), mxb = vmax3(eb0, eb1);
        if (any_gt3(mna - mxb, a.dHat) || any_gt3(mnb - mxa, a.dHat)) continue;
        const d3 u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0;
        auto moll = [&]() {
            const double eps_x =
                G_MUL(G_MUL(1.0e-3, n2(ld(a.X0, a0) - ld(a.X0, a1))), n2(ld(a.X0, b0) - ld(a.X0, b1)));
            return n2(cross(u, v)) < eps_x;
        };
        switch (ee_type_fast(ea0, ea1, eb0, eb1, u, v, w)) {
            case 0:
                if (n2(w) < a.dh2) {
                    if (moll()) emit(a.S, kc_PPM, a0, a1, b0, b1);
                    else emit_merge(a.S, kc_PP, a0, b0, -1);
                }
                break;
            case 1:
                if (pp_d2(ea0, eb1) < a.dh2) {
                    if (moll()) emit(a.S, kc_PPM, a0, a1, b1, b0);
                    else emit_merge(a.S, kc_PP, a0, b1, -1);
                }
                break;
            case 2:
                if (pe_d2(ea0, eb0, eb1) < a.dh2) {
                    if (moll()) emit(a.S, kc_PEM, a0, a1, b0, b1);
                    else emit_merge(a.S, kc_PE, a0, b0, b1);
                }
                break;
            case 3:
                if (pp_d2(ea1, eb0) < a.dh2) {
                    if (moll()) emit(a.S, kc_PPM, a1, a0, b0, b1);
                    else emit_merge(a.S, kc_PP, a1, b0, -1);
                }
                break;
            case 4:
                if (pp_d2(ea1, eb1) < a.dh2) {
                    if (moll()) emit(a.S, kc_PPM, a1, a0, b1, b0);
                    else emit_merge(a.S, kc_PP, a1, b1, -1);
                }
                break;
            case 5:
                if (pe_d2(ea1, eb0, eb1) < a.dh2) {
                    if (moll()) emit(a.S, kc_PEM, a1, a0, b0, b1);
                    else emit_merge(a.S, kc_PE, a1, b0, b1);
                }
                break;
            case 6:
                if (pe_d2(eb0, ea0, ea1) < a.dh2) {
                    if (moll()) emit(a.S, kc_PEM, b0, b1, a0, a1);
                    else emit_merge(a.S, kc_PE, b0, a0, a1);
                }
                break;
            case 7:
                if (pe_d2(eb1, ea0, ea1) < a.dh2) {
                    if (moll()) emit(a.S, kc_PEM, b1, b0, a0, a1);
                    else emit_merge(a.S, kc_PE, b1, a0, a1);
                }
                break;
            default:
                if (ee_d2_w(u, v, w) < a.dh2) emit(a.S, moll() ? kc_EEM : kc_EE, a0, a1, b0, b1);
                break;
        }
    }
}

__global__ void k_cs_compact(ConSink S)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > S.tmask) return;
    const unsigned long long key = S.tkeys[t];
    if (key == ~0ull) return;
    const int pe = (int)(key >> 63);
    const int a = (int)((key >> 42) & 0x1FFFFF), b = (int)((key >> 21) & 0x1FFFFF), c = (int)(key & 0x1FFFFF);
    const unsigned long long i = atomicAdd(S.counter, 1ull);
    if (i < (unsigned long long)S.cap) {
        S.kind[i] = pe ? kc_PE : kc_PP;
        S.verts[i] = make_int4(a, b, pe ? c : -1, -1);
        S.mult[i] = S.tcount[t];
    } else {
        S.counter[1] = 1;
    }
}

// Codimensional nodes (IPC.h:271-350): rod and particle nodes (boundary nodes
// from sv_begin) against the rod segments (the last boundary edges, grid items
// relative to e_begin): point-edge classification, PP / PE merged like the rest.
__global__ void k_cs_codim_pe(CsArgs a, int sv_begin, int e_begin)
{
    const int sv = sv_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (sv >= a.nbn) return;
    const int vI = a.bnode[sv];
    const d3 p = ld(a.x, vI);
    int ql[3], qh[3];
    ql[0] = cellc(p.x - a.dHat, a.G.inv);
    ql[1] = cellc(p.y - a.dHat, a.G.inv);
    ql[2] = cellc(p.z - a.dHat, a.G.inv);
    qh[0] = cellc(p.x + a.dHat, a.G.inv);
    qh[1] = cellc(p.y + a.dHat, a.G.inv);
    qh[2] = cellc(p.z + a.dHat, a.G.inv);
    grid_query(a.G, ql, qh, [&](int el, const float (&)[6]) {
        const int eI = e_begin + el;
        const int e0 = a.bedge[2 * eI], e1 = a.bedge[2 * eI + 1];
        if (vI == e0 || vI == e1) return;
        if (a.dbc[vI] && a.dbc[e0] && a.dbc[e1]) return;
        const d3 x0 = ld(a.x, e0), x1 = ld(a.x, e1);
        const d3 mx = vmax3(x0, x1), mn = vmin3(x0, x1);
        if (any_gt3(p - mx, a.dHat) || any_gt3(mn - p, a.dHat)) return;  // CCD.h:16-30
        switch (pe_type(p, x0, x1)) {
            case 0: if (pp_d2(p, x0) < a.dh2) emit_merge(a.S, kc_PP, vI, e0, -1); break;
            case 1: if (pp_d2(p, x1) < a.dh2) emit_merge(a.S, kc_PP, vI, e1, -1); break;
            default: if (pe_d2(p, x0, x1) < a.dh2) emit_merge(a.S, kc_PE, vI, e0, e1); break;
        }
    });
}

// particles (boundary nodes from sv_begin) against every later boundary node
// (grid over all boundary nodes): point-point, merged
__global__ void k_cs_codim_pp(CsArgs a, int sv_begin)
{
    const int sv = sv_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (sv >= a.nbn) return;
    const int vI = a.bnode[sv];
    const d3 p = ld(a.x, vI);
    int ql[3], qh[3];
    ql[0] = cellc(p.x - a.dHat, a.G.inv);
    ql[1] = cellc(p.y - a.dHat, a.G.inv);
    ql[2] = cellc(p.z - a.dHat, a.G.inv);
    qh[0] = cellc(p.x + a.dHat, a.G.inv);
    qh[1] = cellc(p.y + a.dHat, a.G.inv);
    qh[2] = cellc(p.z + a.dHat, a.G.inv);
    grid_query(a.G, ql, qh, [&](int svJ, const float (&)[6]) {
        if (svJ <= sv) return;
        const int vJ = a.bnode[svJ];
        if (a.dbc[vI] && a.dbc[vJ]) return;
        if (pp_d2(p, ld(a.x, vJ)) < a.dh2) emit_merge(a.S, kc_PP, vI, vJ, -1);
    });
}

// smallest float not below v (host)
static float float_up(double v)
{
    float f = (float)v;
    if ((double)f < v) f = std::nextafter(f, INFINITY);
    return f;
}

int build_constraints(Sim* s, const double* x)
{
    cudaStream_t st = s->stream;
    const double dHat = sqrt(s->prm.dHat2) + s->prm.xi;
    if (s->cap_con == 0) {
        s->cap_con = std::max(4096, 4 * (s->nbn + s->nbe));
        if (s->ckind.alloc(s->cap_con) || s->cverts.alloc(s->cap_con) || s->cmult.alloc(s->cap_con))
            return set_error(CIPC_ERR_CUDA, "constraint buffers");
    }
    for (int attempt = 0; attempt < 8; ++attempt) {
        // merge table: 4x the list capacity, power of two
        unsigned tsz = 1024;
        while (tsz < 4u * (unsigned)s->cap_con) tsz <<= 1;
        const size_t need = grid_bytes(std::max(std::max(s->nbt, s->nbe), s->nbn), 16) + (size_t)tsz * 12 +
                            24 * ((size_t)s->nbt + s->nbe) +
                            8 * (size_t)std::max(s->cap_cand, std::max(1 << 16, 8 * (s->nbn + s->nbe))) + (1 << 20);
        int rc = ensure_scratch(s, need);
        if (rc) return rc;
        Arena ar{s->scratch.p, s->scratch.n};
        unsigned long long* tkeys = ar.take<unsigned long long>(tsz);
        int* tcount = ar.take<int>(tsz);
        float* tbox = ar.take<float>(6 * (size_t)s->nbt + 6);
        float* ebox = ar.take<float>(6 * (size_t)s->nbe + 6);
        if (s->cap_cand == 0) s->cap_cand = std::max(1 << 16, 8 * (s->nbn + s->nbe));
        int2* cand = ar.take<int2>((size_t)s->cap_cand);
        if (ar.used > ar.cap) return set_error(CIPC_ERR_CUDA, "constraint scratch");
        // the two candidate lists share one buffer: counts in cnt[4] (PT) and cnt[5] (EE)
        const CandList Lpt{cand, s->cnt.p + 4, s->cap_cand}, Lee{cand, s->cnt.p + 5, s->cap_cand};
        const int eval_grid = num_sms() * 8;
        if (s->nbt) k_item_boxes<<<nblk(s->nbt, 256), 256, 0, st>>>(s->nbt, 3, s->btri.p, x, tbox);
        if (s->nbe) k_item_boxes<<<nblk(s->nbe, 256), 256, 0, st>>>(s->nbe, 2, s->bedge.p, x, ebox);
        cudaMemsetAsync(tkeys, 0xFF, sizeof(unsigned long long) * tsz, st);
        cudaMemsetAsync(tcount, 0, sizeof(int) * tsz, st);
        cudaMemsetAsync(s->cnt.p, 0, 8 * sizeof(unsigned long long), st);
        ConSink S{s->ckind.p, s->cverts.p, s->cmult.p, s->cap_con, s->cnt.p, tkeys, tcount, tsz - 1};
        size_t mark = ar.used;
        Grid G;
        rc = static_grid(build_grid(s, ar, s->nbt, 3, s->btri.p, x, nullptr, 0, tbox, G));
        if (rc == kNeedScratch) {
            if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
            continue;
        }
        if (rc) return rc;
        CsArgs a{s->nbn, s->nbe, s->bnode.p, s->bedge.p, s->btri.p, x, s->X0.p, s->dbc.p, dHat, dHat * dHat, G, S,
                 tbox, ebox, float_up(dHat)};
        k_cs_pt<<<eval_grid, 256, 0, st>>>(a, Lpt);
        k_cs_pt_eval<<<eval_grid, 128, 0, st>>>(a, Lpt);
        ar.used = mark;
        rc = static_grid(build_grid(s, ar, s->nbe, 2, s->bedge.p, x, nullptr, 0, ebox, G));
        if (rc == kNeedScratch) {
            if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
            continue;
        }
        if (rc) return rc;
        a.G = G;
        k_cs_ee<<<eval_grid, 256, 0, st>>>(a, Lee);
        k_cs_ee_eval<<<eval_grid, 128, 0, st>>>(a, Lee);
        bool again = false;
        if (s->nrod_e > 0 && s->nbn > s->codim0) {
            ar.used = mark;
            const int e_begin = s->nbe - s->nrod_e;
            rc = static_grid(
                build_grid(s, ar, s->nrod_e, 2, s->bedge.p + 2 * (size_t)e_begin, x, nullptr, 0, nullptr, G));
            if (rc == kNeedScratch) {
                if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
                again = true;
            } else if (rc) {
                return rc;
            } else {
                a.G = G;
                k_cs_codim_pe<<<nblk(s->nbn - s->codim0, 128), 128, 0, st>>>(a, s->codim0, e_begin);
            }
        }
        if (!again && s->nbn > s->codim1) {
            ar.used = mark;
            rc = static_grid(build_grid(s, ar, s->nbn, 1, s->bnode.p, x, nullptr, 0, nullptr, G));
            if (rc == kNeedScratch) {
                if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
                again = true;
            } else if (rc) {
                return rc;
            } else {
                a.G = G;
                k_cs_codim_pp<<<nblk(s->nbn - s->codim1, 128), 128, 0, st>>>(a, s->codim1);
            }
        }
        if (again) continue;
        k_cs_compact<<<nblk(tsz, 256), 256, 0, st>>>(S);
        unsigned long long c[6];
        cudaMemcpyAsync(c, s->cnt.p, sizeof(c), cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return set_cuda_error(e, "constraint set");
        const unsigned long long nc = std::max(c[4], c[5]);
        if (nc > (unsigned long long)s->cap_cand) {
            // a candidate list overflowed: rebuild the set with room for all of them
            s->cap_cand = (int)std::min<unsigned long long>(nc + nc / 2 + 4096, 1ull << 30);
            continue;
        }
        if (!c[1] && !c[2]) {
            s->ncon = (int)c[0];
            return CIPC_OK;
        }
        s->cap_con = std::max(2 * s->cap_con, (int)c[0] + 1024);
        if (s->ckind.alloc(s->cap_con) || s->cverts.alloc(s->cap_con) || s->cmult.alloc(s->cap_con))
            return set_error(CIPC_ERR_CUDA, "constraint buffers");
    }
    return set_error(CIPC_ERR_CUDA, "constraint set did not fit after resizing");
}

// ---------------------------------------------------------------------------
// barrier over the constraint list
// ---------------------------------------------------------------------------
struct BarArgs {
    int n;
    const int* kind;
    const int4* verts;
    const int* mult;
    const double* x;
    const double* X0;
    const uint8_t* dbc;
    double xi2, shat, kappa;
    double* g;
    double* red;
    double* flag;  // set to 1 when some s <= 0
    void* hess;    // 78 per constraint (HT), entry h of constraint i at h * hs + i
    size_t hs;
    double* pdiag;
};

template <typename HT, int K>
__device__ void bar_one(const BarArgs& a, int i, const d3 (&v)[4], const int (&id)[4], double s, double& E,
                        bool want_h)
{
    constexpr int NV = (K == kc_PP ? 2 : (K == kc_PE ? 3 : 4));
    d3 vr[4];
    if (K >= kc_EEM) {
#pragma unroll
        for (int q = 0; q < 4; ++q) vr[q] = ld(a.X0, id[q]);
    }
    ConOut<HT, NV> o;
    con_eval<HT, K>(v, vr, s, a.shat, a.kappa, (double)a.mult[i], want_h, o);
    E = o.E;
    if (a.g)
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
            for (int c = 0; c < 3; ++c) atomicAdd(a.g + 3 * id[q] + c, o.g[3 * q + c]);
    if (want_h) {
        HT* out = reinterpret_cast<HT*>(a.hess) + i;
        int w = 0;
        constexpr int m = 3 * NV;
#pragma unroll
        for (int p = 0; p < m; ++p)
#pragma unroll
            for (int q = p; q < m; ++q) {
                const bool keep = !a.dbc[id[p / 3]] && !a.dbc[id[q / 3]];
                out[(w++) * a.hs] = keep ? o.H[p][q] : HT(0);
            }
        // diagonal blocks into the block-Jacobi diagonal
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            if (a.dbc[id[q]]) continue;
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) atomicAdd(a.pdiag + 9 * (size_t)id[q] + 3 * r + c, (double)o.H[3 * q + r][3 * q + c]);
        }
    }
}

template <typename HT>
__global__ void __launch_bounds__(128) k_barrier_cons(BarArgs a, int want_h)
{
    __shared__ double sh[128];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double E = 0;
    if (i < a.n) {
        const int k = a.kind[i];
        const int4 iv = a.verts[i];
        const int id[4] = {iv.x, iv.y, iv.z < 0 ? iv.x : iv.z, iv.w < 0 ? iv.x : iv.w};
        d3 v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = ld(a.x, id[q]);
        const double s = con_d2(k, v) - a.xi2;
        if (!(s > 0)) {
            if (a.flag) *a.flag = 1.0;
            if (want_h) {
                HT* out = reinterpret_cast<HT*>(a.hess) + i;
                for (int w = 0; w < 78; ++w) out[w * a.hs] = HT(0);
            }
        } else if (s < a.shat) {
            switch (k) {
                case kc_PP: bar_one<HT, kc_PP>(a, i, v, id, s, E, want_h); break;
                case kc_PE: bar_one<HT, kc_PE>(a, i, v, id, s, E, want_h); break;
                case kc_PT: bar_one<HT, kc_PT>(a, i, v, id, s, E, want_h); break;
                case kc_EE: bar_one<HT, kc_EE>(a, i, v, id, s, E, want_h); break;
                case kc_EEM: bar_one<HT, kc_EEM>(a, i, v, id, s, E, want_h); break;
                case kc_PEM: bar_one<HT, kc_PEM>(a, i, v, id, s, E, want_h); break;
                default: bar_one<HT, kc_PPM>(a, i, v, id, s, E, want_h); break;
            }
        } else if (want_h) {
            HT* out = reinterpret_cast<HT*>(a.hess) + i;
            for (int w = 0; w < 78; ++w) out[w * a.hs] = HT(0);
        }
    }
    // energy partial
    sh[threadIdx.x] = E;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = sh[0];
}

double barrier_kappa(const Sim* s)
{
    return s->prm.elastic ? s->kappa / (s->prm.dHat2 * s->prm.dHat2) : s->kappa;
}

static BarArgs bar_args(Sim* s, const double* x)
{
    BarArgs a;
    a.n = s->ncon;
    a.kind = s->ckind.p;
    a.verts = s->cverts.p;
    a.mult = s->cmult.p;
    a.x = x;
    a.X0 = s->X0.p;
    a.dbc = s->proj.p;  // Hessian rows / columns removed from the Newton system
    a.xi2 = s->prm.xi * s->prm.xi;
    a.shat = s->prm.dHat2 + 2 * sqrt(s->prm.dHat2) * s->prm.xi;
    a.kappa = barrier_kappa(s);
    a.g = nullptr;
    a.red = nullptr;
    a.flag = nullptr;
    a.hess = nullptr;
    a.pdiag = s->pdiag.p;
    return a;
}

int contact_energy_partials(Sim* s, const double* x, double* red, double* flag)
{
    if (s->ncon == 0) return 0;
    BarArgs a = bar_args(s, x);
    a.red = red;
    a.flag = flag;
    k_barrier_cons<double><<<nblk(s->ncon, 128), 128, 0, s->stream>>>(a, 0);
    return nblk(s->ncon, 128);
}

void contact_grad_hess(Sim* s, const double* x, double* g, bool want_hess)
{
    if (s->ncon == 0) return;
    BarArgs a = bar_args(s, x);
    a.g = g;
    const bool f32 = s->prm.precision == 1;
    if (want_hess) {
        s->chess.alloc((size_t)s->cap_con * 78 * (f32 ? 4 : 8));
        a.hess = s->chess.p;
        a.hs = (size_t)s->cap_con;
    }
    if (f32) k_barrier_cons<float><<<nblk(s->ncon, 128), 128, 0, s->stream>>>(a, want_hess ? 1 : 0);
    else k_barrier_cons<double><<<nblk(s->ncon, 128), 128, 0, s->stream>>>(a, want_hess ? 1 : 0);
}

// minimum of d^2 - xi^2 over the constraint list (device scalar, +inf if empty)
__global__ void k_min_d2(int n, const int* kind, const int4* verts, const double* x, double xi2, double* out)
{
    __shared__ double sh[256];
    double m = 1e300;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 iv = verts[i];
        const int id[4] = {iv.x, iv.y, iv.z < 0 ? iv.x : iv.z, iv.w < 0 ? iv.x : iv.w};
        d3 v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = ld(x, id[q]);
        m = fmin(m, con_d2(kind[i], v) - xi2);
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        // ordered-integer atomic min on a non-negative or negative double
        const double v = sh[0];
        unsigned long long* o = (unsigned long long*)out;
        unsigned long long bits = __double_as_longlong(v);
        unsigned long long key = (bits >> 63) ? ~bits : (bits | 0x8000000000000000ull);
        atomicMin(o, key);
    }
}
__global__ void k_decode_min(double* out)
{
    unsigned long long key = *(unsigned long long*)out;
    unsigned long long bits = (key >> 63) ? (key & 0x7FFFFFFFFFFFFFFFull) : ~key;
    *out = __longlong_as_double(bits);
}

void min_dist2_partials(Sim* s, const double* x, double* out_min)
{
    k_set_u64<<<1, 1, 0, s->stream>>>((unsigned long long*)out_min, 0xFFF0000000000000ull);  // key of +inf
    if (s->ncon > 0)
        k_min_d2<<<std::min(nblk(s->ncon, 256), 1024), 256, 0, s->stream>>>(s->ncon, s->ckind.p, s->cverts.p, x,
                                                                               s->prm.xi * s->prm.xi, out_min);
    k_decode_min<<<1, 1, 0, s->stream>>>(out_min);
}

// ---------------------------------------------------------------------------
// lagged friction (FRICTION.h:16-660)
// ---------------------------------------------------------------------------
__device__ __forceinline__ d3 nrmz(d3 a) { return scl(a, 1.0 / sqrt(n2(a))); }

__global__ void k_fric_basis(int n, const int* kind, const int4* verts, const int* mult, const double* x, double xi2,
                             double shat, double kappa, int* fkind, int4* fverts, int* fmult, double* fw, double* fT,
                             double* flam)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = kind[i];
    const int4 iv = verts[i];
    fkind[i] = k;
    fverts[i] = iv;
    fmult[i] = mult[i];
    double w[4] = {0, 0, 0, 0};
    d3 T0 = mk(1, 0, 0), T1 = mk(0, 1, 0);
    double d2 = 0;
    if (k >= kc_EEM) {  // no friction on mollified constraints
        flam[i] = 0;
        for (int q = 0; q < 4; ++q) fw[4 * i + q] = 0;
        for (int q = 0; q < 6; ++q) fT[6 * i + q] = 0;
        return;
    }
    const d3 v0 = ld(x, iv.x), v1 = ld(x, iv.y);
    if (k == kc_EE) {
        const d3 v2 = ld(x, iv.z), v3 = ld(x, iv.w);
        const d3 e20 = v0 - v2, e01 = v1 - v0, e23 = v3 - v2;
        double g1, g2;
        ldlt2(dot(e01, e01), -dot(e23, e01), dot(e23, e23), -dot(e20, e01), dot(e20, e23), g1, g2);
        w[0] = 1 - g1; w[1] = g1; w[2] = g2 - 1; w[3] = -g2;
        T0 = nrmz(e01);
        T1 = nrmz(cross(cross(e01, e23), e01));
        d2 = ee_d2(v0, v1, v2, v3);
    } else if (k == kc_PP) {
        const d3 v01 = v1 - v0;
        const d3 xc = cross(mk(1, 0, 0), v01), yc = cross(mk(0, 1, 0), v01);
        if (n2(xc) > n2(yc)) {
            T0 = nrmz(xc);
            T1 = nrmz(cross(v01, xc));
        } else {
            T0 = nrmz(yc);
            T1 = nrmz(cross(v01, yc));
        }
        w[0] = 1; w[1] = -1;
        d2 = pp_d2(v0, v1);
    } else if (k == kc_PE) {
        const d3 v2 = ld(x, iv.z);
        const d3 e12 = v2 - v1;
        const double yita = dot(v0 - v1, e12) / n2(e12);
        w[0] = 1; w[1] = yita - 1; w[2] = -yita;
        T0 = nrmz(e12);
        T1 = nrmz(cross(e12, v0 - v1));
        d2 = pe_d2(v0, v1, v2);
    } else {
        const d3 v2 = ld(x, iv.z), v3 = ld(x, iv.w);
        const d3 r0 = v2 - v1, r1 = v3 - v1, q = v0 - v1;
        double b1, b2;
        ldlt2(dot(r0, r0), dot(r1, r0), dot(r1, r1), dot(r0, q), dot(r1, q), b1, b2);
        w[0] = 1; w[1] = -1 + b1 + b2; w[2] = -b1; w[3] = -b2;
        T0 = nrmz(r0);
        T1 = nrmz(cross(cross(r0, r1), r0));
        d2 = pt_d2(v0, v1, v2, v3);
    }
    double bv, bg, bh;
    barrier3(d2 - xi2, shat, kappa, bv, bg, bh);
    flam[i] = -bg * 2 * sqrt(d2);
    for (int q = 0; q < 4; ++q) fw[4 * i + q] = w[q];
    fT[6 * i + 0] = T0.x; fT[6 * i + 1] = T0.y; fT[6 * i + 2] = T0.z;
    fT[6 * i + 3] = T1.x; fT[6 * i + 4] = T1.y; fT[6 * i + 5] = T1.z;
}

int friction_basis(Sim* s, const double* x)
{
    s->nfric = s->ncon;
    if (s->nfric == 0) return CIPC_OK;
    const size_t n = s->nfric;
    if (s->fkind.alloc(n) || s->fmult.alloc(n) || s->fverts.alloc(n) || s->fw.alloc(4 * n) || s->fT.alloc(6 * n) ||
        s->flam.alloc(n) || s->fhess.alloc(3 * sizeof(double) * n))
        return set_error(CIPC_ERR_CUDA, "friction buffers");
    const double shat = s->prm.dHat2 + 2 * sqrt(s->prm.dHat2) * s->prm.xi;
    k_fric_basis<<<nblk(s->nfric, 128), 128, 0, s->stream>>>(s->nfric, s->ckind.p, s->cverts.p, s->cmult.p, x,
                                                             s->prm.xi * s->prm.xi, shat, barrier_kappa(s), s->fkind.p,
                                                             s->fverts.p, s->fmult.p, s->fw.p, s->fT.p, s->flam.p);
    return CIPC_OK;
}

struct FricArgs {
    int n;
    const int* kind;
    const int4* verts;
    const int* mult;
    const double *fw, *fT, *flam;
    const double *x, *xn;
    const uint8_t* dbc;
    double eh, mu;
    double* g;
    double* red;
    double* M;  // 3 per constraint: inner 2x2 (m00, m01, m11), times mu lambda mult
    double* pdiag;
};

__global__ void __launch_bounds__(128) k_friction(FricArgs a, int want_h)
{
    __shared__ double sh[128];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double E = 0;
    if (i < a.n && a.kind[i] < kc_EEM) {
        const int4 iv = a.verts[i];
        const int nv = con_nv(a.kind[i]);
        const int id[4] = {iv.x, iv.y, iv.z, iv.w};
        d3 r = mk(0, 0, 0);
        for (int q = 0; q < nv; ++q) r = r + scl(ld(a.x, id[q]) - ld(a.xn, id[q]), a.fw[4 * i + q]);
        const d3 T0 = ld(a.fT, 2 * (int64_t)i), T1 = ld(a.fT, 2 * (int64_t)i + 1);
        const double u0 = dot(T0, r), u1 = dot(T1, r);
        const double u2 = u0 * u0 + u1 * u1;
        const double ml = a.mu * a.flam[i] * a.mult[i];
        const double eh = a.eh;
        const double f0 = u2 >= eh * eh ? sqrt(u2) : u2 * (-sqrt(u2) / 3.0 + eh) / (eh * eh) + eh / 3.0;
        const double f1 = u2 >= eh * eh ? 1 / sqrt(u2) : (-sqrt(u2) + 2.0 * eh) / (eh * eh);
        E = ml * f0;
        if (a.g) {
            const d3 tu = scl(T0, u0 * f1 * ml) + scl(T1, u1 * f1 * ml);
            for (int q = 0; q < nv; ++q) {
                const double wq = a.fw[4 * i + q];
                atomicAdd(a.g + 3 * id[q], wq * tu.x);
                atomicAdd(a.g + 3 * id[q] + 1, wq * tu.y);
                atomicAdd(a.g + 3 * id[q] + 2, wq * tu.z);
            }
        }
        if (want_h) {
            double m00, m01, m11;
            const double un = sqrt(u2);
            if (u2 >= eh * eh) {
                const double sc = ml * f1 / u2;
                m00 = sc * u1 * u1;
                m01 = -sc * u1 * u0;
                m11 = sc * u0 * u0;
            } else if (un == 0) {
                m00 = ml * f1;
                m01 = 0;
                m11 = ml * f1;
            } else {
                const double f2 = -1 / (eh * eh);
                double A[2][2] = {{f2 / un * u0 * u0 + f1, f2 / un * u0 * u1}, {f2 / un * u1 * u0, f2 / un * u1 * u1 + f1}};
                jacobi_psd<double, 2>(A);
                m00 = A[0][0] * ml;
                m01 = A[0][1] * ml;
                m11 = A[1][1] * ml;
            }
            a.M[3 * i] = m00;
            a.M[3 * i + 1] = m01;
            a.M[3 * i + 2] = m11;
            // diagonal blocks w_q^2 T M T^T
            const double Tm[3][2] = {{T0.x, T1.x}, {T0.y, T1.y}, {T0.z, T1.z}};
            for (int q = 0; q < nv; ++q) {
                if (a.dbc[id[q]]) continue;
                const double w2 = a.fw[4 * i + q] * a.fw[4 * i + q];
                for (int rr = 0; rr < 3; ++rr)
                    for (int cc = 0; cc < 3; ++cc) {
                        const double v = Tm[rr][0] * (m00 * Tm[cc][0] + m01 * Tm[cc][1]) +
                                         Tm[rr][1] * (m01 * Tm[cc][0] + m11 * Tm[cc][1]);
                        atomicAdd(a.pdiag + 9 * (size_t)id[q] + 3 * rr + cc, w2 * v);
                    }
            }
        }
    } else if (i < a.n && want_h) {
        a.M[3 * i] = a.M[3 * i + 1] = a.M[3 * i + 2] = 0;
    }
    sh[threadIdx.x] = E;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = sh[0];
}

static FricArgs fric_args(Sim* s, const double* x)
{
    FricArgs a;
    a.n = s->nfric;
    a.kind = s->fkind.p;
    a.verts = s->fverts.p;
    a.mult = s->fmult.p;
    a.fw = s->fw.p;
    a.fT = s->fT.p;
    a.flam = s->flam.p;
    a.x = x;
    a.xn = s->xn.p;
    a.dbc = s->proj.p;  // Hessian rows / columns removed from the Newton system
    a.eh = sqrt(s->prm.epsv2) * s->prm.h;
    a.mu = s->prm.mu;
    a.g = nullptr;
    a.red = nullptr;
    a.M = (double*)s->fhess.p;
    a.pdiag = s->pdiag.p;
    return a;
}

int friction_energy_partials(Sim* s, const double* x, double* red)
{
    if (s->nfric == 0 || !(s->prm.mu > 0)) return 0;
    FricArgs a = fric_args(s, x);
    a.red = red;
    k_friction<<<nblk(s->nfric, 128), 128, 0, s->stream>>>(a, 0);
    return nblk(s->nfric, 128);
}

void friction_grad_hess(Sim* s, const double* x, double* g, bool want_hess)
{
    if (s->nfric == 0 || !(s->prm.mu > 0)) return;
    FricArgs a = fric_args(s, x);
    a.g = g;
    k_friction<<<nblk(s->nfric, 128), 128, 0, s->stream>>>(a, want_hess ? 1 : 0);
}

// ---------------------------------------------------------------------------
// intersection-free step size (IPC.h:1879-2244 + SPATIAL_HASH.h:477-482)
// ---------------------------------------------------------------------------
__global__ void k_abs_sum_nodes(int n, const int* bnode, const double* p, double* red)
{
    __shared__ double sh[256];
    double v = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = bnode[i];
        v += fabs(p[3 * k]) + fabs(p[3 * k + 1]) + fabs(p[3 * k + 2]);
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) red[blockIdx.x] = sh[0];
}
__global__ void k_edge_len_sum(int n, const int* bedge, const double* x, double* red)
{
    __shared__ double sh[256];
    double v = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        v += sqrt(n2(ld(x, bedge[2 * i]) - ld(x, bedge[2 * i + 1])));
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) red[blockIdx.x] = sh[0];
}

struct CcdCand {
    const int* bnode;
    const int* bedge;
    const int* btri;
    int nbn, nbe;
    const double* x;
    const double* p;
    double alpha, xi;
    const uint8_t* dbc;
    Grid G;
    uint8_t* ptype;
    int4* pidx;
    int cap;
    unsigned long long* counter;  // [0] count, [1] overflow
    // FP32 boxes over {x, x + p} of the boundary triangles and edges (outward
    // rounded) and xi rounded up: the conservative prefilter of the FP64 swept-box
    // test (box_apart)
    const float* tbox;
    const float* ebox;
    float xi_f;
};

// FP32 boxes of n items over their vertices at x and at x + p (the FP64 sums the
// swept-box test forms), rounded outward
__global__ void k_item_swept_boxes(int n, int nvi, const int* verts, const double* x, const double* p, float* box)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < nvi; ++k) {
        const int v = verts[nvi * t + k];
        const d3 a = ld(x, v), b = a + ld(p, v);
        const double av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], fmin(av[d], bv[d]));
            mx[d] = fmax(mx[d], fmax(av[d], bv[d]));
        }
    }
    for (int d = 0; d < 3; ++d) {
        box[6 * t + d] = __double2float_rd(mn[d]);
        box[6 * t + 3 + d] = __double2float_ru(mx[d]);
    }
}

__device__ __forceinline__ void add_pair(const CcdCand& c, int tp, int a, int b, int d, int e)
{
    const unsigned long long i = atomicAdd(c.counter, 1ull);
    if (i < (unsigned long long)c.cap) {
        c.ptype[i] = (uint8_t)tp;
        c.pidx[i] = make_int4(a, b, d, e);
    } else {
        c.counter[1] = 1;
    }
}

__global__ void k_ccd_pt(CcdCand c, CandList L)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kQueryChunk; base < c.nbn;
         base += nw * kQueryChunk) {
        QuerySetup mine{};
        const int sv = base + lane;
        if (lane < kQueryChunk && sv < c.nbn) {
            const int vI = c.bnode[sv];
            const d3 p = ld(c.x, vI), dp = ld(c.p, vI);
            const d3 pe = p + scl(dp, c.alpha);
            const d3 mn = vmin3(p, pe), mx = vmax3(p, pe);
            mine.ql[0] = cellc(mn.x - c.xi, c.G.inv);
            mine.ql[1] = cellc(mn.y - c.xi, c.G.inv);
            mine.ql[2] = cellc(mn.z - c.xi, c.G.inv);
            mine.qh[0] = cellc(mx.x + c.xi, c.G.inv);
            mine.qh[1] = cellc(mx.y + c.xi, c.G.inv);
            mine.qh[2] = cellc(mx.z + c.xi, c.G.inv);
            const d3 pf = p + dp;
            const float pb[6] = {__double2float_rd(fmin(p.x, pf.x)), __double2float_rd(fmin(p.y, pf.y)),
                                 __double2float_rd(fmin(p.z, pf.z)), __double2float_ru(fmax(p.x, pf.x)),
                                 __double2float_ru(fmax(p.y, pf.y)), __double2float_ru(fmax(p.z, pf.z))};
#pragma unroll
            for (int d = 0; d < 6; ++d) mine.box[d] = pb[d];
            mine.id[0] = vI;
        }
        const int nq = min(kQueryChunk, c.nbn - base);
        for (int k = 0; k < nq; ++k) {
            const QuerySetup q = bcast_setup(mine, k);
            const int vI = q.id[0];
            grid_query_warp(c.G, q.ql, q.qh, [&](int t, const float (&bx)[6]) {
                if (box_apart(q.box, bx, c.xi_f)) return;
                const int t0i = c.btri[3 * t], t1i = c.btri[3 * t + 1], t2i = c.btri[3 * t + 2];
                if (vI == t0i || vI == t1i || vI == t2i) return;
                if (c.dbc[vI] && c.dbc[t0i] && c.dbc[t1i] && c.dbc[t2i]) return;
                push_cand(L, vI, t);
            });
        }
    }
}

// point-triangle CCD candidates: the swept-box test of CCD.h:187-211 with the
// full direction, in FP64, then the pair list of the narrow phase
__global__ void __launch_bounds__(128) k_ccd_pt_eval(CcdCand c, CandList L)
{
    const int n = cand_count(L);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int2 q = L.v[k];
        const int vI = q.x, t = q.y;
        const d3 p = ld(c.x, vI), dp = ld(c.p, vI);
        const int t0i = c.btri[3 * t], t1i = c.btri[3 * t + 1], t2i = c.btri[3 * t + 2];
        const d3 t0 = ld(c.x, t0i), t1 = ld(c.x, t1i), t2 = ld(c.x, t2i);
        const d3 d0 = ld(c.p, t0i), d1 = ld(c.p, t1i), d2 = ld(c.p, t2i);
        const d3 mxp = vmax3(p, p + dp), mnp = vmin3(p, p + dp);
        const d3 mxt = vmax3(vmax3(vmax3(t0, t1), t2), vmax3(vmax3(t0 + d0, t1 + d1), t2 + d2));
        const d3 mnt = vmin3(vmin3(vmin3(t0, t1), t2), vmin3(vmin3(t0 + d0, t1 + d1), t2 + d2));
        if (any_gt3(mnp - mxt, c.xi) || any_gt3(mnt - mxp, c.xi)) continue;
        add_pair(c, kPT, vI, t0i, t1i, t2i);
    }
}

__global__ void k_ccd_ee(CcdCand c, CandList L)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kQueryChunk; base < c.nbe;
         base += nw * kQueryChunk) {
        QuerySetup mine{};
        const int e = base + lane;
        if (lane < kQueryChunk && e < c.nbe) {
            const int a0 = c.bedge[2 * e], a1 = c.bedge[2 * e + 1];
            const d3 ea0 = ld(c.x, a0), ea1 = ld(c.x, a1), da0 = ld(c.p, a0), da1 = ld(c.p, a1);
            const d3 s0 = ea0 + scl(da0, c.alpha), s1 = ea1 + scl(da1, c.alpha);
            const d3 mn = vmin3(vmin3(ea0, ea1), vmin3(s0, s1)), mx = vmax3(vmax3(ea0, ea1), vmax3(s0, s1));
            mine.ql[0] = cellc(mn.x - c.xi, c.G.inv);
            mine.ql[1] = cellc(mn.y - c.xi, c.G.inv);
            mine.ql[2] = cellc(mn.z - c.xi, c.G.inv);
            mine.qh[0] = cellc(mx.x + c.xi, c.G.inv);
            mine.qh[1] = cellc(mx.y + c.xi, c.G.inv);
            mine.qh[2] = cellc(mx.z + c.xi, c.G.inv);
#pragma unroll
            for (int d = 0; d < 6; ++d) mine.box[d] = c.ebox[6 * (size_t)e + d];
            mine.id[0] = e;
            mine.id[1] = a0;
            mine.id[2] = a1;
        }
        const int nq = min(kQueryChunk, c.nbe - base);
        for (int k = 0; k < nq; ++k) {
            const QuerySetup q = bcast_setup(mine, k);
            const int eI = q.id[0], a0 = q.id[1], a1 = q.id[2];
            grid_query_warp(c.G, q.ql, q.qh, [&](int eJ, const float (&bx)[6]) {
                if (eJ <= eI) return;
                if (box_apart(q.box, bx, c.xi_f)) return;
                const int b0 = c.bedge[2 * eJ], b1 = c.bedge[2 * eJ + 1];
                if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) return;
                if (c.dbc[a0] && c.dbc[a1] && c.dbc[b0] && c.dbc[b1]) return;
                push_cand(L, eI, eJ);
            });
        }
    }
}

// edge-edge CCD candidates: the FP64 swept-box test (CCD.h), then the pair list
__global__ void __launch_bounds__(128) k_ccd_ee_eval(CcdCand c, CandList L)
{
    const int n = cand_count(L);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int2 q = L.v[k];
        const int eI = q.x, eJ = q.y;
        const int a0 = c.bedge[2 * eI], a1 = c.bedge[2 * eI + 1];
        const int b0 = c.bedge[2 * eJ], b1 = c.bedge[2 * eJ + 1];
        const d3 ea0 = ld(c.x, a0), ea1 = ld(c.x, a1), da0 = ld(c.p, a0), da1 = ld(c.p, a1);
        const d3 eb0 = ld(c.x, b0), eb1 = ld(c.x, b1), db0 = ld(c.p, b0), db1 = ld(c.p, b1);
        const d3 mxa = vmax3(vmax3(ea0, ea1), vmax3(ea0 + da0, ea1 + da1));
        const d3 mna = vmin3(vmin3(ea0, ea1), vmin3(ea0 + da0, ea1 + da1));
        const d3 mxb = vmax3(vmax3(eb0, eb1), vmax3(eb0 + db0, eb1 + db1));
        const d3 mnb = vmin3(vmin3(eb0, eb1), vmin3(eb0 + db0, eb1 + db1));
        if (any_gt3(mna - mxb, c.xi) || any_gt3(mnb - mxa, c.xi)) continue;
        add_pair(c, kEE, a0, a1, b0, b1);
    }
}

// codimensional CCD candidates (IPC.h:2087-2165): particles (boundary nodes from
// sv_begin) against rod segments (grid items relative to e_begin) and against every
// later boundary node (grid over all boundary nodes, e_begin < 0)
__global__ void k_ccd_codim(CcdCand c, int sv_begin, int e_begin)
{
    const int sv = sv_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (sv >= c.nbn) return;
    const int vI = c.bnode[sv];
    const d3 p = ld(c.x, vI), dp = ld(c.p, vI);
    const d3 pe = p + scl(dp, c.alpha);
    const d3 mn = vmin3(p, pe), mx = vmax3(p, pe);
    int ql[3], qh[3];
    ql[0] = cellc(mn.x - c.xi, c.G.inv);
    ql[1] = cellc(mn.y - c.xi, c.G.inv);
    ql[2] = cellc(mn.z - c.xi, c.G.inv);
    qh[0] = cellc(mx.x + c.xi, c.G.inv);
    qh[1] = cellc(mx.y + c.xi, c.G.inv);
    qh[2] = cellc(mx.z + c.xi, c.G.inv);
    const d3 mxp = vmax3(p, p + dp), mnp = vmin3(p, p + dp);
    grid_query(c.G, ql, qh, [&](int it, const float (&)[6]) {
        if (e_begin >= 0) {
            const int eI = e_begin + it;
            const int e0 = c.bedge[2 * eI], e1 = c.bedge[2 * eI + 1];
            if (vI == e0 || vI == e1) return;
            if (c.dbc[vI] && c.dbc[e0] && c.dbc[e1]) return;
            const d3 x0 = ld(c.x, e0), x1 = ld(c.x, e1), d0 = ld(c.p, e0), d1 = ld(c.p, e1);
            const d3 mxe = vmax3(vmax3(x0, x1), vmax3(x0 + d0, x1 + d1));
            const d3 mne = vmin3(vmin3(x0, x1), vmin3(x0 + d0, x1 + d1));
            if (any_gt3(mnp - mxe, c.xi) || any_gt3(mne - mxp, c.xi)) return;  // CCD.h:238-257
            add_pair(c, kPE, vI, e0, e1, -1);
        } else {
            if (it <= sv) return;
            const int vJ = c.bnode[it];
            if (c.dbc[vI] && c.dbc[vJ]) return;
            const d3 q = ld(c.x, vJ), dq = ld(c.p, vJ);
            const d3 mxq = vmax3(q, q + dq), mnq = vmin3(q, q + dq);
            if (any_gt3(mnp - mxq, c.xi) || any_gt3(mnq - mxp, c.xi)) return;  // CCD.h:260-280
            add_pair(c, kPP, vI, vJ, -1, -1);
        }
    });
}

int ccd_step_size(Sim* s, const double* x, const double* p, double alpha, double* alpha_out)
{
    cudaStream_t st = s->stream;
    // span-size cap: mean |p| over boundary nodes vs mean current edge length
    double* red = s->red.p;
    k_abs_sum_nodes<<<64, 256, 0, st>>>(s->nbn, s->bnode.p, p, red);
    k_edge_len_sum<<<64, 256, 0, st>>>(s->nbe, s->bedge.p, x, red + 64);
    double hr[128];
    cudaMemcpyAsync(hr, red, sizeof(hr), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    double ps = 0, el = 0;
    for (int i = 0; i < 64; ++i) {
        ps += hr[i];
        el += hr[64 + i];
    }
    const double pSize = ps / (3.0 * s->nbn), voxel = s->nbe ? el / s->nbe : 1.0;
    const double span = alpha * pSize / voxel;
    if (span > 1) alpha /= span;
    int cap = std::max(4096, 8 * (s->nbn + s->nbe));
    int shrink = 0;
    for (int attempt = 0; attempt < 8; ++attempt) {
        const size_t need = grid_bytes(std::max(std::max(s->nbt, s->nbe), s->nbn), 32) + (size_t)cap * (16 + 1 + 8 + 1) +
                            24 * ((size_t)s->nbt + s->nbe) +
                            8 * (size_t)std::max(s->cap_cand, std::max(1 << 16, 8 * (s->nbn + s->nbe))) + (1 << 20);
        int rc = ensure_scratch(s, need);
        if (rc) return rc;
        Arena ar{s->scratch.p, s->scratch.n};
        uint8_t* ptype = ar.take<uint8_t>(cap);
        int4* pidx = ar.take<int4>(cap);
        double* toc = ar.take<double>(cap);
        uint8_t* hit = ar.take<uint8_t>(cap);
        unsigned long long* ctr = ar.take<unsigned long long>(8);
        double* amin = ar.take<double>(1);
        float* tbox = ar.take<float>(6 * (size_t)s->nbt + 6);
        float* ebox = ar.take<float>(6 * (size_t)s->nbe + 6);
        if (s->cap_cand == 0) s->cap_cand = std::max(1 << 16, 8 * (s->nbn + s->nbe));
        int2* cand = ar.take<int2>((size_t)s->cap_cand);
        if (ar.used > ar.cap) return set_error(CIPC_ERR_CUDA, "CCD scratch");
        // candidate lists (one buffer, used in turn): counts in ctr[6] (PT) and ctr[7] (EE)
        const CandList Lpt{cand, ctr + 6, s->cap_cand}, Lee{cand, ctr + 7, s->cap_cand};
        const int eval_grid = num_sms() * 8;
        if (s->nbt) k_item_swept_boxes<<<nblk(s->nbt, 256), 256, 0, st>>>(s->nbt, 3, s->btri.p, x, p, tbox);
        if (s->nbe) k_item_swept_boxes<<<nblk(s->nbe, 256), 256, 0, st>>>(s->nbe, 2, s->bedge.p, x, p, ebox);
        cudaMemsetAsync(ctr, 0, 8 * sizeof(unsigned long long), st);
        size_t mark = ar.used;
        Grid G;
        rc = build_grid(s, ar, s->nbt, 3, s->btri.p, x, p, alpha, tbox, G);
        if (rc == kSpanTooLarge) {
            if (++shrink > 60) return set_error(CIPC_ERR_NOT_CONVERGED, "CCD: swept boxes span too many cells");
            alpha *= 0.5;  // a smaller trial step: the bound stays conservative
            --attempt;
            continue;
        }
        if (rc == kNeedScratch) {
            if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
            continue;
        }
        if (rc) return rc;
        CcdCand c{s->bnode.p, s->bedge.p, s->btri.p, s->nbn, s->nbe, x, p, alpha, s->prm.xi, s->dbc.p, G,
                  ptype, pidx, cap, ctr, tbox, ebox, float_up(s->prm.xi)};
        k_ccd_pt<<<eval_grid, 256, 0, st>>>(c, Lpt);
        k_ccd_pt_eval<<<eval_grid, 128, 0, st>>>(c, Lpt);
        ar.used = mark;
        rc = build_grid(s, ar, s->nbe, 2, s->bedge.p, x, p, alpha, ebox, G);
        if (rc == kSpanTooLarge) {
            if (++shrink > 60) return set_error(CIPC_ERR_NOT_CONVERGED, "CCD: swept boxes span too many cells");
            alpha *= 0.5;  // a smaller trial step: the bound stays conservative
            --attempt;
            continue;
        }
        if (rc == kNeedScratch) {
            if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
            continue;
        }
        if (rc) return rc;
        c.G = G;
        k_ccd_ee<<<eval_grid, 256, 0, st>>>(c, Lee);
        k_ccd_ee_eval<<<eval_grid, 128, 0, st>>>(c, Lee);
        bool again = false;
        if (s->nrod_e > 0 && s->nbn > s->codim1) {
            ar.used = mark;
            const int e_begin = s->nbe - s->nrod_e;
            rc = build_grid(s, ar, s->nrod_e, 2, s->bedge.p + 2 * (size_t)e_begin, x, p, alpha, nullptr, G);
            if (rc == kSpanTooLarge) {
                if (++shrink > 60) return set_error(CIPC_ERR_NOT_CONVERGED, "CCD: swept boxes span too many cells");
                alpha *= 0.5;  // a smaller trial step: the bound stays conservative
                --attempt;
                continue;
            }
            if (rc == kNeedScratch) {
                if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
                again = true;
            } else if (rc) {
                return rc;
            } else {
                c.G = G;
                k_ccd_codim<<<nblk(s->nbn - s->codim1, 128), 128, 0, st>>>(c, s->codim1, e_begin);
            }
        }
        if (!again && s->nbn > s->codim1) {
            ar.used = mark;
            rc = build_grid(s, ar, s->nbn, 1, s->bnode.p, x, p, alpha, nullptr, G);
            if (rc == kSpanTooLarge) {
                if (++shrink > 60) return set_error(CIPC_ERR_NOT_CONVERGED, "CCD: swept boxes span too many cells");
                alpha *= 0.5;  // a smaller trial step: the bound stays conservative
                --attempt;
                continue;
            }
            if (rc == kNeedScratch) {
                if ((rc = ensure_scratch(s, s->scratch_bytes))) return rc;
                again = true;
            } else if (rc) {
                return rc;
            } else {
                c.G = G;
                k_ccd_codim<<<nblk(s->nbn - s->codim1, 128), 128, 0, st>>>(c, s->codim1, -1);
            }
        }
        if (again) continue;
        unsigned long long cc[8];
        cudaMemcpyAsync(cc, ctr, sizeof(cc), cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return set_cuda_error(e, "ccd candidates");
        const unsigned long long nc = std::max(cc[6], cc[7]);
        if (nc > (unsigned long long)s->cap_cand) {
            // a candidate list overflowed: rerun with room for all of them
            s->cap_cand = (int)std::min<unsigned long long>(nc + nc / 2 + 4096, 1ull << 30);
            continue;
        }
        if (cc[1]) {
            cap = (int)std::min<unsigned long long>(cc[0] + cc[0] / 2 + 1024, 1ull << 30);
            continue;
        }
        const int np = (int)cc[0];
        if (np == 0) {
            *alpha_out = alpha;
            return CIPC_OK;
        }
        CcdArgs a;
        a.n = np;
        a.type = ptype;
        a.idx = pidx;
        a.x = x;
        a.dx = p;
        a.eta = 0.1;
        a.th = s->prm.xi;
        a.toc_in = alpha;
        a.max_iter = s->prm.accd_max_iter;
        a.nv = s->nv;
        a.toc_out = toc;
        a.hit = hit;
        a.iters = nullptr;
        a.counter = ctr + 2;
        a.toc_min = (unsigned long long*)amin;
        cudaMemsetAsync(ctr + 2, 0, 4 * sizeof(unsigned long long), st);
        unsigned long long init_bits;
        memcpy(&init_bits, &alpha, sizeof(double));
        k_set_u64<<<1, 1, 0, st>>>((unsigned long long*)amin, init_bits);
        int grid = num_sms() * accd_exact_blocks_per_sm();
        if ((np + 255) / 256 < grid) grid = (np + 255) / 256;
        e = launch_accd_exact(a, grid, st);
        if (e != cudaSuccess) return set_cuda_error(e, "ccd");
        double res;
        unsigned long long over = 0;
        cudaMemcpyAsync(&res, amin, sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&over, ctr + 3, sizeof(over), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return set_cuda_error(e, "ccd");
        *alpha_out = res;
        // A pair at the cap has lowered the minimum to the time it safely advanced
        // to, so the bound stays conservative; with a cap the caller set
        // explicitly (cipc_step_params.accd_max_iters > 0) reaching it ends the
        // step instead (the reference's ACCD loops without bound there)
        if (over && s->prm.accd_cap_strict)
            return set_error(CIPC_ERR_ITER_CAP, "step size: %llu CCD pairs reached the cap of %lld ACCD steps", over,
                             s->prm.accd_max_iter);
        return CIPC_OK;
    }
    return set_error(CIPC_ERR_CUDA, "ccd candidates did not fit after resizing");
}

}  // namespace cipc
