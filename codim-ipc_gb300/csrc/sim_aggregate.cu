// Aggregate block Jacobi preconditioner for the Newton-system PCG.
//
// The reference solves each Newton system directly (CHOLMOD,
// Library/Math/DIRECT_SOLVER.h:13-88), so it has no preconditioner; the GPU
// solver's default is block Jacobi over 3x3 vertex blocks.  This preconditioner
// groups the vertices into aggregates of up to 32 mesh neighbours (a root vertex
// and its neighbours in the block-row pattern, built once per mesh on the host)
// and inverts, for every Newton system, each aggregate's whole diagonal block of
// the operator: the elastic rows (with the folded constraints) plus the
// intra-aggregate blocks of the constraints still applied matrix-free.  The
// solver applies z_I = (H_II)^-1 r_I inside its update phase (each block owns a
// balanced range of aggregates, agg_rounds), so it costs no extra grid-wide
// barrier; on the draped 200x200 cloth it halves the PCG iterations of block
// Jacobi.
//
// Layout in HBM: vertices by aggregate (voff / verts), the dense m x m inverse of
// aggregate a (m = 3 x its vertices, <= 96) at inv + boff[a], symmetric, so row
// and column order coincide and a warp's loads of one column are coalesced.
// Vertices with no neighbour in the rows (free particles) are packed 32 to an
// aggregate that keeps only each vertex's own 3x3 block (9 entries per vertex,
// boff[a + 1] - boff[a] = 9 x its vertices): block Jacobi for them, without the
// mostly-zero dense block; contact blocks between two of them are left out there.  The
// blocks are assembled in FP64 (atomic adds into the zeroed FP64 staging copy),
// scaled to unit diagonal and inverted by Gauss-Jordan elimination without
// pivoting (the blocks are symmetric positive definite) in shared memory, one CTA
// per aggregate, in the solver's precision.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/cipc.h"
#include "agg_rounds.h"
#include "cipc_util.h"
#include "constraint_eval.cuh"
#include "sim.h"
#include "sim_kernels.h"

namespace cipc {

namespace {

constexpr int kAggMax = 32;  // vertices per aggregate (one warp lane each)
constexpr int kInvThreads = 128;

struct AggState {
    int nv = 0, nagg = 0, max_m = 0;
    long long entries = 0;
    DBuf<int> voff, verts, vagg, vloc, ellmap, flag;
    DBuf<long long> boff;
    std::vector<int> h_voff;        // host copies for the solver's rounds
    std::vector<long long> h_boff;
    int rk_grid = 0, rk_rows = 0, rk_max = 0, rk_loads = 0;  // limits the rounds were built for
    DBuf<int> bround, rstart;
    DBuf<double> A;   // assembled blocks
    DBuf<char> inv;   // inverses (float or double)
    int* flag_host = nullptr;
    ~AggState()
    {
        if (flag_host) cudaFreeHost(flag_host);
        for (DBuf<int>* b : {&voff, &verts, &vagg, &vloc, &ellmap, &flag, &bround, &rstart}) b->release();
        boff.release();
        A.release();
        inv.release();
    }
};

inline int nblk(long long n, int bs) { return n > 0 ? (int)((n + bs - 1) / bs) : 1; }

// Greedy aggregation of the vertex graph given by the block-row pattern (column
// col[k * nv + i] of row i; padding entries repeat i): (1) every vertex whose
// neighbours are all unassigned becomes a root with its neighbours (up to
// kAggMax); (2) a remaining vertex joins the aggregate most of its neighbours
// belong to while it has room, else starts a new one; (3) vertices with no
// neighbours are packed in index order, kAggMax to an aggregate.
void aggregate(int nv, int K, const std::vector<int>& col, std::vector<int>& agg, int& nagg,
               std::vector<uint8_t>& packed)
{
    agg.assign(nv, -1);
    std::vector<int> size;
    auto nbr = [&](int i, std::vector<int>& out) {
        out.clear();
        for (int k = 0; k < K; ++k) {
            const int j = col[(size_t)k * nv + i];
            if (j != i && j >= 0 && j < nv && std::find(out.begin(), out.end(), j) == out.end()) out.push_back(j);
        }
    };
    std::vector<int> nb;
    nagg = 0;
    for (int i = 0; i < nv; ++i) {
        if (agg[i] >= 0) continue;
        nbr(i, nb);
        if (nb.empty()) continue;
        bool free_all = true;
        for (int j : nb) free_all = free_all && agg[j] < 0;
        if (!free_all) continue;
        agg[i] = nagg;
        int n = 1;
        for (int j : nb)
            if (n < kAggMax) {
                agg[j] = nagg;
                ++n;
            }
        size.push_back(n);
        ++nagg;
    }
    for (int i = 0; i < nv; ++i) {
        if (agg[i] >= 0) continue;
        nbr(i, nb);
        if (nb.empty()) continue;
        int best = -1, bc = 0;
        for (int j : nb) {
            const int a = agg[j];
            if (a < 0 || size[a] >= kAggMax) continue;
            int c = 0;
            for (int q : nb) c += agg[q] == a;
            if (c > bc) {
                bc = c;
                best = a;
            }
        }
        if (best < 0) {
            best = nagg++;
            size.push_back(0);
        }
        agg[i] = best;
        ++size[best];
    }
    packed.assign(nagg, 0);
    int open = -1;
    for (int i = 0; i < nv; ++i) {
        if (agg[i] >= 0) continue;
        if (open < 0 || size[open] >= kAggMax) {
            open = nagg++;
            size.push_back(0);
            packed.push_back(1);
        }
        agg[i] = open;
        ++size[open];
    }
}

int build_state(Sim* s, AggState* st)
{
    const int nv = s->nv, K = s->ell_k;
    std::vector<int> col((size_t)K * nv);
    cudaError_t e = cudaMemcpy(col.data(), s->col.p, sizeof(int) * col.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_cuda_error(e, "aggregate set-up");
    std::vector<int> agg;
    std::vector<uint8_t> packed;
    int nagg = 0;
    aggregate(nv, K, col, agg, nagg, packed);
    std::vector<int> voff(nagg + 1, 0), verts(nv), vloc(nv);
    for (int i = 0; i < nv; ++i) ++voff[agg[i] + 1];
    for (int a = 0; a < nagg; ++a) voff[a + 1] += voff[a];
    {
        std::vector<int> cur(voff.begin(), voff.end() - 1);
        for (int i = 0; i < nv; ++i) {
            vloc[i] = cur[agg[i]] - voff[agg[i]];
            verts[cur[agg[i]]++] = i;
        }
    }
    std::vector<long long> boff(nagg + 1, 0);
    int max_m = 0;
    for (int a = 0; a < nagg; ++a) {
        const int m = 3 * (voff[a + 1] - voff[a]);
        max_m = std::max(max_m, m);
        boff[a + 1] = boff[a] + (packed[a] ? 3LL * m : (long long)m * m);
    }
    if (boff[nagg] >= (1ll << 31)) return set_error(CIPC_ERR_INVALID_ARG, "aggregate blocks exceed 2^31 entries");
    std::vector<int> ellmap((size_t)K * nv, -1);
    for (size_t q = 0; q < ellmap.size(); ++q) {
        const int i = (int)(q % nv), j = col[q];
        // (padding entries repeat the row's own column with zero blocks: they map
        // onto the diagonal block and add nothing)
        if (j < 0 || j >= nv || agg[i] != agg[j]) continue;
        const int a = agg[i], m = 3 * (voff[a + 1] - voff[a]);
        if (packed[a]) {
            if (j == i) ellmap[q] = (int)(boff[a] + 9LL * vloc[i]);
            continue;
        }
        ellmap[q] = (int)(boff[a] + (long long)(3 * vloc[i]) * m + 3 * vloc[j]);
    }
    st->nv = nv;
    st->nagg = nagg;
    st->max_m = max_m;
    st->h_voff = voff;
    st->h_boff = boff;
    st->entries = boff[nagg];
    if (st->voff.alloc(nagg + 1) || st->verts.alloc(nv) || st->vagg.alloc(nv) || st->vloc.alloc(nv) ||
        st->ellmap.alloc(ellmap.size()) || st->boff.alloc(nagg + 1) || st->flag.alloc(1) ||
        st->A.alloc((size_t)st->entries) || cudaMallocHost((void**)&st->flag_host, sizeof(int)) != cudaSuccess)
        return set_error(CIPC_ERR_CUDA, "aggregate buffers");
    e = cudaMemcpy(st->voff.p, voff.data(), sizeof(int) * voff.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(st->verts.p, verts.data(), sizeof(int) * nv, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(st->vagg.p, agg.data(), sizeof(int) * nv, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(st->vloc.p, vloc.data(), sizeof(int) * nv, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(st->ellmap.p, ellmap.data(), sizeof(int) * ellmap.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(st->boff.p, boff.data(), sizeof(long long) * boff.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return set_cuda_error(e, "aggregate upload");
    return CIPC_OK;
}

// stored block layout of aggregate a: dense m x m (rows m apart), or for a pack of
// isolated vertices their 3x3 blocks one after another (rows 3 apart)
__device__ __forceinline__ bool agg_packed(const int* voff, const long long* boff, int a)
{
    const int sv = voff[a + 1] - voff[a];
    return sv > 1 && boff[a + 1] - boff[a] == 9LL * sv;
}

// elastic rows: ELL entry q = k nv + i lands at A[ellmap[q]] (rows of the
// aggregate block are m apart, 3 in a pack of isolated vertices)
template <typename VT>
__global__ void k_agg_ell(long long n, int nv, const int* __restrict__ ellmap, const int* __restrict__ vagg,
                          const int* __restrict__ voff, const long long* __restrict__ boff,
                          const VT* __restrict__ val, double* A)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int o = ellmap[q];
    if (o < 0) return;
    const int i = (int)(q % nv), a = vagg[i];
    const int m = agg_packed(voff, boff, a) ? 3 : 3 * (voff[a + 1] - voff[a]);
    const VT* B = val + 9 * q;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const double v = (double)B[3 * r + t];
            if (v != 0) atomicAdd(A + o + (size_t)r * m + t, v);
        }
}

struct AggMaps {
    const int* vagg;
    const int* vloc;
    const int* voff;
    const long long* boff;
    const uint8_t* proj;
};

// intra-aggregate blocks (p, q) of one constraint with vertices id (free vertices
// only); blk(p, q, r, t) gives entry (3p + r, 3q + t) of the constraint matrix
template <typename F>
__device__ __forceinline__ void agg_add_blocks(const AggMaps& M, const int (&id)[4], int cnv, double* A, const F& blk)
{
    for (int p = 0; p < cnv; ++p) {
        if (M.proj[id[p]]) continue;
        const int a = M.vagg[id[p]];
        const bool pk = agg_packed(M.voff, M.boff, a);
        const int m = pk ? 3 : 3 * (M.voff[a + 1] - M.voff[a]);
        for (int q = 0; q < cnv; ++q) {
            if (M.proj[id[q]] || M.vagg[id[q]] != a) continue;
            if (pk && id[q] != id[p]) continue;  // a pack keeps each vertex's own block only
            double* D = pk ? A + M.boff[a] + 9 * (size_t)M.vloc[id[p]]
                           : A + M.boff[a] + (size_t)(3 * M.vloc[id[p]]) * m + 3 * M.vloc[id[q]];
            for (int r = 0; r < 3; ++r)
                for (int t = 0; t < 3; ++t) {
                    const double v = blk(p, q, r, t);
                    if (v != 0) atomicAdd(D + (size_t)r * m + t, v);
                }
        }
    }
}

template <typename VT>
__global__ void k_agg_con(int n, const int* __restrict__ list, const int* __restrict__ nlist,
                          const int* __restrict__ kind, const int4* __restrict__ verts, const VT* __restrict__ hess,
                          size_t hs, AggMaps M, double* A)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || (list && c >= *nlist)) return;
    if (list) c = list[c];
    const int cnv = con_nv(kind[c]), Mm = 3 * cnv;
    const int4 iv = verts[c];
    const int id[4] = {iv.x, iv.y, iv.z, iv.w};
    agg_add_blocks(M, id, cnv, A, [&](int p, int q, int r, int t) {
        const int i = min(3 * p + r, 3 * q + t), j = max(3 * p + r, 3 * q + t);
        return (double)hess[(size_t)(i * Mm - (i * (i - 1)) / 2 + (j - i)) * hs + c];
    });
}

__global__ void k_agg_fric(int n, const int* __restrict__ list, const int* __restrict__ nlist,
                           const int* __restrict__ kind, const int4* __restrict__ verts, const double* __restrict__ fw,
                           const double* __restrict__ fT, const double* __restrict__ fM, AggMaps M, double* A)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || (list && c >= *nlist)) return;
    if (list) c = list[c];
    if (kind[c] >= kc_EEM) return;
    const int cnv = con_nv(kind[c]);
    const int4 iv = verts[c];
    const int id[4] = {iv.x, iv.y, iv.z, iv.w};
    const double* T = fT + 6 * (size_t)c;
    const double m00 = fM[3 * c], m01 = fM[3 * c + 1], m11 = fM[3 * c + 2];
    double S[3][3];
    for (int r = 0; r < 3; ++r)
        for (int t = 0; t < 3; ++t)
            S[r][t] = T[r] * (m00 * T[t] + m01 * T[3 + t]) + T[3 + r] * (m01 * T[t] + m11 * T[3 + t]);
    const double* w = fw + 4 * (size_t)c;
    agg_add_blocks(M, id, cnv, A, [&](int p, int q, int r, int t) { return w[p] * w[q] * S[r][t]; });
}

// Gauss-Jordan inversion in place (no pivoting: the block is symmetric positive
// definite), in GT, one CTA per aggregate; a pivot that is not positive and
// finite sets *flag
template <typename GT, typename PT>
__global__ void __launch_bounds__(kInvThreads) k_agg_invert(const int* __restrict__ voff,
                                                            const long long* __restrict__ boff,
                                                            const double* __restrict__ A, PT* inv, int* flag)
{
    extern __shared__ unsigned char smem_raw[];
    GT* S = reinterpret_cast<GT*>(smem_raw);
    const int a = blockIdx.x;
    const int m = 3 * (voff[a + 1] - voff[a]);
    const double* Ab = A + boff[a];
    if (agg_packed(voff, boff, a)) {
        // pack of isolated vertices: each vertex's 3x3 block (FP64 cofactors)
        PT* out = inv + boff[a];
        for (int v = threadIdx.x; v < m / 3; v += blockDim.x) {
            const double* B = Ab + 9 * v;
            const double c00 = B[4] * B[8] - B[5] * B[7], c01 = B[5] * B[6] - B[3] * B[8],
                         c02 = B[3] * B[7] - B[4] * B[6];
            const double det = B[0] * c00 + B[1] * c01 + B[2] * c02;
            if (!(B[0] > 0) || !(det > 0) || !(det < INFINITY)) {
                atomicExch(flag, 1);
                continue;
            }
            const double id = 1.0 / det;
            const double I[9] = {c00 * id, (B[2] * B[7] - B[1] * B[8]) * id, (B[1] * B[5] - B[2] * B[4]) * id,
                                 c01 * id, (B[0] * B[8] - B[2] * B[6]) * id, (B[2] * B[3] - B[0] * B[5]) * id,
                                 c02 * id, (B[1] * B[6] - B[0] * B[7]) * id, (B[0] * B[4] - B[1] * B[3]) * id};
            for (int r = 0; r < 3; ++r)
                for (int t = 0; t < 3; ++t) out[9 * v + 3 * r + t] = (PT)(0.5 * (I[3 * r + t] + I[3 * t + r]));
        }
        return;
    }
    GT* fcol = S + (size_t)m * m;
    __shared__ double dsc[3 * kAggMax];
    __shared__ GT piv;
    __shared__ int bad;
    // rows to warps, columns to lanes: no index division in the O(m^3) loops (each
    // entry is still updated by one thread with the same arithmetic)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // symmetric diagonal scaling (unit diagonal) before the elimination: the
    // contact blocks make the rows' scales differ by orders of magnitude
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const double d = Ab[(size_t)i * m + i];
        dsc[i] = d > 0 ? 1.0 / sqrt(d) : 1.0;
    }
    __syncthreads();
    for (int i = wid; i < m; i += nw)
        for (int j = lane; j < m; j += 32) S[i * m + j] = (GT)(Ab[(size_t)i * m + j] * dsc[i] * dsc[j]);
    if (threadIdx.x == 0) bad = 0;
    for (int k = 0; k < m; ++k) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const GT p = S[k * m + k];
            if (!(p > GT(0)) || !(p < GT(INFINITY))) bad = 1;
            piv = (p > GT(0) && p < GT(INFINITY)) ? GT(1) / p : GT(1);
        }
        for (int i = threadIdx.x; i < m; i += blockDim.x) fcol[i] = S[i * m + k];
        __syncthreads();
        const GT p = piv;
        for (int j = threadIdx.x; j < m; j += blockDim.x) S[k * m + j] = (j == k ? GT(1) : S[k * m + j]) * p;
        __syncthreads();
        for (int i = wid; i < m; i += nw) {
            if (i == k) continue;
            const GT f = fcol[i];
            for (int j = lane; j < m; j += 32) S[i * m + j] = (j == k ? GT(0) : S[i * m + j]) - f * S[k * m + j];
        }
    }
    __syncthreads();
    PT* out = inv + boff[a];
    // symmetrise (the rounding of the elimination is not symmetric)
    for (int i = wid; i < m; i += nw)
        for (int j = lane; j < m; j += 32)
            out[i * m + j] = (PT)(0.5 * ((double)S[i * m + j] + (double)S[j * m + i]) * dsc[i] * dsc[j]);
    if (threadIdx.x == 0 && bad) atomicExch(flag, 1);
}

template <typename VT>
int setup_impl(Sim* s, AggState* st)
{
    const bool f32 = sizeof(VT) == 4;
    const size_t pbytes = (size_t)st->entries * sizeof(VT);
    if (st->inv.n < pbytes) {
        cudaStreamSynchronize(s->stream);
        if (st->inv.alloc(pbytes) != cudaSuccess) return set_error(CIPC_ERR_CUDA, "aggregate inverses");
    }
    cudaStream_t str = s->stream;
    cudaError_t e = cudaMemsetAsync(st->A.p, 0, sizeof(double) * (size_t)st->entries, str);
    if (e == cudaSuccess) e = cudaMemsetAsync(st->flag.p, 0, sizeof(int), str);
    if (e != cudaSuccess) return set_cuda_error(e, "aggregate set-up");
    const VT* val = reinterpret_cast<const VT*>(s->folded ? s->hval_op.p : s->hval.p);
    const long long ne = (long long)s->ell_k * s->nv;
    k_agg_ell<VT><<<nblk(ne, 256), 256, 0, str>>>(ne, s->nv, st->ellmap.p, st->vagg.p, st->voff.p, st->boff.p, val,
                                                  st->A.p);
    AggMaps M{st->vagg.p, st->vloc.p, st->voff.p, st->boff.p, s->proj.p};
    const int ncon = s->prm.withCollision ? s->ncon : 0;
    const int nfric = (s->prm.withCollision && s->prm.mu > 0) ? s->nfric : 0;
    if (ncon > 0)
        k_agg_con<VT><<<nblk(ncon, 128), 128, 0, str>>>(ncon, s->folded ? s->crest.p : nullptr, s->fold_cnt.p,
                                                        s->ckind.p, s->cverts.p,
                                                        reinterpret_cast<const VT*>(s->chess.p), (size_t)s->cap_con, M,
                                                        st->A.p);
    if (nfric > 0)
        k_agg_fric<<<nblk(nfric, 128), 128, 0, str>>>(nfric, s->folded ? s->frest.p : nullptr, s->fold_cnt.p + 1,
                                                      s->fkind.p, s->fverts.p, s->fw.p, s->fT.p,
                                                      reinterpret_cast<const double*>(s->fhess.p), M, st->A.p);
    const size_t smem = ((size_t)st->max_m * st->max_m + st->max_m) * sizeof(VT);
    if (f32) {
        auto k = k_agg_invert<float, float>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            k<<<st->nagg, kInvThreads, smem, str>>>(st->voff.p, st->boff.p, st->A.p, (float*)st->inv.p, st->flag.p);
    } else {
        auto k = k_agg_invert<double, double>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            k<<<st->nagg, kInvThreads, smem, str>>>(st->voff.p, st->boff.p, st->A.p, (double*)st->inv.p, st->flag.p);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(st->flag_host, st->flag.p, sizeof(int), cudaMemcpyDeviceToHost, str);
    if (e == cudaSuccess) e = cudaStreamSynchronize(str);
    if (e != cudaSuccess) return set_cuda_error(e, "aggregate inverses");
    if (*st->flag_host) return set_error(CIPC_ERR_NOT_CONVERGED, "aggregate block not positive definite");
    return CIPC_OK;
}

}  // namespace

int agg_setup(Sim* s)
{
    s->agg_ready = false;
    AggState* st = static_cast<AggState*>(s->agg);
    if (!st || st->nv != s->nv) {
        delete st;
        st = new AggState();
        s->agg = st;
        const int rc = build_state(s, st);
        if (rc) {
            delete st;
            s->agg = nullptr;
            return rc;
        }
    }
    const int rc = s->prm.precision == 1 ? setup_impl<float>(s, st) : setup_impl<double>(s, st);
    if (rc == CIPC_OK) s->agg_ready = true;
    return rc;
}

AggView agg_view(const Sim* s)
{
    const AggState* st = static_cast<const AggState*>(s->agg);
    if (!st || !s->agg_ready) return AggView{0, nullptr, nullptr, nullptr, nullptr};
    return AggView{st->nagg, st->voff.p, st->verts.p, st->boff.p, st->inv.p};
}

int agg_rounds(Sim* s, int grid, int rows, int maxagg, int loads, const int** bround, const int** rstart)
{
    AggState* st = static_cast<AggState*>(s->agg);
    if (!st || grid < 1 || rows < st->max_m || maxagg < 1 || loads < 3)
        return set_error(CIPC_ERR_INVALID_ARG, "aggregate rounds: no aggregates or limits below the largest block");
    if (st->rk_grid != grid || st->rk_rows != rows || st->rk_max != maxagg || st->rk_loads != loads) {
        std::vector<int> br, rs;
        agg_partition(st->h_voff, st->h_boff, grid, rows, maxagg, loads, br, rs);
        cudaStreamSynchronize(s->stream);
        if (st->bround.alloc(br.size()) != cudaSuccess || st->rstart.alloc(rs.size()) != cudaSuccess)
            return set_error(CIPC_ERR_CUDA, "aggregate rounds");
        cudaError_t e = cudaMemcpy(st->bround.p, br.data(), sizeof(int) * br.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(st->rstart.p, rs.data(), sizeof(int) * rs.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return set_cuda_error(e, "aggregate rounds upload");
        st->rk_grid = grid;
        st->rk_rows = rows;
        st->rk_max = maxagg;
        st->rk_loads = loads;
    }
    *bround = st->bround.p;
    *rstart = st->rstart.p;
    return CIPC_OK;
}

void agg_release(Sim* s)
{
    delete static_cast<AggState*>(s->agg);
    s->agg = nullptr;
    s->agg_ready = false;
}

}  // namespace cipc
