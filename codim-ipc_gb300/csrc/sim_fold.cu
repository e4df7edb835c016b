// Folding of contact and friction constraints into the 3x3 block rows of the
// Newton operator.  The reference assembles every element, barrier and friction
// triplet into one sparse matrix before its direct solve
// (Library/Math/CSR_MATRIX.h:49-54, Library/FEM/Shell/IMPLICIT_EULER.h:500-540).
// Here the elastic rows have a fixed block pattern (one ELL slot per mesh
// neighbour, built once per mesh); a constraint whose free-vertex pairs all have a
// slot in that pattern (a cloth point against an obstacle triangle, a cloth edge
// against an obstacle edge, contacts between neighbouring cloth vertices) is added
// into a copy of the rows, and only the rest (contacts between distant parts of
// the mesh) stay in the matrix-free constraint lists the solver applies.  The
// copy leaves the assembled rows untouched for the preconditioner, the learned
// correction's features and the captured training systems.
#include <cuda_runtime.h>

#include <cstdlib>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "constraint_eval.cuh"
#include "sim.h"
#include "sim_kernels.h"

namespace cipc {

namespace {

inline int nblk(long long n, int bs) { return n > 0 ? (int)((n + bs - 1) / bs) : 1; }

// ELL slot k of row a holding column b, or -1
__device__ __forceinline__ int find_slot(const int* __restrict__ col, int nv, int K, int a, int b)
{
    for (int k = 0; k < K; ++k)
        if (__ldg(col + (size_t)k * nv + a) == b) return k;
    return -1;
}

// Slots of the constraint's free-vertex pairs (slot[p][q] = -2 where a vertex is
// projected out); false if some pair has no block in the rows
__device__ __forceinline__ bool pair_slots(const int (&id)[4], int cnv, const uint8_t* __restrict__ proj,
                                           const int* __restrict__ col, int nv, int K, int (&slot)[4][4])
{
    bool fr[4];
    for (int p = 0; p < 4; ++p) fr[p] = p < cnv && !proj[id[p]];
    for (int p = 0; p < cnv; ++p)
        for (int q = 0; q < cnv; ++q) {
            if (!fr[p] || !fr[q]) {
                slot[p][q] = -2;
                continue;
            }
            const int k = find_slot(col, nv, K, id[p], id[q]);
            if (k < 0) return false;
            slot[p][q] = k;
        }
    return true;
}

template <typename VT>
__global__ void __launch_bounds__(128) k_fold_con(int n, const int* __restrict__ kind, const int4* __restrict__ verts,
                                                  const uint8_t* __restrict__ proj, const int* __restrict__ col, int nv,
                                                  int K, const VT* __restrict__ hess, size_t hs, VT* val, int* rest,
                                                  int* nrest)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int cnv = con_nv(kind[c]), M = 3 * cnv;
    const int4 iv = verts[c];
    const int id[4] = {iv.x, iv.y, iv.z, iv.w};
    int slot[4][4];
    if (!pair_slots(id, cnv, proj, col, nv, K, slot)) {
        rest[atomicAdd(nrest, 1)] = c;
        return;
    }
    // block (p, q) of the packed upper triangle (row by row, entry h at hess[h * hs])
    for (int p = 0; p < cnv; ++p)
        for (int q = 0; q < cnv; ++q) {
            if (slot[p][q] < 0) continue;
            VT* B = val + 9 * ((size_t)slot[p][q] * nv + id[p]);
            for (int r = 0; r < 3; ++r)
                for (int t = 0; t < 3; ++t) {
                    const int i = min(3 * p + r, 3 * q + t), j = max(3 * p + r, 3 * q + t);
                    const VT h = hess[(size_t)(i * M - (i * (i - 1)) / 2 + (j - i)) * hs + c];
                    if (h != VT(0)) atomicAdd(B + 3 * r + t, h);
                }
        }
}

// friction constraint c: blocks w_p w_q T^T M T (T the 2x3 tangent basis, M the
// 2x2 inner matrix), over non-projected vertices
template <typename VT>
__global__ void __launch_bounds__(128) k_fold_fric(int n, const int* __restrict__ kind, const int4* __restrict__ verts,
                                                   const double* __restrict__ fw, const double* __restrict__ fT,
                                                   const double* __restrict__ fM, const uint8_t* __restrict__ proj,
                                                   const int* __restrict__ col, int nv, int K, VT* val, int* rest,
                                                   int* nrest)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || kind[c] >= kc_EEM) return;  // no friction on mollified edge-edge constraints
    const int cnv = con_nv(kind[c]);
    const int4 iv = verts[c];
    const int id[4] = {iv.x, iv.y, iv.z, iv.w};
    int slot[4][4];
    if (!pair_slots(id, cnv, proj, col, nv, K, slot)) {
        rest[atomicAdd(nrest, 1)] = c;
        return;
    }
    const double* T = fT + 6 * (size_t)c;
    const double m00 = fM[3 * c], m01 = fM[3 * c + 1], m11 = fM[3 * c + 2];
    // S = T^T M T (3x3)
    double S[3][3];
    for (int r = 0; r < 3; ++r)
        for (int t = 0; t < 3; ++t)
            S[r][t] = T[r] * (m00 * T[t] + m01 * T[3 + t]) + T[3 + r] * (m01 * T[t] + m11 * T[3 + t]);
    for (int p = 0; p < cnv; ++p)
        for (int q = 0; q < cnv; ++q) {
            if (slot[p][q] < 0) continue;
            const double w = fw[4 * c + p] * fw[4 * c + q];
            if (w == 0) continue;
            VT* B = val + 9 * ((size_t)slot[p][q] * nv + id[p]);
            for (int r = 0; r < 3; ++r)
                for (int t = 0; t < 3; ++t) atomicAdd(B + 3 * r + t, (VT)(w * S[r][t]));
        }
}

template <typename VT>
int fold_impl(Sim* s, int ncon, int nfric)
{
    const size_t bytes = 9 * sizeof(VT) * (size_t)s->nnzb;
    if (s->hval_op.n < bytes || s->crest.n < (size_t)ncon || s->frest.n < (size_t)nfric || s->fold_cnt.n < 2) {
        cudaStreamSynchronize(s->stream);
        if (s->hval_op.alloc(bytes) != cudaSuccess || s->crest.alloc(ncon) != cudaSuccess ||
            s->frest.alloc(nfric) != cudaSuccess || s->fold_cnt.alloc(2) != cudaSuccess)
            return set_error(CIPC_ERR_CUDA, "folded operator allocation");
    }
    cudaError_t e = cudaMemcpyAsync(s->hval_op.p, s->hval.p, bytes, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->fold_cnt.p, 0, 2 * sizeof(int), s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "folded operator copy");
    VT* val = reinterpret_cast<VT*>(s->hval_op.p);
    if (ncon > 0)
        k_fold_con<VT><<<nblk(ncon, 128), 128, 0, s->stream>>>(ncon, s->ckind.p, s->cverts.p, s->proj.p, s->col.p,
                                                               s->nv, s->ell_k, reinterpret_cast<const VT*>(s->chess.p),
                                                               (size_t)s->cap_con, val, s->crest.p, s->fold_cnt.p);
    if (nfric > 0)
        k_fold_fric<VT><<<nblk(nfric, 128), 128, 0, s->stream>>>(
            nfric, s->fkind.p, s->fverts.p, s->fw.p, s->fT.p, reinterpret_cast<const double*>(s->fhess.p), s->proj.p,
            s->col.p, s->nv, s->ell_k, val, s->frest.p, s->fold_cnt.p + 1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "constraint folding");
    s->folded = true;
    return CIPC_OK;
}

}  // namespace

bool fold_enabled()
{
    static const bool off = std::getenv("CIPC_NO_FOLD") != nullptr;
    return !off;
}

int fold_constraints(Sim* s)
{
    s->folded = false;
    if (!fold_enabled()) return CIPC_OK;
    const int ncon = s->prm.withCollision ? s->ncon : 0;
    const int nfric = (s->prm.withCollision && s->prm.mu > 0) ? s->nfric : 0;
    return s->prm.precision == 1 ? fold_impl<float>(s, ncon, nfric) : fold_impl<double>(s, ncon, nfric);
}

}  // namespace cipc
