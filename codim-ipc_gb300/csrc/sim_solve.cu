// Newton-system solve: preconditioned conjugate gradients on the assembled
// Hessian (replaces the reference's per-iteration CHOLMOD factorization,
// Library/Math/DIRECT_SOLVER.h:13-88).
//
// Operator: y = H x with H = (elastic + mass, 3x3 block CSR) + sum over contact
// constraints of their stored PSD blocks + sum over friction constraints of
// w_a w_b T M T^T (applied matrix-free from the 2x2 inner matrix); constraints
// folded into a copy of the block rows (sim_fold.cu) are applied through it.  Dirichlet
// rows/columns were removed at assembly (identity diagonal), so Dirichlet
// entries of every PCG vector stay zero.
//
// Precision modes:
//   FP64:  matrix, vectors and reductions in FP64 (block-Jacobi PCG).
//   mixed: matrix values FP32; inner PCG in FP32 vectors with FP32 block
//          partials; outer iterative refinement in FP64 (r = b - H x with FP64
//          vectors), so the Newton increment meets the same FP64 residual bound.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "constraint_eval.cuh"
#include "sim.h"
#include "sim_kernels.h"
#include "sim_pcg.h"
#include "learned.h"

namespace cipc {

static inline int nblk(long long n, int bs) { return n > 0 ? (int)((n + bs - 1) / bs) : 1; }

template <typename VT, typename XT>
__global__ void __launch_bounds__(256) k_bsr_spmv(int nv, const int* __restrict__ rowlen, const int* __restrict__ col,
                                                  const VT* __restrict__ val, const XT* __restrict__ x,
                                                  XT* __restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    XT a0 = 0, a1 = 0, a2 = 0;
    const int L = rowlen[i];  // the row's real blocks (the rest is zero padding)
    for (int k = 0; k < L; ++k) {
        const size_t e = (size_t)k * nv + i;
        const int j = col[e];
        const VT* B = val + 9 * e;
        const XT x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
        a0 += (XT)B[0] * x0 + (XT)B[1] * x1 + (XT)B[2] * x2;
        a1 += (XT)B[3] * x0 + (XT)B[4] * x1 + (XT)B[5] * x2;
        a2 += (XT)B[6] * x0 + (XT)B[7] * x1 + (XT)B[8] * x2;
    }
    y[3 * i] = a0;
    y[3 * i + 1] = a1;
    y[3 * i + 2] = a2;
}

// contact blocks: packed upper triangle (row by row) of the (3nv x 3nv) constraint
// Hessian, entry h of constraint c at hess[h * hs + c]
template <typename VT, typename XT>
__global__ void __launch_bounds__(128) k_con_spmv(int n, const int* __restrict__ list, const int* __restrict__ nlist,
                                                  const int* __restrict__ kind, const int4* __restrict__ verts,
                                                  const VT* __restrict__ hess, size_t hs, const XT* __restrict__ x,
                                                  XT* __restrict__ y)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || (list && c >= *nlist)) return;
    if (list) c = list[c];
    const int nv = con_nv(kind[c]);
    const int m = 3 * nv;
    const int4 iv = verts[c];
    const int id[4] = {iv.x, iv.y, iv.z, iv.w};
    XT xs[12], ys[12];
    for (int q = 0; q < nv; ++q)
        for (int d = 0; d < 3; ++d) {
            xs[3 * q + d] = x[3 * id[q] + d];
            ys[3 * q + d] = 0;
        }
    const VT* H = hess + c;
    size_t w = 0;
    for (int p = 0; p < m; ++p) {
        ys[p] += (XT)H[w * hs] * xs[p];
        ++w;
        for (int q = p + 1; q < m; ++q, ++w) {
            const XT h = (XT)H[w * hs];
            ys[p] += h * xs[q];
            ys[q] += h * xs[p];
        }
    }
    for (int q = 0; q < nv; ++q)
        for (int d = 0; d < 3; ++d)
            if (ys[3 * q + d] != XT(0)) atomicAdd(y + 3 * id[q] + d, ys[3 * q + d]);
}

// friction: y_a += w_a T M T^T sum_b w_b x_b
template <typename XT>
__global__ void k_fric_spmv(int n, const int* __restrict__ list, const int* __restrict__ nlist,
                            const int* __restrict__ kind, const int4* __restrict__ verts,
                            const double* __restrict__ fw, const double* __restrict__ fT, const double* __restrict__ M,
                            const uint8_t* __restrict__ dbc, const XT* __restrict__ x, XT* __restrict__ y)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || (list && c >= *nlist)) return;
    if (list) c = list[c];
    if (kind[c] >= kc_EEM) return;
    const int nv = con_nv(kind[c]);
    const int4 iv = verts[c];
    const int id[4] = {iv.x, iv.y, iv.z, iv.w};
    double s0 = 0, s1 = 0, s2 = 0;
    for (int q = 0; q < nv; ++q) {
        if (dbc[id[q]]) continue;
        const double w = fw[4 * c + q];
        s0 += w * (double)x[3 * id[q]];
        s1 += w * (double)x[3 * id[q] + 1];
        s2 += w * (double)x[3 * id[q] + 2];
    }
    const double* T = fT + 6 * (size_t)c;
    const double t0 = T[0] * s0 + T[1] * s1 + T[2] * s2, t1 = T[3] * s0 + T[4] * s1 + T[5] * s2;
    const double m00 = M[3 * c], m01 = M[3 * c + 1], m11 = M[3 * c + 2];
    const double u0 = m00 * t0 + m01 * t1, u1 = m01 * t0 + m11 * t1;
    const double o0 = T[0] * u0 + T[3] * u1, o1 = T[1] * u0 + T[4] * u1, o2 = T[2] * u0 + T[5] * u1;
    for (int q = 0; q < nv; ++q) {
        if (dbc[id[q]]) continue;
        const double w = fw[4 * c + q];
        atomicAdd(y + 3 * id[q], (XT)(w * o0));
        atomicAdd(y + 3 * id[q] + 1, (XT)(w * o1));
        atomicAdd(y + 3 * id[q] + 2, (XT)(w * o2));
    }
}

// block-Jacobi: pdiag (already holding contact / friction diagonal blocks) += BSR
// diagonal blocks, then inverted (3x3, FP64)
template <typename VT, typename PT>
__global__ void k_precond(int nv, const int* diag, const VT* val, const double* pdiag, PT* pinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    double A[9];
    const VT* B = val + 9 * (size_t)diag[i];
    for (int k = 0; k < 9; ++k) A[k] = (double)B[k] + pdiag[9 * (size_t)i + k];
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    double inv[9];
    if (!(fabs(det) > 0)) {
        for (int k = 0; k < 9; ++k) inv[k] = (k % 4 == 0) ? 1.0 : 0.0;
    } else {
        const double id = 1.0 / det;
        inv[0] = c00 * id;
        inv[3] = c01 * id;
        inv[6] = c02 * id;
        inv[1] = (A[2] * A[7] - A[1] * A[8]) * id;
        inv[4] = (A[0] * A[8] - A[2] * A[6]) * id;
        inv[7] = (A[1] * A[6] - A[0] * A[7]) * id;
        inv[2] = (A[1] * A[5] - A[2] * A[4]) * id;
        inv[5] = (A[2] * A[3] - A[0] * A[5]) * id;
        inv[8] = (A[0] * A[4] - A[1] * A[3]) * id;
    }
    for (int k = 0; k < 9; ++k) pinv[9 * (size_t)i + k] = (PT)inv[k];
}

// dot product partials (block sums in XT, written as double)
template <typename XT>
__global__ void k_dot(int n, const XT* __restrict__ a, const XT* __restrict__ b, double* part)
{
    __shared__ XT sh[256];
    XT s = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = (double)sh[0];
}
__global__ void k_dot_final(const double* part, int n, double* out)
{
    __shared__ double sh[256];
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

template <typename A, typename B>
__global__ void k_convert(int n, const A* a, B* b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (B)a[i];
}
// r = b - y (FP64)
__global__ void k_residual(int n, const double* b, const double* y, double* r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - y[i];
}
template <typename XT>
__global__ void k_axpy_into(int n, const XT* d, double* x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)d[i];
}
// b = (float)(a * scale): the refinement hands the FP32 solver a unit-norm
// residual, so that its dot products neither underflow nor overflow
__global__ void k_convert_scaled(int n, const double* a, double scale, float* b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)(a[i] * scale);
}
// x += scale * d
__global__ void k_axpy_scaled(int n, const float* d, double scale, double* x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += scale * (double)d[i];
}

struct SolveCtx {
    Sim* s;
    cudaStream_t st;
    int n3;
    double* part;   // dot partials
    double* sc;     // device scalars
    int nparts;
};

template <typename XT>
static void dot(SolveCtx& C, const XT* a, const XT* b, double* out)
{
    k_dot<XT><<<C.nparts, 256, 0, C.st>>>(C.n3, a, b, C.part);
    k_dot_final<<<1, 256, 0, C.st>>>(C.part, C.nparts, out);
}

template <typename VT, typename XT>
static void apply_H(SolveCtx& C, const XT* x, XT* y)
{
    Sim* s = C.s;
    const bool fo = s->folded;
    k_bsr_spmv<VT, XT><<<nblk(s->nv, 256), 256, 0, C.st>>>(s->nv, s->rowlen.p, s->col.p,
                                                            (const VT*)(fo ? s->hval_op.p : s->hval.p), x, y);
    const int ncon = s->prm.withCollision ? s->ncon : 0;
    const int nfric = (s->prm.withCollision && s->prm.mu > 0) ? s->nfric : 0;
    if (ncon > 0)
        k_con_spmv<VT, XT><<<nblk(ncon, 128), 128, 0, C.st>>>(ncon, fo ? s->crest.p : nullptr, s->fold_cnt.p,
                                                               s->ckind.p, s->cverts.p, (const VT*)s->chess.p,
                                                               (size_t)s->cap_con, x, y);
    if (nfric > 0)
        k_fric_spmv<XT><<<nblk(nfric, 128), 128, 0, C.st>>>(nfric, fo ? s->frest.p : nullptr, s->fold_cnt.p + 1,
                                                             s->fkind.p, s->fverts.p, s->fw.p, s->fT.p,
                                                             (const double*)s->fhess.p, s->proj.p, x, y);
}

// Finalizes the block-Jacobi preconditioner from the assembled matrix
static void build_precond(Sim* s)
{
    if (s->prm.precision == 1)
        k_precond<float, float><<<nblk(s->nv, 256), 256, 0, s->stream>>>(s->nv, s->diag.p, (const float*)s->hval.p,
                                                                          s->pdiag.p, (float*)s->pinv.p);
    else
        k_precond<double, double><<<nblk(s->nv, 256), 256, 0, s->stream>>>(s->nv, s->diag.p, (const double*)s->hval.p,
                                                                            s->pdiag.p, (double*)s->pinv.p);
}

// PCG (FP64, or FP32 inside FP64 refinement) with the preconditioner already in s->pinv
static int solve_with_precond(Sim* s, const double* rhs, double* sol, int* iters)
{
    const int n3 = 3 * s->nv;
    const double tol = s->solve_tol > 0 ? s->solve_tol : s->prm.pcg_tol;
    int total = 0;
    double rel = 0;
    int rc = CIPC_OK;
    if (s->prm.precision != 1) {
        rc = pcg_solve_fp64(s, rhs, sol, tol, s->prm.pcg_maxit, &total, &rel);
    } else {
        // mixed: FP32 inner PCG, FP64 iterative refinement of the residual
        const size_t need = (size_t)n3 * 2 * sizeof(double) + 4096 * sizeof(double) + (1 << 16);
        if (s->scratch.n < need) {
            cudaStreamSynchronize(s->stream);
            if (s->scratch.alloc(need) != cudaSuccess) return set_error(CIPC_ERR_CUDA, "solver scratch");
        }
        char* base = s->scratch.p;
        size_t off = 0;
        auto take = [&](size_t bytes) {
            off = (off + 255) & ~(size_t)255;
            char* p = base + off;
            off += bytes;
            return p;
        };
        SolveCtx C;
        C.s = s;
        C.st = s->stream;
        C.n3 = n3;
        C.nparts = std::min(nblk(n3, 256), 1024);
        C.part = (double*)take(1024 * sizeof(double));
        C.sc = (double*)take(64 * sizeof(double));
        double* r64 = (double*)take((size_t)n3 * 8);
        double* y64 = (double*)take((size_t)n3 * 8);
        float *b32 = nullptr, *d32 = nullptr;
        if ((rc = pcg_fp32_io(s, &b32, &d32))) return rc;
        cudaMemsetAsync(sol, 0, sizeof(double) * n3, s->stream);
        cudaMemcpyAsync(r64, rhs, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s->stream);
        double* sc = C.sc;
        dot<double>(C, rhs, rhs, sc + 10);
        double bb = 0;
        cudaMemcpyAsync(&bb, sc + 10, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
        cudaStreamSynchronize(s->stream);
        // each pass asks the FP32 solver for what is still missing (with a margin
        // for the gap between its recurrence and the true residual), down to the
        // 1e-5 an FP32 Krylov recurrence reliably reaches; a pass restarts the
        // Krylov space, so fewer, deeper passes take fewer iterations in total
        double rr = bb;
        for (int outer = 0; outer < 20 && bb > 0; ++outer) {
            const double rn = std::sqrt(rr);
            const double inner_tol = std::min(0.5, std::max(0.5 * tol * std::sqrt(bb / rr), 1e-5));
            k_convert_scaled<<<nblk(n3, 256), 256, 0, s->stream>>>(n3, r64, 1.0 / rn, b32);
            double relin = 0;
            int it = 0;
            const int lr = pcg_solve_fp32(s, b32, d32, inner_tol, std::max(1, s->prm.pcg_maxit - total), &it, &relin);
            total += it;
            if (lr == CIPC_ERR_NAN || (lr != CIPC_OK && lr != CIPC_ERR_NOT_CONVERGED)) return lr;
            if (it == 0 && lr != CIPC_OK) break;  // no progress possible (non-positive curvature)
            k_axpy_scaled<<<nblk(n3, 256), 256, 0, s->stream>>>(n3, d32, rn, sol);
            apply_H<float, double>(C, sol, y64);
            k_residual<<<nblk(n3, 256), 256, 0, s->stream>>>(n3, rhs, y64, r64);
            dot<double>(C, r64, r64, sc + 11);
            cudaMemcpyAsync(&rr, sc + 11, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
            cudaStreamSynchronize(s->stream);
            rel = std::sqrt(rr / bb);
            if (s->trace)
                std::fprintf(stderr, "cipc refine %d: inner %.3e outer %.3e pcg %d\n", outer, relin, rel, total);
            if (rel <= tol || total >= s->prm.pcg_maxit) break;
        }
        rc = rel <= tol ? CIPC_OK : set_error(CIPC_ERR_NOT_CONVERGED, "PCG stopped at relative residual %g", rel);
    }
    if (iters) *iters = total;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "linear solve");
    if (!(rel == rel)) return set_error(CIPC_ERR_NAN, "linear solve produced NaN");
    return rc;
}

int linear_solve(Sim* s, const double* rhs, double* sol, int* iters)
{
    // The learned correction is used once a block-Jacobi solve of this time step
    // (its first) has set the yardstick, and not after it has stalled twice in
    // the step.  It stalls when it needs more than three times the iterations of
    // the latest block-Jacobi solve (at least 100; consecutive Newton systems of
    // a step differ in difficulty by up to ~2x, while across steps the count
    // drifts upward as contacts build up, hence the per-step yardstick), breaks
    // down or yields NaN; block Jacobi then solves the same system, so a poor
    // network costs at most ~4x a plain solve.
    bool learned = false;
    if (s->prm.precond == 1 && s->learned && s->bj_last_iters > 0 && s->solve_fallbacks < 2)
        learned = lp_precond(s, static_cast<LpModel*>(s->learned)) == CIPC_OK;
    if (!learned) build_precond(s);
    {
        const int frc = fold_constraints(s);
        if (frc) return frc;
    }
    // aggregate block Jacobi: the inverses of the aggregates' diagonal blocks of
    // this system (after folding); a block that is not positive definite in the
    // solver's precision leaves the solve to block Jacobi
    s->agg_ready = false;
    bool aggregate = false;
    if (s->prm.precond == 2) {
        const int arc = agg_setup(s);
        if (arc && arc != CIPC_ERR_NOT_CONVERGED) return arc;
        aggregate = arc == CIPC_OK;
        if (!aggregate) ++s->solve_fallbacks;
    }
    int total = 0, it = 0;
    const int maxit = s->prm.pcg_maxit;
    if (learned) s->prm.pcg_maxit = std::min(maxit, std::max(100, 3 * s->bj_last_iters));
    int rc = solve_with_precond(s, rhs, sol, &it);
    s->prm.pcg_maxit = maxit;
    total += it;
    if (aggregate && (rc == CIPC_ERR_NOT_CONVERGED || rc == CIPC_ERR_NAN)) {
        // breakdown with the aggregate inverses (an FP32 inverse can lose
        // definiteness): block Jacobi solves the same system
        ++s->solve_fallbacks;
        s->agg_ready = false;
        rc = solve_with_precond(s, rhs, sol, &it);
        total += it;
    }
    if (learned) {
        ++s->solve_learned;
        if (rc == CIPC_ERR_NOT_CONVERGED || rc == CIPC_ERR_NAN) {
            // the learned preconditioner stalled or broke down: plain block Jacobi
            // solves the same system (and is the yardstick for the network)
            ++s->solve_fallbacks;
            build_precond(s);
            rc = solve_with_precond(s, rhs, sol, &it);
            total += it;
            s->bj_last_iters = std::max(1, it);
        }
    } else {
        s->bj_last_iters = std::max(1, it);
    }
    if (iters) *iters = total;
    if (rc == CIPC_OK && s->capture) {
        const int crc = lp_capture(s, static_cast<LpModel*>(s->capture), rhs, sol);
        if (crc) return crc;
    }
    return rc;
}

}  // namespace cipc
