// One implicit-Euler time step on the GPU and the simulation C ABI.
//
// Restates Advance_One_Step_IE_Discrete_Shell (Library/FEM/Shell/IMPLICIT_EULER.h:
// 151-902) and Line_Search (:9-149): x~ = x + h v + h^2 M^-1 b; Dirichlet targets
// applied when the Dirichlet step is intersection free; constraint set and lagged
// friction basis; Newton iterations with an intersection-free (CCD) step bound and
// backtracking on the incremental potential, the min-distance safeguard, the
// barrier-stiffness doubling when a tiny distance keeps shrinking, the
// max-of-last-three RMS(step)/h stopping rule (at least three iterations) and the
// gradient-descent fallback; finally v = (x - x^n) / h.  All per-element and
// per-constraint work runs in kernels; the host only reads back scalars
// (energies, step sizes, residual norms) to drive the loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "sim_handle.h"
#include "constraint_eval.cuh"
#include "sim.h"
#include "sim_host.h"
#include "sim_kernels.h"
#include "sim_pcg.h"
#include "learned.h"

namespace cipc {

static inline int nblk(long long n, int bs) { return n > 0 ? (int)((n + bs - 1) / bs) : 1; }

__global__ void k_axpby(int n, const double* a, double alpha, const double* d, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] + alpha * d[i];
}
__global__ void k_neg(int n, const double* a, double* b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = -a[i];
}
__global__ void k_velocity(int n, const double* x, const double* xn, double h, double* v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (x[i] - xn[i]) / h;
}
__global__ void k_dbc_disp(int nd, const int* idx, const double* tgt, const double* x, double* disp)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nd) return;
    const int v = idx[k];
    for (int d = 0; d < 3; ++d) disp[3 * v + d] = tgt[3 * k + d] - x[3 * v + d];
}
// Dirichlet vertices whose displacement this step is exactly zero
__global__ void k_dbc_fixed(int nd, const int* idx, const double* disp, uint8_t* fixed)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nd) return;
    const int v = idx[k];
    fixed[v] = (disp[3 * v] == 0 && disp[3 * v + 1] == 0 && disp[3 * v + 2] == 0) ? 1 : 0;
}
__global__ void k_dbc_apply(int nd, const int* idx, const double* tgt, double* x)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nd) return;
    const int v = idx[k];
    for (int d = 0; d < 3; ++d) x[3 * v + d] = tgt[3 * k + d];
}
__global__ void k_sumsq(int n, const double* a, double* part)
{
    __shared__ double sh[256];
    double s = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += a[i] * a[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
// d^2 - xi^2 for a constraint list
__global__ void k_con_d2(int n, const int* kind, const int4* verts, const double* x, double xi2, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 iv = verts[i];
    const int id[4] = {iv.x, iv.y, iv.z < 0 ? iv.x : iv.z, iv.w < 0 ? iv.x : iv.w};
    d3 v[4];
    for (int q = 0; q < 4; ++q) v[q] = ld(x, id[q]);
    out[i] = con_d2(kind[i], v) - xi2;
}
// flag = 1 if some previous constraint had d2 < 1e-18 and shrank (IMPLICIT_EULER.h:566-580)
__global__ void k_kappa_flag(int n, const int* kind, const int4* verts, const double* prev, const double* x, double xi2,
                             unsigned long long* flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 iv = verts[i];
    const int id[4] = {iv.x, iv.y, iv.z < 0 ? iv.x : iv.z, iv.w < 0 ? iv.x : iv.w};
    d3 v[4];
    for (int q = 0; q < 4; ++q) v[q] = ld(x, id[q]);
    const double cur = con_d2(kind[i], v) - xi2;
    if (prev[i] < 1e-18 && cur < prev[i]) *flag = 1;
}

// energy of the incremental potential at x (FP64).  *ok = false when some
// constraint distance is at or below the offset.
static int eval_energy(Sim* s, const double* x, double* E, bool* ok)
{
    const int worst = nblk(s->nv, 256) + 2 * nblk(s->nt, 128) + nblk(s->nh, 128) + nblk(s->nrs, 128) + nblk(s->nrh, 128) +
                      nblk(s->ntet, 128) +
                      (s->prm.withCollision ? nblk(s->ncon, 128) + nblk(s->nfric, 128) : 0) + 16;
    if ((int)s->red.n < worst + 16) {
        cudaStreamSynchronize(s->stream);
        if (s->red.alloc(2 * worst + 64) != cudaSuccess) return set_error(CIPC_ERR_CUDA, "reduction buffer");
    }
    double* red = s->red.p;
    double* out = red + s->red.n - 2;  // [E, flag]
    cudaMemsetAsync(out, 0, 2 * sizeof(double), s->stream);
    int n = elastic_energy_partials(s, x, red, out + 1);
    n += dbc_penalty_partials(s, x, red + n, nullptr);
    if (s->prm.withCollision) {
        n += contact_energy_partials(s, x, red + n, out + 1);
        if (s->prm.mu > 0) n += friction_energy_partials(s, x, red + n);
    }
    sum_partials(s, red, n, out);
    double h[2];
    cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "energy");
    *E = h[0];
    *ok = h[1] == 0;
    return CIPC_OK;
}

// gradient (DBC rows zeroed) and, optionally, the Hessian with its preconditioner diagonal
static void eval_grad_hess(Sim* s, const double* x, double* g, bool want_h)
{
    if (want_h) cudaMemsetAsync(s->pdiag.p, 0, 9 * sizeof(double) * (size_t)s->nv, s->stream);
    elastic_grad_hess(s, x, g, want_h);
    dbc_penalty_partials(s, x, nullptr, g);
    if (s->prm.withCollision) {
        contact_grad_hess(s, x, g, want_h);
        if (s->prm.mu > 0) friction_grad_hess(s, x, g, want_h);
    }
    zero_dbc(s, g);
}

static double sum_sq(Sim* s, const double* a, int n)
{
    double* part = s->red.p;
    k_sumsq<<<64, 256, 0, s->stream>>>(n, a, part);
    double h[64];
    cudaMemcpyAsync(h, part, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
    cudaStreamSynchronize(s->stream);
    double t = 0;
    for (double v : h) t += v;
    return t;
}

static int min_d2(Sim* s, const double* x, double* out)
{
    double* dev = s->red.p + s->red.n - 3;
    min_dist2_partials(s, x, dev);
    cudaMemcpyAsync(out, dev, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "min distance");
}

// Run logs in the reference's formats, appended in the simulation's output
// folder when one is set (cipc_sim_set_output): residual.txt one line per Newton
// iteration, "PNIter avgResMag maxRes Eprev L2Norm" (IMPLICIT_EULER.h:647-670);
// counter.txt one line per step, "PNIter[ #constraints]" (:868-875);
// Hessian_info.txt when a Newton system could not be solved (:531-534, there a
// non-SPD factorisation); and steps.jsonl, one JSON object of step statistics
// per step (no reference counterpart).
static void log_line(Sim* s, const char* file, const char* fmt, ...)
{
    FILE* f = std::fopen((s->out_dir + "/" + file).c_str(), "a+");
    if (!f) return;
    va_list ap;
    va_start(ap, fmt);
    std::vfprintf(f, fmt, ap);
    va_end(ap);
    std::fclose(f);
}

// per-vertex magnitudes of the Newton step: sum of |p_i| and max |p_ij|
__global__ void k_resmag(int nv, const double* p, double* part)
{
    __shared__ double ss[256], sm[256];
    double sum = 0, mx = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
        const double a = p[3 * i], b = p[3 * i + 1], c = p[3 * i + 2];
        sum += sqrt(a * a + b * b + c * c);
        mx = fmax(mx, fmax(fabs(a), fmax(fabs(b), fabs(c))));
    }
    ss[threadIdx.x] = sum;
    sm[threadIdx.x] = mx;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            ss[threadIdx.x] += ss[threadIdx.x + w];
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = ss[0];
        part[2 * blockIdx.x + 1] = sm[0];
    }
}

static void log_residual(Sim* s, int pn_iter, int n_free, double Eprev, double L2)
{
    double* part = s->red.p;
    k_resmag<<<64, 256, 0, s->stream>>>(s->nv, s->dir.p, part);
    double h[128];
    cudaMemcpyAsync(h, part, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return;
    double avg = 0, mx = 0;
    for (int b = 0; b < 64; ++b) {
        avg += h[2 * b];
        mx = std::max(mx, h[2 * b + 1]);
    }
    avg /= n_free;
    const double hh = s->prm.h;
    log_line(s, "residual.txt", "%d %le %le %le %le\n", pn_iter, avg / hh, mx / hh, Eprev, L2);
}

static void log_step(Sim* s, const StepStats& S, bool with_collision)
{
    if (with_collision)
        log_line(s, "counter.txt", "%d %lu\n", S.newton_iters, (unsigned long)S.n_constraints);
    else
        log_line(s, "counter.txt", "%d\n", S.newton_iters);
    log_line(s, "steps.jsonl",
             "{\"step\": %d, \"newton_iters\": %d, \"pcg_iters\": %d, \"line_search_trials\": %d, "
             "\"n_constraints\": %d, \"status\": %d, \"min_dist2\": %.17g, \"kappa\": %.17g, \"ms\": %.3f, "
             "\"precond_fallbacks\": %d, \"learned_solves\": %d, \"solve_ms\": %.3f}\n",
             s->step_count, S.newton_iters, S.pcg_iters, S.line_search_trials, S.n_constraints, S.status, S.min_dist2,
             S.kappa, S.ms, S.precond_fallbacks, S.learned_solves, S.solve_ms);
}

// 1 in *flag when some entry is NaN or infinite
__global__ void k_nonfinite(int n, const double* a, unsigned long long* flag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (!isfinite(a[i])) {
            *flag = 1;
            return;
        }
}

static int check_finite_state(Sim* s)
{
    unsigned long long* flag = s->cnt.p + 33;
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(unsigned long long), s->stream);
    const int n3 = 3 * s->nv;
    if (e == cudaSuccess) {
        k_nonfinite<<<nblk(n3, 256) < 304 ? nblk(n3, 256) : 304, 256, 0, s->stream>>>(n3, s->x.p, flag);
        k_nonfinite<<<nblk(n3, 256) < 304 ? nblk(n3, 256) : 304, 256, 0, s->stream>>>(n3, s->v.p, flag);
        e = cudaGetLastError();
    }
    unsigned long long hf = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hf, flag, sizeof(hf), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "state check");
    return hf ? set_error(CIPC_ERR_NAN, "the state holds a NaN or infinite position or velocity") : CIPC_OK;
}

static void save_prev(Sim* s, const double* x)
{
    s->npcon = s->ncon;
    if (s->ncon == 0) return;
    s->pkind.alloc(s->ncon);
    s->pverts.alloc(s->ncon);
    s->pd2.alloc(s->ncon);
    cudaMemcpyAsync(s->pkind.p, s->ckind.p, sizeof(int) * s->ncon, cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(s->pverts.p, s->cverts.p, sizeof(int4) * s->ncon, cudaMemcpyDeviceToDevice, s->stream);
    k_con_d2<<<nblk(s->ncon, 256), 256, 0, s->stream>>>(s->ncon, s->ckind.p, s->cverts.p, x,
                                                        s->prm.xi * s->prm.xi, s->pd2.p);
}

int sim_step(Sim* s, StepStats* st)
{
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    StepStats S;
    s->solve_fallbacks = 0;
    s->solve_learned = 0;
    s->solve_ms = 0;
    s->bj_last_iters = 0;  // the step's first solve is block Jacobi: a fresh yardstick
    s->sl_have_prev = false;  // strain history is per step (IMPLICIT_EULER.h:444)
    const SimParams& P = s->prm;
    const int nv = s->nv, n3 = 3 * nv, nd = (int)s->dbc_idx_h.size();
    cudaStream_t str = s->stream;
    int rc = CIPC_OK;
    // per-phase wall time, only with CIPC_TRACE (each mark waits for the stream):
    // 0 setup, 1 constraint sets, 2 friction basis, 3 energies, 4 gradient +
    // Hessian, 5 linear solves, 6 CCD step sizes, 7 other
    double ph[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    auto tmark = clk::now();
    auto mark = [&](int k) {
        if (!s->trace) return;
        cudaStreamSynchronize(str);
        const auto now = clk::now();
        ph[k] += std::chrono::duration<double, std::milli>(now - tmark).count();
        tmark = now;
    };
    // a non-finite position or velocity would propagate silently through every
    // kernel; the step refuses it up front
    if ((rc = check_finite_state(s))) {
        S.status = -5;
        *st = S;
        return rc;
    }
    cudaMemcpyAsync(s->xn.p, s->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
    launch_xtilde(s);
    // Dirichlet step (IMPLICIT_EULER.h:304-401): move the Dirichlet vertices to
    // their targets when that motion is intersection free, otherwise keep them at
    // x^n and pull them with the augmented-Lagrangian penalty
    s->dbc_stiff = 0;
    double dbcPenaltyXn = 0;
    cudaMemcpyAsync(s->proj.p, s->dbc.p, nv, cudaMemcpyDeviceToDevice, str);
    if (nd > 0) {
        cudaMemsetAsync(s->disp.p, 0, sizeof(double) * n3, str);
        k_dbc_disp<<<nblk(nd, 128), 128, 0, str>>>(nd, s->dbc_idx.p, s->dbc_tgt.p, s->x.p, s->disp.p);
        cudaMemsetAsync(s->dbc_fixed.p, 0, nv, str);
        k_dbc_fixed<<<nblk(nd, 128), 128, 0, str>>>(nd, s->dbc_idx.p, s->disp.p, s->dbc_fixed.p);
        double dbcAlpha = 1.0;
        if (P.withCollision) {
            rc = ccd_step_size(s, s->x.p, s->disp.p, 1.0, &dbcAlpha);
            if (rc) return rc;
        }
        if (dbcAlpha == 1.0) {
            k_dbc_apply<<<nblk(nd, 128), 128, 0, str>>>(nd, s->dbc_idx.p, s->dbc_tgt.p, s->x.p);
        } else {
            s->dbc_stiff = 1e6;
            dbcPenaltyXn = dbc_dist2(s, s->xn.p);
            cudaMemcpyAsync(s->proj.p, s->dbc_fixed.p, nv, cudaMemcpyDeviceToDevice, str);
            S.status = 1;  // penalty path taken
        }
    }
    mark(0);
    s->ncon = 0;
    s->nfric = 0;
    s->npcon = 0;
    if (P.withCollision) {
        if ((rc = build_constraints(s, s->x.p))) return rc;
        mark(1);
        if (P.mu > 0 && (rc = friction_basis(s, s->x.p))) return rc;
        mark(2);
    }
    double Eprev;
    bool ok;
    if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
    // the reference exits where a constraint's d^2 - xi^2 is not positive
    // (IPC.h:773-776); a start state inside the offset cannot be stepped from
    if (!ok) {
        S.status = -4;
        *st = S;
        return set_error(CIPC_ERR_NONPOSITIVE_DISTANCE, "the step's start state has a contact at or inside the offset");
    }
    if (!std::isfinite(Eprev)) {
        S.status = -5;
        *st = S;
        return set_error(CIPC_ERR_NAN, "the incremental potential at the step's start is not finite");
    }
    mark(3);
    std::deque<double> res;
    int fricIterI = 0, it = 0;
    bool useGD = false;
    double L2 = 0;
    // inexact Newton: Eisenstat-Walker forcing term, choice 2 (gamma 0.9, alpha 2)
    // with its safeguard, clamped to [pcg_tol, 0.1]; full accuracy once the last
    // step was within 10x of the Newton tolerance, so the stopping test (and the
    // friction re-solve below) always sees a direction solved to pcg_tol
    double gnorm_prev = -1, eta_prev = 0.1;
    s->solve_tol = 0;
    do {
        if (it >= P.maxIter) {
            S.status = -1;
            rc = set_error(CIPC_ERR_NOT_CONVERGED, "Newton iteration cap %d reached", P.maxIter);
            break;
        }
        eval_grad_hess(s, s->x.p, s->g.p, !useGD);
        k_neg<<<nblk(n3, 256), 256, 0, str>>>(n3, s->g.p, s->rhs.p);
        mark(4);
        if (useGD) {
            cudaMemcpyAsync(s->dir.p, s->rhs.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
        } else {
            // the forcing term is not combined with the learned correction: its
            // early-stopped solves (trained on tight ones) gave directions of
            // ~100 m/s and Newton loops of 50+ iterations on the cloth-on-sphere scene
            if (P.forcing && !(P.precond == 1 && s->learned)) {
                const double gn = std::sqrt(sum_sq(s, s->rhs.p, n3));
                double eta = 0.1;
                if (gnorm_prev > 0) {
                    eta = 0.9 * (gn / gnorm_prev) * (gn / gnorm_prev);
                    const double safe = 0.9 * eta_prev * eta_prev;
                    if (safe > 0.1) eta = std::max(eta, safe);
                }
                eta = std::min(0.1, std::max(P.pcg_tol, eta));
                if (!res.empty() && res.back() < 10 * P.tol) eta = P.pcg_tol;
                gnorm_prev = gn;
                eta_prev = eta;
                s->solve_tol = eta;
            }
            int pit = 0;
            const int lr = linear_solve(s, s->rhs.p, s->dir.p, &pit);
            s->solve_tol = 0;
            S.pcg_iters += pit;
            if (lr == CIPC_ERR_NAN && !s->out_dir.empty()) log_line(s, "Hessian_info.txt", "Hessian not SPD in PNIter%d\n", it);
            if (lr == CIPC_ERR_NAN) {
                useGD = true;
                cudaMemcpyAsync(s->dir.p, s->rhs.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
            } else if (lr != CIPC_OK && lr != CIPC_ERR_NOT_CONVERGED) {
                return lr;
            }
        }
        mark(5);
        // line search (IMPLICIT_EULER.h:9-149)
        cudaMemcpyAsync(s->xprev.p, s->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
        double alpha = 1.0;
        if (s->sl.k0 > 0 || s->ntet > 0) {
            // elastic feasibility first (IMPLICIT_EULER.h:74-94): halve until every
            // stretch is inside the limits and no tetrahedron is inverted
            for (int k = 0;; ++k) {
                if (k > 200) return set_error(CIPC_ERR_NOT_CONVERGED, "no feasible step");
                k_axpby<<<nblk(n3, 256), 256, 0, str>>>(n3, s->xprev.p, alpha, s->dir.p, s->x.p);
                bool feas = true;
                if ((rc = elastic_feasible(s, s->x.p, &feas))) return rc;
                if (feas) break;
                alpha /= 2;
            }
        }
        if (P.withCollision && (rc = ccd_step_size(s, s->xprev.p, s->dir.p, alpha, &alpha))) return rc;
        mark(6);
        const double feasible = alpha;
        double E = Eprev;
        int trials = 0;
        do {
            if (++trials > 200) {
                S.status = -3;
                return set_error(CIPC_ERR_NOT_CONVERGED, "line search did not find a decrease");
            }
            k_axpby<<<nblk(n3, 256), 256, 0, str>>>(n3, s->xprev.p, alpha, s->dir.p, s->x.p);
            if (P.withCollision) {
                if ((rc = build_constraints(s, s->x.p))) return rc;
                mark(1);
                if (s->ncon > 0) {
                    double md;
                    if ((rc = min_d2(s, s->x.p, &md))) return rc;
                    mark(7);
                    if (md <= 0) {
                        alpha /= 2;
                        E = Eprev + 1;
                        ok = true;
                        continue;
                    }
                }
            }
            if ((rc = eval_energy(s, s->x.p, &E, &ok))) return rc;
            mark(3);
            alpha /= 2;
        } while (E > Eprev || !ok);
        S.line_search_trials += trials;
        if (s->trace)
            std::fprintf(stderr, "cipc newton %d: step %.3e feasible %.3e trials %d E %.17g dE %.3e gd %d\n", it,
                         2 * alpha, feasible, trials, E, E - Eprev, (int)useGD);
        Eprev = E;
        // barrier stiffness update (IMPLICIT_EULER.h:566-595; offset IPC only)
        if (s->npcon > 0 && !P.elastic) {
            unsigned long long* flag = s->cnt.p + 32;
            cudaError_t ce = cudaMemsetAsync(flag, 0, sizeof(unsigned long long), str);
            if (ce != cudaSuccess) return set_cuda_error(ce, "kappa update: clearing the flag");
            k_kappa_flag<<<nblk(s->npcon, 256), 256, 0, str>>>(s->npcon, s->pkind.p, s->pverts.p, s->pd2.p, s->x.p,
                                                               P.xi * P.xi, flag);
            if ((ce = cudaGetLastError()) != cudaSuccess) return set_cuda_error(ce, "kappa update: k_kappa_flag");
            unsigned long long hf = 0;
            if ((ce = cudaMemcpyAsync(&hf, flag, sizeof(hf), cudaMemcpyDeviceToHost, str)) != cudaSuccess)
                return set_cuda_error(ce, "kappa update: reading the flag");
            if ((ce = cudaStreamSynchronize(str)) != cudaSuccess)
                return set_cuda_error(ce, "kappa update: synchronize");
            if (hf && s->kappa < s->kappa_max) {
                s->kappa *= 2;
                if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
            }
        }
        save_prev(s, s->x.p);
        // strain-limit stiffness update (IMPLICIT_EULER.h:606-645)
        if (s->sl.k0 > 0) {
            bool raise = false;
            if ((rc = strain_kappa_update(s, s->x.p, &raise))) return rc;
            if (raise && s->sl.k0 < 1e5) {
                s->sl.k0 *= 2;
                if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
            }
        }
        // convergence (IMPLICIT_EULER.h:647-710)
        L2 = std::sqrt(sum_sq(s, s->dir.p, n3) / (nv - nd)) / P.h;
        ++it;
        if (!s->out_dir.empty()) log_residual(s, it, nv - nd, Eprev, L2);
        res.push_back(L2);
        if (res.size() > 3) res.pop_front();
        const double cur = L2;
        L2 = *std::max_element(res.begin(), res.end());
        if (useGD) L2 = P.tol * 10;
        if (alpha * 2 < 1e-8 && feasible > 1e-8) {
            if (!useGD) {
                if (cur < P.tol) res.assign(3, cur);
                else useGD = true;
            }
        } else {
            useGD = false;
        }
        if (s->trace)
            std::fprintf(stderr, "cipc newton %d: res %.3e L2 %.3e kappa %.6g dbc_stiff %.3g ncon %d\n", it, cur, L2,
                         s->kappa, s->dbc_stiff, s->ncon);
        mark(7);
        // augmented-Lagrangian Dirichlet progress (IMPLICIT_EULER.h:713-764)
        if (s->dbc_stiff != 0) {
            const double progress = 1 - std::sqrt(dbc_dist2(s, s->x.p) / dbcPenaltyXn);
            if (progress < 0.99) {
                if (L2 < P.tol * 10 && s->dbc_stiff < 1e8) {
                    s->dbc_stiff *= 2;
                    if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
                }
                L2 = P.tol * 10;
            } else {
                s->dbc_stiff = 0;
                cudaMemcpyAsync(s->proj.p, s->dbc.p, nv, cudaMemcpyDeviceToDevice, str);
                if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
            }
        }
        if (res.size() == 3 && L2 <= P.tol) {
            ++fricIterI;
            if ((fricIterI < P.fricIterAmt || P.fricIterAmt <= 0) && P.withCollision && P.mu > 0) {
                if ((rc = friction_basis(s, s->x.p))) return rc;
                eval_grad_hess(s, s->x.p, s->g.p, true);
                k_neg<<<nblk(n3, 256), 256, 0, str>>>(n3, s->g.p, s->rhs.p);
                int pit = 0;
                const int lr = linear_solve(s, s->rhs.p, s->dir.p, &pit);
                S.pcg_iters += pit;
                if (lr != CIPC_OK && lr != CIPC_ERR_NOT_CONVERGED) return lr;
                L2 = std::sqrt(sum_sq(s, s->dir.p, n3) / (nv - nd)) / P.h;
                if (L2 > P.tol && (rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
            }
        }
    } while (res.size() < 3 || L2 > P.tol);
    mark(7);
    k_velocity<<<nblk(n3, 256), 256, 0, str>>>(n3, s->x.p, s->xn.p, P.h, s->v.p);
    S.newton_iters = it;
    S.n_constraints = s->ncon;
    if (s->ncon > 0) min_d2(s, s->x.p, &S.min_dist2);
    S.kappa = s->kappa;
    cudaError_t e = cudaStreamSynchronize(str);
    if (e != cudaSuccess) return set_cuda_error(e, "step");
    S.ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    S.precond_fallbacks = s->solve_fallbacks;
    S.learned_solves = s->solve_learned;
    S.solve_ms = s->solve_ms;
    if (s->trace)
        std::fprintf(stderr,
                     "cipc step: %.2f ms  setup %.2f  sets %.2f  fbasis %.2f  energy %.2f  gradhess %.2f  solve %.2f  "
                     "ccd %.2f  other %.2f  (newton %d pcg %d)\n",
                     S.ms, ph[0], ph[1], ph[2], ph[3], ph[4], ph[5], ph[6], ph[7], it, S.pcg_iters);
    if (!s->out_dir.empty()) log_step(s, S, P.withCollision != 0);
    *st = S;
    return rc;
}

// Split stepper (Advance_One_Step_SIE_Discrete_Shell, SPLITTING_IE.h:362-729):
// an elastodynamic implicit-Euler substep without contact and without strain
// limiting gives x'; a projection substep then minimises, from x^n,
//   1/2 (x - x')^T M (x - x') + strain-limit barrier + contact barrier
//   + lagged friction (+ Dirichlet penalty)
// (Compute_SLP_Energy, :7-69) with its own Dirichlet handling (DBC_Info_Init
// :218-301: the Dirichlet vertices move by the largest strain-feasible fraction of
// their motion; if that is not all of it, a penalty of stiffness 1e8 pulls them,
// doubled up to 1e10 while progress < 99%, DBC_Dual_Update :303-360) and line
// search (CCD bound, then halving on infeasible strain, non-positive distance or
// no decrease).
int sim_step_split(Sim* s, StepStats* st)
{
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    SimParams& P = s->prm;
    const int nv = s->nv, n3 = 3 * nv, nd = (int)s->dbc_idx_h.size();
    cudaStream_t str = s->stream;
    int rc = CIPC_OK;
    if ((rc = check_finite_state(s))) {
        st->status = -5;
        return rc;
    }
    if (s->xsplit.alloc(n3) != cudaSuccess) return set_error(CIPC_ERR_CUDA, "split stepper buffer");
    cudaMemcpyAsync(s->xsplit.p, s->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
    // elastodynamic substep: no contact, no strain limiting
    StepStats S1;
    {
        const SlParams sl = s->sl;
        const int wc = P.withCollision;
        s->sl.k0 = s->sl.k1 = 0;
        P.withCollision = 0;
        rc = sim_step(s, &S1);
        s->sl = sl;
        P.withCollision = wc;
        if (rc != CIPC_OK && rc != CIPC_ERR_NOT_CONVERGED) return rc;
    }
    // projection substep from x^n towards x'
    StepStats S;
    S.pcg_iters = S1.pcg_iters;
    S.line_search_trials = S1.line_search_trials;
    cudaMemcpyAsync(s->xt.p, s->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);  // x'
    cudaMemcpyAsync(s->x.p, s->xsplit.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
    cudaMemcpyAsync(s->xn.p, s->xsplit.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
    s->elastic_off = 1;
    struct Restore {
        Sim* s;
        ~Restore() { s->elastic_off = 0; }
    } restore{s};
    s->solve_fallbacks = 0;
    s->solve_learned = 0;
    s->solve_ms = 0;
    s->bj_last_iters = 0;
    s->dbc_stiff = 0;
    double dbcPenaltyXn = 0;
    cudaMemcpyAsync(s->proj.p, s->dbc.p, nv, cudaMemcpyDeviceToDevice, str);
    if (nd > 0) {
        cudaMemsetAsync(s->disp.p, 0, sizeof(double) * n3, str);
        k_dbc_disp<<<nblk(nd, 128), 128, 0, str>>>(nd, s->dbc_idx.p, s->dbc_tgt.p, s->x.p, s->disp.p);
        cudaMemsetAsync(s->dbc_fixed.p, 0, nv, str);
        k_dbc_fixed<<<nblk(nd, 128), 128, 0, str>>>(nd, s->dbc_idx.p, s->disp.p, s->dbc_fixed.p);
        double dbcAlpha = 1.0;
        if (s->sl.k0 > 0) {
            for (int k = 0;; ++k) {
                if (k > 200) return set_error(CIPC_ERR_NOT_CONVERGED, "no strain-feasible Dirichlet motion");
                k_axpby<<<nblk(n3, 256), 256, 0, str>>>(n3, s->xsplit.p, dbcAlpha, s->disp.p, s->x.p);
                bool feas = true;
                if ((rc = elastic_feasible(s, s->x.p, &feas))) return rc;
                if (feas) break;
                dbcAlpha /= 2;
            }
            cudaMemcpyAsync(s->x.p, s->xsplit.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
        }
        if (dbcAlpha == 1.0) {
            k_dbc_apply<<<nblk(nd, 128), 128, 0, str>>>(nd, s->dbc_idx.p, s->dbc_tgt.p, s->x.p);
        } else {
            s->dbc_stiff = 1e8;
            dbcPenaltyXn = dbc_dist2(s, s->xn.p);
            cudaMemcpyAsync(s->proj.p, s->dbc_fixed.p, nv, cudaMemcpyDeviceToDevice, str);
            S.status = 1;
        }
    }
    s->ncon = s->nfric = s->npcon = 0;
    if (P.withCollision) {
        if ((rc = build_constraints(s, s->x.p))) return rc;
        if (P.mu > 0 && (rc = friction_basis(s, s->x.p))) return rc;
    }
    double Eprev;
    bool ok;
    if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
    if (!ok) return set_error(CIPC_ERR_NONPOSITIVE_DISTANCE, "split step: the start of the projection is infeasible");
    std::deque<double> res;
    bool useGD = false;
    double L2 = 0;
    int it = 0;
    s->solve_tol = 0;
    do {
        if (it >= P.maxIter) {
            S.status = -1;
            rc = set_error(CIPC_ERR_NOT_CONVERGED, "Newton iteration cap %d reached", P.maxIter);
            break;
        }
        eval_grad_hess(s, s->x.p, s->g.p, !useGD);
        k_neg<<<nblk(n3, 256), 256, 0, str>>>(n3, s->g.p, s->rhs.p);
        if (useGD) {
            cudaMemcpyAsync(s->dir.p, s->rhs.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
        } else {
            int pit = 0;
            const int lr = linear_solve(s, s->rhs.p, s->dir.p, &pit);
            S.pcg_iters += pit;
            if (lr == CIPC_ERR_NAN) {
                useGD = true;
                cudaMemcpyAsync(s->dir.p, s->rhs.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
            } else if (lr != CIPC_OK && lr != CIPC_ERR_NOT_CONVERGED) {
                return lr;
            }
        }
        cudaMemcpyAsync(s->xprev.p, s->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, str);
        double alpha = 1.0, feasible = 0, E = Eprev;
        if (P.withCollision && (rc = ccd_step_size(s, s->xprev.p, s->dir.p, 1.0, &alpha))) return rc;
        bool valid = true;
        int trials = 0;
        do {
            if (++trials > 200) {
                S.status = -3;
                return set_error(CIPC_ERR_NOT_CONVERGED, "line search did not find a decrease");
            }
            k_axpby<<<nblk(n3, 256), 256, 0, str>>>(n3, s->xprev.p, alpha, s->dir.p, s->x.p);
            if ((rc = elastic_feasible(s, s->x.p, &valid))) return rc;
            if (valid) {
                if (feasible == 0) feasible = alpha;
                if (P.withCollision) {
                    if ((rc = build_constraints(s, s->x.p))) return rc;
                    if (s->ncon > 0) {
                        double md;
                        if ((rc = min_d2(s, s->x.p, &md))) return rc;
                        if (md <= 0) {
                            alpha /= 2;
                            valid = false;
                            feasible = 0;
                            continue;
                        }
                    }
                }
                bool eok;
                if ((rc = eval_energy(s, s->x.p, &E, &eok))) return rc;
                valid = valid && eok;
            }
            alpha /= 2;
        } while (E > Eprev || !valid);
        S.line_search_trials += trials;
        Eprev = E;
        L2 = std::sqrt(sum_sq(s, s->dir.p, n3) / (nv - nd)) / P.h;
        ++it;
        if (!s->out_dir.empty()) log_residual(s, it, nv - nd, Eprev, L2);
        res.push_back(L2);
        if (res.size() > 3) res.pop_front();
        L2 = *std::max_element(res.begin(), res.end());
        if (useGD) L2 = P.tol * 10;
        if (alpha * 2 < 1e-6 && feasible > 1e-6) useGD = true;
        else useGD = false;
        if (s->trace)
            std::fprintf(stderr, "cipc split %d: step %.3e feasible %.3e L2 %.3e dbc_stiff %.3g ncon %d\n", it,
                         2 * alpha, feasible, L2, s->dbc_stiff, s->ncon);
        if (s->dbc_stiff != 0) {
            const double progress = 1 - std::sqrt(dbc_dist2(s, s->x.p) / dbcPenaltyXn);
            if (progress < 0.99) {
                if (L2 < P.tol * 10 && s->dbc_stiff < 1e10) {
                    s->dbc_stiff *= 2;
                    if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
                }
                L2 = P.tol * 10;
            } else {
                s->dbc_stiff = 0;
                cudaMemcpyAsync(s->proj.p, s->dbc.p, nv, cudaMemcpyDeviceToDevice, str);
                if ((rc = eval_energy(s, s->x.p, &Eprev, &ok))) return rc;
            }
        }
    } while (res.size() < 3 || L2 > P.tol);
    k_velocity<<<nblk(n3, 256), 256, 0, str>>>(n3, s->x.p, s->xsplit.p, P.h, s->v.p);
    S.newton_iters = S1.newton_iters + it;
    S.n_constraints = s->ncon;
    if (s->ncon > 0) min_d2(s, s->x.p, &S.min_dist2);
    S.kappa = s->kappa;
    cudaError_t e = cudaStreamSynchronize(str);
    if (e != cudaSuccess) return set_cuda_error(e, "split step");
    S.ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    S.precond_fallbacks = s->solve_fallbacks;
    S.learned_solves = s->solve_learned;
    S.solve_ms = s->solve_ms;
    if (!s->out_dir.empty()) log_step(s, S, P.withCollision != 0);
    *st = S;
    return rc;
}

void sim_destroy(Sim* s)
{
    if (!s) return;
    cudaStreamSynchronize(s->stream);
    pcg_release(s);
    agg_release(s);
    s->hval_op.release();
    s->crest.release();
    s->frest.release();
    s->fold_cnt.release();
    for (DBuf<int>* b : {&s->tri, &s->hinge, &s->bnode, &s->bedge, &s->btri, &s->dbc_idx, &s->col, &s->rowlen,
                         &s->diag, &s->tri_slot, &s->hinge_slot, &s->ckind, &s->cmult, &s->fkind, &s->fmult,
                         &s->rseg, &s->rhinge, &s->rseg_slot, &s->rhinge_slot, &s->tet, &s->tet_slot,
                         &s->pkind})
        b->release();
    for (DBuf<double>* b : {&s->P, &s->vol, &s->hinfo, &s->mass, &s->b, &s->X0, &s->dbc_tgt, &s->x, &s->xn, &s->xt,
                            &s->v, &s->g, &s->dir, &s->xprev, &s->rhs, &s->disp, &s->fw, &s->fT, &s->flam, &s->pdiag,
                            &s->red, &s->pd2, &s->rinfo, &s->rhinfo, &s->tDinv, &s->tvol, &s->sl_prev, &s->xsplit})
        b->release();
    s->dbc.release();
    s->proj.release();
    s->dbc_fixed.release();
    s->hval.release();
    s->chess.release();
    s->fhess.release();
    s->pinv.release();
    s->scratch.release();
    s->cnt.release();
    s->cverts.release();
    s->fverts.release();
    s->pverts.release();
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

}  // namespace cipc

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace cipc;


extern "C" int cipc_sim_create(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                               double thickness, const double* gravity, double bend_stiff_mult, int membrane_model,
                               cipc_sim** out)
{
    if (!out || !gravity) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_create: null output or gravity");
    if (nv >= (1 << 21) - 1) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_create: at most 2^21-2 vertices");
    Sim* s = nullptr;
    int rc = sim_create(&s, nv, X, nt, tri, rho, E, nu, thickness, gravity, bend_stiff_mult, membrane_model);
    if (rc) return rc;
    *out = new cipc_sim{s};
    return CIPC_OK;
}

extern "C" int cipc_sim_create_codim(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                                     double thickness, const double* gravity, double bend_stiff_mult,
                                     int membrane_model, const cipc_codim_desc* codim, cipc_sim** out)
{
    if (!out || !gravity || !codim) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_create_codim: null argument");
    if (nv >= (1 << 21) - 1) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_create_codim: at most 2^21-2 vertices");
    CodimDesc cd;
    cd.nseg = codim->n_segments;
    cd.seg = codim->segments;
    cd.rod_E = codim->rod_E;
    cd.rod_rho = codim->rod_rho;
    cd.rod_thickness = codim->rod_thickness;
    cd.rod_bend_mult = codim->rod_bend_mult;
    cd.npart = codim->n_particles;
    cd.part = codim->particles;
    cd.part_rho = codim->particle_rho;
    cd.part_thickness = codim->particle_thickness;
    Sim* s = nullptr;
    int rc = sim_create(&s, nv, X, nt, tri, rho, E, nu, thickness, gravity, bend_stiff_mult, membrane_model, &cd);
    if (rc) return rc;
    *out = new cipc_sim{s};
    return CIPC_OK;
}

extern "C" int cipc_sim_create_full(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                                    double thickness, const double* gravity, double bend_stiff_mult,
                                    int membrane_model, const cipc_codim_desc* codim, const cipc_tet_desc* tets,
                                    cipc_sim** out)
{
    if (!out || !gravity) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_create_full: null argument");
    if (nv >= (1 << 21) - 1) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_create_full: at most 2^21-2 vertices");
    CodimDesc cd;
    if (codim) {
        cd.nseg = codim->n_segments;
        cd.seg = codim->segments;
        cd.rod_E = codim->rod_E;
        cd.rod_rho = codim->rod_rho;
        cd.rod_thickness = codim->rod_thickness;
        cd.rod_bend_mult = codim->rod_bend_mult;
        cd.npart = codim->n_particles;
        cd.part = codim->particles;
        cd.part_rho = codim->particle_rho;
        cd.part_thickness = codim->particle_thickness;
    }
    TetDesc td;
    if (tets) {
        td.ntet = tets->n_tets;
        td.tet = tets->tets;
        td.E = tets->E;
        td.nu = tets->nu;
        td.rho = tets->rho;
    }
    Sim* s = nullptr;
    int rc = sim_create(&s, nv, X, nt, tri, rho, E, nu, thickness, gravity, bend_stiff_mult, membrane_model,
                        codim ? &cd : nullptr, tets ? &td : nullptr);
    if (rc) return rc;
    *out = new cipc_sim{s};
    return CIPC_OK;
}

extern "C" int cipc_sim_destroy(cipc_sim* h)
{
    if (!h) return CIPC_OK;
    sim_destroy(h->s);
    delete h;
    return CIPC_OK;
}

extern "C" int cipc_sim_init_oipc(cipc_sim* h, double dhat, double stiff_mult, double* kappa2, double* dhat2)
{
    if (int rc = check_sim(h)) return rc;
    double k2[2];
    const double d2 = oipc_kappa(h->s->host_mass, dhat, stiff_mult, k2);
    h->s->kappa = k2[0];
    h->s->kappa_max = k2[1];
    if (kappa2) {
        kappa2[0] = k2[0];
        kappa2[1] = k2[1];
    }
    if (dhat2) *dhat2 = d2;
    return CIPC_OK;
}

extern "C" int cipc_scene_oipc_kappa(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                                     double thickness, const double* gravity, double bend_stiff_mult,
                                     int membrane_model, const cipc_codim_desc* codim, const cipc_tet_desc* tets,
                                     double dhat, double stiff_mult, double* kappa2, double* dhat2)
{
    if (!gravity || !kappa2) return set_error(CIPC_ERR_INVALID_ARG, "cipc_scene_oipc_kappa: null argument");
    CodimDesc cd;
    if (codim) {
        cd.nseg = codim->n_segments;
        cd.seg = codim->segments;
        cd.rod_E = codim->rod_E;
        cd.rod_rho = codim->rod_rho;
        cd.rod_thickness = codim->rod_thickness;
        cd.rod_bend_mult = codim->rod_bend_mult;
        cd.npart = codim->n_particles;
        cd.part = codim->particles;
        cd.part_rho = codim->particle_rho;
        cd.part_thickness = codim->particle_thickness;
    }
    TetDesc td;
    if (tets) {
        td.ntet = tets->n_tets;
        td.tet = tets->tets;
        td.E = tets->E;
        td.nu = tets->nu;
        td.rho = tets->rho;
    }
    HostScene S;  // host only: no device is touched
    int rc = build_host_scene(S, nv, X, nt, tri, rho, E, nu, thickness, gravity, bend_stiff_mult, membrane_model,
                              codim ? &cd : nullptr, tets ? &td : nullptr);
    if (rc) return rc;
    const double d2 = oipc_kappa(S.mass, dhat, stiff_mult, kappa2);
    if (dhat2) *dhat2 = d2;
    return CIPC_OK;
}

extern "C" int cipc_sim_init_eipc(cipc_sim* h, double E, double nu, double thickness, double dt, double* kappa3,
                                  double* dhat2)
{
    if (int rc = check_sim(h)) return rc;
    if (!(E > 0) || !(nu > -1 && nu < 0.5) || !(thickness > 0) || !(dt > 0))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_init_eipc: bad material or step");
    const double lambda = E * nu / (1 - nu * nu), mu = E / (2 * (1 + nu)), h2 = dt * dt;
    h->s->kappa = h2 * mu;
    h->s->kappa_max = h2 * lambda;
    if (kappa3) {
        kappa3[0] = h2 * mu;
        kappa3[1] = h2 * lambda;
        kappa3[2] = nu;
    }
    if (dhat2) *dhat2 = thickness * thickness;
    return CIPC_OK;
}

extern "C" int cipc_sim_set_kappa(cipc_sim* h, double kappa, double kappa_max)
{
    if (int rc = check_sim(h)) return rc;
    h->s->kappa = kappa;
    h->s->kappa_max = kappa_max;
    return CIPC_OK;
}

extern "C" int cipc_sim_get_kappa(cipc_sim* h, double* kappa2)
{
    if (int rc = check_sim(h)) return rc;
    kappa2[0] = h->s->kappa;
    kappa2[1] = h->s->kappa_max;
    return CIPC_OK;
}

extern "C" int cipc_sim_set_strain_limit(cipc_sim* h, const double* s, const double* s_hat, const double* kappa_s)
{
    if (int rc = check_sim(h)) return rc;
    if (!s || !s_hat || !kappa_s || !(kappa_s[0] >= 0) || !(kappa_s[1] >= 0) ||
        (kappa_s[0] > 0 && !(s[0] > s_hat[0])) || (kappa_s[1] > 0 && !(s[1] < s_hat[1])))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_set_strain_limit: need s[0] > s_hat[0] (and s[1] < s_hat[1])");
    SlParams& p = h->s->sl;
    p.s0 = s[0];
    p.s1 = s[1];
    p.sh0 = s_hat[0];
    p.sh1 = s_hat[1];
    p.k0 = kappa_s[0];
    p.k1 = kappa_s[1];
    return CIPC_OK;
}

extern "C" int cipc_sim_get_strain_limit(cipc_sim* h, double* kappa_s)
{
    if (int rc = check_sim(h)) return rc;
    kappa_s[0] = h->s->sl.k0;
    kappa_s[1] = h->s->sl.k1;
    return CIPC_OK;
}

extern "C" int cipc_sim_set_state(cipc_sim* h, const double* x, const double* v)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    const size_t b = sizeof(double) * 3 * s->nv;
    if (x) cudaMemcpyAsync(s->x.p, x, b, cudaMemcpyHostToDevice, s->stream);
    if (v) cudaMemcpyAsync(s->v.p, v, b, cudaMemcpyHostToDevice, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_sim_set_state");
}

extern "C" int cipc_sim_get_state(cipc_sim* h, double* x, double* v)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    const size_t b = sizeof(double) * 3 * s->nv;
    if (x) cudaMemcpyAsync(x, s->x.p, b, cudaMemcpyDeviceToHost, s->stream);
    if (v) cudaMemcpyAsync(v, s->v.p, b, cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_sim_get_state");
}

extern "C" int cipc_sim_set_dbc(cipc_sim* h, int n, const int* idx, const double* targets)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    if (n < 0 || (n > 0 && (!idx || !targets))) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_set_dbc: bad arrays");
    for (int k = 0; k < n; ++k)
        if (idx[k] < 0 || idx[k] >= s->nv) return set_error(CIPC_ERR_INDEX_RANGE, "cipc_sim_set_dbc: vertex index");
    s->dbc_idx_h.assign(idx, idx + n);
    s->dbc_motion.clear();  // explicit targets replace any device-side motion
    std::vector<uint8_t> mask(s->nv, 0);
    for (int k = 0; k < n; ++k) mask[idx[k]] = 1;
    cudaError_t e = cudaMemcpyAsync(s->dbc.p, mask.data(), s->nv, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->proj.p, mask.data(), s->nv, cudaMemcpyHostToDevice, s->stream);
    s->dbc_stiff = 0;
    if (n > 0) {
        if (s->dbc_idx.alloc(n) || s->dbc_tgt.alloc(3 * (size_t)n)) return set_error(CIPC_ERR_CUDA, "dbc buffers");
        cudaMemcpyAsync(s->dbc_idx.p, idx, sizeof(int) * n, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->dbc_tgt.p, targets, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_sim_set_dbc");
}

static void to_params(const cipc_step_params* p, SimParams& q)
{
    q.h = p->h;
    q.dHat2 = p->dhat2;
    q.xi = p->xi;
    q.mu = p->mu;
    q.epsv2 = p->epsv2;
    q.fricIterAmt = p->fric_iters;
    q.tol = p->newton_tol;
    q.withCollision = p->with_collision;
    q.maxIter = p->max_newton_iters > 0 ? p->max_newton_iters : 200;
    q.precision = p->precision;
    q.pcg_tol = p->pcg_tol > 0 ? p->pcg_tol : 1e-6;
    q.pcg_maxit = p->pcg_max_iters > 0 ? p->pcg_max_iters : 10000;
    q.precond = p->preconditioner;
    q.forcing = p->forcing;
    // elastic IPC (Advance_One_Step_IE_Hinge_EIPC): no offset anywhere
    // (IPC.h:49-51, 752-754, FRICTION.h:28-30)
    q.elastic = p->barrier_model == CIPC_BARRIER_ELASTIC;
    q.accd_max_iter = p->accd_max_iters > 0 ? p->accd_max_iters : (1 << 20);
    q.accd_cap_strict = p->accd_max_iters > 0;
    q.pcg_wait_polls = p->pcg_wait_polls > 0 ? p->pcg_wait_polls : 0;
    if (q.elastic) q.xi = 0;
}

static int step_entry(cipc_sim* h, const cipc_step_params* p, cipc_step_stats* stats, bool split)
{
    if (int rc = check_sim(h)) return rc;
    if (!p || !(p->h > 0) || !(p->dhat2 > 0) || !(p->xi >= 0) || !(p->newton_tol > 0) ||
        (p->precision != CIPC_PRECISION_FP64 && p->precision != CIPC_PRECISION_MIXED) ||
        p->preconditioner < CIPC_PRECOND_BLOCK_JACOBI || p->preconditioner > CIPC_PRECOND_AGGREGATE)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_step: bad parameters");
    Sim* s = h->s;
    const int old_prec = s->prm.precision;
    to_params(p, s->prm);
    if (old_prec != s->prm.precision) s->hval.alloc(9 * sizeof(double) * (size_t)s->nnzb);
    StepStats S;
    ++s->step_count;
    const int rc = split ? sim_step_split(s, &S) : sim_step(s, &S);
    if (stats) {
        stats->newton_iters = S.newton_iters;
        stats->pcg_iters = S.pcg_iters;
        stats->line_search_trials = S.line_search_trials;
        stats->n_constraints = S.n_constraints;
        stats->status = S.status;
        stats->min_dist2 = S.min_dist2;
        stats->kappa = S.kappa;
        stats->ms = S.ms;
        stats->precond_fallbacks = S.precond_fallbacks;
        stats->learned_solves = S.learned_solves;
        stats->solve_ms = S.solve_ms;
    }
    return rc;
}

extern "C" int cipc_sim_step(cipc_sim* h, const cipc_step_params* p, cipc_step_stats* stats)
{
    return step_entry(h, p, stats, false);
}

extern "C" int cipc_sim_step_split(cipc_sim* h, const cipc_step_params* p, cipc_step_stats* stats)
{
    return step_entry(h, p, stats, true);
}

extern "C" int cipc_sim_constraints(cipc_sim* h, const cipc_step_params* p, const double* x, int cap, int* out6,
                                    int* count)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    to_params(p, s->prm);
    cudaMemcpyAsync(s->xprev.p, x, sizeof(double) * 3 * s->nv, cudaMemcpyHostToDevice, s->stream);
    int rc = build_constraints(s, s->xprev.p);
    if (rc) return rc;
    *count = s->ncon;
    const int n = std::min(cap, s->ncon);
    std::vector<int> k(n), m(n);
    std::vector<int4> v(n);
    if (n > 0) {
        cudaMemcpy(k.data(), s->ckind.p, sizeof(int) * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(m.data(), s->cmult.p, sizeof(int) * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(v.data(), s->cverts.p, sizeof(int4) * n, cudaMemcpyDeviceToHost);
    }
    for (int i = 0; i < n; ++i) {
        out6[6 * i] = k[i];
        out6[6 * i + 1] = v[i].x;
        out6[6 * i + 2] = v[i].y;
        out6[6 * i + 3] = v[i].z;
        out6[6 * i + 4] = v[i].w;
        out6[6 * i + 5] = m[i];
    }
    return CIPC_OK;
}

extern "C" int cipc_sim_eval(cipc_sim* h, const cipc_step_params* p, const double* x, const double* xtilde,
                             double* energy, double* grad)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    to_params(p, s->prm);
    const size_t b = sizeof(double) * 3 * s->nv;
    cudaMemcpyAsync(s->xprev.p, x, b, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->xt.p, xtilde, b, cudaMemcpyHostToDevice, s->stream);
    s->nfric = 0;
    int rc = CIPC_OK;
    if (p->with_collision && (rc = build_constraints(s, s->xprev.p))) return rc;
    bool ok = true;
    if ((rc = eval_energy(s, s->xprev.p, energy, &ok))) return rc;
    if (!ok) *energy = NAN;
    if (grad) {
        eval_grad_hess(s, s->xprev.p, s->g.p, false);
        cudaMemcpyAsync(grad, s->g.p, b, cudaMemcpyDeviceToHost, s->stream);
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_sim_eval");
}

extern "C" int cipc_sim_ccd(cipc_sim* h, const cipc_step_params* p, const double* x, const double* dir, double alpha,
                            double* alpha_out)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    to_params(p, s->prm);
    const size_t b = sizeof(double) * 3 * s->nv;
    cudaMemcpyAsync(s->xprev.p, x, b, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->disp.p, dir, b, cudaMemcpyHostToDevice, s->stream);
    return ccd_step_size(s, s->xprev.p, s->disp.p, alpha, alpha_out);
}

extern "C" int cipc_sim_capture_systems(cipc_sim* h, cipc_precond* p, int max_systems)
{
    if (int rc = check_sim(h)) return rc;
    LpModel* m = lp_model(p);
    if (p && !m) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_capture_systems: bad preconditioner handle");
    if (m) m->capture_max = std::max(0, max_systems);
    h->s->capture = (m && max_systems > 0) ? m : nullptr;
    return CIPC_OK;
}

extern "C" int cipc_sim_set_precond(cipc_sim* h, cipc_precond* p)
{
    if (int rc = check_sim(h)) return rc;
    LpModel* m = lp_model(p);
    if (p && !m) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_set_precond: bad preconditioner handle");
    h->s->learned = m;
    return CIPC_OK;
}
