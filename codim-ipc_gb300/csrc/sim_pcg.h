// Graph-replayed fused PCG on the Newton system (sim_pcg.cu).
#pragma once

namespace cipc {

struct Sim;

// Solves H x = b to |r| <= tol |b| with the preconditioner in s->pinv.  x starts
// at zero.  Returns CIPC_OK, CIPC_ERR_NOT_CONVERGED (iteration cap or
// non-positive curvature; x holds the last iterate) or CIPC_ERR_NAN.
int pcg_solve_fp64(Sim* s, const double* b, double* x, double tol, int maxit, int* iters, double* rel);
// FP32 matrix values, vectors and preconditioner; FP64 reductions
int pcg_solve_fp32(Sim* s, const float* b, float* x, double tol, int maxit, int* iters, double* rel);
// the solver-owned FP32 right-hand side and solution vectors (3 nv floats each)
int pcg_fp32_io(Sim* s, float** b, float** x);
// frees the solver's buffers and graph
void pcg_release(Sim* s);

}  // namespace cipc
