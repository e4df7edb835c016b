// Learned block-Jacobi correction for the Newton-system PCG (learned.cu).
//
// A small message-passing network over the vertices of the Newton system (edges:
// the elastic off-diagonal blocks, plus the vertex groups of the active contact
// constraints) maps scale-free features of each vertex's diagonal block and
// couplings to a lower-triangular 3x3 Cm_i; the preconditioner block is
// P_i = Cm_i D_i^-1 Cm_i^T (SPD whenever D_i is), so with the output layer at zero
// it is plain block Jacobi.  It is trained on (H, r, p) triples captured from the
// plain solver: loss 1 - (z.r)^2 / ((z.Hz)(r.p)) with z = P r, the relative
// H-norm error left after one preconditioned step.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/cipc.h"
#include "sim.h"

namespace cipc {

constexpr int kLpFeatures = 10, kLpOut = 6, kLpPsdSteps = 8;

// One captured Newton system, FP32, on the device.
struct LpTriple {
    int nv = 0, K = 0, ncon = 0, nfric = 0;
    DBuf<int> col, diag;     // ELL pattern (K*nv) and each row's diagonal block index
    DBuf<float> val;         // 9 per ELL block
    DBuf<float> cdiag;       // 9 per vertex: contact + friction part of the diagonal block
    DBuf<uint8_t> proj;      // Dirichlet rows
    DBuf<int> ckind;         // contact constraints
    DBuf<int4> cverts;
    DBuf<float> chess;       // 78 per constraint, entry h of constraint c at h * ncon + c
    DBuf<int> fkind;         // friction constraints
    DBuf<int4> fverts;
    DBuf<float> fw, fT, fM;  // 4, 6, 3 per friction constraint
    DBuf<float> r, p;        // right-hand side and solution (3 nv)
    void release();
};

// Network parameters, Adam state, captured triples and work buffers.
struct LpModel {
    int H = 32, L = 2, nparams = 0;
    // 0: 1 - (z.r)^2/((z.Hz)(r.p)); 1: |z - p|_H^2 / |p|_H^2; 2: |e_k|_H^2 / |p|_H^2
    // after k steps of preconditioned steepest descent from 0 (kLpPsdSteps)
    int loss_kind = 2;
    uint64_t seed = 0;
    DBuf<float> params, grad, adam_m, adam_v;
    DBuf<uint16_t> wbf16;    // BF16 copy of the dense-layer weights for inference
    bool wbf16_valid = false;
    int adam_t = 0;
    std::vector<LpTriple*> data;
    int capture_max = 0;
    // work buffers (sized for the largest system seen)
    int cap_nv = 0, cap_k = 0, cap_con = 0;
    DBuf<float> X, E, Dn, a, s, u0, o, z, hz, dz, dout, dh, dh2, du, dg, dc, acc;
    DBuf<float> h, g, c, u;  // (L+1) or L layers of nv x H
    DBuf<float> Pm, Gb, psd;  // preconditioner blocks, their adjoint, steepest-descent vectors
    DBuf<int> ncnt;
    DBuf<double> red;
    cudaStream_t stream = nullptr;
    ~LpModel();
};

// A Newton system as the network sees it (live simulation or captured triple).
template <typename VT, typename CT>
struct LpSys {
    int nv, K;
    const int* col;
    const int* diag;
    const VT* val;
    const CT* cdiag;
    const uint8_t* proj;
    int ncon;
    const int* ckind;
    const int4* cverts;
};

int lp_create(int hidden, int layers, uint64_t seed, LpModel** out);
// Writes the learned preconditioner of the simulation's current Newton system
// into s->pinv (precision of the solve); returns CIPC_OK or an error.
int lp_precond(Sim* s, LpModel* m);
// Appends the simulation's current Newton system and its solution to m's data.
int lp_capture(Sim* s, LpModel* m, const double* rhs, const double* sol);
// Adam on the captured systems; mean loss before / after (optional)
int lp_train(LpModel* m, int epochs, int batch, double lr, uint64_t seed, double* before, double* after);
// the model behind a C-ABI handle (nullptr for a null handle)
LpModel* lp_model(::cipc_precond* p);

}  // namespace cipc
