// Device-resident state of one shell simulation (one CUDA stream per handle) and
// the internal entry points of the time-step kernels.
#pragma once
#include <string>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <vector>

#include "sl_params.h"

namespace cipc {

// constraint kinds: PP, PE, PT, EE and the mollified edge-edge family whose
// four vertices are the two edges (EEM: ea0 ea1 eb0 eb1, PEM: p p' e0 e1,
// PPM: p p' q q', primed = the other endpoint of the point's edge)
enum ConKind : int { cPP = 0, cPE = 1, cPT = 2, cEE = 3, cEEM = 4, cPEM = 5, cPPM = 6 };

inline bool poison_buffers()
{
    static const bool on = std::getenv("CIPC_POISON") != nullptr;
    return on;
}

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count)
    {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc((void**)&p, (count ? count : 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        // CIPC_POISON set: new buffers start as all-ones bytes (NaN for floating
        // point, -1 for integers) so that a read before the first write shows
        if (e == cudaSuccess && poison_buffers()) e = cudaMemset(p, 0xFF, (count ? count : 1) * sizeof(T));
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct Sim;
// barrier stiffness applied to the constraints: kappa for offset IPC; for elastic
// IPC the reference's normalised barrier -kappa (d/dhat - 1)^2 ln(d/dhat) on
// squared distances (Math/BARRIER.h:9-62, elastic branch) is the offset form with
// kappa / dhat^4
double barrier_kappa(const Sim* s);

// one Init_Dirichlet group: list entries [begin, end) move by rotation about the
// axis through center at ang_deg degrees per second, then by velocity v
struct DbcMotion {
    int begin, end;
    double v[3], center[3], axis[3], ang_deg;
};

struct SimParams {
    double h = 0.04;          // time step
    double dHat2 = 1e-6;      // dhat^2
    double xi = 0;            // offset (thickness)
    double mu = 0;            // friction coefficient
    double epsv2 = 1e-6;      // friction smoothing epsv^2 (times h^2 inside)
    int fricIterAmt = 1;      // friction basis updates per step
    double tol = 1e-2;        // Newton tolerance on RMS(step)/h
    int withCollision = 1;
    int maxIter = 200;        // Newton iteration cap
    int precision = 0;        // 0 FP64 Hessians / PCG, 1 FP32 Hessians + FP32 PCG with FP64 refinement
    double pcg_tol = 1e-6;    // relative residual of the Newton system (FP64)
    int pcg_maxit = 10000;
    int precond = 0;          // 0 block-Jacobi, 1 learned correction (when a model is loaded), 2 aggregate block Jacobi
    int forcing = 0;          // 1: inexact Newton (Eisenstat-Walker forcing term)
    int elastic = 0;          // 1: elastic IPC (no offset, barrier scaled by 1/dhat^4, kappa fixed)
    long long accd_max_iter = 1 << 20;  // ACCD steps per pair in the step-size search
    int accd_cap_strict = 0;  // 1: a pair reaching accd_max_iter ends the step with CIPC_ERR_ITER_CAP
    int pcg_wait_polls = 0;   // PCG grid-wait poll limit (0: the solver's default, over a second)
};

struct StepStats {
    int newton_iters = 0;
    int pcg_iters = 0;        // total inner iterations
    int line_search_trials = 0;
    int n_constraints = 0;
    int status = 0;
    double min_dist2 = 0;
    double kappa = 0;
    double ms = 0;
    int precond_fallbacks = 0;
    int learned_solves = 0;
    double solve_ms = 0;      // device time of the PCG kernels
};

struct Sim {
    // sizes
    int nv = 0, nt = 0, nh = 0, nbn = 0, nbe = 0, nbt = 0;
    int nh_model = 1;
    double lam = 0, mu = 0, kbend = 0;
    double cell = 1;  // broad-phase cell size (mean rest edge length)
    double kappa = 1, kappa_max = 100;
    SlParams sl;              // strain limiting (kappa_s doubles during steps, like kappa)
    int elastic_off = 0;      // energies without membrane, bending, rods, tets (split stepper projection)
    DBuf<double> xsplit;      // split stepper: positions at the start of the step
    DBuf<double> sl_prev;     // per-triangle largest stretch after the previous Newton iteration
    bool sl_have_prev = false;
    int trace = 0;    // CIPC_TRACE set: one stderr line per Newton iteration and refinement pass
    std::string out_dir;  // run logs (residual.txt, counter.txt, Hessian_info.txt, steps.jsonl) when set
    int step_count = 0;   // steps taken (successful or not) since creation or the last restore
    // static device data
    DBuf<int> tri, hinge, bnode, bedge, btri;
    DBuf<double> P, vol, hinfo, mass, b, X0;
    DBuf<uint8_t> dbc;        // Dirichlet vertices (element / constraint exclusion)
    DBuf<uint8_t> proj;       // rows/columns projected out of the Newton system
    DBuf<uint8_t> dbc_fixed;  // Dirichlet vertices whose target equals their position
    double dbc_stiff = 0;     // penalty stiffness of the augmented-Lagrangian Dirichlet path (0 = projection)
    std::vector<int> dbc_idx_h;
    DBuf<int> dbc_idx;
    DBuf<double> dbc_tgt;
    std::vector<DbcMotion> dbc_motion;  // device-side Dirichlet motion groups (ranges of the list above)
    DBuf<DbcMotion> dbc_motion_d;
    // block sparsity of the elastic part (vertex blocks, 3x3) in ELL form: row i's
    // k-th block is block k * nv + i (k < ell_k), column col[k * nv + i]; padding
    // blocks are zero with the row's own column; nnzb = ell_k * nv
    int nnzb = 0, ell_k = 0;
    DBuf<int> col, diag, tri_slot, hinge_slot;
    DBuf<int> rowlen;  // real blocks per row: the rest of a row is zero padding that products skip
    bool rows_uniform = false;  // at least 90% of the row slots are real blocks (products keep the fixed length)
    // rods: segments (2 ints, info E L t), hinges (3 ints, info E*bendMult lsum t), block slots
    int nrs = 0, nrh = 0;
    DBuf<int> rseg, rhinge, rseg_slot, rhinge_slot;
    DBuf<double> rinfo, rhinfo;
    // volumetric Neo-Hookean tetrahedra (Dm^-1 row-major, volume, ELL slots)
    int ntet = 0;
    double tlam = 0, tmu = 0;
    DBuf<int> tet, tet_slot;
    DBuf<double> tDinv, tvol;
    // boundary layout: bnode = [shell | rod nodes from codim0 | particles from codim1],
    // the last nrod_e boundary edges are rod segments
    int codim0 = 0, codim1 = 0, nrod_e = 0;
    // dynamic
    DBuf<double> x, xn, xt, v, g, dir, xprev, rhs, disp;
    DBuf<char> hval;  // BSR values, float or double per precision
    // contact constraint list
    int ncon = 0, cap_con = 0;
    int cap_cand = 0;  // capacity of the broad phase's candidate-pair lists (grown on overflow)
    DBuf<int> ckind, cmult;
    DBuf<int4> cverts;
    DBuf<char> chess;  // 78 entries per constraint (float/double)
    // previous iterate's constraint list and its distances (barrier stiffness update)
    int npcon = 0;
    DBuf<int> pkind;
    DBuf<int4> pverts;
    DBuf<double> pd2;
    // friction (lagged)
    int nfric = 0;
    DBuf<int> fkind, fmult;
    DBuf<int4> fverts;
    DBuf<double> fw, fT, flam;  // 4 weights, 6 basis entries, normal force per friction constraint
    DBuf<char> fhess;
    // block-Jacobi diagonal (9 per vertex, double) and its inverse (float/double)
    DBuf<double> pdiag;
    DBuf<char> pinv;
    // Newton operator of the linear solve: the block rows with every contact and
    // friction constraint folded in whose free-vertex pairs all have a block there
    // (hval_op, float/double per precision), and the constraints left to apply
    // matrix-free (crest, frest; their counts on the device in fold_cnt[0..1])
    bool folded = false;
    DBuf<char> hval_op;
    DBuf<int> crest, frest, fold_cnt;
    // aggregate block Jacobi (sim_aggregate.cu): vertex aggregates built once per
    // mesh and the inverses of their diagonal blocks; agg_ready: the inverses
    // belong to the current Newton system
    void* agg = nullptr;
    bool agg_ready = false;
    // scratch
    DBuf<double> red;               // reduction partials
    DBuf<unsigned long long> cnt;   // counters
    DBuf<char> scratch;             // broad-phase / solver work space
    size_t scratch_bytes = 0;
    cudaStream_t stream = nullptr;
    SimParams prm;
    StepStats last;
    // graph-replayed PCG (sim_pcg.cu)
    void* pcg = nullptr;
    // learned preconditioner (LpModel, optional): used when prm.precond == 1;
    // capture: every solved Newton system is appended to that model's data
    void* learned = nullptr;
    void* capture = nullptr;
    int solve_fallbacks = 0, solve_learned = 0;  // counts of the current step
    double solve_ms = 0;                         // device time of the current step's PCG kernels
    int bj_last_iters = 0;                       // iterations of the step's latest block-Jacobi solve (0: none yet)
    double solve_tol = 0;                        // relative tolerance of the next linear solve (0: prm.pcg_tol)
    std::vector<double> host_mass;
};

// host-side construction (sim_setup.cpp)
struct CodimDesc;
struct TetDesc;
int sim_create(Sim** out, int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
               double thickness, const double* gravity, double bendMult, int nh_model, const CodimDesc* cd = nullptr,
               const TetDesc* td = nullptr);
void sim_destroy(Sim* s);
int sim_step(Sim* s, StepStats* st);
int sim_step_split(Sim* s, StepStats* st);

}  // namespace cipc
