// Launchers of the time-step kernels (all enqueue on Sim::stream).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "sim.h"

namespace cipc {

struct ElasticArgs {
    int nt, nh;
    const int *tri, *hinge;
    const double *P, *vol, *hinfo;
    const int *tri_slot, *hinge_slot;
    const uint8_t* dbc;   // element skip: all vertices Dirichlet
    const uint8_t* proj;  // Hessian rows/columns projected out
    const double* x;
    double* g;
    double h, lam, mu, kbend;
    int nh_model;
    double* red;
    // rods
    int nrs, nrh;
    const int *rseg, *rhinge, *rseg_slot, *rhinge_slot;
    const double *rinfo, *rhinfo;
    // strain limiting (on when sl.k0 > 0); flag set to 1 by an infeasible triangle
    // or tetrahedron
    SlParams sl;
    double* flag;
    // membrane off (the split stepper's projection substep keeps only inertia,
    // strain limiting and contact)
    int skip_membrane;
    // volumetric Neo-Hookean tetrahedra
    int ntet;
    const int *tet, *tet_slot;
    const double *tDinv, *tvol;
    double tlam, tmu;
};

// sim_elastic.cu
void launch_xtilde(Sim* s);
int elastic_energy_partials(Sim* s, const double* x, double* red, double* flag);  // returns #partials written
int elastic_feasible(Sim* s, const double* x, bool* ok);         // stretches within the strain limits, tets not inverted
int strain_kappa_update(Sim* s, const double* x, bool* raise);   // kappa_s doubling test; updates the history
void elastic_grad_hess(Sim* s, const double* x, double* g, bool want_hess);
void zero_dbc(Sim* s, double* g);
int dbc_penalty_partials(Sim* s, const double* x, double* red, double* g);  // energy partials (+ gradient if g)
double dbc_dist2(Sim* s, const double* x);                                   // sum |target - x|^2 (host value)
void sum_partials(Sim* s, const double* red, int n, double* out);

// sim_contact.cu
int build_constraints(Sim* s, const double* x);           // fills the constraint list; status code
int contact_energy_partials(Sim* s, const double* x, double* red, double* flag);  // #partials; flag: s <= 0 seen
void contact_grad_hess(Sim* s, const double* x, double* g, bool want_hess);
void min_dist2_partials(Sim* s, const double* x, double* out_min);  // device scalar
int friction_basis(Sim* s, const double* x);               // lagged basis from the current constraint list
int friction_energy_partials(Sim* s, const double* x, double* red);
void friction_grad_hess(Sim* s, const double* x, double* g, bool want_hess);
int ccd_step_size(Sim* s, const double* x, const double* p, double alpha_in, double* alpha_out);
void kappa_check(Sim* s, const double* x, int* update_flag_dev);  // uses the previous constraint list

// sim_solve.cu
int linear_solve(Sim* s, const double* rhs, double* sol, int* iters);

// sim_fold.cu: builds the solver's operator (s->hval_op and the matrix-free rest
// lists; s->folded) from the assembled rows and constraint Hessians
int fold_constraints(Sim* s);
bool fold_enabled();

// sim_aggregate.cu: aggregate block Jacobi.  agg_setup builds (once per mesh) the
// vertex aggregates and, for the current Newton system (after fold_constraints),
// the inverses of the aggregates' diagonal blocks; sets s->agg_ready, or returns
// CIPC_ERR_NOT_CONVERGED when a block is not positive definite (the caller then
// uses block Jacobi).  agg_view fills the solver's view of the inverses.
int agg_setup(Sim* s);
struct AggView {
    int nagg;
    const int* voff;        // nagg + 1 offsets into verts
    const int* verts;       // vertices by aggregate
    const long long* boff;  // nagg + 1 offsets of the dense inverse blocks (entries)
    const void* inv;        // inverses (float or double per precision), symmetric m x m, m = 3 x vertices
};
AggView agg_view(const Sim* s);
// The solver's rounds of aggregates for a grid of `grid` blocks: block b owns a
// contiguous range of aggregates of about equal cost (the solver's items, of
// `loads` loads per lane, and rows), cut into rounds of at most `rows` scalar
// rows and `maxagg` aggregates; rounds [bround[b], bround[b + 1]) of block b,
// round q = aggregates [rstart[q], rstart[q + 1]).  Built on the host when the
// grid or the limits change (device arrays owned by the aggregate state).
int agg_rounds(Sim* s, int grid, int rows, int maxagg, int loads, const int** bround, const int** rstart);
void agg_release(Sim* s);

}  // namespace cipc
