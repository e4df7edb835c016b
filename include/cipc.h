/*
 * cipc.h — C ABI of the GB300 contact + Newton hot path for codimensional IPC.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (CIPC_OK = 0).  Buffers are host memory when `mem` is CIPC_MEM_HOST (the call
 * copies them to the GPU, runs, copies results back and waits) or device memory
 * when `mem` is CIPC_MEM_DEVICE (the call only enqueues work on `stream`; scalar
 * out-parameters such as counts are host pointers and, when non-NULL, make the
 * call wait for the stream).  `stream` is a cudaStream_t or NULL for the legacy
 * default stream.  A status other than CIPC_OK leaves a message for
 * cipc_last_error() on the calling thread.
 *
 * Pair encoding.  A contact pair is type[i] in {0 PP, 1 PE, 2 PT, 3 EE} and four
 * vertex indices idx[4*i .. 4*i+3]:
 *   PP (p0, p1, -, -)   PE (p, e0, e1, -)   PT (p, t0, t1, t2)   EE (ea0, ea1, eb0, eb1)
 * Unused slots are ignored.  Positions are n_verts x 3 doubles.  The reference
 * packs the same four cases into sign-encoded Vector4i constraint codes
 * (Library/FEM/IPC.h:571-661); cipc_encode_reference_constraint converts.
 */
#ifndef CIPC_H
#define CIPC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CIPC_OK 0
#define CIPC_ERR_INVALID_ARG 1
#define CIPC_ERR_CUDA 2
#define CIPC_ERR_ITER_CAP 3
#define CIPC_ERR_NONPOSITIVE_DISTANCE 4
#define CIPC_ERR_NOT_CONVERGED 5
#define CIPC_ERR_NAN 6
#define CIPC_ERR_NO_DEVICE 7
#define CIPC_ERR_INDEX_RANGE 8
#define CIPC_ERR_TIMEOUT 9 /* a bounded device-side wait gave up (the kernel returned, the context is usable) */

/* CIPC_PRECISION_FP64: every value that reaches a result is FP64; decisions and
 * results are bit-identical to the CPU restatement.  Distance-type decisions are
 * taken by a certified FP32 evaluation when it is certain (it returns the FP64
 * decision or defers to FP64), which does not change any result.
 * CIPC_PRECISION_MIXED: for the pair CCD, distances and times in float-float (FP32
 * pairs, ~47 bits) from FP64 vertex differences -- NOT bit-exact and NOT
 * guaranteed conservative: on seeded benchmark pairs ~1e-5 of the hit/miss
 * decisions differ from FP64, in both directions, and a shared hit's time can be
 * later than FP64's.  For the barrier pairs and the time step: FP32 Hessians and
 * PCG (inside FP64 iterative refinement); distances, constraint sets, CCD step
 * sizes, energies and gradients stay FP64. */
#define CIPC_PRECISION_FP64 0
#define CIPC_PRECISION_MIXED 1
#define CIPC_BARRIER_OFFSET 0  /* offset IPC (C-IPC): barrier on d^2 - xi^2 */
#define CIPC_BARRIER_ELASTIC 1 /* elastic IPC: no offset, barrier normalised by dhat */
#define CIPC_PRECOND_BLOCK_JACOBI 0
#define CIPC_PRECOND_LEARNED 1
#define CIPC_PRECOND_AGGREGATE 2

#define CIPC_MEM_HOST 0
#define CIPC_MEM_DEVICE 1

#define CIPC_PAIR_PP 0
#define CIPC_PAIR_PE 1
#define CIPC_PAIR_PT 2
#define CIPC_PAIR_EE 3

/* Library identification and error reporting. */
const char* cipc_version(void);
const char* cipc_last_error(void);
const char* cipc_status_string(int status);
int cipc_device_count(void);

/*
 * Additive CCD over candidate pairs.
 *
 * Replaces the narrow-phase calls Point_Triangle_CCD / Edge_Edge_CCD /
 * Point_Edge_CCD / Point_Point_CCD (Library/Math/Distance/CCD.h:279-483) that
 * Compute_Intersection_Free_StepSize makes per candidate
 * (Library/FEM/IPC.h:1959-2242).  dx is the full displacement, toc_in the step
 * fraction the reference passes as `toc` (its largest allowed step).
 * Outputs per pair: hit[i] = 1 when a time of impact below toc_in exists, and
 * toc_out[i] = that conservative time (eta-scaled, thickness-offset), else toc_in.
 * *n_overflow (optional) receives the number of pairs that reached the
 * iteration cap (2^20 steps) — they are reported as no hit; with any overflow the
 * call returns CIPC_ERR_ITER_CAP.  Pairs with an index outside [0, n_verts) or a
 * type above 3 are not evaluated and make the call return CIPC_ERR_INDEX_RANGE.
 * With CIPC_MEM_HOST the call returns after the results are back.  Page-locked
 * host buffers (cudaHostAlloc / cudaHostRegister, e.g. pinned tensors) are read
 * and written in place by the kernel over the CPU-GPU link (NVLink-C2C on
 * Grace-Blackwell), with no staging copies.  Pageable host buffers are staged
 * in stream-ordered allocations; n_pairs above 2.5M are then streamed in chunks
 * (records in, results out) around the kernel on internal streams.
 */
int cipc_ccd_pairs(int64_t n_pairs, const uint8_t* type, const int32_t* idx, int64_t n_verts,
                   const double* x, const double* dx, double eta, double thickness, double toc_in,
                   int precision, int mem, double* toc_out, uint8_t* hit, int64_t* n_overflow,
                   void* stream);

/*
 * cipc_ccd_pairs for callers that must not allocate device memory (no reference
 * counterpart: the reference's CCD runs on the host).
 *
 * Same pairs, same kernels and the same outputs and status codes as
 * cipc_ccd_pairs with mem = CIPC_MEM_DEVICE, but the three counters the kernel
 * needs (work counter, overflow count, invalid-pair count) come from a fixed
 * scratch array compiled into the library instead of cudaMallocAsync: no
 * cudaMalloc / cudaMallocAsync / cudaFree call, and no library call that
 * allocates.  All buffers must already be in device memory of the current device.
 *
 * The scratch holds CIPC_NOALLOC_SLOTS slots of CIPC_NOALLOC_SLOT_BYTES; `slot`
 * picks one (0 <= slot < CIPC_NOALLOC_SLOTS, anything else is rejected with
 * CIPC_ERR_INVALID_ARG).  The call zeroes its slot on `stream` before the launch
 * (the counters must start at zero).  Two calls that overlap in time on the same
 * device and the same slot race on its counters and give wrong results: give
 * each stream that may run concurrently its own slot, or order the calls.
 * The first call on each device, and the first call after the device's context
 * was replaced (cudaDeviceReset), looks up the scratch array's device address
 * (cudaGetSymbolAddress, which may load the library's kernels on that device);
 * make that first call outside any stream capture.  With n_overflow == NULL the
 * call only enqueues work on `stream` and reports no kernel-side counts.
 */
#define CIPC_NOALLOC_SLOTS 16
#define CIPC_NOALLOC_SLOT_BYTES 128
int cipc_ccd_pairs_noalloc(int64_t n_pairs, const uint8_t* type, const int32_t* idx, int64_t n_verts,
                           const double* x, const double* dx, double eta, double thickness, double toc_in,
                           int precision, int slot, double* toc_out, uint8_t* hit, int64_t* n_overflow,
                           void* stream);

/*
 * Barrier energy, gradient and PSD-projected Hessian per contact pair.
 *
 * Replaces the per-constraint bodies of Compute_Barrier, Compute_Barrier_Gradient
 * and Compute_Barrier_Hessian (Library/FEM/IPC.h:742-1731) for weight 1 and
 * multiplicity 1, using the thickness-offset barrier of IPC.h:756-757 and
 * Library/Math/BARRIER.h:9-62: s = d^2 - xi^2, shat = dhat2 + 2 sqrt(dhat2) xi,
 * b(s) = -kappa (s - shat)^2 ln(s / shat).  EE pairs take the mollified form when
 * |ea x eb|^2 < 1e-3 |ea_rest|^2 |eb_rest|^2 (EDGE_EDGE_MOLLIFIER.h:582-591).
 * Outputs: energy[i]; grad[12*i + k] (first 3*nv used, rest zero); hess[78*i + k] =
 * upper triangle of the (3nv x 3nv) Hessian packed row by row (first
 * 3nv(3nv+1)/2 used, rest zero), doubles for CIPC_PRECISION_FP64 and floats for
 * CIPC_PRECISION_MIXED.  Pairs with s >= shat are inactive (all zeros).  Pairs
 * with s <= 0 are counted in *n_nonpositive (optional) and make the call return
 * CIPC_ERR_NONPOSITIVE_DISTANCE (the reference exits there, IPC.h:773-776).
 */
int cipc_barrier_pairs(int64_t n_pairs, const uint8_t* type, const int32_t* idx, int64_t n_verts,
                       const double* x, const double* x_rest, double dhat2, double xi, double kappa,
                       int project_pd, int precision, int mem, double* energy, double* grad, void* hess,
                       int64_t* n_nonpositive, void* stream);

/*
 * Converts one pair to the reference's sign-encoded constraint code
 * (Library/FEM/IPC.h:571-661 for the 3D merge, :776-930 for decoding):
 *   PT (-p-1, t0, t1, t2)  PE (-p-1, e0, e1, -mult)  PP (-p0-1, p1, -1, -mult)
 *   EE (ea0, ea1, eb0, eb1);  mollified EE (ea0, ea1, -eb0-1, eb1).
 * mult is the PE/PP multiplicity (1 when not merged).  Returns CIPC_OK.
 */
int cipc_encode_reference_constraint(int type, const int32_t* idx4, int mollified, int multiplicity,
                                     int32_t* code4);

/* ------------------------------------------------------------------------
 * Shell simulation: one implicit-Euler time step of codimensional shells with
 * offset IPC contact and lagged friction, on one GPU.
 * ------------------------------------------------------------------------ */

/* Step parameters; the fields mirror the arguments of the reference's
 * FEM.DiscreteShell.Advance_One_Step_IE_Hinge (Library/FEM/Shell/DISCRETE_SHELL.h:1108,
 * IMPLICIT_EULER.h:151-187) that this path uses. */
typedef struct cipc_step_params {
    double h;              /* dt */
    double dhat2;          /* dHat2 (dhat squared) */
    double xi;             /* thickness offset of the barrier (the driver's `thickness`) */
    double mu;             /* friction coefficient */
    double epsv2;          /* friction smoothing epsv^2 (scaled by h^2 inside) */
    int fric_iters;        /* fricIterAmt */
    double newton_tol;     /* PNTol: RMS(Newton step) / h */
    int with_collision;    /* withCollision */
    int max_newton_iters;  /* safety cap (0 = 200) */
    int precision;         /* CIPC_PRECISION_FP64 or CIPC_PRECISION_MIXED */
    double pcg_tol;        /* relative residual of each Newton system (0 = 1e-6) */
    int pcg_max_iters;     /* 0 = 10000 */
    int preconditioner;    /* CIPC_PRECOND_BLOCK_JACOBI (0), CIPC_PRECOND_LEARNED (1: the
                              learned correction when a model is set, else block Jacobi) or
                              CIPC_PRECOND_AGGREGATE (2: exact inverses of the diagonal blocks
                              of vertex aggregates of up to 32 mesh neighbours; block Jacobi
                              for a system where one is not positive definite) */
    int forcing;           /* 0: every Newton system to pcg_tol; 1: inexact Newton, the
                              Eisenstat-Walker forcing term (choice 2, gamma 0.9, alpha 2)
                              clamped to [pcg_tol, 0.1], pcg_tol once RMS(step)/h < 10 tol;
                              ignored while the learned preconditioner is in use */
    int barrier_model;     /* CIPC_BARRIER_OFFSET (0, Advance_One_Step_IE_Hinge) or
                              CIPC_BARRIER_ELASTIC (1, Advance_One_Step_IE_Hinge_EIPC:
                              no offset, normalised barrier, kappa not adapted) */
    int accd_max_iters;    /* ACCD steps per candidate pair in the step-size search (the
                              reference's CCD loop has no bound, CCD.h:279-483).  0: 2^20, and
                              a pair that reaches it lowers the step to the time it has safely
                              advanced to (a conservative bound; grazing, sliding contact can
                              take that long).  > 0: that cap, and a pair that reaches it ends
                              the step with CIPC_ERR_ITER_CAP */
    int pcg_wait_polls;    /* polls of a grid-wide wait inside the PCG kernel before it gives
                              up (0 = 2^22, over a second); giving up ends the linear solve,
                              and the step, with CIPC_ERR_TIMEOUT */
} cipc_step_params;

typedef struct cipc_step_stats {
    int newton_iters;       /* the reference's return value (PNIter) */
    int pcg_iters;
    int line_search_trials;
    int n_constraints;
    int status;
    double min_dist2;       /* min over constraints of d^2 - xi^2 at the end of the step */
    double kappa;           /* barrier stiffness after the step (kappaVec[0]) */
    double ms;              /* wall time of the step */
    int precond_fallbacks;  /* linear solves where the learned preconditioner stalled and block Jacobi re-solved */
    int learned_solves;     /* linear solves that used the learned preconditioner */
    double solve_ms;        /* device time of the step's PCG kernels (CUDA events on the
                               simulation's stream around each launch) */
} cipc_step_stats;

typedef struct cipc_sim cipc_sim;

/* Creates a simulation of the shell mesh (nv vertices, nt triangles) with the
 * reference's shell initialization (Initialize_Shell_Hinge_EIPC ->
 * Initialize_Discrete_Shell, DISCRETE_SHELL.h:218-357): lumped mass, body force
 * mass*gravity, inverse rest fundamental forms, hinges, plane-stress material.
 * membrane_model: 1 Neo-Hookean (the reference's default useNH), 0 StVK. */
int cipc_sim_create(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                    double thickness, const double* gravity, double bend_stiff_mult, int membrane_model,
                    cipc_sim** out);
/* Codimensional parts added to a shell scene (all vertices live in X):
 * discrete rods (Make_Rod + Initialize_Discrete_Rod, Library/FEM/Shell/Rod/
 * DISCRETE_ROD.h:85-150: segment mass, stretching and bending with hinges between
 * every pair of segments meeting at a vertex) and particles
 * (Initialize_Discrete_Particle, Library/FEM/Shell/DISCRETE_PARTICLE.h:52-75).
 * Rod nodes and particles take part in contact as the reference's codimensional
 * boundary nodes, rod segments as boundary edges (IMPLICIT_EULER.h:242-277). */
typedef struct cipc_codim_desc {
    int n_segments;
    const int32_t* segments;  /* 2 vertex indices per rod segment */
    double rod_E, rod_rho, rod_thickness, rod_bend_mult;
    int n_particles;
    const int32_t* particles; /* particle vertex indices */
    double particle_rho, particle_thickness;
} cipc_codim_desc;
int cipc_sim_create_codim(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                          double thickness, const double* gravity, double bend_stiff_mult, int membrane_model,
                          const cipc_codim_desc* codim, cipc_sim** out);
/* Volumetric tetrahedra (the drivers' add_object_3D + initialize of a tet mesh:
 * FEM.Compute_Vol_And_Inv_Basis, DEFORMATION_GRADIENT.h:39-76; lumped mass;
 * Neo-Hookean material, NEOHOOKEAN.h, in the step via INC_POTENTIAL.h:97-109,
 * 228-229, 354-364).  Their surface triangles (Find_Surface_TriMesh,
 * MESHIO.h:486-544) take part in contact ahead of the shell triangles
 * (IMPLICIT_EULER.h:235-241).  Tetrahedra must be positively oriented. */
typedef struct cipc_tet_desc {
    int n_tets;
    const int32_t* tets; /* 4 vertex indices per tetrahedron */
    double E, nu, rho;
} cipc_tet_desc;
/* Shell + optional codimensional parts + optional tetrahedra (either may be NULL). */
int cipc_sim_create_full(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                         double thickness, const double* gravity, double bend_stiff_mult, int membrane_model,
                         const cipc_codim_desc* codim, const cipc_tet_desc* tets, cipc_sim** out);
int cipc_sim_destroy(cipc_sim* sim);
/* Offset-IPC barrier stiffness; replaces FEM.DiscreteShell.Initialize_OIPC
 * (DISCRETE_SHELL.h:555-577, export :1103).  Writes (kappa, kappa_max) and dhat^2. */
int cipc_sim_init_oipc(cipc_sim* sim, double dhat, double stiff_mult, double* kappa2, double* dhat2);
/* The same stiffness from a scene description alone (the arguments of
 * cipc_sim_create_full), computed on the host with no device: what
 * FEM.DiscreteShell.Initialize_OIPC returns at set-up time, before a simulation
 * exists on the GPU. */
int cipc_scene_oipc_kappa(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                          double thickness, const double* gravity, double bend_stiff_mult, int membrane_model,
                          const cipc_codim_desc* codim, const cipc_tet_desc* tets, double dhat, double stiff_mult,
                          double* kappa2, double* dhat2);
/* Elastic-IPC stiffness; replaces FEM.DiscreteShell.Initialize_EIPC
 * (DISCRETE_SHELL.h:555-577, export :1102): kappa3 = (h^2 mu, h^2 lambda, nu) of the
 * plane-stress material, dhat^2 = thickness^2; sets the simulation's kappa. */
int cipc_sim_init_eipc(cipc_sim* sim, double E, double nu, double thickness, double dt, double* kappa3,
                       double* dhat2);
int cipc_sim_set_kappa(cipc_sim* sim, double kappa, double kappa_max);
int cipc_sim_get_kappa(cipc_sim* sim, double* kappa2);
/* Isotropic strain limiting (Library/FEM/Shell/INEXT.h; the driver's s, sHat and
 * kappa_s, passed to Advance_One_Step_IE_Hinge, IMPLICIT_EULER.h:162): a barrier
 * keeps every triangle's stretches (singular values of its deformation) below
 * s[0], active above s_hat[0] with stiffness h^2 vol kappa_s[0], and above s[1]
 * when kappa_s[1] > 0.  kappa_s[0] = 0 (the default) turns it off.  kappa_s[0]
 * doubles (up to 1e5) when a triangle stays within 1e-4 (s[0] - s_hat[0]) of the
 * limit, and keeps its value across steps (read it back with
 * cipc_sim_get_strain_limit). */
int cipc_sim_set_strain_limit(cipc_sim* sim, const double* s, const double* s_hat, const double* kappa_s);
int cipc_sim_get_strain_limit(cipc_sim* sim, double* kappa_s);
/* Positions / velocities, host arrays nv x 3 (either may be NULL). */
int cipc_sim_set_state(cipc_sim* sim, const double* x, const double* v);
int cipc_sim_get_state(cipc_sim* sim, double* x, double* v);
/* Dirichlet vertices and their targets for the next step (the DBC storage of the
 * reference, moved by FEM.Step_Dirichlet on the host). */
int cipc_sim_set_dbc(cipc_sim* sim, int n, const int* idx, const double* targets);
/* Device-side Dirichlet motion; replaces FEM.Init_Dirichlet / FEM.Step_Dirichlet
 * (Library/FEM/BOUNDARY_CONDITION.h:16-157).  init: the vertices of [v_begin,
 * v_end) (v_end < 0: to the last vertex) whose current positions lie in the box
 * rel_min..rel_max, relative to that range's bounding box, are appended to the
 * Dirichlet list with their positions as targets, as one motion group (velocity
 * v; rotation about rot_axis through rot_center at ang_vel_deg degrees per
 * second); *added = their count.  step: advances every group's targets by dt on
 * the device (rotation, then translation).  cipc_sim_set_dbc replaces the list
 * and drops the motions.  get: copies up to cap indices / targets of the list. */
int cipc_sim_init_dirichlet(cipc_sim* sim, const double* rel_min, const double* rel_max, const double* v,
                            const double* rot_center, const double* rot_axis, double ang_vel_deg, int v_begin,
                            int v_end, int* added);
int cipc_sim_step_dirichlet(cipc_sim* sim, double dt);
int cipc_sim_get_dbc(cipc_sim* sim, int cap, int* idx, double* targets, int* count);
/* Writes the current positions and the shell triangles as an OBJ file in the
 * reference's format (Write_TriMesh_Obj, Library/Utils/MESHIO.h:182-213). */
int cipc_sim_write_obj(cipc_sim* sim, const char* path);
/* Run logs in the reference's formats, appended in `folder` during steps
 * (Advance_One_Step_IE_Hinge's outputFolder argument): residual.txt, one line
 * "PNIter avgResMag maxRes Eprev L2Norm" per Newton iteration
 * (IMPLICIT_EULER.h:647-670); counter.txt, "PNIter #constraints" per step
 * (:868-875); Hessian_info.txt when a Newton system could not be solved
 * (:531-534); steps.jsonl, one JSON object of cipc_step_stats per step.
 * NULL or "" turns logging off (the default). */
int cipc_sim_set_output(cipc_sim* sim, const char* folder);
/* Checkpoint of a run: positions and velocities (bit for bit), the barrier
 * stiffness and its maximum (kappaVec, kept across steps by the reference only
 * in memory, IMPLICIT_EULER.h:578-580), the strain-limit stiffness and the step
 * count.  load checks the vertex count; the mesh, materials and Dirichlet setup
 * come from the simulation it is loaded into. */
int cipc_sim_save_state(cipc_sim* sim, const char* path);
int cipc_sim_load_state(cipc_sim* sim, const char* path);
/* The reference drivers' restart (load_frame + load_velocity,
 * Python/Drivers/FEMDiscreteShellBase.py:244-253; Load_Velocity,
 * Library/Utils/MESHIO.h:967-984): positions from the vertex lines of obj_last,
 * velocities (obj_last - obj_prev) / dt, or zero when obj_prev is NULL. */
int cipc_sim_load_obj_frames(cipc_sim* sim, const char* obj_prev, const char* obj_last, double dt);
/* One time step; replaces Advance_One_Step_IE_Hinge (IMPLICIT_EULER.h:151-902).
 * Returns CIPC_OK, or CIPC_ERR_NOT_CONVERGED when the Newton cap is reached or
 * the Dirichlet motion is blocked by contact (stats->status -1 / -2). */
int cipc_sim_step(cipc_sim* sim, const cipc_step_params* params, cipc_step_stats* stats);
/* Split stepper; replaces Advance_One_Step_SIE_Hinge (SPLITTING_IE.h:362-729,
 * export DISCRETE_SHELL.h:1115): an implicit-Euler substep without contact and
 * strain limiting, then a projection substep minimising 1/2 |x - x'|_M^2 + strain
 * barrier + contact barrier + friction from x^n.  stats->newton_iters counts both
 * substeps' Newton iterations. */
int cipc_sim_step_split(cipc_sim* sim, const cipc_step_params* params, cipc_step_stats* stats);
/* Parity entry points: the constraint set at x (rows of kind, v0..v3, multiplicity;
 * kinds 0 PP 1 PE 2 PT 3 EE 4 mollified EE 5 mollified PE 6 mollified PP), the
 * incremental potential and its gradient at x for a given x~, and the
 * intersection-free step size along dir (Compute_Intersection_Free_StepSize). */
int cipc_sim_constraints(cipc_sim* sim, const cipc_step_params* params, const double* x, int cap, int* out6,
                         int* count);
int cipc_sim_eval(cipc_sim* sim, const cipc_step_params* params, const double* x, const double* xtilde,
                  double* energy, double* grad);
int cipc_sim_ccd(cipc_sim* sim, const cipc_step_params* params, const double* x, const double* dir, double alpha,
                 double* alpha_out);

/* ------------------------------------------------------------------------
 * Learned block-Jacobi correction for the Newton-system PCG (no reference
 * counterpart: the reference factorizes every Newton system with CHOLMOD,
 * Library/Math/DIRECT_SOLVER.h:13-88, and has no iterative solver to precondition).
 *
 * A message-passing network over the vertices of the Newton system (edges: the
 * elastic off-diagonal blocks and the active contact constraints) maps
 * scale-free features of each vertex's 3x3 diagonal block D_i and couplings to a
 * lower-triangular Cm_i; the preconditioner block is Cm_i D_i^-1 Cm_i^T, so the
 * untrained network (zero output layer) is plain block Jacobi.  PCG still stops
 * at the same relative residual, so the network changes iteration counts, not
 * answers; a solve that stalls or breaks down is repeated with block Jacobi.
 * Training data are the (H, r, p) systems the solver itself produces: attach a
 * preconditioner with cipc_sim_capture_systems, step, then train.  Loss per
 * system: 1 - (z.r)^2 / ((z.Hz)(r.p)), z = M^-1 r, the relative H-norm error
 * left after one preconditioned step.  All work runs on the current device;
 * a handle is not thread-safe and must outlive the simulations using it.
 * ------------------------------------------------------------------------ */
typedef struct cipc_precond cipc_precond;

/* hidden: 16 or 32 channels; layers: 1..8 message-passing layers; seed fixes the
 * initial weights. */
int cipc_precond_create(int hidden, int layers, uint64_t seed, cipc_precond** out);
int cipc_precond_destroy(cipc_precond* p);
/* number of float parameters (or -1 for a bad handle); get/set copy them host-side */
int cipc_precond_num_params(const cipc_precond* p);
int cipc_precond_get_params(const cipc_precond* p, float* out);
int cipc_precond_set_params(cipc_precond* p, const float* in);
/* training loss per system (z = M^-1 r, p = H^-1 r, errors in the H-norm relative to
 * |p|_H): 0 the error after one optimally scaled preconditioned step,
 * 1 - (z.r)^2 / ((z.Hz)(r.p)); 1 the error of the unit step |z - p|_H^2 / |p|_H^2;
 * 2 (default) the error after 8 steps of preconditioned steepest descent from 0,
 * which depends on the whole spectrum of M^-1 H as PCG's convergence does */
int cipc_precond_set_loss(cipc_precond* p, int kind);
/* captured Newton systems: count (or -1) and clearing */
int cipc_precond_num_systems(const cipc_precond* p);
int cipc_precond_clear_systems(cipc_precond* p);
/* Adam over the captured systems (minibatches of `batch` systems, `epochs` passes,
 * order shuffled with `seed`); mean loss before and after training (optional). */
int cipc_precond_train(cipc_precond* p, int epochs, int batch, double lr, uint64_t seed, double* loss_before,
                       double* loss_after);
/* Loss of captured system `system` and the parameter gradient (num_params floats,
 * optional) at the current parameters. */
int cipc_precond_loss_grad(cipc_precond* p, int system, double* loss, float* grad);
/* sizes4 = (n_verts, ell_k, n_contacts, n_friction) of a captured system, and its
 * arrays: ELL columns (ell_k x n_verts, block k of row i at k*n_verts+i), ELL blocks
 * (9 floats each), contact/friction part of the diagonal blocks (9 per vertex),
 * Dirichlet mask, contact kinds and vertices (4 per contact), contact blocks (78
 * per contact, packed upper triangle row by row), right-hand side and solution
 * (3 per vertex).  Any output may be NULL. */
int cipc_precond_system_sizes(const cipc_precond* p, int system, int32_t* sizes4);
/* Network outputs (6 per vertex) and preconditioner blocks (9 per vertex) for
 * captured system `system`: bf16 = 1 runs the inference path the solver uses
 * (message-passing layers on the BF16 tensor cores, FP32 accumulate), 0 the FP32
 * training forward.  Either output may be NULL. */
int cipc_precond_infer(cipc_precond* p, int system, int bf16, float* out6, float* blocks9);
int cipc_precond_system_export(const cipc_precond* p, int system, int32_t* col, float* val, float* cdiag,
                               uint8_t* proj, int32_t* ckind, int32_t* cverts, float* chess, float* rhs,
                               float* sol);
/* Append every Newton system the simulation solves (up to max_systems in p) to p's
 * training data; p = NULL or max_systems = 0 stops capturing. */
int cipc_sim_capture_systems(cipc_sim* sim, cipc_precond* p, int max_systems);
/* Preconditioner used by steps with params.preconditioner = 1 (NULL: block Jacobi). */
int cipc_sim_set_precond(cipc_sim* sim, cipc_precond* p);

#ifdef __cplusplus
}
#endif

#endif /* CIPC_H */
