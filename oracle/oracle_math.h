// CPU ORACLE — test infrastructure only.
//
// This directory is a plain C++ restatement of the reference's per-pair contact
// math (Codim-IPC, Library/Math/Distance/*, Library/Math/BARRIER.h,
// Library/Math/UTILS.h).  It exists to check the CUDA product path: only the test
// suite, the smoke check and the bench's CPU-baseline leg may load it.  Nothing in
// the product links or calls it.
//
// Canonical arithmetic.  The reference is compiled with -O3 -mfma and lets GCC
// contract a*b+c.  This oracle fixes the contractions GCC 13 makes there on the
// reference's own source (measured by compiling the reference's distance-type,
// distance and ACCD routines against oracle/eigen_shim.h with the reference's
// flags and its vectorizer off, oracle/build.py:build_ref_ccd; the bit-for-bit
// pin is tests/test_oracle_reference_ccd.py), and the CUDA kernels follow the
// same rule, so that accept/reject decisions and FP64 values agree bit for bit:
//   dot3(a,b)   = fma(a2,b2, fma(a0,b0, a1*b1))
//   cross(a,b)  = (fma(a1,b2,-(a2*b1)), fma(a2,b0,-(a0*b2)), fma(a0,b1,-(a1*b0)))
//   x + t*d     = fma(t,d,x)
// and every other expression is evaluated left to right with no contraction
// (compiled with -ffp-contract=off).
#pragma once
#include <cmath>
#include <cstdint>

namespace orc {

struct V3 {
    double x, y, z;
};

static inline V3 v3(double a, double b, double c) { return V3{a, b, c}; }
static inline V3 ld3(const double* p) { return V3{p[0], p[1], p[2]}; }
static inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 scale(V3 a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
static inline V3 divs(V3 a, double s) { return V3{a.x / s, a.y / s, a.z / s}; }
static inline double dot(V3 a, V3 b) { return std::fma(a.z, b.z, std::fma(a.x, b.x, a.y * b.y)); }
static inline double norm2(V3 a) { return dot(a, a); }
static inline V3 cross(V3 a, V3 b)
{
    return V3{std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)),
              std::fma(a.x, b.y, -(a.y * b.x))};
}
// x + t*d with one rounding per component
static inline V3 axpy(double t, V3 d, V3 x)
{
    return V3{std::fma(t, d.x, x.x), std::fma(t, d.y, x.y), std::fma(t, d.z, x.z)};
}

// ---- distance types (Library/Math/Distance/DISTANCE_TYPE.h) -----------------
int pe_type(V3 p, V3 e0, V3 e1);
int pt_type(V3 p, V3 t0, V3 t1, V3 t2);
int ee_type(V3 ea0, V3 ea1, V3 eb0, V3 eb1);

// ---- squared distances (POINT_POINT.h, POINT_EDGE.h, POINT_TRIANGLE.h, EDGE_EDGE.h)
double pp_d2(V3 a, V3 b);
double pe_d2(V3 p, V3 e0, V3 e1);
double pt_d2(V3 p, V3 t0, V3 t1, V3 t2);
double ee_d2(V3 ea0, V3 ea1, V3 eb0, V3 eb1);
double ee_cross_n2(V3 ea0, V3 ea1, V3 eb0, V3 eb1);
// DISTANCE_UNCLASSIFIED.h
double pt_d2_unclassified(V3 p, V3 t0, V3 t1, V3 t2);
double ee_d2_unclassified(V3 ea0, V3 ea1, V3 eb0, V3 eb1);
double pe_d2_unclassified(V3 p, V3 e0, V3 e1);

// Gradient (n) and full Hessian (n*n row-major) of a squared distance.
// kind: 0 PP (6), 1 PE (9), 2 PT (12), 3 EE (12), 4 EE cross-norm^2 (12)
void d2_grad_hess(int kind, const double* x, double* g, double* H);

// ---- barrier (Library/Math/BARRIER.h, non-elastic branch) --------------------
void barrier3(double d, double dHat, double kappa, double* b, double* g, double* h);

// ---- EE mollifier (EDGE_EDGE_MOLLIFIER.h) -----------------------------------
double mollifier_threshold(V3 a0r, V3 a1r, V3 b0r, V3 b1r);
// e, de (12), d2e (144); returns e
double mollifier(const double* x12, double eps_x, double* g, double* H);

// ---- PSD projection (Library/Math/UTILS.h makePD) ---------------------------
void make_pd(int n, double* H);
// symmetric eigen-decomposition, ascending eigenvalues, V column-major eigvecs
void sym_eigen(int n, const double* A, double* w, double* V);

// ---- ACCD (Library/Math/Distance/CCD.h) -------------------------------------
// Each returns 1 on "hit before toc_in" with *toc = time of impact lower bound,
// 0 on "no hit" (then *toc is left as the reference leaves it: the running toc),
// -1 on iteration-cap overflow.  *iters counts loop iterations.
int accd_pt(V3 p, V3 t0, V3 t1, V3 t2, V3 dp, V3 dt0, V3 dt1, V3 dt2, double eta,
            double thickness, double* toc, int64_t max_iter, int64_t* iters);
int accd_ee(V3 ea0, V3 ea1, V3 eb0, V3 eb1, V3 dea0, V3 dea1, V3 deb0, V3 deb1, double eta,
            double thickness, double* toc, int64_t max_iter, int64_t* iters);
int accd_pe(V3 p, V3 e0, V3 e1, V3 dp, V3 de0, V3 de1, double eta, double thickness,
            double* toc, int64_t max_iter, int64_t* iters);
int accd_pp(V3 p0, V3 p1, V3 dp0, V3 dp1, double eta, double thickness, double* toc,
            int64_t max_iter, int64_t* iters);

}  // namespace orc
