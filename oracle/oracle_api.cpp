// CPU ORACLE — test infrastructure only.  C entry points over oracle_math.cpp for
// ctypes: single-primitive checks and the batched contact-pair microbenchmark
// (ACCD time of impact, barrier energy/gradient/PSD-projected Hessian).
#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include "oracle_math.h"

using namespace orc;

extern "C" {

int orc_num_threads() { return omp_get_max_threads(); }
void orc_set_threads(int n) { omp_set_num_threads(n); }

int orc_pt_type(const double* x) { return pt_type(ld3(x), ld3(x + 3), ld3(x + 6), ld3(x + 9)); }
int orc_ee_type(const double* x) { return ee_type(ld3(x), ld3(x + 3), ld3(x + 6), ld3(x + 9)); }
int orc_pe_type(const double* x) { return pe_type(ld3(x), ld3(x + 3), ld3(x + 6)); }

// kind: 0 PP, 1 PE, 2 PT, 3 EE, 4 EE cross norm^2, 5 PT unclassified,
//       6 EE unclassified, 7 PE unclassified
double orc_d2(int kind, const double* x)
{
    V3 a = ld3(x), b = ld3(x + 3), c = ld3(x + 6), d = ld3(x + 9);
    switch (kind) {
        case 0: return pp_d2(a, b);
        case 1: return pe_d2(a, b, c);
        case 2: return pt_d2(a, b, c, d);
        case 3: return ee_d2(a, b, c, d);
        case 4: return ee_cross_n2(a, b, c, d);
        case 5: return pt_d2_unclassified(a, b, c, d);
        case 6: return ee_d2_unclassified(a, b, c, d);
        case 7: return pe_d2_unclassified(a, b, c);
    }
    return NAN;
}

void orc_d2_grad_hess(int kind, const double* x, double* g, double* H) { d2_grad_hess(kind, x, g, H); }
void orc_barrier(double d, double dHat, double kappa, double* out3)
{
    barrier3(d, dHat, kappa, out3, out3 + 1, out3 + 2);
}
double orc_mollifier(const double* x12, double eps_x, double* g, double* H) { return mollifier(x12, eps_x, g, H); }
void orc_make_pd(int n, double* H) { make_pd(n, H); }
void orc_sym_eigen(int n, const double* A, double* w, double* V) { sym_eigen(n, A, w, V); }

// Pair types of the microbenchmark / constraint list: 0 PP, 1 PE, 2 PT, 3 EE.
static const int kNV[4] = {2, 3, 4, 4};

// ACCD over n pairs, one step of displacement dx scaled by toc_in (the reference
// calls CCD with displacement alpha*p and toc = 1; here dx is the full
// displacement and toc_in the step fraction).  hit[i] = 1 when a time of impact
// below toc_in was found; toc_out[i] = that time, else toc_in.  status[i] = -1
// marks an iteration-cap overflow.  Returns the number of cap overflows.
int64_t orc_ccd_pairs(int64_t n, const uint8_t* type, const int32_t* idx, const double* x,
                      const double* dx, double eta, double thickness, double toc_in,
                      int64_t max_iter, double* toc_out, uint8_t* hit, int32_t* iters)
{
    int64_t overflow = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : overflow)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t* id = idx + 4 * i;
        V3 p[4], d[4];
        int nv = kNV[type[i]];
        for (int k = 0; k < nv; ++k) {
            p[k] = ld3(x + 3 * (int64_t)id[k]);
            d[k] = ld3(dx + 3 * (int64_t)id[k]);
        }
        double t = toc_in;
        int64_t it = 0;
        int r = 0;
        switch (type[i]) {
            case 0: r = accd_pp(p[0], p[1], d[0], d[1], eta, thickness, &t, max_iter, &it); break;
            case 1: r = accd_pe(p[0], p[1], p[2], d[0], d[1], d[2], eta, thickness, &t, max_iter, &it); break;
            case 2: r = accd_pt(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], eta, thickness, &t, max_iter, &it); break;
            case 3: r = accd_ee(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], eta, thickness, &t, max_iter, &it); break;
        }
        if (r < 0) ++overflow;
        hit[i] = (r == 1) ? 1 : 0;
        toc_out[i] = (r == 1) ? t : toc_in;
        if (iters) iters[i] = (int32_t)it;
    }
    return overflow;
}

// Barrier of one contact pair, following IPC.h Compute_Barrier / _Gradient /
// _Hessian (IPC.h:742-1731) with stencil weight 1 and multiplicity 1:
//   s = d^2 - xi^2, shat = dHat2 + 2 sqrt(dHat2) xi (IPC.h:756-757),
//   E = b(s), grad = b'(s) grad d^2, H = makePD(b'' grad d^2 grad d^2^T + b' hess d^2).
// EE pairs whose |ea x eb|^2 is below 1e-3 |ea_rest|^2 |eb_rest|^2 take the
// mollified form E = e b (IPC.h:1472-1478).  Inactive pairs (s >= shat) give zeros.
// Outputs: E[i]; grad[i*12 + k] (first 3*nv used); hess[i*78 + ...] = upper
// triangle of the (3nv)x(3nv) Hessian packed row by row.  Returns the number of
// pairs with s <= 0 (the reference exits on those, IPC.h:773-776).
int64_t orc_barrier_pairs(int64_t n, const uint8_t* type, const int32_t* idx, const double* x,
                          const double* x_rest, double dHat2, double xi, double kappa,
                          int project_pd, double* E, double* grad, double* hess)
{
    int64_t bad = 0;
    const double shat = dHat2 + 2 * std::sqrt(dHat2) * xi;
    const double xi2 = xi * xi;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : bad)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t* id = idx + 4 * i;
        int tp = type[i];
        int nv = kNV[tp];
        int m = 3 * nv;
        double xv[12];
        for (int k = 0; k < nv; ++k)
            for (int c = 0; c < 3; ++c) xv[3 * k + c] = x[3 * (int64_t)id[k] + c];
        V3 a = ld3(xv), b = ld3(xv + 3), c = ld3(xv + 6), d = ld3(xv + 9);
        double d2 = 0;
        switch (tp) {
            case 0: d2 = pp_d2(a, b); break;
            case 1: d2 = pe_d2(a, b, c); break;
            case 2: d2 = pt_d2(a, b, c, d); break;
            case 3: d2 = ee_d2(a, b, c, d); break;
        }
        double s = d2 - xi2;
        double* g = grad + 12 * i;
        double* hp = hess + 78 * i;
        for (int k = 0; k < 12; ++k) g[k] = 0;
        for (int k = 0; k < 78; ++k) hp[k] = 0;
        E[i] = 0;
        if (!(s > 0)) {
            ++bad;
            continue;
        }
        if (s >= shat) continue;
        double bv, bg, bh;
        barrier3(s, shat, kappa, &bv, &bg, &bh);
        double gd[12], Hd[144];
        static const int kindOf[4] = {0, 1, 2, 3};
        d2_grad_hess(kindOf[tp], xv, gd, Hd);
        double H[144];
        double e = 1.0;
        bool moll = false;
        double ge[12], He[144];
        if (tp == 3) {
            double xr[12];
            for (int k = 0; k < 4; ++k)
                for (int cc = 0; cc < 3; ++cc) xr[3 * k + cc] = x_rest[3 * (int64_t)id[k] + cc];
            double eps_x = mollifier_threshold(ld3(xr), ld3(xr + 3), ld3(xr + 6), ld3(xr + 9));
            if (ee_cross_n2(a, b, c, d) < eps_x) {
                moll = true;
                e = mollifier(xv, eps_x, ge, He);
            }
        }
        if (!moll) {
            E[i] = bv;
            for (int k = 0; k < m; ++k) g[k] = bg * gd[k];
            for (int r = 0; r < m; ++r)
                for (int q = 0; q < m; ++q) H[r * m + q] = bh * gd[r] * gd[q] + bg * Hd[r * m + q];
        } else {
            E[i] = e * bv;
            for (int k = 0; k < 12; ++k) g[k] = e * bg * gd[k] + bv * ge[k];
            for (int r = 0; r < 12; ++r)
                for (int q = 0; q < 12; ++q)
                    H[r * 12 + q] = bg * gd[r] * ge[q] + ge[r] * bg * gd[q] + bv * He[r * 12 + q] +
                                    e * bh * gd[r] * gd[q] + e * bg * Hd[r * 12 + q];
        }
        if (project_pd) make_pd(m, H);
        int o = 0;
        for (int r = 0; r < m; ++r)
            for (int q = r; q < m; ++q) hp[o++] = H[r * m + q];
    }
    return bad;
}

}  // extern "C"
