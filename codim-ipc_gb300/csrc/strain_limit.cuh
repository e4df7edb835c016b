// Isotropic strain-limiting barrier of the shell step (Library/FEM/Shell/INEXT.h):
// per triangle, the singular values sigma of the deformation F = A B^-1 (A the
// two edge vectors, B^T B the rest first fundamental form) are kept below s0 (and
// above s1 when kappa1 > 0) by
//   b(sigma) = k f(sigma),  f(s) = -(sh - s)^2 ln((sl - s)/(sl - sh)) / (sl - sh)^2,
// active for sigma > sh0 (upper) or sigma < sh1 (lower), k = h^2 vol kappa_s;
// sigma >= s0 (or <= s1) makes the state infeasible.  f is C2 at sh.
//
// Derivatives are analytic in the singular frame: with F = U diag(s1, s2) V^T,
// the Hessian of sum_i b(sigma_i) in F is diagonal in the orthonormal basis
//   u1 v1^T: b''(s1)      u2 v2^T: b''(s2)
//   (u1 v2^T + u2 v1^T)/sqrt2: (b'(s1) - b'(s2)) / (s1 - s2)
//   (u1 v2^T - u2 v1^T)/sqrt2: (b'(s1) + b'(s2)) / (s1 + s2)
//   u3 v1^T: b'(s1) / s1  u3 v2^T: b'(s2) / s2
// so the PSD projection of the 6x6 F-Hessian (the reference's makePD) clamps
// these six eigenvalues at zero; the 9x9 vertex Hessian follows from the linear
// map x -> F.
#pragma once
#include "geom.cuh"
#include "sl_params.h"

namespace cipc {

// f, f', f'' of the barrier for limit sl and activation sh
CIPC_HD double sl_f(double s, double sl, double sh)
{
    const double a = sh - s, D = sl - sh;
    return -a * a * log((sl - s) / D) / (D * D);
}
CIPC_HD double sl_df(double s, double sl, double sh)
{
    const double a = sh - s, b = sl - s, D = sl - sh;
    return (2 * a * log(b / D) + a * a / b) / (D * D);
}
CIPC_HD double sl_d2f(double s, double sl, double sh)
{
    const double a = sh - s, b = sl - s, D = sl - sh, c = a / b;
    return (-2 * log(b / D) + c * (c - 4)) / (D * D);
}

// barrier value and derivatives of one singular value (zero outside the active
// ranges); returns false if sigma is infeasible.  kh = h^2 vol.
CIPC_HD bool sl_sigma(double s, const SlParams& p, double kh, double& e, double& g, double& hh)
{
    e = g = hh = 0;
    bool ok = true;
    if (s >= p.s0) {
        ok = false;
    } else if (s > p.sh0) {
        const double k = kh * p.k0;
        e += k * sl_f(s, p.s0, p.sh0);
        g += k * sl_df(s, p.s0, p.sh0);
        hh += k * sl_d2f(s, p.s0, p.sh0);
    }
    if (p.k1 > 0) {
        if (s <= p.s1) {
            ok = false;
        } else if (s < p.sh1) {
            const double k = kh * p.k1;
            e += k * sl_f(s, p.s1, p.sh1);
            g += k * sl_df(s, p.s1, p.sh1);
            hh += k * sl_d2f(s, p.s1, p.sh1);
        }
    }
    return ok;
}

// F = A B^-1 (3x2, F[i][k]) and c[k][v] = dF[:,k] / dx_v, from the inverse rest
// fundamental form P = (p00, p01, p11): B^T B = P^-1 with B upper triangular
CIPC_HD void sl_deform(const d3 (&x)[3], const double* P, double (&F)[3][2], double (&c)[2][3])
{
    const double det = P[0] * P[2] - P[1] * P[1];
    const double q00 = P[2] / det, q01 = -P[1] / det, q11 = P[0] / det;  // rest form
    const double b00 = sqrt(q00), b01 = q01 / b00, b11 = sqrt(q11 - q01 * q01 / q00);
    // B^-1 (upper triangular)
    const double i00 = 1 / b00, i01 = -b01 / (b00 * b11), i11 = 1 / b11;
    const d3 e1 = x[1] - x[0], e2 = x[2] - x[0];
    const double E1[3] = {e1.x, e1.y, e1.z}, E2[3] = {e2.x, e2.y, e2.z};
    for (int i = 0; i < 3; ++i) {
        F[i][0] = E1[i] * i00;
        F[i][1] = E1[i] * i01 + E2[i] * i11;
    }
    c[0][0] = -i00;
    c[0][1] = i00;
    c[0][2] = 0;
    c[1][0] = -(i01 + i11);
    c[1][1] = i01;
    c[1][2] = i11;
}

// singular values s1 >= s2 of F (3x2), right vectors v[k] (columns), left u[0..2]
CIPC_HD void sl_svd(const double (&F)[3][2], double& s1, double& s2, double (&v)[2][2], double (&u)[3][3])
{
    double c00 = 0, c01 = 0, c11 = 0;
    for (int i = 0; i < 3; ++i) {
        c00 += F[i][0] * F[i][0];
        c01 += F[i][0] * F[i][1];
        c11 += F[i][1] * F[i][1];
    }
    const double m = 0.5 * (c00 + c11), d = 0.5 * (c00 - c11);
    const double r = sqrt(d * d + c01 * c01);
    s1 = sqrt(m + r);
    s2 = sqrt(fmax(m - r, 0.0));
    const double th = (r > 0) ? 0.5 * atan2(2 * c01, c00 - c11) : 0.0;
    const double cs = cos(th), sn = sin(th);
    v[0][0] = cs;
    v[0][1] = sn;  // v1
    v[1][0] = -sn;
    v[1][1] = cs;  // v2
    for (int a = 0; a < 2; ++a) {
        const double sa = a == 0 ? s1 : s2;
        for (int i = 0; i < 3; ++i) u[a][i] = (F[i][0] * v[a][0] + F[i][1] * v[a][1]) / sa;
    }
    u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
    u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
    u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
}

// largest singular value (the reference's per-triangle strain, INEXT.h:72-118)
CIPC_HD double sl_max_strain(const d3 (&x)[3], const double* P)
{
    double F[3][2], c[2][3], v[2][2], u[3][3], s1, s2;
    sl_deform(x, P, F, c);
    sl_svd(F, s1, s2, v, u);
    return s1;
}

// energy and gradient (g[9], may be null); returns false if infeasible
CIPC_HD bool sl_eg(const d3 (&x)[3], const double* P, const SlParams& p, double kh, double& E, double* g)
{
    double F[3][2], c[2][3], v[2][2], u[3][3], s1, s2;
    sl_deform(x, P, F, c);
    sl_svd(F, s1, s2, v, u);
    double e1, g1, h1, e2, g2, h2;
    const bool ok = sl_sigma(s1, p, kh, e1, g1, h1) & sl_sigma(s2, p, kh, e2, g2, h2);
    E = e1 + e2;
    if (g) {
        // dE/dF = g1 u1 v1^T + g2 u2 v2^T; dE/dx_v = sum_k c[k][v] dE/dF[:, k]
        for (int w = 0; w < 3; ++w)
            for (int i = 0; i < 3; ++i) {
                double s = 0;
                for (int k = 0; k < 2; ++k) s += c[k][w] * (g1 * u[0][i] * v[0][k] + g2 * u[1][i] * v[1][k]);
                g[3 * w + i] = s;
            }
    }
    return ok;
}

// 9x9 Hessian, PSD-projected in F (project) or not; returns false (H untouched)
// when no singular value is in an active range
template <typename HT>
CIPC_HD bool sl_hess(const d3 (&x)[3], const double* P, const SlParams& p, double kh, bool project, HT (&H)[9][9])
{
    double F[3][2], c[2][3], v[2][2], u[3][3], s1, s2;
    sl_deform(x, P, F, c);
    sl_svd(F, s1, s2, v, u);
    double e1, g1, h1, e2, g2, h2;
    sl_sigma(s1, p, kh, e1, g1, h1);
    sl_sigma(s2, p, kh, e2, g2, h2);
    if (g1 == 0 && g2 == 0 && h1 == 0 && h2 == 0) return false;
    const double ds = s1 - s2;
    const double lam[6] = {h1, h2, fabs(ds) > 1e-12 * fmax(s1, 1.0) ? (g1 - g2) / ds : 0.5 * (h1 + h2),
                           (g1 + g2) / (s1 + s2), g1 / s1, g2 / s2};
    // mode matrices Q[m][i][k] (3x2) of the orthonormal eigenbasis
    const double r2 = 0.70710678118654752440;
    double Q[6][3][2];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 2; ++k) {
            Q[0][i][k] = u[0][i] * v[0][k];
            Q[1][i][k] = u[1][i] * v[1][k];
            Q[2][i][k] = r2 * (u[0][i] * v[1][k] + u[1][i] * v[0][k]);
            Q[3][i][k] = r2 * (u[0][i] * v[1][k] - u[1][i] * v[0][k]);
            Q[4][i][k] = u[2][i] * v[0][k];
            Q[5][i][k] = u[2][i] * v[1][k];
        }
    // modes mapped to the vertices: W[m][3w + i] = sum_k c[k][w] Q[m][i][k]
    double W[6][9];
    for (int m = 0; m < 6; ++m)
        for (int w = 0; w < 3; ++w)
            for (int i = 0; i < 3; ++i) W[m][3 * w + i] = c[0][w] * Q[m][i][0] + c[1][w] * Q[m][i][1];
    double L[6];
    for (int m = 0; m < 6; ++m) L[m] = project ? fmax(lam[m], 0.0) : lam[m];
    for (int a = 0; a < 9; ++a)
        for (int b = a; b < 9; ++b) {
            double s = 0;
            for (int m = 0; m < 6; ++m) s += L[m] * W[m][a] * W[m][b];
            H[a][b] = (HT)s;
            H[b][a] = (HT)s;
        }
    return true;
}

}  // namespace cipc
