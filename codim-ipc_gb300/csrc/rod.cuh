// Discrete rod elements of the shell step (Library/FEM/Shell/Rod/ROD_STRETCHING.h:9-107,
// ROD_BENDING.h:9-120):
//   stretching  E = K L / 2 (l / L - 1)^2, l = |x0 - x1|, K = h^2 pi t^2 / 4 E_young;
//   bending     E = Kb |kb|^2 / lsum, kb = 2 a x b / (|a||b| + a.b), a = x1 - x0,
//               b = x2 - x1, Kb = h^2 E_young bendMult t^4 pi / 64.
// Stretching has a closed-form PSD Hessian: with d = x0 - x1 the 6x6 Hessian is
// [[B, -B], [-B, B]], B = K (dd^T / (L l^2) + (1/L - 1/l)(I - dd^T/l^2)), whose
// eigen-decomposition is that of B, so clamping B's (perpendicular) eigenvalue at
// zero is the reference's makePD exactly.  Bending: analytic gradient in (a, b);
// Hessian by forward-mode differentiation of that gradient in (a, b), mapped to the
// vertices and projected to PSD in the translation-free basis.
#pragma once
#include "elements.cuh"

namespace cipc {

// stretching: energy and gradient (g[6] = d/dx0, d/dx1)
CIPC_HD double rod_spring_eg(const d3& x0, const d3& x1, double L, double K, double* g)
{
    const d3 d = x0 - x1;
    const double l = sqrt(n2(d));
    const double s = l / L - 1;
    if (g) {
        const double c = l > 0 ? K * s / l : 0.0;
        g[0] = c * d.x;
        g[1] = c * d.y;
        g[2] = c * d.z;
        g[3] = -g[0];
        g[4] = -g[1];
        g[5] = -g[2];
    }
    return 0.5 * K * L * s * s;
}

// stretching: PSD Hessian
template <typename HT>
CIPC_HD void rod_spring_hess(const d3& x0, const d3& x1, double L, double K, HT (&H)[6][6])
{
    const d3 d = x0 - x1;
    const double l2 = n2(d), l = sqrt(l2);
    const double par = K / L, perp = (l > 0) ? fmax(0.0, K * (1.0 / L - 1.0 / l)) : 0.0;
    const double dv[3] = {d.x, d.y, d.z};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double dd = l2 > 0 ? dv[i] * dv[j] / l2 : 0.0;
            const double b = par * dd + perp * ((i == j ? 1.0 : 0.0) - dd);
            H[i][j] = (HT)b;
            H[3 + i][3 + j] = (HT)b;
            H[i][3 + j] = (HT)(-b);
            H[3 + i][j] = (HT)(-b);
        }
}

// forward-mode dual over the 6 reduced variables (a, b)
struct dual6 {
    double v, d[6];
};
CIPC_HD dual6 dv6(double v)
{
    dual6 r;
    r.v = v;
    for (int k = 0; k < 6; ++k) r.d[k] = 0;
    return r;
}
CIPC_HD dual6 operator+(const dual6& a, const dual6& b)
{
    dual6 r;
    r.v = a.v + b.v;
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
CIPC_HD dual6 operator-(const dual6& a, const dual6& b)
{
    dual6 r;
    r.v = a.v - b.v;
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
CIPC_HD dual6 operator*(const dual6& a, const dual6& b)
{
    dual6 r;
    r.v = a.v * b.v;
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
CIPC_HD dual6 operator/(const dual6& a, const dual6& b)
{
    dual6 r;
    r.v = a.v / b.v;
    const double ib2 = 1.0 / (b.v * b.v);
    for (int k = 0; k < 6; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) * ib2;
    return r;
}
CIPC_HD dual6 dsqrt(const dual6& a)
{
    dual6 r;
    r.v = sqrt(a.v);
    const double h = 0.5 / r.v;
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] * h;
    return r;
}
CIPC_HD double dsqrt(double a) { return sqrt(a); }
// constant of the scalar type of the second argument
CIPC_HD double cst(double c, double) { return c; }
CIPC_HD dual6 cst(double c, const dual6&) { return dv6(c); }

// gradient of f = |kb|^2 = 4 |a x b|^2 / s^2, s = |a||b| + a.b, in (a, b):
//   df/da = 8 (b x c) / s^2 - 8 |c|^2 (|b|/|a| a + b) / s^3, c = a x b
//   df/db = 8 (c x a) / s^2 - 8 |c|^2 (|a|/|b| b + a) / s^3
template <typename T>
CIPC_HD void kb2_grad(const T (&a)[3], const T (&b)[3], T (&ga)[3], T (&gb)[3])
{
    const T c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const T la = dsqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    const T lb = dsqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    const T s = la * lb + (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
    const T c2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    const T eight = cst(8.0, s);
    const T f1 = eight / (s * s), f2 = eight * c2 / (s * s * s);
    const T bc[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
    const T ca[3] = {c[1] * a[2] - c[2] * a[1], c[2] * a[0] - c[0] * a[2], c[0] * a[1] - c[1] * a[0]};
    const T ra = lb / la, rb = la / lb;
    for (int k = 0; k < 3; ++k) {
        ga[k] = f1 * bc[k] - f2 * (ra * a[k] + b[k]);
        gb[k] = f1 * ca[k] - f2 * (rb * b[k] + a[k]);
    }
}

// bending: energy and gradient (g[9] = d/dx0, d/dx1, d/dx2)
CIPC_HD double rod_bend_eg(const d3& x0, const d3& x1, const d3& x2, double lsum, double Kb, double* g)
{
    const d3 a = x1 - x0, b = x2 - x1;
    const d3 c = cross(a, b);
    const double s = sqrt(n2(a) * n2(b)) + dot(a, b);
    const double w = Kb / lsum;
    const double E = w * 4.0 * n2(c) / (s * s);
    if (g) {
        const double av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
        double ga[3], gb[3];
        kb2_grad<double>(av, bv, ga, gb);
        for (int k = 0; k < 3; ++k) {
            g[k] = -w * ga[k];
            g[3 + k] = w * (ga[k] - gb[k]);
            g[6 + k] = w * gb[k];
        }
    }
    return E;
}

// bending: PSD Hessian (9x9)
template <typename HT>
CIPC_HD void rod_bend_hess(const d3& x0, const d3& x1, const d3& x2, double lsum, double Kb, HT (&H)[9][9])
{
    const d3 a = x1 - x0, b = x2 - x1;
    dual6 ad[3], bd[3];
    const double av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
    for (int k = 0; k < 3; ++k) {
        ad[k] = dv6(av[k]);
        ad[k].d[k] = 1.0;
        bd[k] = dv6(bv[k]);
        bd[k].d[3 + k] = 1.0;
    }
    dual6 ga[3], gb[3];
    kb2_grad<dual6>(ad, bd, ga, gb);
    const double w = Kb / lsum;
    // reduced Hessian R (6x6) over (a, b), symmetrized
    double R[6][6];
    for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 6; ++j) {
            R[k][j] = w * ga[k].d[j];
            R[3 + k][j] = w * gb[k].d[j];
        }
    for (int i = 0; i < 6; ++i)
        for (int j = i + 1; j < 6; ++j) {
            const double m = 0.5 * (R[i][j] + R[j][i]);
            R[i][j] = R[j][i] = m;
        }
    // vertex map: x0 -> -a, x1 -> +a -b, x2 -> +b
    const double inc[3][2] = {{-1, 0}, {1, -1}, {0, 1}};
    for (int u = 0; u < 3; ++u)
        for (int v = 0; v < 3; ++v)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double t = 0;
                    for (int p = 0; p < 2; ++p)
                        for (int q = 0; q < 2; ++q) t += inc[u][p] * inc[v][q] * R[3 * p + i][3 * q + j];
                    H[3 * u + i][3 * v + j] = (HT)t;
                }
    project_translation_free<HT, 3>(H);
}

}  // namespace cipc
