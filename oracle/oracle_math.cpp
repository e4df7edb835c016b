// CPU ORACLE — test infrastructure only (see oracle_math.h for the arithmetic rule).
// Each function cites the reference function it restates (paths relative to the
// Codim-IPC source tree).
#include "oracle_math.h"

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// Distance types — Library/Math/Distance/DISTANCE_TYPE.h
// ---------------------------------------------------------------------------

// DISTANCE_TYPE.h:11-27 (3D use: ratio of projection onto the edge)
int pe_type(V3 p, V3 e0, V3 e1)
{
    V3 e = e1 - e0;
    double ratio = dot(e, p - e0) / norm2(e);
    if (ratio < 0) return 0;
    if (ratio > 1) return 1;
    return 2;
}

// Restates Eigen's pivoted LDL^T (LDLT::compute + LDLT::solve) for a symmetric 2x2
// system [a00 a10; a10 a11] y = (b0,b1), as used through `.ldlt().solve()` in
// DISTANCE_TYPE.h:46,54,62.  Pivot = larger |diagonal| (first on ties); a zero
// pivot gives the zero solution; D entries with |d| <= DBL_MIN are pseudo-inverted
// to zero.
static inline void ldlt2_solve(double a00, double a10, double a11, double b0, double b1,
                               double* y0, double* y1)
{
    bool swap = std::fabs(a11) > std::fabs(a00);
    double d0 = swap ? a11 : a00;
    double m11 = swap ? a00 : a11;
    if (swap) std::swap(b0, b1);
    if (d0 == 0.0) {
        *y0 = 0.0;
        *y1 = 0.0;
        return;
    }
    double l10 = a10 / d0;
    double d1 = std::fma(-l10, d0 * l10, m11);
    double z0 = b0;
    double z1 = std::fma(-l10, z0, b1);
    z0 = (std::fabs(d0) > DBL_MIN) ? z0 / d0 : 0.0;
    z1 = (std::fabs(d1) > DBL_MIN) ? z1 / d1 : 0.0;
    z0 = std::fma(-l10, z1, z0);
    if (swap) std::swap(z0, z1);
    *y0 = z0;
    *y1 = z1;
}

// Parametric coordinates of p - o in the basis (r0, r0 x n): DISTANCE_TYPE.h:44-47.
static inline void pt_param(V3 r0, V3 n, V3 v, double* s, double* q)
{
    V3 r1 = cross(r0, n);
    double a00 = dot(r0, r0);
    double a10 = dot(r1, r0);
    double a11 = dot(r1, r1);
    double b0 = dot(r0, v);
    double b1 = dot(r1, v);
    ldlt2_solve(a00, a10, a11, b0, b1, s, q);
}

// DISTANCE_TYPE.h:30-82
int pt_type(V3 p, V3 t0, V3 t1, V3 t2)
{
    V3 n = cross(t1 - t0, t2 - t0);
    double s0, q0, s1, q1, s2, q2;
    pt_param(t1 - t0, n, p - t0, &s0, &q0);
    if (s0 > 0.0 && s0 < 1.0 && q0 >= 0.0) return 3;
    pt_param(t2 - t1, n, p - t1, &s1, &q1);
    if (s1 > 0.0 && s1 < 1.0 && q1 >= 0.0) return 4;
    pt_param(t0 - t2, n, p - t2, &s2, &q2);
    if (s2 > 0.0 && s2 < 1.0 && q2 >= 0.0) return 5;
    if (s0 <= 0.0 && s2 >= 1.0) return 0;
    if (s1 <= 0.0 && s0 >= 1.0) return 1;
    if (s2 <= 0.0 && s1 >= 1.0) return 2;
    return 6;
}

// DISTANCE_TYPE.h:84-164
int ee_type(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    V3 u = ea1 - ea0;
    V3 v = eb1 - eb0;
    V3 w = ea0 - eb0;
    double a = dot(u, u);
    double b = dot(u, v);
    double c = dot(v, v);
    double d = dot(u, w);
    double e = dot(v, w);
    double D = std::fma(a, c, -(b * b));
    double tD = D;
    double sN, tN;
    int defaultCase = 8;
    sN = std::fma(b, e, -(c * d));
    if (sN <= 0.0) {
        tN = e;
        tD = c;
        defaultCase = 2;
    } else if (sN >= D) {
        tN = e + b;
        tD = c;
        defaultCase = 5;
    } else {
        tN = std::fma(a, e, -(b * d));
        if (tN > 0.0 && tN < tD) {
            V3 uxv = cross(u, v);
            if (dot(uxv, w) == 0.0 || norm2(uxv) < 1.0e-20 * a * c) {
                if (sN < D / 2) {
                    tN = e;
                    tD = c;
                    defaultCase = 2;
                } else {
                    tN = e + b;
                    tD = c;
                    defaultCase = 5;
                }
            }
        }
    }
    if (tN <= 0.0) {
        if (-d <= 0.0) return 0;
        if (-d >= a) return 3;
        return 6;
    } else if (tN >= tD) {
        if ((-d + b) <= 0.0) return 1;
        if ((-d + b) >= a) return 4;
        return 7;
    }
    return defaultCase;
}

// ---------------------------------------------------------------------------
// Squared distances
// ---------------------------------------------------------------------------

// POINT_POINT.h:11-17
double pp_d2(V3 a, V3 b) { return norm2(a - b); }

// POINT_EDGE.h:11-25 (3D branch)
double pe_d2(V3 p, V3 e0, V3 e1) { return norm2(cross(e0 - p, e1 - p)) / norm2(e1 - e0); }

// POINT_TRIANGLE.h:11-22
double pt_d2(V3 p, V3 t0, V3 t1, V3 t2)
{
    V3 b = cross(t1 - t0, t2 - t0);
    double aTb = dot(p - t0, b);
    return aTb * aTb / norm2(b);
}

// EDGE_EDGE.h:11-22
double ee_d2(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    V3 b = cross(ea1 - ea0, eb1 - eb0);
    double aTb = dot(eb0 - ea0, b);
    return aTb * aTb / norm2(b);
}

// EDGE_EDGE_MOLLIFIER.h:9-18
double ee_cross_n2(V3 ea0, V3 ea1, V3 eb0, V3 eb1) { return norm2(cross(ea1 - ea0, eb1 - eb0)); }

// DISTANCE_UNCLASSIFIED.h:15-58
double pt_d2_unclassified(V3 p, V3 t0, V3 t1, V3 t2)
{
    switch (pt_type(p, t0, t1, t2)) {
        case 0: return pp_d2(p, t0);
        case 1: return pp_d2(p, t1);
        case 2: return pp_d2(p, t2);
        case 3: return pe_d2(p, t0, t1);
        case 4: return pe_d2(p, t1, t2);
        case 5: return pe_d2(p, t2, t0);
        default: return pt_d2(p, t0, t1, t2);
    }
}

// DISTANCE_UNCLASSIFIED.h:60-125
double ee_d2_unclassified(V3 ea0, V3 ea1, V3 eb0, V3 eb1)
{
    switch (ee_type(ea0, ea1, eb0, eb1)) {
        case 0: return pp_d2(ea0, eb0);
        case 1: return pp_d2(ea0, eb1);
        case 2: return pe_d2(ea0, eb0, eb1);
        case 3: return pp_d2(ea1, eb0);
        case 4: return pp_d2(ea1, eb1);
        case 5: return pe_d2(ea1, eb0, eb1);
        case 6: return pe_d2(eb0, ea0, ea1);
        case 7: return pe_d2(eb1, ea0, ea1);
        default: return ee_d2(ea0, ea1, eb0, eb1);
    }
}

// DISTANCE_UNCLASSIFIED.h:127-148 (projection form, not the cross-product form)
double pe_d2_unclassified(V3 p, V3 e0, V3 e1)
{
    V3 v = e1 - e0;
    V3 w = p - e0;
    double c1 = dot(w, v);
    if (c1 <= 0.0) return pp_d2(p, e0);
    double c2 = dot(v, v);
    if (c2 <= c1) return pp_d2(p, e1);
    double b = c1 / c2;
    return pp_d2(p, axpy(b, v, e0));
}

// ---------------------------------------------------------------------------
// Derivatives of squared distances.  Written from the closed forms
//   PT/EE:  f = u^2/w,  u = a.(e1 x e2),  w = |e1 x e2|^2
//   PE:     f = |a x b|^2 / |b - a|^2
// differentiated in the reduced variables (a, e1, e2) and mapped to vertex
// coordinates by a constant +-1 incidence matrix.  They agree with the reference's
// generated g_PT/H_PT, g_EE/H_EE, g_PE3D/H_PE3D, g_EECN2/H_EECN2
// (POINT_TRIANGLE.h:24-565, EDGE_EDGE.h:24-748, POINT_EDGE.h:60-605,
// EDGE_EDGE_MOLLIFIER.h:20-380) to rounding.
// ---------------------------------------------------------------------------

static void skew(V3 v, double M[9])  // [v]x
{
    M[0] = 0; M[1] = -v.z; M[2] = v.y;
    M[3] = v.z; M[4] = 0; M[5] = -v.x;
    M[6] = -v.y; M[7] = v.x; M[8] = 0;
}

// place 3x3 block B (scaled) at block (bi,bj) of an m x m (m = 3*nb) matrix, plus transpose at (bj,bi)
static void put_block_sym(double* H, int m, int bi, int bj, const double B[9], double s)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            H[(3 * bi + i) * m + 3 * bj + j] += s * B[3 * i + j];
            if (bi != bj) H[(3 * bj + j) * m + 3 * bi + i] += s * B[3 * i + j];
        }
}

// Gradient/Hessian of w = |e1 x e2|^2 w.r.t. (e1, e2), written into the (k1,k2)
// variable blocks of an m x m Hessian / m gradient.
static void crossn2_derivs(V3 e1, V3 e2, int k1, int k2, int m, double* g, double* H)
{
    V3 n = cross(e1, e2);
    V3 g1 = scale(cross(e2, n), 2.0);
    V3 g2 = scale(cross(n, e1), 2.0);
    g[3 * k1 + 0] += g1.x; g[3 * k1 + 1] += g1.y; g[3 * k1 + 2] += g1.z;
    g[3 * k2 + 0] += g2.x; g[3 * k2 + 1] += g2.y; g[3 * k2 + 2] += g2.z;
    double B[9];
    double e1v[3] = {e1.x, e1.y, e1.z}, e2v[3] = {e2.x, e2.y, e2.z};
    double n22 = norm2(e2), n11 = norm2(e1), d12 = dot(e1, e2);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[3 * i + j] = (i == j ? n22 : 0.0) - e2v[i] * e2v[j];
    put_block_sym(H, m, k1, k1, B, 2.0);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[3 * i + j] = (i == j ? n11 : 0.0) - e1v[i] * e1v[j];
    put_block_sym(H, m, k2, k2, B, 2.0);
    double S[9];
    skew(n, S);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            B[3 * i + j] = e1v[i] * e2v[j] - (i == j ? d12 : 0.0) - S[3 * i + j];
    put_block_sym(H, m, k1, k2, B, 2.0);
}

// Map reduced derivatives (nr variable 3-blocks) to vertex derivatives (nv vertices)
// through the incidence matrix C (nr x nv, entries -1/0/1).
static void map_to_vertices(int nr, int nv, const int* C, const double* gr, const double* Hr,
                            double* g, double* H)
{
    int mr = 3 * nr, m = 3 * nv;
    for (int v = 0; v < nv; ++v)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int r = 0; r < nr; ++r) s += C[r * nv + v] * gr[3 * r + c];
            g[3 * v + c] = s;
        }
    for (int v = 0; v < nv; ++v)
        for (int c = 0; c < 3; ++c)
            for (int v2 = 0; v2 < nv; ++v2)
                for (int c2 = 0; c2 < 3; ++c2) {
                    double s = 0;
                    for (int r = 0; r < nr; ++r)
                        for (int r2 = 0; r2 < nr; ++r2) {
                            int w = C[r * nv + v] * C[r2 * nv + v2];
                            if (w) s += w * Hr[(3 * r + c) * mr + 3 * r2 + c2];
                        }
                    H[(3 * v + c) * m + 3 * v2 + c2] = s;
                }
}

// f = u^2 / w with u = a.(e1 x e2), w = |e1 x e2|^2; reduced variables (a, e1, e2)
static void u2w_reduced(V3 a, V3 e1, V3 e2, double gr[9], double Hr[81])
{
    V3 n = cross(e1, e2);
    double u = dot(a, n);
    double w = norm2(n);
    double gu[9] = {0}, Hu[81] = {0}, gw[9] = {0}, Hw[81] = {0};
    V3 t1 = cross(e2, a), t2 = cross(a, e1);
    double gu_[9] = {n.x, n.y, n.z, t1.x, t1.y, t1.z, t2.x, t2.y, t2.z};
    std::memcpy(gu, gu_, sizeof(gu));
    double S[9];
    skew(e2, S);
    put_block_sym(Hu, 9, 0, 1, S, -1.0);
    skew(e1, S);
    put_block_sym(Hu, 9, 0, 2, S, 1.0);
    skew(a, S);
    put_block_sym(Hu, 9, 1, 2, S, -1.0);
    crossn2_derivs(e1, e2, 1, 2, 9, gw, Hw);
    double r = u / w;
    double gv[9];
    for (int i = 0; i < 9; ++i) {
        gv[i] = gu[i] - r * gw[i];
        gr[i] = r * (2.0 * gu[i] - r * gw[i]);
    }
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j)
            Hr[9 * i + j] = (2.0 / w) * gv[i] * gv[j] + 2.0 * r * Hu[9 * i + j] - r * r * Hw[9 * i + j];
}

void d2_grad_hess(int kind, const double* x, double* g, double* H)
{
    if (kind == 0) {  // PP, POINT_POINT.h:19-41
        for (int c = 0; c < 3; ++c) {
            g[c] = 2.0 * (x[c] - x[3 + c]);
            g[3 + c] = -g[c];
        }
        std::memset(H, 0, sizeof(double) * 36);
        for (int i = 0; i < 6; ++i) H[7 * i] = 2.0;
        for (int c = 0; c < 3; ++c) H[c * 6 + 3 + c] = H[(3 + c) * 6 + c] = -2.0;
        return;
    }
    if (kind == 1) {  // PE: x = (p, e0, e1); a = e0 - p, b = e1 - p
        V3 p = ld3(x), e0 = ld3(x + 3), e1 = ld3(x + 6);
        V3 a = e0 - p, b = e1 - p;
        double gN[6] = {0}, HN[36] = {0};
        crossn2_derivs(a, b, 0, 1, 6, gN, HN);
        V3 ba = b - a;
        double N = norm2(cross(a, b));
        double D = norm2(ba);
        double f = N / D;
        double gD[6] = {-2 * ba.x, -2 * ba.y, -2 * ba.z, 2 * ba.x, 2 * ba.y, 2 * ba.z};
        double gf[6], Hr[36];
        for (int i = 0; i < 6; ++i) gf[i] = (gN[i] - f * gD[i]) / D;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                double HD = (i % 3 == j % 3) ? ((i / 3 == j / 3) ? 2.0 : -2.0) : 0.0;
                Hr[6 * i + j] = (HN[6 * i + j] - f * HD - gD[i] * gf[j] - gf[i] * gD[j]) / D;
            }
        static const int C[6] = {-1, 1, 0, -1, 0, 1};
        map_to_vertices(2, 3, C, gf, Hr, g, H);
        return;
    }
    if (kind == 2 || kind == 3) {
        V3 v0 = ld3(x), v1 = ld3(x + 3), v2 = ld3(x + 6), v3 = ld3(x + 9);
        double gr[9], Hr[81];
        if (kind == 2) {  // PT: a = p - t0, e1 = t1 - t0, e2 = t2 - t0
            u2w_reduced(v0 - v1, v2 - v1, v3 - v1, gr, Hr);
            static const int C[12] = {1, -1, 0, 0, 0, -1, 1, 0, 0, -1, 0, 1};
            map_to_vertices(3, 4, C, gr, Hr, g, H);
        } else {  // EE: a = eb0 - ea0, e1 = ea1 - ea0, e2 = eb1 - eb0
            u2w_reduced(v2 - v0, v1 - v0, v3 - v2, gr, Hr);
            static const int C[12] = {-1, 0, 1, 0, -1, 1, 0, 0, 0, 0, -1, 1};
            map_to_vertices(3, 4, C, gr, Hr, g, H);
        }
        return;
    }
    if (kind == 4) {  // |ea x eb|^2: e1 = ea1 - ea0, e2 = eb1 - eb0
        V3 v0 = ld3(x), v1 = ld3(x + 3), v2 = ld3(x + 6), v3 = ld3(x + 9);
        double gr[6] = {0}, Hr[36] = {0};
        crossn2_derivs(v1 - v0, v3 - v2, 0, 1, 6, gr, Hr);
        static const int C[8] = {-1, 1, 0, 0, 0, 0, -1, 1};
        map_to_vertices(2, 4, C, gr, Hr, g, H);
        return;
    }
}

// ---------------------------------------------------------------------------
// Barrier — Library/Math/BARRIER.h:9-62 (elastic == false)
// ---------------------------------------------------------------------------
void barrier3(double d, double dHat, double kappa, double* b, double* g, double* h)
{
    double t2 = d - dHat;
    double lg = std::log(d / dHat);
    if (b) *b = -kappa * t2 * t2 * lg;
    if (g) *g = kappa * (t2 * lg * -2.0 - (t2 * t2) / d);
    if (h) *h = kappa * ((lg * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2));
}

// ---------------------------------------------------------------------------
// Mollifier — EDGE_EDGE_MOLLIFIER.h:440-591
// ---------------------------------------------------------------------------
double mollifier_threshold(V3 a0r, V3 a1r, V3 b0r, V3 b1r)
{
    return 1.0e-3 * norm2(a0r - a1r) * norm2(b0r - b1r);
}

double mollifier(const double* x12, double eps_x, double* g, double* H)
{
    V3 ea0 = ld3(x12), ea1 = ld3(x12 + 3), eb0 = ld3(x12 + 6), eb1 = ld3(x12 + 9);
    double c = ee_cross_n2(ea0, ea1, eb0, eb1);
    if (!(c < eps_x)) {
        if (g) std::memset(g, 0, sizeof(double) * 12);
        if (H) std::memset(H, 0, sizeof(double) * 144);
        return 1.0;
    }
    double r = c / eps_x;
    double e = (-r + 2.0) * r;
    if (g || H) {
        double gc[12], Hc[144];
        d2_grad_hess(4, x12, gc, Hc);
        double one = 1.0 / eps_x;
        double qg = 2.0 * one * (-one * c + 1.0);
        double qH = -2.0 / (eps_x * eps_x);
        if (g)
            for (int i = 0; i < 12; ++i) g[i] = qg * gc[i];
        if (H)
            for (int i = 0; i < 12; ++i)
                for (int j = 0; j < 12; ++j) H[12 * i + j] = qg * Hc[12 * i + j] + qH * gc[i] * gc[j];
    }
    return e;
}

// ---------------------------------------------------------------------------
// Symmetric eigen-decomposition (cyclic Jacobi) and makePD — Library/Math/UTILS.h:9-27.
// The clamped reconstruction V max(L,0) V^T is the unique nearest PSD matrix, so any
// convergent eigen-solver reproduces Eigen's SelfAdjointEigenSolver result to rounding.
// ---------------------------------------------------------------------------
void sym_eigen(int n, const double* A0, double* w, double* V)
{
    std::vector<double> A(A0, A0 + n * n);
    for (int i = 0; i < n * n; ++i) V[i] = 0;
    for (int i = 0; i < n; ++i) V[i * n + i] = 1;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0, tot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double a = A[i * n + j] * A[i * n + j];
                tot += a;
                if (i != j) off += a;
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = A[p * n + q];
                if (apq == 0.0) continue;
                double app = A[p * n + p], aqq = A[q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    // sort ascending
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return A[a * n + a] < A[b * n + b]; });
    std::vector<double> Vs(n * n);
    for (int j = 0; j < n; ++j) {
        w[j] = A[idx[j] * n + idx[j]];
        for (int k = 0; k < n; ++k) Vs[k * n + j] = V[k * n + idx[j]];
    }
    std::memcpy(V, Vs.data(), sizeof(double) * n * n);
}

void make_pd(int n, double* H)
{
    std::vector<double> w(n), V(n * n);
    sym_eigen(n, H, w.data(), V.data());
    if (w[0] >= 0) return;
    for (int i = 0; i < n; ++i) {
        if (w[i] < 0) w[i] = 0;
        else break;
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += V[i * n + k] * w[k] * V[j * n + k];
            H[i * n + j] = s;
        }
}

// ---------------------------------------------------------------------------
// Additive CCD — Library/Math/Distance/CCD.h:279-483.  The reference loops without
// bound; here a cap turns a runaway loop into status -1.
// ---------------------------------------------------------------------------
int accd_pt(V3 p, V3 t0, V3 t1, V3 t2, V3 dp, V3 dt0, V3 dt1, V3 dt2, double eta,
            double thickness, double* toc, int64_t max_iter, int64_t* iters)
{
    // CCD.h:290-299
    V3 mov = scale(((dt0 + dt1) + dt2) + dp, 0.25);
    dt0 = dt0 - mov;
    dt1 = dt1 - mov;
    dt2 = dt2 - mov;
    dp = dp - mov;
    double m2 = std::max(std::max(norm2(dt0), norm2(dt1)), norm2(dt2));
    double maxDispMag = std::sqrt(norm2(dp)) + std::sqrt(m2);
    *iters = 0;
    if (maxDispMag == 0) return 0;
    double th2 = thickness * thickness;
    double dist2 = pt_d2_unclassified(p, t0, t1, t2);
    double dist = std::sqrt(dist2);
    double gap = eta * (dist2 - th2) / (dist + thickness);
    double toc_prev = *toc;
    double t = 0;
    for (int64_t it = 0;; ++it) {
        if (it >= max_iter) { *iters = it; *toc = t; return -1; }
        double tlb = (1 - eta) * (dist2 - th2) / ((dist + thickness) * maxDispMag);
        p = axpy(tlb, dp, p);
        t0 = axpy(tlb, dt0, t0);
        t1 = axpy(tlb, dt1, t1);
        t2 = axpy(tlb, dt2, t2);
        dist2 = pt_d2_unclassified(p, t0, t1, t2);
        dist = std::sqrt(dist2);
        if (t != 0 && ((dist2 - th2) / (dist + thickness) < gap)) { *iters = it + 1; break; }
        t += tlb;
        if (t > toc_prev) { *iters = it + 1; *toc = t; return 0; }
    }
    *toc = t;
    return 1;
}

static inline double ee_dfunc(V3 ea0, V3 ea1, V3 eb0, V3 eb1, double th2, double* dist2)
{
    double d2 = ee_d2_unclassified(ea0, ea1, eb0, eb1);
    double f = d2 - th2;
    if (f <= 0) {  // CCD.h:339-345
        double a = pp_d2(ea0, eb0), b = pp_d2(ea0, eb1), c = pp_d2(ea1, eb0), d = pp_d2(ea1, eb1);
        d2 = std::min(std::min(std::min(a, b), c), d);
        f = d2 - th2;
    }
    *dist2 = d2;
    return f;
}

int accd_ee(V3 ea0, V3 ea1, V3 eb0, V3 eb1, V3 dea0, V3 dea1, V3 deb0, V3 deb1, double eta,
            double thickness, double* toc, int64_t max_iter, int64_t* iters)
{
    // CCD.h:320-380
    V3 mov = scale(((dea0 + dea1) + deb0) + deb1, 0.25);
    dea0 = dea0 - mov;
    dea1 = dea1 - mov;
    deb0 = deb0 - mov;
    deb1 = deb1 - mov;
    double maxDispMag = std::sqrt(std::max(norm2(dea0), norm2(dea1))) +
                        std::sqrt(std::max(norm2(deb0), norm2(deb1)));
    *iters = 0;
    if (maxDispMag == 0) return 0;
    double th2 = thickness * thickness;
    double dist2;
    double dFunc = ee_dfunc(ea0, ea1, eb0, eb1, th2, &dist2);
    double dist = std::sqrt(dist2);
    double gap = eta * dFunc / (dist + thickness);
    double toc_prev = *toc;
    double t = 0;
    for (int64_t it = 0;; ++it) {
        if (it >= max_iter) { *iters = it; *toc = t; return -1; }
        double tlb = (1 - eta) * dFunc / ((dist + thickness) * maxDispMag);
        ea0 = axpy(tlb, dea0, ea0);
        ea1 = axpy(tlb, dea1, ea1);
        eb0 = axpy(tlb, deb0, eb0);
        eb1 = axpy(tlb, deb1, eb1);
        dFunc = ee_dfunc(ea0, ea1, eb0, eb1, th2, &dist2);
        dist = std::sqrt(dist2);
        if (t != 0 && (dFunc / (dist + thickness) < gap)) { *iters = it + 1; break; }
        t += tlb;
        if (t > toc_prev) { *iters = it + 1; *toc = t; return 0; }
    }
    *toc = t;
    return 1;
}

int accd_pe(V3 p, V3 e0, V3 e1, V3 dp, V3 de0, V3 de1, double eta, double thickness,
            double* toc, int64_t max_iter, int64_t* iters)
{
    // CCD.h:383-432
    V3 mov = divs((dp + de0) + de1, 3.0);
    de0 = de0 - mov;
    de1 = de1 - mov;
    dp = dp - mov;
    double maxDispMag = std::sqrt(norm2(dp)) + std::sqrt(std::max(norm2(de0), norm2(de1)));
    *iters = 0;
    if (maxDispMag == 0) return 0;
    double th2 = thickness * thickness;
    double dist2 = pe_d2_unclassified(p, e0, e1);
    double dist = std::sqrt(dist2);
    double gap = eta * (dist2 - th2) / (dist + thickness);
    double toc_prev = *toc;
    double t = 0;
    for (int64_t it = 0;; ++it) {
        if (it >= max_iter) { *iters = it; *toc = t; return -1; }
        double tlb = (1 - eta) * (dist2 - th2) / ((dist + thickness) * maxDispMag);
        p = axpy(tlb, dp, p);
        e0 = axpy(tlb, de0, e0);
        e1 = axpy(tlb, de1, e1);
        dist2 = pe_d2_unclassified(p, e0, e1);
        dist = std::sqrt(dist2);
        if (t != 0 && (dist2 - th2) / (dist + thickness) < gap) { *iters = it + 1; break; }
        t += tlb;
        if (t > toc_prev) { *iters = it + 1; *toc = t; return 0; }
    }
    *toc = t;
    return 1;
}

int accd_pp(V3 p0, V3 p1, V3 dp0, V3 dp1, double eta, double thickness, double* toc,
            int64_t max_iter, int64_t* iters)
{
    // CCD.h:434-482
    V3 mov = scale(dp0 + dp1, 0.5);
    dp1 = dp1 - mov;
    dp0 = dp0 - mov;
    double maxDispMag = std::sqrt(norm2(dp0)) + std::sqrt(norm2(dp1));
    *iters = 0;
    if (maxDispMag == 0) return 0;
    double th2 = thickness * thickness;
    double dist2 = pp_d2(p0, p1);
    double dist = std::sqrt(dist2);
    double gap = eta * (dist2 - th2) / (dist + thickness);
    double toc_prev = *toc;
    double t = 0;
    for (int64_t it = 0;; ++it) {
        if (it >= max_iter) { *iters = it; *toc = t; return -1; }
        double tlb = (1 - eta) * (dist2 - th2) / ((dist + thickness) * maxDispMag);
        p0 = axpy(tlb, dp0, p0);
        p1 = axpy(tlb, dp1, p1);
        dist2 = pp_d2(p0, p1);
        dist = std::sqrt(dist2);
        if (t != 0 && (dist2 - th2) / (dist + thickness) < gap) { *iters = it + 1; break; }
        t += tlb;
        if (t > toc_prev) { *iters = it + 1; *toc = t; return 0; }
    }
    *toc = t;
    return 1;
}

}  // namespace orc
