// Device derivatives of contact squared distances, the log barrier and the EE
// mollifier, plus the symmetric Jacobi PSD projection.
//
// Squared distances are written in reduced (translation-free) variables:
//   PT: a = p - t0,  e1 = t1 - t0,  e2 = t2 - t0      f = (a.(e1 x e2))^2 / |e1 x e2|^2
//   EE: a = eb0 - ea0, e1 = ea1 - ea0, e2 = eb1 - eb0  (same form)
//   PE: a = e0 - p,  b = e1 - p                       f = |a x b|^2 / |b - a|^2
//   PP: d = p0 - p1                                   f = |d|^2
// A pair's vertex Hessian is J^T Hr J with J = C (x) I3 for a constant incidence
// matrix C.  Writing C = M Q with Q the orthonormal (Helmert) basis of the
// translation complement, J^T Hr J = (Q (x) I)^T K (Q (x) I) with K = M^T Hr M,
// and its PSD projection is (Q (x) I)^T PSD(K) (Q (x) I).  The eigen-problem is
// therefore 9x9 (PT, EE), 6x6 (PE) or 3x3 (PP) instead of 12x12/9x9/6x6, and the
// result equals the reference's makePD of the full matrix (Math/UTILS.h:9-27).
#pragma once
#include "geom.cuh"

namespace cipc {

template <typename T>
struct t3 {
    T x, y, z;
};
template <typename T>
CIPC_HD t3<T> tv(d3 v)
{
    return t3<T>{(T)v.x, (T)v.y, (T)v.z};
}
template <typename T>
CIPC_HD T tdot(t3<T> a, t3<T> b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
CIPC_HD t3<T> tcross(t3<T> a, t3<T> b)
{
    return t3<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
CIPC_HD t3<T> tsub(t3<T> a, t3<T> b)
{
    return t3<T>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
CIPC_HD T comp(t3<T> a, int i)
{
    return i == 0 ? a.x : (i == 1 ? a.y : a.z);
}

// H[3bi+i][3bj+j] += s * B_ij (and the mirrored block when bi != bj), where
// B = [v]x (kind 0), |v|^2 I - v v^T (kind 1), u v^T - (u.v) I (kind 2)
template <typename T, int N>
CIPC_HD void add_skew(T (&H)[N][N], int bi, int bj, t3<T> v, T s)
{
    // [v]x = [[0,-vz,vy],[vz,0,-vx],[-vy,vx,0]]
    const T B[3][3] = {{0, -v.z, v.y}, {v.z, 0, -v.x}, {-v.y, v.x, 0}};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            H[3 * bi + i][3 * bj + j] += s * B[i][j];
            H[3 * bj + j][3 * bi + i] += s * B[i][j];
        }
}

// Gradient / Hessian of |e1 x e2|^2 into variable blocks k1, k2.
// n = e1 x e2 is passed in: it is computed in FP64 by the caller because it
// cancels for nearly parallel e1, e2.
template <typename T, int N>
CIPC_HD void crossn2_add(t3<T> e1, t3<T> e2, t3<T> n, int k1, int k2, T s, T (&g)[N], T (&H)[N][N])
{
    const t3<T> g1 = tcross(e2, n), g2 = tcross(n, e1);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        g[3 * k1 + i] += s * 2 * comp(g1, i);
        g[3 * k2 + i] += s * 2 * comp(g2, i);
    }
    const T n11 = tdot(e1, e1), n22 = tdot(e2, e2), d12 = tdot(e1, e2);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const T b11 = (i == j ? n22 : T(0)) - comp(e2, i) * comp(e2, j);
            const T b22 = (i == j ? n11 : T(0)) - comp(e1, i) * comp(e1, j);
            const T b12 = comp(e1, i) * comp(e2, j) - (i == j ? d12 : T(0));
            H[3 * k1 + i][3 * k1 + j] += s * 2 * b11;
            H[3 * k2 + i][3 * k2 + j] += s * 2 * b22;
            H[3 * k1 + i][3 * k2 + j] += s * 2 * b12;
            H[3 * k2 + j][3 * k1 + i] += s * 2 * b12;
        }
    add_skew<T, N>(H, k1, k2, n, T(-2) * s);
}

// f = u^2/w (PT, EE): reduced gradient and Hessian over (a, e1, e2).  n = e1 x e2
// and r = u / w are passed in from FP64: u = a.n cancels when the separation is
// small against the primitive size.
template <typename T>
CIPC_HD void u2w_derivs(t3<T> a, t3<T> e1, t3<T> e2, t3<T> n, T r, T (&g)[9], T (&H)[9][9])
{
    const T w = tdot(n, n);
    T gu[9], gw[9];
    T Hw[9][9];
    const t3<T> t1 = tcross(e2, a), t2 = tcross(a, e1);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gu[i] = comp(n, i);
        gu[3 + i] = comp(t1, i);
        gu[6 + i] = comp(t2, i);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        gw[i] = 0;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            H[i][j] = 0;
            Hw[i][j] = 0;
        }
    }
    // 2 r Hu: blocks (a,e1) = -[e2]x, (a,e2) = [e1]x, (e1,e2) = -[a]x
    add_skew<T, 9>(H, 0, 1, e2, T(-2) * r);
    add_skew<T, 9>(H, 0, 2, e1, T(2) * r);
    add_skew<T, 9>(H, 1, 2, a, T(-2) * r);
    crossn2_add<T, 9>(e1, e2, n, 1, 2, T(1), gw, Hw);
    const T c2w = T(2) / w, r2 = r * r;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const T gvi = gu[i] - r * gw[i];
        g[i] = r * (T(2) * gu[i] - r * gw[i]);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const T gvj = gu[j] - r * gw[j];
            H[i][j] += c2w * gvi * gvj - r2 * Hw[i][j];
        }
    }
}

// gradient only of u^2/w, FP64 (the Newton residual); u uses the same
// fma-chain dot product as the squared distance itself
CIPC_HD void u2w_grad(d3 a, d3 e1, d3 e2, double (&g)[9])
{
    using T = double;
    const d3 n = cross(e1, e2);
    const T u = dot(a, n), w = dot(n, n);
    const T r = u / w;
    const d3 t1 = cross(e2, a), t2 = cross(a, e1);
    const d3 w1 = cross(e2, n), w2 = cross(n, e1);
    const double nn[3] = {n.x, n.y, n.z}, a1[3] = {t1.x, t1.y, t1.z}, a2[3] = {t2.x, t2.y, t2.z};
    const double b1[3] = {w1.x, w1.y, w1.z}, b2[3] = {w2.x, w2.y, w2.z};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        g[i] = r * (T(2) * nn[i]);
        g[3 + i] = r * (T(2) * a1[i] - r * T(2) * b1[i]);
        g[6 + i] = r * (T(2) * a2[i] - r * T(2) * b2[i]);
    }
}

// gradient only of |a x b|^2 / |b - a|^2 (PE), FP64
CIPC_HD void pe_grad(d3 a, d3 b, double (&g)[6])
{
    const d3 n = cross(a, b);
    const d3 g1 = cross(b, n), g2 = cross(n, a);
    const d3 ba = b - a;
    const double N = dot(n, n), D = dot(ba, ba);
    const double f = N / D;
    const double gN[6] = {2 * g1.x, 2 * g1.y, 2 * g1.z, 2 * g2.x, 2 * g2.y, 2 * g2.z};
    const double gD[6] = {-2 * ba.x, -2 * ba.y, -2 * ba.z, 2 * ba.x, 2 * ba.y, 2 * ba.z};
#pragma unroll
    for (int i = 0; i < 6; ++i) g[i] = (gN[i] - f * gD[i]) / D;
}

// f = |a x b|^2 / |b - a|^2 (PE) over (a, b); n = a x b and f come from FP64
// (a x b cancels for a point close to the line).
template <typename T>
CIPC_HD void pe_derivs(t3<T> a, t3<T> b, t3<T> n, T f, T (&g)[6], T (&H)[6][6])
{
    T gN[6] = {0, 0, 0, 0, 0, 0};
    T HN[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) HN[i][j] = 0;
    crossn2_add<T, 6>(a, b, n, 0, 1, T(1), gN, HN);
    const t3<T> ba = tsub(b, a);
    const T D = tdot(ba, ba);
    const T iD = T(1) / D;
    T gD[6];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gD[i] = T(-2) * comp(ba, i);
        gD[3 + i] = T(2) * comp(ba, i);
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) g[i] = (gN[i] - f * gD[i]) * iD;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const T HD = (i % 3 == j % 3) ? ((i / 3 == j / 3) ? T(2) : T(-2)) : T(0);
            H[i][j] = (HN[i][j] - f * HD - gD[i] * g[j] - g[i] * gD[j]) * iD;
        }
}

// ---------------------------------------------------------------------------
// Cyclic Jacobi PSD projection of a symmetric N x N matrix held in registers.
// A is overwritten by V max(L, 0) V^T when its smallest eigenvalue is negative
// and left unchanged otherwise (the reference's makePD early return).
// ---------------------------------------------------------------------------
template <typename T, int N>
CIPC_HD void jacobi_psd(T (&A)[N][N])
{
    T scale = 0;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) scale = fmax(scale, fabs(A[i][j]));
    if (!(scale > 0)) return;
    const T inv = T(1) / scale;
    T B[N][N], V[N][N];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) {
            B[i][j] = A[i][j] * inv;
            V[i][j] = (i == j) ? T(1) : T(0);
        }
    const int max_sweeps = sizeof(T) == 8 ? 14 : 10;
    const T tol = sizeof(T) == 8 ? T(1e-30) : T(1e-13);
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        T off = 0, tot = 0;
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) {
                const T b2 = B[i][j] * B[i][j];
                tot += b2;
                if (i != j) off += b2;
            }
        if (off <= tol * tot) break;
#pragma unroll
        for (int p = 0; p < N - 1; ++p)
#pragma unroll
            for (int q = p + 1; q < N; ++q) {
                const T apq = B[p][q];
                if (apq != T(0)) {
                    const T theta = (B[q][q] - B[p][p]) / (T(2) * apq);
                    const T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
                    const T c = T(1) / sqrt(t * t + T(1));
                    const T s = t * c;
                    B[p][p] = B[p][p] - t * apq;
                    B[q][q] = B[q][q] + t * apq;
                    B[p][q] = T(0);
                    B[q][p] = T(0);
#pragma unroll
                    for (int k = 0; k < N; ++k) {
                        if (k != p && k != q) {
                            const T akp = B[k][p], akq = B[k][q];
                            const T nkp = c * akp - s * akq;
                            const T nkq = s * akp + c * akq;
                            B[k][p] = nkp;
                            B[p][k] = nkp;
                            B[k][q] = nkq;
                            B[q][k] = nkq;
                        }
                        const T vkp = V[k][p], vkq = V[k][q];
                        V[k][p] = c * vkp - s * vkq;
                        V[k][q] = s * vkp + c * vkq;
                    }
                }
            }
    }
    T lam[N];
    bool neg = false;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        lam[i] = B[i][i];
        if (lam[i] < T(0)) {
            neg = true;
            lam[i] = T(0);
        }
    }
    if (!neg) return;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) {
            T s = 0;
#pragma unroll
            for (int k = 0; k < N; ++k) s += V[i][k] * lam[k] * V[j][k];
            A[i][j] = s * scale;
            A[j][i] = s * scale;
        }
}

// ---------------------------------------------------------------------------
// Log barrier b(s) = -kappa (s - shat)^2 ln(s / shat) and its first two
// derivatives (Math/BARRIER.h:9-62, non-elastic branch).
// ---------------------------------------------------------------------------
CIPC_HD void barrier3(double d, double dHat, double kappa, double& b, double& g, double& h)
{
    const double t2 = d - dHat;
    const double lg = log(d / dHat);
    b = -kappa * t2 * t2 * lg;
    g = kappa * (t2 * lg * -2.0 - (t2 * t2) / d);
    h = kappa * ((lg * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2));
}

}  // namespace cipc
