// Shell element energies, FP64 gradients and PSD-projected Hessians (FP64 or FP32).
//
// Membrane (Library/FEM/Shell/MEMBRANE.h:7-290): with e1 = x2 - x1, e2 = x3 - x1,
// A_ab = e_a . e_b and P the inverse rest first fundamental form,
//   NH:   psi = k (mu/2 (tr(PA) - 2 - 2 lnJ) + lambda/2 lnJ^2),  lnJ = ln(det A det P)/2, k = h^2 vol
//   StVK: psi = k/4 (lambda/2 tr(M)^2 + mu tr(M^2)),  M = PA - I
// S = dpsi/dA gives dpsi/de_a = 2 sum_d S_ad e_d, and the e-space Hessian block
//   H_ab = 2 S_ab I + 2 sum_{d,f} (C_{ad,bf} + C_{ad,fb}) e_d e_f^T,  C = dS/dA,
// which reduces to
//   StVK: 2 S_ab I + k [lambda q_a q_b^T + mu P_ab G + mu q_b q_a^T],      q_a = sum_d P_ad e_d,
//                                                                        G = sum_df P_df e_d e_f^T
//   NH:   2 S_ab I + 2k [lambda/2 r_a r_b^T - c Q_ab R - c r_b r_a^T],   Q = A^-1, c = (lambda lnJ - mu)/2,
//                                                                        r_a = sum_d Q_ad e_d, R = sum Q_df e_d e_f^T
// (for StVK k already carries the 1/4, so the bracket coefficient is 4k/4).
//
// Hinge bending (BENDING.h:52-77, 175-210; DIHEDRAL_ANGLE.h): psi = c (theta - thetabar)^2,
// c = h^2 k_b |ebar| / hbar.  With stencil (x0, x1, x2, x3), hinge edge x1-x2,
// e0 = x2 - x1, n1 = e0 x (x0 - x1), n2 = (x3 - x1) x e0, every component of
// grad theta has the form s(x) n/|n|^2; its Jacobian is assembled from
// d(n/|n|^2) = (I/|n|^2 - 2 n n^T/|n|^4) dn and the gradients of the scalars s.
//
// All element Hessians are translation invariant; they are PSD-projected in the
// orthonormal complement of translations (K = Q H Q^T, 6x6 for triangles, 9x9 for
// hinges), which equals makePD of the full matrix.
#pragma once
#include "derivs.cuh"

namespace cipc {

// Helmert rows q_i (orthonormal, orthogonal to the all-ones vector), i < nv - 1
CIPC_HD double helmert(int nv, int i, int v)
{
    const double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637, r12 = 0.28867513459481288225;
    if (i == 0) return v == 0 ? r2 : (v == 1 ? -r2 : 0.0);
    if (i == 1) return v < 2 ? r6 : (v == 2 ? -2 * r6 : 0.0);
    (void)nv;
    return v < 3 ? r12 : (v == 3 ? -3 * r12 : 0.0);
}

// H (m x m, m = 3 NV) translation invariant -> PSD projection in place
template <typename T, int NV>
CIPC_HD void project_translation_free(T (&H)[3 * NV][3 * NV])
{
    constexpr int M = 3 * (NV - 1);
    constexpr int MX = 3 * NV;
    T K[M][M];
    // W = Q H  (M x MX)
    T W[M][MX];
#pragma unroll
    for (int i = 0; i < NV - 1; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int q = 0; q < MX; ++q) {
                T s = 0;
#pragma unroll
                for (int v = 0; v < NV; ++v) s += (T)helmert(NV, i, v) * H[3 * v + c][q];
                W[3 * i + c][q] = s;
            }
#pragma unroll
    for (int p = 0; p < M; ++p)
#pragma unroll
        for (int j = 0; j < NV - 1; ++j)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                T s = 0;
#pragma unroll
                for (int v = 0; v < NV; ++v) s += W[p][3 * v + c] * (T)helmert(NV, j, v);
                K[p][3 * j + c] = s;
            }
    jacobi_psd<T, M>(K);
#pragma unroll
    for (int p = 0; p < MX; ++p)
#pragma unroll
        for (int q = p; q < MX; ++q) {
            const int v = p / 3, c = p % 3, v2 = q / 3, c2 = q % 3;
            T s = 0;
#pragma unroll
            for (int i = 0; i < NV - 1; ++i)
#pragma unroll
                for (int j = 0; j < NV - 1; ++j)
                    s += (T)(helmert(NV, i, v) * helmert(NV, j, v2)) * K[3 * i + c][3 * j + c2];
            H[p][q] = s;
            H[q][p] = s;
        }
}

// ---------------------------------------------------------------------------
// Membrane
// ---------------------------------------------------------------------------
struct MembraneOut {
    double E;
    double g[9];
};

// energy and FP64 gradient; S (dpsi/dA, entries s00 s01 s11) returned for the Hessian
CIPC_HD void membrane_eg(const d3 (&x)[3], const double* P, double k, double lam, double mu, int nh, MembraneOut& o,
                         double (&S)[3], double& cNH)
{
    const d3 e1 = x[1] - x[0], e2 = x[2] - x[0];
    const double a00 = dot(e1, e1), a01 = dot(e1, e2), a11 = dot(e2, e2);
    const double p00 = P[0], p01 = P[1], p11 = P[2];
    if (nh) {
        const double det = a00 * a11 - a01 * a01;
        const double lnJ = log(det * (p00 * p11 - p01 * p01)) / 2;
        const double tr = p00 * a00 + 2 * p01 * a01 + p11 * a11;
        o.E = k * (mu / 2 * (tr - 2 - 2 * lnJ) + lam / 2 * lnJ * lnJ);
        const double c = (-mu + lam * lnJ) / 2;
        cNH = c;
        S[0] = k * (mu / 2 * p00 + c * a11 / det);
        S[1] = k * (mu / 2 * p01 - c * a01 / det);
        S[2] = k * (mu / 2 * p11 + c * a00 / det);
    } else {
        const double m00 = p00 * a00 + p01 * a01 - 1, m01 = p00 * a01 + p01 * a11;
        const double m10 = p01 * a00 + p11 * a01, m11 = p01 * a01 + p11 * a11 - 1;
        const double trM = m00 + m11;
        o.E = k / 4 * (0.5 * lam * trM * trM + mu * (m00 * m00 + 2 * m01 * m10 + m11 * m11));
        const double mp00 = m00 * p00 + m01 * p01, mp01 = m00 * p01 + m01 * p11;
        const double mp10 = m10 * p00 + m11 * p01, mp11 = m10 * p01 + m11 * p11;
        const double c4 = k / 4;
        S[0] = c4 * (lam * trM * p00 + 2 * mu * mp00);
        S[1] = c4 * (lam * trM * p01 + mu * (mp01 + mp10));
        S[2] = c4 * (lam * trM * p11 + 2 * mu * mp11);
        cNH = 0;
    }
    const d3 g2 = scl(e1, 2 * S[0]) + scl(e2, 2 * S[1]);
    const d3 g3 = scl(e1, 2 * S[1]) + scl(e2, 2 * S[2]);
    o.g[3] = g2.x; o.g[4] = g2.y; o.g[5] = g2.z;
    o.g[6] = g3.x; o.g[7] = g3.y; o.g[8] = g3.z;
    o.g[0] = -(g2.x + g3.x);
    o.g[1] = -(g2.y + g3.y);
    o.g[2] = -(g2.z + g3.z);
}

// 9x9 vertex Hessian (before projection) in T
template <typename T>
CIPC_HD void membrane_hess(const d3 (&x)[3], const double* P, double k, double lam, double mu, int nh,
                           const double (&S)[3], double cNH, T (&H)[9][9])
{
    const d3 e1 = x[1] - x[0], e2 = x[2] - x[0];
    const double ev[2][3] = {{e1.x, e1.y, e1.z}, {e2.x, e2.y, e2.z}};
    double Mt[2][2];  // P (StVK) or Q = A^-1 (NH)
    if (nh) {
        const double a00 = dot(e1, e1), a01 = dot(e1, e2), a11 = dot(e2, e2);
        const double det = a00 * a11 - a01 * a01;
        Mt[0][0] = a11 / det;
        Mt[0][1] = Mt[1][0] = -a01 / det;
        Mt[1][1] = a00 / det;
    } else {
        Mt[0][0] = P[0];
        Mt[0][1] = Mt[1][0] = P[1];
        Mt[1][1] = P[2];
    }
    double qv[2][3], G[3][3];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i) qv[a][i] = Mt[a][0] * ev[0][i] + Mt[a][1] * ev[1][i];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) G[i][j] = ev[0][i] * qv[0][j] + ev[1][i] * qv[1][j];
    const double Sm[2][2] = {{S[0], S[1]}, {S[1], S[2]}};
    double HE[6][6];
    // coefficients of (q_a q_b^T, M_ab G, q_b q_a^T)
    double c1, c2, c3;
    if (nh) {
        c1 = 2 * k * lam / 2;
        c2 = -2 * k * cNH;
        c3 = -2 * k * cNH;
    } else {
        c1 = k * lam;
        c2 = k * mu;
        c3 = k * mu;
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    HE[3 * a + i][3 * b + j] = (i == j ? 2 * Sm[a][b] : 0.0) + c1 * qv[a][i] * qv[b][j] +
                                               c2 * Mt[a][b] * G[i][j] + c3 * qv[b][i] * qv[a][j];
    // vertex Hessian: x1 = -(e1 + e2) direction
#pragma unroll
    for (int va = 0; va < 3; ++va)
#pragma unroll
        for (int vb = 0; vb < 3; ++vb)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    double s = 0;
#pragma unroll
                    for (int a = 0; a < 2; ++a)
#pragma unroll
                        for (int b = 0; b < 2; ++b) {
                            const int ca = (va == 0) ? -1 : (va == a + 1 ? 1 : 0);
                            const int cb = (vb == 0) ? -1 : (vb == b + 1 ? 1 : 0);
                            if (ca && cb) s += ca * cb * HE[3 * a + i][3 * b + j];
                        }
                    H[3 * va + i][3 * vb + j] = (T)s;
                }
}

// ---------------------------------------------------------------------------
// Hinge bending
// ---------------------------------------------------------------------------
// dihedral angle (atan2 form: equal to the reference's acos form, better
// conditioned near flat), sign by (nB x nA).(x1 - x2)
CIPC_HD double dihedral_angle(const d3 (&x)[4])
{
    const d3 nA = cross(x[1] - x[0], x[2] - x[0]);
    const d3 nB = cross(x[2] - x[3], x[1] - x[3]);
    const d3 c = cross(nB, nA);
    double th = atan2(sqrt(n2(c)), dot(nA, nB));
    if (dot(c, x[1] - x[2]) < 0) th = -th;
    return th;
}

// grad theta (12) in FP64
CIPC_HD void dihedral_grad(const d3 (&x)[4], double (&g)[12])
{
    const d3 e0 = x[2] - x[1], e1 = x[0] - x[1], e2 = x[3] - x[1], e3 = x[0] - x[2], e4 = x[3] - x[2];
    const d3 nA = cross(e0, e1), nB = cross(e2, e0);
    const double nAs = n2(nA), nBs = n2(nB), e0n = sqrt(n2(e0));
    const d3 ga = scl(nA, -e0n / nAs);
    const d3 gb = scl(nA, -dot(e0, e3) / (e0n * nAs)) + scl(nB, -dot(e0, e4) / (e0n * nBs));
    const d3 gc = scl(nA, dot(e0, e1) / (e0n * nAs)) + scl(nB, dot(e0, e2) / (e0n * nBs));
    const d3 gd = scl(nB, -e0n / nBs);
    const d3 gg[4] = {ga, gb, gc, gd};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        g[3 * k] = gg[k].x;
        g[3 * k + 1] = gg[k].y;
        g[3 * k + 2] = gg[k].z;
    }
}

// Hessian of theta (12x12), full, in double
CIPC_HD void dihedral_hess(const d3 (&x)[4], double (&H)[12][12])
{
    const d3 e0 = x[2] - x[1], e1 = x[0] - x[1], e2 = x[3] - x[1], e3 = x[0] - x[2], e4 = x[3] - x[2];
    const d3 nA = cross(e0, e1), nB = cross(e2, e0);
    const double nAs = n2(nA), nBs = n2(nB), e0n = sqrt(n2(e0));
#pragma unroll
    for (int i = 0; i < 12; ++i)
#pragma unroll
        for (int j = 0; j < 12; ++j) H[i][j] = 0;
    // dn/dx_v for nA = e0 x e1 (e0 = x2 - x1, e1 = x0 - x1) and nB = e2 x e0 (e2 = x3 - x1):
    //   dn1/dx0 = [e0]x, dn1/dx2 = -[e1]x, dn1/dx1 = -[e0]x + [e1]x
    //   dn2/dx3 = -[e0]x, dn2/dx2 = [e2]x, dn2/dx1 = [e0]x - [e2]x
    auto skewm = [](d3 v, double (&S)[3][3], double s) {
        S[0][0] = 0; S[0][1] = -v.z * s; S[0][2] = v.y * s;
        S[1][0] = v.z * s; S[1][1] = 0; S[1][2] = -v.x * s;
        S[2][0] = -v.y * s; S[2][1] = v.x * s; S[2][2] = 0;
    };
    double Dn1[4][3][3], Dn2[4][3][3];
    {
        double A[3][3], B[3][3];
        skewm(e0, Dn1[0], 1.0);
        skewm(e1, Dn1[2], -1.0);
        skewm(e0, A, -1.0);
        skewm(e1, B, 1.0);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                Dn1[1][i][j] = A[i][j] + B[i][j];
                Dn1[3][i][j] = 0;
            }
        skewm(e0, Dn2[3], -1.0);
        skewm(e2, Dn2[2], 1.0);
        skewm(e0, A, 1.0);
        skewm(e2, B, -1.0);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                Dn2[1][i][j] = A[i][j] + B[i][j];
                Dn2[0][i][j] = 0;
            }
    }
    // Pi = I/|n|^2 - 2 n n^T / |n|^4, du/dx_v = Pi dn/dx_v for u = n/|n|^2
    double Du1[4][3][3], Du2[4][3][3];
    const double nv1[3] = {nA.x, nA.y, nA.z}, nv2[3] = {nB.x, nB.y, nB.z};
    for (int v = 0; v < 4; ++v)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s1 = Dn1[v][i][j] / nAs, s2 = Dn2[v][i][j] / nBs;
                double t1 = 0, t2 = 0;
                for (int k = 0; k < 3; ++k) {
                    t1 += nv1[k] * Dn1[v][k][j];
                    t2 += nv2[k] * Dn2[v][k][j];
                }
                Du1[v][i][j] = s1 - 2 * nv1[i] * t1 / (nAs * nAs);
                Du2[v][i][j] = s2 - 2 * nv2[i] * t2 / (nBs * nBs);
            }
    const double u1[3] = {nA.x / nAs, nA.y / nAs, nA.z / nAs}, u2[3] = {nB.x / nBs, nB.y / nBs, nB.z / nBs};
    // scalar gradients: |e0| -> d/dx1 = -e0/|e0|, d/dx2 = e0/|e0|
    const d3 ue0 = scl(e0, 1.0 / e0n);
    // row block 0: s = -|e0| u1 ; row block 3: s = -|e0| u2
    // row block 1: s = -(e0.e3)/|e0| u1 - (e0.e4)/|e0| u2
    // row block 2: s = (e0.e1)/|e0| u1 + (e0.e2)/|e0| u2
    // gradient of f(x) = (e0.w)/|e0| with w = xa - xb: df = (w.de0 + e0.dw)/|e0| - (e0.w) ue0.de0/|e0|^2
    auto ratio_grad = [&](d3 w, int a, int b, double (&gs)[12]) {
        // w = x_a - x_b
        for (int k = 0; k < 12; ++k) gs[k] = 0;
        const double ew = dot(e0, w);
        const d3 de0 = scl(w, 1.0 / e0n) - scl(ue0, ew / (e0n * e0n));  // derivative wrt e0
        // e0 = x2 - x1
        gs[6] += de0.x; gs[7] += de0.y; gs[8] += de0.z;
        gs[3] -= de0.x; gs[4] -= de0.y; gs[5] -= de0.z;
        const d3 dw = scl(e0, 1.0 / e0n);
        gs[3 * a] += dw.x; gs[3 * a + 1] += dw.y; gs[3 * a + 2] += dw.z;
        gs[3 * b] -= dw.x; gs[3 * b + 1] -= dw.y; gs[3 * b + 2] -= dw.z;
    };
    double gs[12];
    auto add_term = [&](int row, double s, const double* gsv, const double (&u)[3], const double (&Du)[4][3][3]) {
        for (int i = 0; i < 3; ++i)
            for (int v = 0; v < 4; ++v)
                for (int j = 0; j < 3; ++j)
                    H[3 * row + i][3 * v + j] += u[i] * gsv[3 * v + j] + s * Du[v][i][j];
    };
    // |e0| gradient
    double ge0[12] = {0};
    ge0[3] = -ue0.x; ge0[4] = -ue0.y; ge0[5] = -ue0.z;
    ge0[6] = ue0.x; ge0[7] = ue0.y; ge0[8] = ue0.z;
    double mge0[12];
    for (int k = 0; k < 12; ++k) mge0[k] = -ge0[k];
    add_term(0, -e0n, mge0, u1, Du1);
    add_term(3, -e0n, mge0, u2, Du2);
    // row 1
    ratio_grad(e3, 0, 2, gs);
    for (int k = 0; k < 12; ++k) gs[k] = -gs[k];
    add_term(1, -dot(e0, e3) / e0n, gs, u1, Du1);
    ratio_grad(e4, 3, 2, gs);
    for (int k = 0; k < 12; ++k) gs[k] = -gs[k];
    add_term(1, -dot(e0, e4) / e0n, gs, u2, Du2);
    // row 2
    ratio_grad(e1, 0, 1, gs);
    add_term(2, dot(e0, e1) / e0n, gs, u1, Du1);
    ratio_grad(e2, 3, 1, gs);
    add_term(2, dot(e0, e2) / e0n, gs, u2, Du2);
    // symmetrize rounding
    for (int i = 0; i < 12; ++i)
        for (int j = i + 1; j < 12; ++j) {
            const double s = 0.5 * (H[i][j] + H[j][i]);
            H[i][j] = H[j][i] = s;
        }
}

// Hessian of theta (12x12) in T from the hinge's edge vectors (taken in FP64 by
// the caller: e0 = x2 - x1, e1 = x0 - x1, e2 = x3 - x1, e3 = x0 - x2, e4 = x3 - x2),
// the same expressions as dihedral_hess, formed in the caller's Hessian array:
// the bending kernel's form in both precisions (FP32 for the mixed-precision
// Hessians, which takes it off GB300's narrow FP64 pipe)
template <typename T>
CIPC_HD void dihedral_hess_t(const T (&E)[5][3], T (&H)[12][12])
{
    auto crs = [](const T* a, const T* b, T* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto dt = [](const T* a, const T* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    const T *e0 = E[0], *e1 = E[1], *e2 = E[2], *e3 = E[3], *e4 = E[4];
    T nA[3], nB[3];
    crs(e0, e1, nA);
    crs(e2, e0, nB);
    const T nAs = dt(nA, nA), nBs = dt(nB, nB), e0n = sqrt(dt(e0, e0));
#pragma unroll
    for (int i = 0; i < 12; ++i)
#pragma unroll
        for (int j = 0; j < 12; ++j) H[i][j] = 0;
    auto skewm = [](const T* v, T (&S)[3][3], T s) {
        S[0][0] = 0; S[0][1] = -v[2] * s; S[0][2] = v[1] * s;
        S[1][0] = v[2] * s; S[1][1] = 0; S[1][2] = -v[0] * s;
        S[2][0] = -v[1] * s; S[2][1] = v[0] * s; S[2][2] = 0;
    };
    T Dn1[4][3][3], Dn2[4][3][3];
    {
        T A[3][3], B[3][3];
        skewm(e0, Dn1[0], T(1));
        skewm(e1, Dn1[2], T(-1));
        skewm(e0, A, T(-1));
        skewm(e1, B, T(1));
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                Dn1[1][i][j] = A[i][j] + B[i][j];
                Dn1[3][i][j] = 0;
            }
        skewm(e0, Dn2[3], T(-1));
        skewm(e2, Dn2[2], T(1));
        skewm(e0, A, T(1));
        skewm(e2, B, T(-1));
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                Dn2[1][i][j] = A[i][j] + B[i][j];
                Dn2[0][i][j] = 0;
            }
    }
    T Du1[4][3][3], Du2[4][3][3];
    const T iA = T(1) / nAs, iB = T(1) / nBs;
    for (int v = 0; v < 4; ++v)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                T t1 = 0, t2 = 0;
                for (int k = 0; k < 3; ++k) {
                    t1 += nA[k] * Dn1[v][k][j];
                    t2 += nB[k] * Dn2[v][k][j];
                }
                Du1[v][i][j] = Dn1[v][i][j] * iA - 2 * nA[i] * t1 * iA * iA;
                Du2[v][i][j] = Dn2[v][i][j] * iB - 2 * nB[i] * t2 * iB * iB;
            }
    const T u1[3] = {nA[0] * iA, nA[1] * iA, nA[2] * iA}, u2[3] = {nB[0] * iB, nB[1] * iB, nB[2] * iB};
    const T ie0 = T(1) / e0n;
    const T ue0[3] = {e0[0] * ie0, e0[1] * ie0, e0[2] * ie0};
    auto ratio_grad = [&](const T* w, int a, int b, T (&gs)[12]) {
        for (int k = 0; k < 12; ++k) gs[k] = 0;
        const T ew = dt(e0, w);
        for (int d = 0; d < 3; ++d) {
            const T de0 = w[d] * ie0 - ue0[d] * ew * ie0 * ie0;
            gs[6 + d] += de0;
            gs[3 + d] -= de0;
            const T dw = e0[d] * ie0;
            gs[3 * a + d] += dw;
            gs[3 * b + d] -= dw;
        }
    };
    auto add_term = [&](int row, T sc, const T* gsv, const T (&u)[3], const T (&Du)[4][3][3]) {
        for (int i = 0; i < 3; ++i)
            for (int v = 0; v < 4; ++v)
                for (int j = 0; j < 3; ++j) H[3 * row + i][3 * v + j] += u[i] * gsv[3 * v + j] + sc * Du[v][i][j];
    };
    T gs[12];
    T mge0[12] = {0, 0, 0, ue0[0], ue0[1], ue0[2], -ue0[0], -ue0[1], -ue0[2], 0, 0, 0};
    add_term(0, -e0n, mge0, u1, Du1);
    add_term(3, -e0n, mge0, u2, Du2);
    ratio_grad(e3, 0, 2, gs);
    for (int k = 0; k < 12; ++k) gs[k] = -gs[k];
    add_term(1, -dt(e0, e3) * ie0, gs, u1, Du1);
    ratio_grad(e4, 3, 2, gs);
    for (int k = 0; k < 12; ++k) gs[k] = -gs[k];
    add_term(1, -dt(e0, e4) * ie0, gs, u2, Du2);
    ratio_grad(e1, 0, 1, gs);
    add_term(2, dt(e0, e1) * ie0, gs, u1, Du1);
    ratio_grad(e2, 3, 1, gs);
    add_term(2, dt(e0, e2) * ie0, gs, u2, Du2);
    for (int i = 0; i < 12; ++i)
        for (int j = i + 1; j < 12; ++j) {
            const T s = T(0.5) * (H[i][j] + H[j][i]);
            H[i][j] = H[j][i] = s;
        }
}

}  // namespace cipc
