// Volumetric Neo-Hookean tetrahedra of the shell step (Library/Physics/NEOHOOKEAN.h,
// called from Library/FEM/Shell/INC_POTENTIAL.h:97-109, 228-229, 354-364):
//   F = Ds Dm^-1, Ds = [x1 - x0, x2 - x0, x3 - x0],
//   psi(F) = mu/2 (|F|^2 - 3) - mu ln J + lambda/2 ln^2 J,  J = det F,
// scaled by h^2 vol; J <= 0 makes the state infeasible.  The first Piola stress is
// P = mu (F - F^-T) + lambda ln J F^-T and its derivative
//   dP_ij/dF_kl = mu d_ik d_jl + (mu - lambda ln J) (F^-1)_jk (F^-1)_li
//                 + lambda (F^-T)_ij (F^-T)_kl,
// which is projected to PSD as one 9x9 matrix (the reference projects the same
// matrix block by block in its singular frame) before the map to the 12x12 vertex
// Hessian.
#pragma once
#include "derivs.cuh"
#include "geom.cuh"

namespace cipc {

// F (row-major 3x3) and c[m][j] = dF_ij / dx_m,i (m = 0..3)
CIPC_HD void tet_deform(const d3 (&x)[4], const double* Dinv, double (&F)[3][3], double (&c)[4][3])
{
    const d3 e[3] = {x[1] - x[0], x[2] - x[0], x[3] - x[0]};
    const double E[3][3] = {{e[0].x, e[1].x, e[2].x}, {e[0].y, e[1].y, e[2].y}, {e[0].z, e[1].z, e[2].z}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) F[i][j] = E[i][0] * Dinv[j] + E[i][1] * Dinv[3 + j] + E[i][2] * Dinv[6 + j];
    for (int j = 0; j < 3; ++j) {
        c[1][j] = Dinv[j];
        c[2][j] = Dinv[3 + j];
        c[3][j] = Dinv[6 + j];
        c[0][j] = -(c[1][j] + c[2][j] + c[3][j]);
    }
}

// determinant and inverse of a 3x3 matrix
CIPC_HD double inv33(const double (&F)[3][3], double (&Fi)[3][3])
{
    const double c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    const double c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    const double c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    const double J = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    const double iJ = 1 / J;
    Fi[0][0] = c00 * iJ;
    Fi[1][0] = c01 * iJ;
    Fi[2][0] = c02 * iJ;
    Fi[0][1] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * iJ;
    Fi[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * iJ;
    Fi[2][1] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * iJ;
    Fi[0][2] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * iJ;
    Fi[1][2] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * iJ;
    Fi[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * iJ;
    return J;
}

// energy and gradient (g[12], may be null); w = h^2 vol; false if J <= 0
CIPC_HD bool tet_nh_eg(const d3 (&x)[4], const double* Dinv, double w, double lam, double mu, double& E, double* g)
{
    double F[3][3], c[4][3], Fi[3][3];
    tet_deform(x, Dinv, F, c);
    const double J = inv33(F, Fi);
    if (!(J > 0)) {
        E = 0;
        if (g)
            for (int k = 0; k < 12; ++k) g[k] = 0;
        return false;
    }
    const double lnJ = log(J);
    double f2 = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) f2 += F[i][j] * F[i][j];
    E = w * (0.5 * mu * (f2 - 3) - mu * lnJ + 0.5 * lam * lnJ * lnJ);
    if (g) {
        double P[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) P[i][j] = w * (mu * (F[i][j] - Fi[j][i]) + lam * lnJ * Fi[j][i]);
        for (int m = 0; m < 4; ++m)
            for (int i = 0; i < 3; ++i) g[3 * m + i] = P[i][0] * c[m][0] + P[i][1] * c[m][1] + P[i][2] * c[m][2];
    }
    return true;
}

// 12x12 Hessian with the 9x9 stress derivative projected to PSD (project)
template <typename HT>
CIPC_HD void tet_nh_hess(const d3 (&x)[4], const double* Dinv, double w, double lam, double mu, bool project,
                         HT (&H)[12][12])
{
    double F[3][3], c[4][3], Fi[3][3];
    tet_deform(x, Dinv, F, c);
    const double J = inv33(F, Fi);
    const double lnJ = log(J);
    double A[9][9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l)
                    A[3 * i + j][3 * k + l] = w * ((i == k && j == l ? mu : 0.0) + (mu - lam * lnJ) * Fi[j][k] * Fi[l][i] +
                                                   lam * Fi[j][i] * Fi[l][k]);
    if (project) jacobi_psd<double, 9>(A);
    for (int m = 0; m < 4; ++m)
        for (int n = 0; n < 4; ++n)
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) {
                    double s = 0;
                    for (int j = 0; j < 3; ++j)
                        for (int l = 0; l < 3; ++l) s += c[m][j] * c[n][l] * A[3 * i + j][3 * k + l];
                    H[3 * m + i][3 * n + k] = (HT)s;
                }
}

}  // namespace cipc
