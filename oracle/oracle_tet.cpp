// Test infrastructure: CPU restatement of the volumetric Neo-Hookean tetrahedron
// of the shell step (Library/Physics/NEOHOOKEAN.h: Compute_E, first Piola stress,
// Compute_DP_Div_DF with projection; used by Library/FEM/Shell/INC_POTENTIAL.h:
// 97-109, 228-229, 354-364), with derivatives by nested forward-mode duals over
// the nine entries of F (independent of the GPU's closed-form stress derivative).
//
//   F = [x1-x0, x2-x0, x3-x0] Dm^-1,  psi = mu/2 (|F|^2 - 3) - mu ln J + lambda/2 ln^2 J,
//   energy w psi with w = h^2 vol; infeasible if det F <= 0.  The 9x9 Hessian in F
//   is made PSD (the reference's per-block projection in the singular frame is the
//   projection of the same matrix) and mapped to the 12x12 vertex Hessian.
#include <cmath>

#include "oracle_dual.h"
#include "oracle_math.h"

namespace orc_tet {

using namespace orc_dual;

template <typename T>
T psi(const T* f, double lam, double mu)
{
    // f row-major: f[3 i + j] = F_ij
    const T J = f[0] * (f[4] * f[8] - f[5] * f[7]) - f[1] * (f[3] * f[8] - f[5] * f[6]) +
                f[2] * (f[3] * f[7] - f[4] * f[6]);
    T n2 = C<T>(0.0);
    for (int k = 0; k < 9; ++k) n2 = n2 + f[k] * f[k];
    const T lnJ = ln(J);
    return C<T>(0.5 * mu) * (n2 - C<T>(3.0)) - C<T>(mu) * lnJ + C<T>(0.5 * lam) * lnJ * lnJ;
}

}  // namespace orc_tet

extern "C" {

// One tetrahedron: x12 its vertices, Dinv = Dm^-1 (row-major), w = h^2 vol.
// Returns the energy (0 if inverted); g (12) and H (144) when non-null;
// *valid = 0 if det F <= 0.
double orc_tet_nh(const double* x12, const double* Dinv, double w, double lam, double mu, int project, double* g,
                  double* H, int* valid)
{
    using namespace orc_tet;
    double c[4][3];
    for (int j = 0; j < 3; ++j) {
        c[1][j] = Dinv[j];
        c[2][j] = Dinv[3 + j];
        c[3][j] = Dinv[6 + j];
        c[0][j] = -(c[1][j] + c[2][j] + c[3][j]);
    }
    double f[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int m = 0; m < 4; ++m) s += c[m][j] * x12[3 * m + i];
            f[3 * i + j] = s;
        }
    const double J = f[0] * (f[4] * f[8] - f[5] * f[7]) - f[1] * (f[3] * f[8] - f[5] * f[6]) +
                     f[2] * (f[3] * f[7] - f[4] * f[6]);
    if (valid) *valid = J > 0 ? 1 : 0;
    if (!(J > 0)) {
        if (g)
            for (int k = 0; k < 12; ++k) g[k] = 0;
        if (H)
            for (int k = 0; k < 144; ++k) H[k] = 0;
        return 0;
    }
    D2<9> fd[9];
    for (int k = 0; k < 9; ++k) fd[k] = seed<9>(f[k], k);
    const D2<9> E = psi(fd, lam, mu);
    if (g)
        for (int m = 0; m < 4; ++m)
            for (int i = 0; i < 3; ++i) {
                double s = 0;
                for (int j = 0; j < 3; ++j) s += c[m][j] * E.v.d[3 * i + j];
                g[3 * m + i] = w * s;
            }
    if (H) {
        double HF[81];
        for (int a = 0; a < 9; ++a)
            for (int b = 0; b < 9; ++b) HF[9 * a + b] = w * 0.5 * (E.d[a].d[b] + E.d[b].d[a]);
        if (project) orc::make_pd(9, HF);
        for (int m = 0; m < 4; ++m)
            for (int i = 0; i < 3; ++i)
                for (int n = 0; n < 4; ++n)
                    for (int k = 0; k < 3; ++k) {
                        double s = 0;
                        for (int j = 0; j < 3; ++j)
                            for (int l = 0; l < 3; ++l) s += c[m][j] * c[n][l] * HF[9 * (3 * i + j) + 3 * k + l];
                        H[12 * (3 * m + i) + 3 * n + k] = s;
                    }
    }
    return w * E.v.v;
}

}  // extern "C"
