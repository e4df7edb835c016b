// Test infrastructure: CPU restatement of the discrete rod elements of the shell
// step (Library/FEM/Shell/Rod/ROD_STRETCHING.h:9-107, ROD_BENDING.h:9-120,
// DISCRETE_ROD.h:85-150), with derivatives by nested forward-mode dual numbers
// (independent of the GPU's closed forms and of the reference's generated code,
// which the tests compare against).
//
//   stretching (segment x0 x1, rest length L):  E = K L / 2 (|x0 - x1| / L - 1)^2,
//       K = h^2 pi t^2 / 4 * E_young                      (ROD_STRETCHING.h:23-24)
//   bending (hinge x0 x1 x2, lsum = rest |e0| + |e1|):  E = Kb |kb|^2 / lsum,
//       kb = 2 e0 x e1 / (|e0||e1| + e0.e1), e0 = x1 - x0, e1 = x2 - x1,
//       Kb = h^2 E_young bendMult t^4 pi / 64               (ROD_BENDING.h:24-29)
// Hessians are projected to PSD by an eigen-decomposition of the full element
// Hessian (the reference's makePD, Math/UTILS.h:9-27).
#include <cmath>
#include <cstring>

#include "oracle_dual.h"
#include "oracle_math.h"

namespace orc_rod {

using namespace orc_dual;

template <typename T>
T spring_energy(const T* x, double L, double K)
{
    const T dx = x[0] - x[3], dy = x[1] - x[4], dz = x[2] - x[5];
    const T l = sq_root(dx * dx + dy * dy + dz * dz);
    const T s = l / C<T>(L) - C<T>(1.0);
    return C<T>(0.5 * K * L) * s * s;
}

template <typename T>
T bending_energy(const T* x, double lsum, double Kb)
{
    T a[3], b[3];
    for (int k = 0; k < 3; ++k) {
        a[k] = x[3 + k] - x[k];
        b[k] = x[6 + k] - x[3 + k];
    }
    const T c0 = a[1] * b[2] - a[2] * b[1], c1 = a[2] * b[0] - a[0] * b[2], c2 = a[0] * b[1] - a[1] * b[0];
    const T la = sq_root(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    const T lb = sq_root(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    const T s = la * lb + (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
    const T k2 = C<T>(4.0) * (c0 * c0 + c1 * c1 + c2 * c2) / (s * s);
    return C<T>(Kb / lsum) * k2;
}

template <int N, typename F>
double eval_all(const double* x, F f, double* g, double* H, bool project)
{
    D2<N> xs[N];
    for (int k = 0; k < N; ++k) xs[k] = seed<N>(x[k], k);
    const D2<N> e = f(xs);
    if (g)
        for (int k = 0; k < N; ++k) g[k] = e.v.d[k];
    if (H) {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) H[N * i + j] = 0.5 * (e.d[j].d[i] + e.d[i].d[j]);
        if (project) orc::make_pd(N, H);
    }
    return e.v.v;
}

}  // namespace orc_rod

extern "C" {

// E, gradient (6) and Hessian (36, PSD-projected when project) of one stretching segment
double orc_rod_spring(const double* x6, double L, double K, double* g, double* H, int project)
{
    return orc_rod::eval_all<6>(
        x6, [&](const orc_rod::D2<6>* xs) { return orc_rod::spring_energy(xs, L, K); }, g, H, project != 0);
}

// E, gradient (9) and Hessian (81) of one rod hinge
double orc_rod_bending(const double* x9, double lsum, double Kb, double* g, double* H, int project)
{
    return orc_rod::eval_all<9>(
        x9, [&](const orc_rod::D2<9>* xs) { return orc_rod::bending_energy(xs, lsum, Kb); }, g, H, project != 0);
}

}  // extern "C"
