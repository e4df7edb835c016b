// Host check of the hinge-bending Hessian forms of codim-ipc_gb300/csrc/elements.cuh:
// dihedral_hess_t<T> (the FP32 form used for mixed-precision Hessians, here also
// instantiated in FP64) against dihedral_hess (FP64) and against central finite
// differences of dihedral_grad, on seeded hinges of cloth-like shape (edge lengths
// 1e-3..1e-1 m, dihedral angles up to ~170 degrees).
// Prints "name value bound" lines; exits 1 when a value exceeds its bound.
#include <cmath>
#include <cstdio>
#include <random>

#define CIPC_HD inline
#include "../../codim-ipc_gb300/csrc/elements.cuh"

using namespace cipc;

int main()
{
    std::mt19937_64 rng(7);
    auto U = [&](double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); };
    double worst_t64 = 0, worst_t32 = 0, worst_fd = 0;
    const int n = 20000;
    for (int c = 0; c < n; ++c) {
        const double L = std::pow(10.0, U(-3, -1));
        // shared edge x1-x2 along a random axis, x0 and x3 on either side
        d3 x[4];
        x[1] = mk(U(-1, 1), U(-1, 1), U(-1, 1));
        const d3 ax = mk(U(-1, 1), U(-1, 1), U(-1, 1));
        const double an = std::sqrt(n2(ax));
        x[2] = x[1] + scl(ax, L / an);
        const d3 mid = x[1] + scl(ax, 0.5 * L / an);
        const double th = U(-2.9, 2.9);
        d3 p = cross(ax, mk(0.3, 1.0, -0.2));
        p = scl(p, 1.0 / std::sqrt(n2(p)));
        const d3 q = scl(cross(ax, p), 1.0 / an);
        const double h0 = L * U(0.4, 1.2), h3 = L * U(0.4, 1.2);
        x[0] = mid + scl(p, h0) + scl(ax, U(-0.3, 0.3) * L / an);
        x[3] = mid + scl(p, h3 * std::cos(th)) + scl(q, h3 * std::sin(th)) + scl(ax, U(-0.3, 0.3) * L / an);
        double H[12][12];
        dihedral_hess(x, H);
        const d3 ev[5] = {x[2] - x[1], x[0] - x[1], x[3] - x[1], x[0] - x[2], x[3] - x[2]};
        double E64[5][3];
        float E32[5][3];
        for (int k = 0; k < 5; ++k) {
            E64[k][0] = ev[k].x; E64[k][1] = ev[k].y; E64[k][2] = ev[k].z;
            for (int d = 0; d < 3; ++d) E32[k][d] = (float)E64[k][d];
        }
        double H64[12][12];
        float H32[12][12];
        dihedral_hess_t<double>(E64, H64);
        dihedral_hess_t<float>(E32, H32);
        double nrm = 0, d64 = 0, d32 = 0;
        for (int i = 0; i < 12; ++i)
            for (int j = 0; j < 12; ++j) {
                nrm += H[i][j] * H[i][j];
                d64 += (H64[i][j] - H[i][j]) * (H64[i][j] - H[i][j]);
                d32 += ((double)H32[i][j] - H[i][j]) * ((double)H32[i][j] - H[i][j]);
            }
        worst_t64 = std::fmax(worst_t64, std::sqrt(d64 / nrm));
        worst_t32 = std::fmax(worst_t32, std::sqrt(d32 / nrm));
        if (c < 2000) {
            // central differences of the FP64 gradient, step 1e-6 of the edge length
            double dfd = 0;
            const double hstep = 1e-6 * L;
            for (int k = 0; k < 12; ++k) {
                d3 xp[4] = {x[0], x[1], x[2], x[3]}, xm[4] = {x[0], x[1], x[2], x[3]};
                double* pp = &xp[k / 3].x;
                double* pm = &xm[k / 3].x;
                pp[k % 3] += hstep;
                pm[k % 3] -= hstep;
                double gp[12], gm[12];
                dihedral_grad(xp, gp);
                dihedral_grad(xm, gm);
                for (int j = 0; j < 12; ++j) {
                    const double f = (gp[j] - gm[j]) / (2 * hstep);
                    dfd += (f - H[k][j]) * (f - H[k][j]);
                }
            }
            worst_fd = std::fmax(worst_fd, std::sqrt(dfd / nrm));
        }
    }
    const double b64 = 1e-11, b32 = 2e-3, bfd = 1e-5;
    std::printf("hess_t64_rel %.3e %.1e\n", worst_t64, b64);
    std::printf("hess_t32_rel %.3e %.1e\n", worst_t32, b32);
    std::printf("hess_fd_rel %.3e %.1e\n", worst_fd, bfd);
    return (worst_t64 <= b64 && worst_t32 <= b32 && worst_fd <= bfd) ? 0 : 1;
}
