// Test infrastructure: CPU restatement of the isotropic strain-limiting barrier of
// the shell step (Library/FEM/Shell/INEXT.h: barrier f_sl_u/g_sl_u/h_sl_u :5-39 in
// its C2 form, energy :120-190, gradient :192-253, Hessian :337-466), with
// derivatives by nested forward-mode dual numbers over the six entries of the
// deformation F (independent of the GPU's singular-frame closed form).
//
// Per triangle (skipped when all three vertices are Dirichlet): B upper
// triangular with B^T B = the rest first fundamental form, F = [x1-x0, x2-x0] B^-1,
// sigma_1 >= sigma_2 its singular values (square roots of the eigenvalues of
// F^T F).  For each sigma: infeasible if sigma >= s0; energy
// h^2 vol kappa_s0 f(sigma; s0, sHat0) if sigma > sHat0, with
// f(s; l, h) = -(h - s)^2 ln((l - s)/(l - h)) / (l - h)^2; the same with
// (s1, sHat1, kappa_s1) below sHat1 when kappa_s1 > 0.  The Hessian in F is made
// PSD (the reference's makePD, Math/UTILS.h:9-27) before it is mapped to the
// vertices.
#include <cmath>

#include "oracle_dual.h"
#include "oracle_math.h"

namespace orc_sl {

using namespace orc_dual;

template <typename T>
T barrier(const T& s, double lim, double hat)
{
    const T a = C<T>(hat) - s;
    const double D = lim - hat;
    return C<T>(-1.0 / (D * D)) * a * a * ln((C<T>(lim) - s) / C<T>(D));
}

// f[0..2] column 0 of F, f[3..5] column 1
// sv0: the singular values that decide feasibility and which terms are active
// (those of the unperturbed F, also when f is split at equal singular values)
template <typename T>
T energy_F(const T* f, const double* sv0, const double* s, const double* sh, const double* ks, double kh,
           bool* valid)
{
    const T c00 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    const T c01 = f[0] * f[3] + f[1] * f[4] + f[2] * f[5];
    const T c11 = f[3] * f[3] + f[4] * f[4] + f[5] * f[5];
    const T m = (c00 + c11) * C<T>(0.5), d = (c00 - c11) * C<T>(0.5);
    const T r = sq_root(d * d + c01 * c01);
    const T sig[2] = {sq_root(m + r), sq_root(m - r)};
    T E = C<T>(0.0);
    for (int i = 0; i < 2; ++i) {
        const double sv = sv0[i];
        if (sv >= s[0]) *valid = false;
        else if (sv > sh[0]) E = E + C<T>(kh * ks[0]) * barrier(sig[i], s[0], sh[0]);
        if (ks[1] > 0) {
            if (sv <= s[1]) *valid = false;
            else if (sv < sh[1]) E = E + C<T>(kh * ks[1]) * barrier(sig[i], s[1], sh[1]);
        }
    }
    return E;
}

}  // namespace orc_sl

extern "C" {

// One triangle: x9 its vertices, P the inverse rest fundamental form (p00, p01,
// p11), kh = h^2 vol, s/s_hat/kappa_s the reference's pairs.  Returns the energy;
// g (9) and H (81) when non-null; *valid = 0 if a stretch is outside the limits.
double orc_sl_elem(const double* x9, const double* P, double kh, const double* s, const double* s_hat,
                   const double* kappa_s, int project, double* g, double* H, int* valid)
{
    using namespace orc_sl;
    const double det = P[0] * P[2] - P[1] * P[1];
    const double q00 = P[2] / det, q01 = -P[1] / det, q11 = P[0] / det;
    const double b00 = std::sqrt(q00), b01 = q01 / b00, b11 = std::sqrt(q11 - q01 * q01 / q00);
    const double i00 = 1 / b00, i01 = -b01 / (b00 * b11), i11 = 1 / b11;
    // dF[:,k]/dx_v = c[k][v] I
    const double c[2][3] = {{-i00, i00, 0.0}, {-(i01 + i11), i01, i11}};
    double f[6];
    for (int i = 0; i < 3; ++i) {
        f[i] = 0;
        f[3 + i] = 0;
        for (int v = 0; v < 3; ++v) {
            f[i] += c[0][v] * x9[3 * v + i];
            f[3 + i] += c[1][v] * x9[3 * v + i];
        }
    }
    // At (numerically) equal singular values, e.g. a triangle at rest, the
    // singular values are not differentiable one by one, although the energy is:
    // there the value and derivatives are the mean of two evaluations at
    // F +- eps e00 (eps = 1e-7 |F|), which split them (error O(eps^2))
    const double c00 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2], c01 = f[0] * f[3] + f[1] * f[4] + f[2] * f[5];
    const double c11 = f[3] * f[3] + f[4] * f[4] + f[5] * f[5];
    const double m = 0.5 * (c00 + c11), dd = 0.5 * (c00 - c11), r = std::sqrt(dd * dd + c01 * c01);
    const bool degenerate = !(r > 1e-14 * m);
    const double eps = 1e-7 * std::sqrt(c00 + c11);
    const double sv0[2] = {std::sqrt(m + r), std::sqrt(m - r)};
    const int nev = degenerate ? 2 : 1;
    double Ev = 0, gF[6] = {0, 0, 0, 0, 0, 0}, HFs[36];
    for (int k = 0; k < 36; ++k) HFs[k] = 0;
    bool ok = true;
    for (int e = 0; e < nev; ++e) {
        double fe[6];
        for (int k = 0; k < 6; ++k) fe[k] = f[k];
        if (degenerate) fe[0] += (e == 0 ? eps : -eps);
        D2<6> fd[6];
        for (int k = 0; k < 6; ++k) fd[k] = seed<6>(fe[k], k);
        const D2<6> E = energy_F(fd, sv0, s, s_hat, kappa_s, kh, &ok);
        Ev += E.v.v / nev;
        for (int k = 0; k < 6; ++k) gF[k] += E.v.d[k] / nev;
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b) HFs[6 * a + b] += 0.5 * (E.d[a].d[b] + E.d[b].d[a]) / nev;
    }
    if (valid) *valid = ok ? 1 : 0;
    if (g) {
        for (int v = 0; v < 3; ++v)
            for (int i = 0; i < 3; ++i) g[3 * v + i] = c[0][v] * gF[i] + c[1][v] * gF[3 + i];
    }
    if (H) {
        double HF[36];
        for (int k = 0; k < 36; ++k) HF[k] = HFs[k];
        if (project) orc::make_pd(6, HF);
        for (int v = 0; v < 3; ++v)
            for (int i = 0; i < 3; ++i)
                for (int w = 0; w < 3; ++w)
                    for (int j = 0; j < 3; ++j) {
                        double t = 0;
                        for (int k = 0; k < 2; ++k)
                            for (int l = 0; l < 2; ++l) t += c[k][v] * c[l][w] * HF[6 * (3 * k + i) + 3 * l + j];
                        H[9 * (3 * v + i) + 3 * w + j] = t;
                    }
    }
    return Ev;
}

// The barrier of one singular value s against the limit lim with activation
// threshold hat (upper: hat < s < lim; lower: lim < s < hat): out = value,
// first and second derivative in s, by the same dual numbers as the element.
void orc_sl_barrier(double s, double lim, double hat, double* out)
{
    using namespace orc_sl;
    const D2<1> sd = seed<1>(s, 0);
    const D2<1> f = barrier(sd, lim, hat);
    out[0] = f.v.v;
    out[1] = f.v.d[0];
    out[2] = f.d[0].d[0];
}

// largest stretch of one triangle (the reference's Compute_Inextensibility)
double orc_sl_strain(const double* x9, const double* P)
{
    const double det = P[0] * P[2] - P[1] * P[1];
    const double q00 = P[2] / det, q01 = -P[1] / det, q11 = P[0] / det;
    const double b00 = std::sqrt(q00), b01 = q01 / b00, b11 = std::sqrt(q11 - q01 * q01 / q00);
    const double i00 = 1 / b00, i01 = -b01 / (b00 * b11), i11 = 1 / b11;
    const double c[2][3] = {{-i00, i00, 0.0}, {-(i01 + i11), i01, i11}};
    double f[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 3; ++i)
        for (int v = 0; v < 3; ++v) {
            f[i] += c[0][v] * x9[3 * v + i];
            f[3 + i] += c[1][v] * x9[3 * v + i];
        }
    const double c00 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    const double c01 = f[0] * f[3] + f[1] * f[4] + f[2] * f[5];
    const double c11 = f[3] * f[3] + f[4] * f[4] + f[5] * f[5];
    const double m = 0.5 * (c00 + c11), d = 0.5 * (c00 - c11);
    return std::sqrt(m + std::sqrt(d * d + c01 * c01));
}

}  // extern "C"
