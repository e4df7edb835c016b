// Test infrastructure: CPU restatement (double precision) of the learned
// block-Jacobi correction used by the GPU PCG.  Only the tests and the bench's
// CPU leg call it; it checks the GPU's features, forward pass, loss and
// parameter gradients.
//
// Network (per vertex i of the Newton system H dx = r):
//   features x_i (10): log(D_aa / dbar) a=0..2; normalised off-diagonals of D_i;
//     log(1e-6 + s_i); contact share |Dc_i|_F / |D_i|_F; Dirichlet flag;
//     min(#contacts, 8) / 8.  D_i = diagonal 3x3 block of H (elastic + mass +
//     contact + friction), Dc_i its contact and friction part, dbar = mean of
//     trace(D_i)/3 over free vertices, s_i = sum_j a_ij.
//   edge weights a_ij = |B_ij|_F / sqrt(|D_i|_F |D_j|_F) over the elastic
//     off-diagonal blocks (zero for padding, self and blocks that are zero).
//   h0 = relu(W0 x + b0)
//   layer l: g_i = sum_j a_ij h_j / s_i ; c_i = mean over constraints touching
//     i of the constraint's mean h ; h <- relu(A h + B g + C c + b) + h
//   o = Wo h + bo (6) ; e_a = exp(0.5 clamp(o_a, -2, 2)), l_a = clamp(o_a, -1, 1)
//   Cm = [[e0,0,0],[o3,e1,0],[o4,o5,e2]] ; P_i = Cm D_i^-1 Cm^T ; z_i = P_i r_i
// With Wo = 0, bo = 0 (the initial state) P_i = D_i^-1: plain block Jacobi.
// Loss of one (H, r, p) triple, p = H^-1 r, kind 0:  L = 1 - (z.r)^2 / ((z.Hz)(r.p)),
// the relative H-norm error left after one optimally scaled preconditioned step;
// kind 1:  L = |z - p|_H^2 / |p|_H^2, the same error for the unit step.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int F = 10, O = 6;

struct Net {
    int H, L;
    const double* W0;
    const double* b0;
    std::vector<const double*> A, B, C, b;
    const double* Wo;
    const double* bo;
    Net(int H_, int L_, const double* p) : H(H_), L(L_)
    {
        W0 = p;
        p += H * F;
        b0 = p;
        p += H;
        for (int l = 0; l < L; ++l) {
            A.push_back(p);
            p += H * H;
            B.push_back(p);
            p += H * H;
            C.push_back(p);
            p += H * H;
            b.push_back(p);
            p += H;
        }
        Wo = p;
        p += O * H;
        bo = p;
    }
};

struct Graph {
    int nv, K;
    const int* col;      // K*nv, block k of row i at k*nv+i
    const float* val;    // 9 per block
    const float* cdiag;  // 9 per vertex: contact + friction part of the diagonal block
    const uint8_t* proj;
    int ncon;
    const int* ckind;    // constraint kind (vertex count 2 for 0, 3 for 1, else 4)
    const int* cverts;   // 4 per constraint
    const float* chess;  // 78 per constraint (packed upper triangle, row by row)
};

int con_nv(int k) { return k == 0 ? 2 : (k == 1 ? 3 : 4); }

void inv3(const double* A, double* inv)
{
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    if (!(std::fabs(det) > 0)) {
        for (int k = 0; k < 9; ++k) inv[k] = (k % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    const double id = 1.0 / det;
    inv[0] = c00 * id;
    inv[3] = c01 * id;
    inv[6] = c02 * id;
    inv[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    inv[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    inv[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    inv[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    inv[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    inv[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

double fro_f(const float* A)
{
    double s = 0;
    for (int k = 0; k < 9; ++k) s += (double)A[k] * A[k];
    return std::sqrt(s);
}

double fro(const double* A)
{
    double s = 0;
    for (int k = 0; k < 9; ++k) s += A[k] * A[k];
    return std::sqrt(s);
}

struct Prep {
    std::vector<double> D, E, x, a, s;  // D 9nv, E = D^-1 9nv, x F*nv, a K*nv, s nv
    std::vector<int> ncnt;
};

void prepare(const Graph& G, Prep& P)
{
    const int nv = G.nv, K = G.K;
    P.D.assign(9 * (size_t)nv, 0);
    P.E.assign(9 * (size_t)nv, 0);
    P.x.assign((size_t)F * nv, 0);
    P.a.assign((size_t)K * nv, 0);
    P.s.assign(nv, 0);
    P.ncnt.assign(nv, 0);
    std::vector<double> Dn(nv);
    for (int i = 0; i < nv; ++i) {
        for (int k = 0; k < K; ++k)
            if (G.col[(size_t)k * nv + i] == i) {
                const float* B = G.val + 9 * ((size_t)k * nv + i);
                for (int q = 0; q < 9; ++q) P.D[9 * (size_t)i + q] += B[q];
            }
        for (int q = 0; q < 9; ++q) P.D[9 * (size_t)i + q] += G.cdiag[9 * (size_t)i + q];
        inv3(&P.D[9 * (size_t)i], &P.E[9 * (size_t)i]);
        Dn[i] = fro(&P.D[9 * (size_t)i]);
    }
    for (int c = 0; c < G.ncon; ++c)
        for (int q = 0; q < con_nv(G.ckind[c]); ++q) P.ncnt[G.cverts[4 * c + q]] += 1;
    double dsum = 0;
    int nfree = 0;
    for (int i = 0; i < nv; ++i)
        if (!G.proj[i]) {
            const double* D = &P.D[9 * (size_t)i];
            dsum += (D[0] + D[4] + D[8]) / 3;
            ++nfree;
        }
    const double dbar = nfree ? dsum / nfree : 1.0;
    for (int i = 0; i < nv; ++i) {
        double s = 0;
        for (int k = 0; k < K; ++k) {
            const int j = G.col[(size_t)k * nv + i];
            const float* B = G.val + 9 * ((size_t)k * nv + i);
            double bn = 0;
            for (int q = 0; q < 9; ++q) bn += (double)B[q] * B[q];
            bn = std::sqrt(bn);
            double w = 0;
            if (j != i && bn > 0 && Dn[i] > 0 && Dn[j] > 0) w = bn / std::sqrt(Dn[i] * Dn[j]);
            P.a[(size_t)k * nv + i] = w;
            s += w;
        }
        P.s[i] = s;
        const double* D = &P.D[9 * (size_t)i];
        double* x = &P.x[(size_t)F * i];
        for (int q = 0; q < 3; ++q) x[q] = std::log(std::fmax(D[4 * q], 1e-30) / dbar);
        const double d0 = std::sqrt(std::fmax(D[0], 1e-30)), d1 = std::sqrt(std::fmax(D[4], 1e-30)),
                     d2 = std::sqrt(std::fmax(D[8], 1e-30));
        x[3] = D[1] / (d0 * d1);
        x[4] = D[2] / (d0 * d2);
        x[5] = D[5] / (d1 * d2);
        x[6] = std::log(1e-6 + s);
        x[7] = Dn[i] > 0 ? fro_f(G.cdiag + 9 * (size_t)i) / Dn[i] : 0.0;
        x[8] = G.proj[i] ? 1.0 : 0.0;
        x[9] = std::fmin((double)P.ncnt[i], 8.0) / 8.0;
    }
}

struct Acts {
    std::vector<double> u0;
    std::vector<std::vector<double>> h, g, c, u;  // h[0..L], g/c/u[0..L-1]
    std::vector<double> o, z;
};

void dense(int nv, int Ho, int Hi, const double* W, const std::vector<double>& in, std::vector<double>& out, bool acc)
{
    if (!acc) out.assign((size_t)Ho * nv, 0);
    for (int i = 0; i < nv; ++i)
        for (int r = 0; r < Ho; ++r) {
            double t = 0;
            for (int q = 0; q < Hi; ++q) t += W[r * Hi + q] * in[(size_t)Hi * i + q];
            out[(size_t)Ho * i + r] += t;
        }
}

void gather_ell(const Graph& G, const Prep& P, int H, const std::vector<double>& h, std::vector<double>& g)
{
    const int nv = G.nv;
    g.assign((size_t)H * nv, 0);
    for (int i = 0; i < nv; ++i) {
        if (!(P.s[i] > 0)) continue;
        for (int k = 0; k < G.K; ++k) {
            const double w = P.a[(size_t)k * nv + i] / P.s[i];
            if (w == 0) continue;
            const int j = G.col[(size_t)k * nv + i];
            for (int q = 0; q < H; ++q) g[(size_t)H * i + q] += w * h[(size_t)H * j + q];
        }
    }
}

void gather_con(const Graph& G, const Prep& P, int H, const std::vector<double>& h, std::vector<double>& c)
{
    const int nv = G.nv;
    c.assign((size_t)H * nv, 0);
    std::vector<double> m(H);
    for (int k = 0; k < G.ncon; ++k) {
        const int n = con_nv(G.ckind[k]);
        for (int q = 0; q < H; ++q) m[q] = 0;
        for (int t = 0; t < n; ++t)
            for (int q = 0; q < H; ++q) m[q] += h[(size_t)H * G.cverts[4 * k + t] + q] / n;
        for (int t = 0; t < n; ++t)
            for (int q = 0; q < H; ++q) c[(size_t)H * G.cverts[4 * k + t] + q] += m[q];
    }
    for (int i = 0; i < nv; ++i) {
        const double inv = 1.0 / std::fmax(1.0, (double)P.ncnt[i]);
        for (int q = 0; q < H; ++q) c[(size_t)H * i + q] *= inv;
    }
}

void precond_block(const double* o, const double* E, double* Pm, double* Cm)
{
    double e[3];
    for (int a = 0; a < 3; ++a) e[a] = std::exp(0.5 * std::fmin(2.0, std::fmax(-2.0, o[a])));
    double l[3];
    for (int a = 0; a < 3; ++a) l[a] = std::fmin(1.0, std::fmax(-1.0, o[3 + a]));
    const double C[9] = {e[0], 0, 0, l[0], e[1], 0, l[1], l[2], e[2]};
    double CE[9];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) CE[3 * r + q] = C[3 * r] * E[q] + C[3 * r + 1] * E[3 + q] + C[3 * r + 2] * E[6 + q];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) Pm[3 * r + q] = CE[3 * r] * C[3 * q] + CE[3 * r + 1] * C[3 * q + 1] + CE[3 * r + 2] * C[3 * q + 2];
    if (Cm) std::memcpy(Cm, C, sizeof(C));
}

void forward(const Net& N, const Graph& G, const Prep& P, const double* r, Acts& A)
{
    const int nv = G.nv, H = N.H, L = N.L;
    A.u0.clear();
    dense(nv, H, F, N.W0, P.x, A.u0, false);
    A.h.assign(L + 1, {});
    A.g.assign(L, {});
    A.c.assign(L, {});
    A.u.assign(L, {});
    A.h[0].resize((size_t)H * nv);
    for (int i = 0; i < nv; ++i)
        for (int q = 0; q < H; ++q) {
            const double v = A.u0[(size_t)H * i + q] + N.b0[q];
            A.u0[(size_t)H * i + q] = v;
            A.h[0][(size_t)H * i + q] = v > 0 ? v : 0;
        }
    for (int l = 0; l < L; ++l) {
        gather_ell(G, P, H, A.h[l], A.g[l]);
        gather_con(G, P, H, A.h[l], A.c[l]);
        dense(nv, H, H, N.A[l], A.h[l], A.u[l], false);
        dense(nv, H, H, N.B[l], A.g[l], A.u[l], true);
        dense(nv, H, H, N.C[l], A.c[l], A.u[l], true);
        A.h[l + 1].resize((size_t)H * nv);
        for (int i = 0; i < nv; ++i)
            for (int q = 0; q < H; ++q) {
                const double v = A.u[l][(size_t)H * i + q] + N.b[l][q];
                A.u[l][(size_t)H * i + q] = v;
                A.h[l + 1][(size_t)H * i + q] = (v > 0 ? v : 0) + A.h[l][(size_t)H * i + q];
            }
    }
    A.o.clear();
    dense(nv, O, H, N.Wo, A.h[L], A.o, false);
    A.z.assign(3 * (size_t)nv, 0);
    for (int i = 0; i < nv; ++i) {
        for (int q = 0; q < O; ++q) A.o[(size_t)O * i + q] += N.bo[q];
        double Pm[9];
        precond_block(&A.o[(size_t)O * i], &P.E[9 * (size_t)i], Pm, nullptr);
        for (int a = 0; a < 3; ++a)
            A.z[3 * i + a] = Pm[3 * a] * r[3 * i] + Pm[3 * a + 1] * r[3 * i + 1] + Pm[3 * a + 2] * r[3 * i + 2];
    }
}

// y = H x (elastic ELL blocks + contact blocks)
void apply_H(const Graph& G, const double* x, double* y)
{
    const int nv = G.nv;
    for (int i = 0; i < 3 * nv; ++i) y[i] = 0;
    for (int i = 0; i < nv; ++i)
        for (int k = 0; k < G.K; ++k) {
            const int j = G.col[(size_t)k * nv + i];
            const float* B = G.val + 9 * ((size_t)k * nv + i);
            for (int a = 0; a < 3; ++a)
                for (int q = 0; q < 3; ++q) y[3 * i + a] += (double)B[3 * a + q] * x[3 * j + q];
        }
    for (int c = 0; c < G.ncon; ++c) {
        const int n = con_nv(G.ckind[c]), m = 3 * n;
        const float* Hc = G.chess + 78 * (size_t)c;
        int w = 0;
        for (int p = 0; p < m; ++p)
            for (int q = p; q < m; ++q, ++w) {
                const int vp = G.cverts[4 * c + p / 3], vq = G.cverts[4 * c + q / 3];
                y[3 * vp + p % 3] += (double)Hc[w] * x[3 * vq + q % 3];
                if (q != p) y[3 * vq + q % 3] += (double)Hc[w] * x[3 * vp + p % 3];
            }
    }
}

}  // namespace

namespace {

// dW (Ho x Hi) += sum_i du_i in_i^T ; db += sum_i du_i
void wgrad(int nv, int Ho, int Hi, const std::vector<double>& du, const std::vector<double>& in, double* dW, double* db)
{
    for (int i = 0; i < nv; ++i)
        for (int r = 0; r < Ho; ++r) {
            const double d = du[(size_t)Ho * i + r];
            if (d == 0) continue;
            for (int q = 0; q < Hi; ++q) dW[r * Hi + q] += d * in[(size_t)Hi * i + q];
            if (db) db[r] += d;
        }
}

// din += W^T du
void dgrad(int nv, int Ho, int Hi, const double* W, const std::vector<double>& du, std::vector<double>& din)
{
    for (int i = 0; i < nv; ++i)
        for (int r = 0; r < Ho; ++r) {
            const double d = du[(size_t)Ho * i + r];
            if (d == 0) continue;
            for (int q = 0; q < Hi; ++q) din[(size_t)Hi * i + q] += W[r * Hi + q] * d;
        }
}

// loss and its gradient with respect to the parameters; returns the loss
double loss_grad(const Net& N, const Graph& G, const Prep& P, const double* r, const double* p, Acts& A, double* grad,
                 int nparams, int kind)
{
    const int nv = G.nv, H = N.H, L = N.L;
    const size_t n3 = 3 * (size_t)nv;
    forward(N, G, P, r, A);
    for (int k = 0; k < nparams; ++k) grad[k] = 0;
    double c = 0;
    for (size_t i = 0; i < n3; ++i) c += r[i] * p[i];
    if (!(c > 0)) return 0;
    // per-vertex adjoint of the preconditioner blocks, as S = G + G^T
    std::vector<double> Sadj(9 * (size_t)nv, 0);
    double loss = 0;
    if (kind == 2) {
        // |p - x_k|_H^2 / |p|_H^2 after k steps of preconditioned steepest descent
        const int ks = 8;
        std::vector<double> Pm(9 * (size_t)nv);
        for (int i = 0; i < nv; ++i) precond_block(&A.o[(size_t)O * i], &P.E[9 * (size_t)i], &Pm[9 * (size_t)i], nullptr);
        auto pmul = [&](const std::vector<double>& x, std::vector<double>& y, bool acc) {
            if (!acc) y.assign(n3, 0);
            for (int i = 0; i < nv; ++i)
                for (int q = 0; q < 3; ++q)
                    y[3 * i + q] += Pm[9 * i + 3 * q] * x[3 * i] + Pm[9 * i + 3 * q + 1] * x[3 * i + 1] +
                                    Pm[9 * i + 3 * q + 2] * x[3 * i + 2];
        };
        auto dotv = [&](const std::vector<double>& x, const std::vector<double>& y) {
            double t = 0;
            for (size_t i = 0; i < n3; ++i) t += x[i] * y[i];
            return t;
        };
        std::vector<std::vector<double>> R(1, std::vector<double>(r, r + n3)), Z, W;
        std::vector<double> a, b, al;
        for (int j = 0; j < ks; ++j) {
            std::vector<double> z, w(n3);
            pmul(R[j], z, false);
            apply_H(G, z.data(), w.data());
            const double aj = dotv(z, R[j]), bj = dotv(z, w);
            if (!(bj > 0) || !(aj == aj)) break;
            Z.push_back(z);
            W.push_back(w);
            a.push_back(aj);
            b.push_back(bj);
            al.push_back(aj / bj);
            std::vector<double> rn(n3);
            for (size_t i = 0; i < n3; ++i) rn[i] = R[j][i] - al.back() * w[i];
            R.push_back(rn);
        }
        const int kk = (int)Z.size();
        if (kk == 0) return 0;
        std::vector<double> x(n3, 0);
        for (int j = 0; j < kk; ++j)
            for (size_t i = 0; i < n3; ++i) x[i] += al[j] * Z[j][i];
        const double xr = dotv(x, R[0]), xHx = xr - dotv(x, R[kk]);
        loss = (c - 2 * xr + xHx) / c;
        std::vector<double> xb(n3), rb(n3, 0), zb(n3), wb(n3), tmp(n3);
        for (size_t i = 0; i < n3; ++i) xb[i] = -2.0 / c * R[kk][i];
        for (int j = kk - 1; j >= 0; --j) {
            const double ab = -dotv(rb, W[j]) + dotv(xb, Z[j]);
            const double abar = ab / b[j], bbar = -ab * a[j] / (b[j] * b[j]);
            for (size_t i = 0; i < n3; ++i) {
                zb[i] = al[j] * xb[i] + abar * R[j][i] + bbar * W[j][i];
                wb[i] = -al[j] * rb[i] + bbar * Z[j][i];
                rb[i] += abar * Z[j][i];
            }
            apply_H(G, wb.data(), tmp.data());
            for (size_t i = 0; i < n3; ++i) zb[i] += tmp[i];
            for (int i = 0; i < nv; ++i)
                for (int x1 = 0; x1 < 3; ++x1)
                    for (int y1 = 0; y1 < 3; ++y1) {
                        const double g = zb[3 * i + x1] * R[j][3 * i + y1];
                        Sadj[9 * i + 3 * x1 + y1] += g;
                        Sadj[9 * i + 3 * y1 + x1] += g;
                    }
            pmul(zb, rb, true);
        }
    } else {
        std::vector<double> Hz(n3);
        apply_H(G, A.z.data(), Hz.data());
        double a = 0, b = 0;
        for (size_t i = 0; i < n3; ++i) {
            a += A.z[i] * r[i];
            b += A.z[i] * Hz[i];
        }
        if (!(b > 0)) return 0;
        // kind 0: 1 - a^2/(bc), dL/dz = (2a/(bc)) (-r + (a/b) Hz)
        // kind 1: |z - p|_H^2 / |p|_H^2 = (b - 2a + c)/c, dL/dz = (2/c) (-r + Hz)
        loss = kind == 1 ? (b - 2 * a + c) / c : 1 - a * a / (b * c);
        const double f = kind == 1 ? 2 / c : 2 * a / (b * c), t = kind == 1 ? 1.0 : a / b;
        for (int i = 0; i < nv; ++i) {
            double dz[3];
            for (int q = 0; q < 3; ++q) dz[q] = f * (-r[3 * i + q] + t * Hz[3 * i + q]);
            for (int x1 = 0; x1 < 3; ++x1)
                for (int y1 = 0; y1 < 3; ++y1)
                    Sadj[9 * i + 3 * x1 + y1] = dz[x1] * r[3 * i + y1] + dz[y1] * r[3 * i + x1];
        }
    }
    // parameter gradient views (same layout as Net)
    double* gW0 = grad;
    double* gb0 = gW0 + H * F;
    double* gp = gb0 + H;
    std::vector<double*> gA(L), gB(L), gC(L), gb(L);
    for (int l = 0; l < L; ++l) {
        gA[l] = gp;
        gp += H * H;
        gB[l] = gp;
        gp += H * H;
        gC[l] = gp;
        gp += H * H;
        gb[l] = gp;
        gp += H;
    }
    double* gWo = gp;
    double* gbo = gWo + O * H;
    std::vector<double> dout((size_t)O * nv, 0);
    for (int i = 0; i < nv; ++i) {
        const double* o = &A.o[(size_t)O * i];
        const double* E = &P.E[9 * (size_t)i];
        double Pm[9], C[9];
        precond_block(o, E, Pm, C);
        // dC = (G + G^T) C E with G the adjoint of the block
        const double* S = &Sadj[9 * (size_t)i];
        double CE[9];
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) CE[3 * x + y] = C[3 * x] * E[y] + C[3 * x + 1] * E[3 + y] + C[3 * x + 2] * E[6 + y];
        double dC[9];
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) dC[3 * x + y] = S[3 * x] * CE[y] + S[3 * x + 1] * CE[3 + y] + S[3 * x + 2] * CE[6 + y];
        double* d = &dout[(size_t)O * i];
        for (int q = 0; q < 3; ++q) {
            const bool in = o[q] > -2.0 && o[q] < 2.0;
            d[q] = in ? dC[4 * q] * 0.5 * C[4 * q] : 0.0;
        }
        d[3] = std::fabs(o[3]) < 1.0 ? dC[3] : 0.0;
        d[4] = std::fabs(o[4]) < 1.0 ? dC[6] : 0.0;
        d[5] = std::fabs(o[5]) < 1.0 ? dC[7] : 0.0;
    }
    wgrad(nv, O, H, dout, A.h[L], gWo, gbo);
    std::vector<double> dh((size_t)H * nv, 0);
    dgrad(nv, O, H, N.Wo, dout, dh);
    for (int l = L - 1; l >= 0; --l) {
        std::vector<double> du(dh);
        for (size_t k = 0; k < du.size(); ++k)
            if (!(A.u[l][k] > 0)) du[k] = 0;
        wgrad(nv, H, H, du, A.h[l], gA[l], gb[l]);
        wgrad(nv, H, H, du, A.g[l], gB[l], nullptr);
        wgrad(nv, H, H, du, A.c[l], gC[l], nullptr);
        std::vector<double> dprev(dh);  // residual path
        dgrad(nv, H, H, N.A[l], du, dprev);
        std::vector<double> dg((size_t)H * nv, 0), dc((size_t)H * nv, 0);
        dgrad(nv, H, H, N.B[l], du, dg);
        dgrad(nv, H, H, N.C[l], du, dc);
        // transpose of the ELL gather
        for (int i = 0; i < nv; ++i) {
            if (!(P.s[i] > 0)) continue;
            for (int k = 0; k < G.K; ++k) {
                const double w = P.a[(size_t)k * nv + i] / P.s[i];
                if (w == 0) continue;
                const int j = G.col[(size_t)k * nv + i];
                for (int q = 0; q < H; ++q) dprev[(size_t)H * j + q] += w * dg[(size_t)H * i + q];
            }
        }
        // transpose of the contact gather
        std::vector<double> tsum(H);
        for (int k = 0; k < G.ncon; ++k) {
            const int n = con_nv(G.ckind[k]);
            for (int q = 0; q < H; ++q) tsum[q] = 0;
            for (int s = 0; s < n; ++s) {
                const int v = G.cverts[4 * k + s];
                const double inv = 1.0 / std::fmax(1.0, (double)P.ncnt[v]);
                for (int q = 0; q < H; ++q) tsum[q] += dc[(size_t)H * v + q] * inv / n;
            }
            for (int s = 0; s < n; ++s)
                for (int q = 0; q < H; ++q) dprev[(size_t)H * G.cverts[4 * k + s] + q] += tsum[q];
        }
        dh.swap(dprev);
    }
    std::vector<double> du0(dh);
    for (size_t k = 0; k < du0.size(); ++k)
        if (!(A.u0[k] > 0)) du0[k] = 0;
    wgrad(nv, H, F, du0, P.x, gW0, gb0);
    return loss;
}

}  // namespace

extern "C" {

int orc_lp_num_params(int H, int L) { return H * F + H + L * (3 * H * H + H) + O * H + O; }

// Features, block-Jacobi inverse and edge weights of one system.
void orc_lp_features(int nv, int K, const int* col, const float* val, const float* cdiag, const uint8_t* proj,
                     int ncon, const int* ckind, const int* cverts, double* x_out, double* a_out, double* E_out)
{
    Graph G{nv, K, col, val, cdiag, proj, ncon, ckind, cverts, nullptr};
    Prep P;
    prepare(G, P);
    if (x_out) std::memcpy(x_out, P.x.data(), sizeof(double) * P.x.size());
    if (a_out) std::memcpy(a_out, P.a.data(), sizeof(double) * P.a.size());
    if (E_out) std::memcpy(E_out, P.E.data(), sizeof(double) * P.E.size());
}

// Loss, parameter gradient (nparams doubles) and preconditioned residual z (3nv)
// of one (H, r, p) triple.
double orc_lp_loss_grad(int H, int L, const double* params, int nv, int K, const int* col, const float* val,
                        const float* cdiag, const uint8_t* proj, int ncon, const int* ckind, const int* cverts,
                        const float* chess, const double* r, const double* p, double* grad, double* z_out, int kind)
{
    Graph G{nv, K, col, val, cdiag, proj, ncon, ckind, cverts, chess};
    Prep P;
    prepare(G, P);
    Net N(H, L, params);
    Acts A;
    std::vector<double> gtmp(orc_lp_num_params(H, L));
    const double loss = loss_grad(N, G, P, r, p, A, grad ? grad : gtmp.data(), orc_lp_num_params(H, L), kind);
    if (z_out) std::memcpy(z_out, A.z.data(), sizeof(double) * A.z.size());
    return loss;
}

// y = H x of a triple's operator (elastic ELL blocks + contact blocks)
void orc_lp_apply(int nv, int K, const int* col, const float* val, int ncon, const int* ckind, const int* cverts,
                  const float* chess, const double* x, double* y)
{
    Graph G{nv, K, col, val, nullptr, nullptr, ncon, ckind, cverts, chess};
    apply_H(G, x, y);
}

}  // extern "C"
