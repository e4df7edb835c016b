// CPU ORACLE — test infrastructure only.
//
// Restatement of one implicit-Euler time step of codimensional shells with
// offset IPC contact and lagged friction, following
//   Library/FEM/Shell/IMPLICIT_EULER.h:151-902   (Newton loop, line search :9-149)
//   Library/FEM/Shell/INC_POTENTIAL.h:15-395     (incremental potential)
//   Library/FEM/Shell/MEMBRANE.h, BENDING.h, DISCRETE_SHELL.h:218-357, 555-577
//   Library/FEM/IPC.h (constraint set, barrier, CCD step size, min distance)
//   Library/FEM/FRICTION.h, FRICTION_UTILS.h
// The direct CHOLMOD solve is replaced by a skyline LDL^T after a reverse
// Cuthill-McKee ordering (exact up to rounding).  Element Hessians are obtained by
// forward-mode differentiation of the closed-form gradients (exact to rounding),
// then projected to PSD like the reference's makePD.
#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <set>
#include <vector>

#include "oracle_math.h"
#include "oracle_shell.h"

namespace orc {

// ---------------------------------------------------------------------------
// forward-mode dual numbers (value + one directional derivative)
// ---------------------------------------------------------------------------
struct Du {
    double v, d;
};
static inline Du dc(double v) { return Du{v, 0}; }
static inline Du operator+(Du a, Du b) { return Du{a.v + b.v, a.d + b.d}; }
static inline Du operator-(Du a, Du b) { return Du{a.v - b.v, a.d - b.d}; }
static inline Du operator-(Du a) { return Du{-a.v, -a.d}; }
static inline Du operator*(Du a, Du b) { return Du{a.v * b.v, a.d * b.v + a.v * b.d}; }
static inline Du operator/(Du a, Du b) { return Du{a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
static inline Du operator*(double s, Du a) { return Du{s * a.v, s * a.d}; }
static inline Du operator*(Du a, double s) { return Du{s * a.v, s * a.d}; }
static inline Du operator+(Du a, double b) { return Du{a.v + b, a.d}; }
static inline Du operator+(double b, Du a) { return Du{a.v + b, a.d}; }
static inline Du operator-(Du a, double b) { return Du{a.v - b, a.d}; }
static inline Du operator-(double b, Du a) { return Du{b - a.v, -a.d}; }
static inline Du operator/(Du a, double b) { return Du{a.v / b, a.d / b}; }
static inline Du operator/(double b, Du a) { return Du{b / a.v, -b * a.d / (a.v * a.v)}; }
static inline Du sqrt(Du a)
{
    double s = std::sqrt(a.v);
    return Du{s, a.d / (2 * s)};
}
static inline Du log(Du a) { return Du{std::log(a.v), a.d / a.v}; }
static inline Du atan2(Du y, Du x)
{
    double r2 = x.v * x.v + y.v * y.v;
    return Du{std::atan2(y.v, x.v), (x.v * y.d - y.v * x.d) / r2};
}
static inline double sqrt(double a) { return std::sqrt(a); }
static inline double log(double a) { return std::log(a); }
static inline double atan2(double y, double x) { return std::atan2(y, x); }
static inline double val(double a) { return a; }
static inline double val(Du a) { return a.v; }

template <typename S>
struct T3 {
    S x, y, z;
};
template <typename S>
static inline T3<S> sub(T3<S> a, T3<S> b) { return T3<S>{a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename S>
static inline T3<S> add(T3<S> a, T3<S> b) { return T3<S>{a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename S>
static inline S tdot(T3<S> a, T3<S> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename S>
static inline T3<S> tcross(T3<S> a, T3<S> b)
{
    return T3<S>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename S>
static inline T3<S> tscale(T3<S> a, S s) { return T3<S>{a.x * s, a.y * s, a.z * s}; }
template <typename S>
static inline T3<S> ld3s(const S* p) { return T3<S>{p[0], p[1], p[2]}; }

// Hessian of a function whose gradient is given by G<Du>(xd, gd): column j is the
// directional derivative of the gradient along e_j.
template <int N, typename F>
static void hess_from_grad(const double* x, F gradfun, double* H)
{
    Du xd[N], gd[N];
    for (int j = 0; j < N; ++j) {
        for (int k = 0; k < N; ++k) xd[k] = Du{x[k], k == j ? 1.0 : 0.0};
        gradfun(xd, gd);
        for (int i = 0; i < N; ++i) H[i * N + j] = gd[i].d;
    }
    for (int i = 0; i < N; ++i)  // symmetrize rounding
        for (int j = i + 1; j < N; ++j) {
            double s = 0.5 * (H[i * N + j] + H[j * N + i]);
            H[i * N + j] = H[j * N + i] = s;
        }
}

// ---------------------------------------------------------------------------
// Membrane — MEMBRANE.h:7-290.  psi(A) with A = [e01.e01, e01.e02; ., e02.e02],
// P = inverse rest first fundamental form; scaled by h^2 vol.
//   NH:   mu/2 (tr(PA) - 2 - 2 lnJ) + lambda/2 lnJ^2,  lnJ = ln(det A det P)/2
//   StVK: 1/4 (lambda/2 tr(M)^2 + mu tr(M^2)),  M = PA - I
// dpsi/dA (4-entry convention, MEMBRANE.h:80-86) chained through dA/dx.
// ---------------------------------------------------------------------------
template <typename S>
static void membrane_grad(const S* x, const double* P, double coef, double lam, double mu, int nh, S* g)
{
    T3<S> x1 = ld3s(x), x2 = ld3s(x + 3), x3 = ld3s(x + 6);
    T3<S> e1 = sub(x2, x1), e2 = sub(x3, x1);
    S a00 = tdot(e1, e1), a01 = tdot(e1, e2), a11 = tdot(e2, e2);
    // temp = dpsi/dA, symmetric 2x2: t00, t01 (= t10), t11
    S t00, t01, t11;
    const double p00 = P[0], p01 = P[1], p11 = P[2];
    if (nh) {
        S det = a00 * a11 - a01 * a01;
        S ia00 = a11 / det, ia01 = (-1.0) * a01 / det, ia11 = a00 / det;
        double detP = p00 * p11 - p01 * p01;
        S lnJ = 0.5 * log(det * dc(detP));
        S c = (-mu + lam * lnJ) * dc(0.5);
        t00 = coef * (dc(mu / 2 * p00) + c * ia00);
        t01 = coef * (dc(mu / 2 * p01) + c * ia01);
        t11 = coef * (dc(mu / 2 * p11) + c * ia11);
    } else {
        // M = P A - I
        S m00 = p00 * a00 + p01 * a01 - dc(1.0), m01 = p00 * a01 + p01 * a11;
        S m10 = p01 * a00 + p11 * a01, m11 = p01 * a01 + p11 * a11 - dc(1.0);
        S tr = m00 + m11;
        // temp = coef/4 (lambda tr(M) P + 2 mu M P)
        S mp00 = m00 * dc(p00) + m01 * dc(p01), mp01 = m00 * dc(p01) + m01 * dc(p11);
        S mp10 = m10 * dc(p00) + m11 * dc(p01), mp11 = m10 * dc(p01) + m11 * dc(p11);
        double c4 = coef / 4;
        t00 = c4 * (lam * tr * dc(p00) + 2 * mu * mp00);
        t01 = c4 * (lam * tr * dc(p01) + mu * (mp01 + mp10));
        t11 = c4 * (lam * tr * dc(p11) + 2 * mu * mp11);
    }
    // dpsi/de1 = 2 t00 e1 + 2 t01 e2, dpsi/de2 = 2 t01 e1 + 2 t11 e2
    T3<S> g2 = add(tscale(e1, 2.0 * t00), tscale(e2, 2.0 * t01));
    T3<S> g3 = add(tscale(e1, 2.0 * t01), tscale(e2, 2.0 * t11));
    g[3] = g2.x; g[4] = g2.y; g[5] = g2.z;
    g[6] = g3.x; g[7] = g3.y; g[8] = g3.z;
    g[0] = (-1.0) * (g2.x + g3.x);
    g[1] = (-1.0) * (g2.y + g3.y);
    g[2] = (-1.0) * (g2.z + g3.z);
}

static double membrane_energy(const double* x, const double* P, double coef, double lam, double mu, int nh)
{
    V3 x1 = ld3(x), x2 = ld3(x + 3), x3 = ld3(x + 6);
    V3 e1 = x2 - x1, e2 = x3 - x1;
    double a00 = dot(e1, e1), a01 = dot(e1, e2), a11 = dot(e2, e2);
    double p00 = P[0], p01 = P[1], p11 = P[2];
    double tr = p00 * a00 + 2 * p01 * a01 + p11 * a11;  // tr(PA)
    if (nh) {
        double lnJ = std::log((a00 * a11 - a01 * a01) * (p00 * p11 - p01 * p01)) / 2;
        return coef * (mu / 2 * (tr - 2 - 2 * lnJ) + lam / 2 * lnJ * lnJ);
    }
    double m00 = p00 * a00 + p01 * a01 - 1, m01 = p00 * a01 + p01 * a11;
    double m10 = p01 * a00 + p11 * a01, m11 = p01 * a01 + p11 * a11 - 1;
    double trM = m00 + m11;
    double trM2 = m00 * m00 + m01 * m10 + m10 * m01 + m11 * m11;
    return coef / 4 * (0.5 * lam * trM * trM + mu * trM2);
}

// ---------------------------------------------------------------------------
// Discrete-shell hinge bending — BENDING.h:52-77 (energy), 175-210 (gradient);
// dihedral angle and its gradient as in Math/DIHEDRAL_ANGLE.h:9-24, 175-200.
// Stencil (x0, x1, x2, x3): x1-x2 is the hinge edge, x0 / x3 the opposite vertices.
// ---------------------------------------------------------------------------
template <typename S>
static S dihedral(T3<S> v0, T3<S> v1, T3<S> v2, T3<S> v3)
{
    T3<S> n1 = tcross(sub(v1, v0), sub(v2, v0));
    T3<S> n2 = tcross(sub(v2, v3), sub(v1, v3));
    // theta = angle between n1 and n2, signed by (n2 x n1).(v1 - v2).  n2 x n1 is
    // parallel to the hinge edge, so its signed length along the unit edge is
    // smooth through flat hinges (|n2 x n1| is not differentiable there).
    T3<S> c = tcross(n2, n1);
    T3<S> e = sub(v1, v2);
    S sn = tdot(c, e) / sqrt(tdot(e, e));
    S cs = tdot(n1, n2);
    return atan2(sn, cs);
}

static double dihedral_value(V3 v0, V3 v1, V3 v2, V3 v3)
{
    V3 n1 = cross(v1 - v0, v2 - v0);
    V3 n2 = cross(v2 - v3, v1 - v3);
    double c = dot(n1, n2) / std::sqrt(norm2(n1) * norm2(n2));
    double th = std::acos(std::max(-1.0, std::min(1.0, c)));
    if (dot(cross(n2, n1), v1 - v2) < 0) th = -th;
    return th;
}

// gradient of theta: with (w2, w0, w1, w3) = (x0, x1, x2, x3), e0 = w1 - w0 ...
template <typename S>
static void dihedral_grad(const S* x, S* g)
{
    T3<S> w2 = ld3s(x), w0 = ld3s(x + 3), w1 = ld3s(x + 6), w3 = ld3s(x + 9);
    T3<S> e0 = sub(w1, w0), e1 = sub(w2, w0), e2 = sub(w3, w0), e3 = sub(w2, w1), e4 = sub(w3, w1);
    T3<S> n1 = tcross(e0, e1), n2 = tcross(e2, e0);
    S n1s = tdot(n1, n1), n2s = tdot(n2, n2), e0n = sqrt(tdot(e0, e0));
    T3<S> ga = tscale(n1, (-1.0) * e0n / n1s);
    T3<S> gb = add(tscale(n1, (-1.0) * tdot(e0, e3) / (e0n * n1s)), tscale(n2, (-1.0) * tdot(e0, e4) / (e0n * n2s)));
    T3<S> gc = add(tscale(n1, tdot(e0, e1) / (e0n * n1s)), tscale(n2, tdot(e0, e2) / (e0n * n2s)));
    T3<S> gd = tscale(n2, (-1.0) * e0n / n2s);
    S* o[4] = {g, g + 3, g + 6, g + 9};
    T3<S> gg[4] = {ga, gb, gc, gd};
    for (int k = 0; k < 4; ++k) {
        o[k][0] = gg[k].x;
        o[k][1] = gg[k].y;
        o[k][2] = gg[k].z;
    }
}

// bending energy gradient: 2 c (theta - thetabar) grad theta, c = h^2 k ebar/hbar
template <typename S>
static void bending_grad(const S* x, double thetabar, double c, S* g)
{
    S th = dihedral(ld3s(x), ld3s(x + 3), ld3s(x + 6), ld3s(x + 9));
    S gt[12];
    dihedral_grad(x, gt);
    S f = 2.0 * c * (th - dc(thetabar));
    for (int i = 0; i < 12; ++i) g[i] = f * gt[i];
}
static void bending_grad_d(const double* x, double thetabar, double c, double* g)
{
    // value path uses the reference's acos form of theta
    double th = dihedral_value(ld3(x), ld3(x + 3), ld3(x + 6), ld3(x + 9));
    double gt[12];
    dihedral_grad<double>(x, gt);
    for (int i = 0; i < 12; ++i) g[i] = 2.0 * c * (th - thetabar) * gt[i];
}


// ---------------------------------------------------------------------------
// Scene setup — DISCRETE_SHELL.h:218-357 (Initialize_Discrete_Shell),
// :131-216 (hinge stencils and rest data), MESHIO.h:728-767 (surface primitives),
// DISCRETE_SHELL.h:555-577 (offset-IPC stiffness).
// ---------------------------------------------------------------------------
// surface triangles of a tetrahedral mesh (Find_Surface_TriMesh, MESHIO.h:486-544):
// the outward faces (0,2,1), (0,3,2), (0,1,3), (1,2,3) of every tetrahedron as
// keys; a key without a reversed twin (in any rotation) is on the surface; key order
static std::vector<int> tet_surface(int ntet, const int* tet)
{
    std::set<std::array<int, 3>> keys;
    for (int t = 0; t < ntet; ++t) {
        const int* v = tet + 4 * t;
        keys.insert({v[0], v[2], v[1]});
        keys.insert({v[0], v[3], v[2]});
        keys.insert({v[0], v[1], v[3]});
        keys.insert({v[1], v[2], v[3]});
    }
    std::vector<int> out;
    for (const auto& k : keys)
        if (!keys.count({k[2], k[1], k[0]}) && !keys.count({k[1], k[0], k[2]}) && !keys.count({k[0], k[2], k[1]}))
            out.insert(out.end(), k.begin(), k.end());
    return out;
}

static void shell_init(Shell& S, int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                       double thickness, const double* gravity, double bendMult, int nh_model, int ntet = 0,
                       const int* tets = nullptr)
{
    S.nv = nv;
    S.X0.assign(X, X + 3 * nv);
    S.nh_model = nh_model;
    S.tri.clear();
    for (int t = 0; t < nt; ++t) {  // drop degenerate triangles
        V3 x1 = ld3(X + 3 * tri[3 * t]), x2 = ld3(X + 3 * tri[3 * t + 1]), x3 = ld3(X + 3 * tri[3 * t + 2]);
        V3 e01 = x2 - x1, e02 = x3 - x1;
        double a00 = dot(e01, e01), a01 = dot(e01, e02), a11 = dot(e02, e02);
        if (a00 * a11 - a01 * a01 != 0)
            for (int k = 0; k < 3; ++k) S.tri.push_back(tri[3 * t + k]);
    }
    nt = (int)S.tri.size() / 3;
    // directed edge -> triangle
    std::map<std::pair<int, int>, int> e2t;
    for (int t = 0; t < nt; ++t) {
        const int* v = &S.tri[3 * t];
        e2t[{v[0], v[1]}] = t;
        e2t[{v[1], v[2]}] = t;
        e2t[{v[2], v[0]}] = t;
    }
    // surface primitives over the tetrahedral surface then the shell
    // (IMPLICIT_EULER.h:235-241): an edge keeps the orientation of its first occurrence
    std::vector<int> ctri = tet_surface(ntet, tets);
    ctri.insert(ctri.end(), S.tri.begin(), S.tri.end());
    std::set<std::pair<int, int>> es;
    std::vector<char> isb(nv, 0);
    S.btri.clear();
    for (int t = 0; t < (int)ctri.size() / 3; ++t) {
        const int* v = &ctri[3 * t];
        for (int k = 0; k < 3; ++k) S.btri.push_back(v[k]);
        for (int k = 0; k < 3; ++k) {
            int a = v[k], b = v[(k + 1) % 3];
            if (!es.count({b, a})) es.insert({a, b});
        }
        isb[v[0]] = isb[v[1]] = isb[v[2]] = 1;
    }
    S.bedge.clear();
    for (auto& e : es) {
        S.bedge.push_back(e.first);
        S.bedge.push_back(e.second);
    }
    S.bnode.clear();
    for (int i = 0; i < nv; ++i)
        if (isb[i]) S.bnode.push_back(i);
    // no rod nodes or particles until codim_init adds them after the shell nodes
    // (the codimensional contact loops start at these indices)
    S.codim0 = S.codim1 = (int)S.bnode.size();
    // rest first fundamental form, stored inverted (P)
    S.P.resize(3 * nt);
    S.vol.resize(nt);
    for (int t = 0; t < nt; ++t) {
        V3 x1 = ld3(X + 3 * S.tri[3 * t]), x2 = ld3(X + 3 * S.tri[3 * t + 1]), x3 = ld3(X + 3 * S.tri[3 * t + 2]);
        V3 e01 = x2 - x1, e02 = x3 - x1;
        double a00 = dot(e01, e01), a01 = dot(e01, e02), a11 = dot(e02, e02);
        double det = a00 * a11 - a01 * a01;
        S.P[3 * t] = a11 / det;
        S.P[3 * t + 1] = -a01 / det;
        S.P[3 * t + 2] = a00 / det;
        S.vol[t] = std::sqrt(norm2(cross(e01, e02))) / 2 * thickness;
    }
    // hinges (non-Kirchhoff-Love branch, DISCRETE_SHELL.h:169-213)
    S.hinge.clear();
    S.hinfo.clear();
    for (auto& e : es) {
        auto f = e2t.find({e.first, e.second});
        if (f == e2t.end()) continue;
        const int* tv = &S.tri[3 * f->second];
        int v0 = -1;
        for (int j = 0; j < 3; ++j)
            if (tv[j] == e.second) v0 = tv[(j + 1) % 3];
        int v1 = e.first, v2 = e.second;
        auto g = e2t.find({v2, v1});
        if (g == e2t.end()) continue;
        const int* ov = &S.tri[3 * g->second];
        int v3 = 0;
        for (int j = 0; j < 3; ++j)
            if (ov[j] == v1) v3 = ov[(j + 1) % 3];
        S.hinge.insert(S.hinge.end(), {v0, v1, v2, v3});
        V3 X0v = ld3(X + 3 * v0), X1v = ld3(X + 3 * v1), X2v = ld3(X + 3 * v2), X3v = ld3(X + 3 * v3);
        double th = dihedral_value(X0v, X1v, X2v, X3v);
        double el = std::sqrt(norm2(X1v - X2v));
        V3 n1 = cross(X1v - X0v, X2v - X0v), n2 = cross(X2v - X3v, X1v - X3v);
        double hb = (std::sqrt(norm2(n1)) + std::sqrt(norm2(n2))) / (el * 6);
        S.hinfo.insert(S.hinfo.end(), {th, el, hb});
    }
    // lumped mass and body force
    S.mass.assign(nv, 0.0);
    S.b.assign(3 * nv, 0.0);
    for (int t = 0; t < nt; ++t) {
        V3 x1 = ld3(X + 3 * S.tri[3 * t]), x2 = ld3(X + 3 * S.tri[3 * t + 1]), x3 = ld3(X + 3 * S.tri[3 * t + 2]);
        double mp = std::sqrt(norm2(cross(x2 - x1, x3 - x1))) / 2 * thickness * rho / 3;
        for (int k = 0; k < 3; ++k) {
            int v = S.tri[3 * t + k];
            S.mass[v] += mp;
            for (int d = 0; d < 3; ++d) S.b[3 * v + d] += mp * gravity[d];
        }
    }
    S.lam = E * nu / (1 - nu * nu);
    S.mu = E / (2 * (1 + nu));
    S.kbend = bendMult * (E * std::pow(thickness, 3) / (24 * (1 - nu * nu)));
    S.dbc.assign(nv, 0);
}

// offset-IPC barrier stiffness (DISCRETE_SHELL.h:555-577 with elasticIPC = false):
// kappa = mult * 1e11 * mean(diag M) * 3 / (4e-16 * b''(1e-16; dHat^2, kappa = 1)),
// kappa_max = 100 kappa.  Returns dHat^2.
// Rods (DISCRETE_ROD.h:85-150) and particles (DISCRETE_PARTICLE.h:52-75) added to
// a shell scene, with the boundary layout of IMPLICIT_EULER.h:242-277.
static void codim_init(Shell& S, const double* X, int nseg, const int* seg, double rodE, double rodRho, double rodT,
                       double rodBendMult, int npart, const int* part, double partRho, double partT,
                       const double* gravity)
{
    S.codim0 = (int)S.bnode.size();
    std::map<int, std::vector<int>> nb;
    std::map<int, int> rod_node;
    for (int i = 0; i < nseg; ++i) {
        const int a = seg[2 * i], b = seg[2 * i + 1];
        nb[a].push_back(b);
        nb[b].push_back(a);
        const double L = std::sqrt(norm2(ld3(X + 3 * a) - ld3(X + 3 * b)));
        S.rseg.insert(S.rseg.end(), {a, b});
        S.rinfo.insert(S.rinfo.end(), {rodE, L, rodT});
        const double mp = L * M_PI * rodT * rodT / 4 * rodRho / 2;
        for (int v : {a, b}) {
            S.mass[v] += mp;
            for (int k = 0; k < 3; ++k) S.b[3 * v + k] += mp * gravity[k];
            rod_node[v] = 1;
        }
        S.bedge.insert(S.bedge.end(), {a, b});
    }
    for (auto& kv : nb)
        if (kv.second.size() >= 2)
            for (size_t i = 0; i < kv.second.size(); ++i)
                for (size_t j = i + 1; j < kv.second.size(); ++j) {
                    const int x0 = kv.second[i], x1 = kv.first, x2 = kv.second[j];
                    const double l0 = std::sqrt(norm2(ld3(X + 3 * x1) - ld3(X + 3 * x0)));
                    const double l1 = std::sqrt(norm2(ld3(X + 3 * x2) - ld3(X + 3 * x1)));
                    S.rhinge.insert(S.rhinge.end(), {x0, x1, x2});
                    S.rhinfo.insert(S.rhinfo.end(), {rodE * rodBendMult, l0 + l1, rodT});
                }
    for (auto& kv : rod_node) S.bnode.push_back(kv.first);
    S.nrod_e = nseg;
    S.codim1 = (int)S.bnode.size();
    if (npart) {
        const double m = 4.0 / 3.0 * M_PI * partT * partT * partT / 8 * partRho;
        for (int i = 0; i < npart; ++i) {
            const int v = part[i];
            S.mass[v] += m;
            for (int k = 0; k < 3; ++k) S.b[3 * v + k] += m * gravity[k];
            S.bnode.push_back(v);
        }
    }
}

static double shell_oipc_kappa(const Shell& S, double dhat, double stiffMult, double* kappa)
{
    double dHat2 = dhat * dhat;
    double Hb;
    barrier3(1.0e-16, dHat2, 1.0, nullptr, nullptr, &Hb);
    double msum = 0;
    for (int i = 0; i < S.nv; ++i) msum += 3 * S.mass[i];
    double mmean = msum / (3.0 * S.nv);
    kappa[0] = stiffMult * 1.0e11 * mmean * 3 / (4.0e-16 * Hb);
    kappa[1] = 100 * kappa[0];
    return dHat2;
}

// ---------------------------------------------------------------------------
// Sparse symmetric assembly (triplets) with the Dirichlet projection of
// CSR_MATRIX::Project_DBC (CSR_MATRIX.h:130-141): DBC rows / columns removed,
// unit diagonal.
// ---------------------------------------------------------------------------
struct Trip {
    int r, c;
    double v;
};
struct Asm {
    std::vector<Trip> t;
    const std::vector<char>* dbc = nullptr;
    bool skipdbc = true;
    void add_block(const int* vid, int nvb, const double* H)  // H is (3nvb)^2 row-major
    {
        int m = 3 * nvb;
        for (int a = 0; a < nvb; ++a)
            for (int b = 0; b < nvb; ++b) {
                if (skipdbc && ((*dbc)[vid[a]] || (*dbc)[vid[b]])) continue;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        double v = H[(3 * a + i) * m + 3 * b + j];
                        if (v != 0) t.push_back({3 * vid[a] + i, 3 * vid[b] + j, v});
                    }
            }
    }
};

// ---------------------------------------------------------------------------
// Element terms.  E += ..., g += ..., Hessians assembled (makePD per element).
// ---------------------------------------------------------------------------
static inline void gather(const double* x, const int* vid, int n, double* out)
{
    for (int a = 0; a < n; ++a)
        for (int d = 0; d < 3; ++d) out[3 * a + d] = x[3 * vid[a] + d];
}
static inline void scatter_add(double* g, const int* vid, int n, const double* in)
{
    for (int a = 0; a < n; ++a)
        for (int d = 0; d < 3; ++d) g[3 * vid[a] + d] += in[3 * a + d];
}
extern "C" double orc_rod_spring(const double* x6, double L, double K, double* g, double* H, int project);
extern "C" double orc_rod_bending(const double* x9, double lsum, double Kb, double* g, double* H, int project);

static inline bool all_dbc(const Shell& S, const int* v, int n)
{
    for (int k = 0; k < n; ++k)
        if (!S.dbc[v[k]]) return false;
    return true;
}

// rod stretching and bending (ROD_STRETCHING.h:9-107, ROD_BENDING.h:9-120)
static double rod_terms(const Shell& S, const double* x, double h, double* g, Asm* A)
{
    double E = 0;
    const int nrs = (int)S.rseg.size() / 2, nrh = (int)S.rhinge.size() / 3;
    for (int e = 0; e < nrs; ++e) {
        const int* v = &S.rseg[2 * e];
        if (all_dbc(S, v, 2)) continue;
        double xe[6], ge[6], H[36];
        gather(x, v, 2, xe);
        const double* ri = &S.rinfo[3 * e];
        const double K = h * h * M_PI * ri[2] * ri[2] / 4 * ri[0];
        E += orc_rod_spring(xe, ri[1], K, ge, A ? H : nullptr, 1);
        if (g) scatter_add(g, v, 2, ge);
        if (A) A->add_block(v, 2, H);
    }
    for (int e = 0; e < nrh; ++e) {
        const int* v = &S.rhinge[3 * e];
        if (all_dbc(S, v, 3)) continue;
        double xe[9], ge[9], H[81];
        gather(x, v, 3, xe);
        const double* ri = &S.rhinfo[3 * e];
        const double Kb = h * h * ri[0] * std::pow(ri[2], 4) * M_PI / 64;
        E += orc_rod_bending(xe, ri[1], Kb, ge, A ? H : nullptr, 1);
        if (g) scatter_add(g, v, 3, ge);
        if (A) A->add_block(v, 3, H);
    }
    return E;
}

extern "C" double orc_tet_nh(const double* x12, const double* Dinv, double w, double lam, double mu, int project,
                              double* g, double* H, int* valid);

// volumetric Neo-Hookean tetrahedra (INC_POTENTIAL.h:97-109, 228-229, 354-364);
// *valid cleared by an inverted tetrahedron
static double tet_terms(const Shell& S, const double* x, double h, double* g, Asm* A, bool* valid)
{
    double E = 0;
    const int nt = (int)S.tvol.size();
    for (int t = 0; t < nt; ++t) {
        const int* v = &S.tet[4 * t];
        if (all_dbc(S, v, 4)) continue;
        double xe[12], ge[12], H[144];
        gather(x, v, 4, xe);
        int ok = 1;
        E += orc_tet_nh(xe, &S.tDinv[9 * t], h * h * S.tvol[t], S.tlam, S.tmu, 1, g ? ge : nullptr, A ? H : nullptr,
                        &ok);
        if (!ok && valid) *valid = false;
        if (g) scatter_add(g, v, 4, ge);
        if (A && ok) A->add_block(v, 4, H);
    }
    return E;
}

// tetrahedra (DEFORMATION_GRADIENT.h:39-76): Dm^-1, vol = det Dm / 6, mass vol rho / 4
static void tet_init(Shell& S, const double* X, int ntet, const int* tets, double E, double nu, double rho,
                     const double* gravity)
{
    S.tlam = E * nu / ((1 + nu) * (1 - 2 * nu));
    S.tmu = E / (2 * (1 + nu));
    for (int t = 0; t < ntet; ++t) {
        const int* v = tets + 4 * t;
        double D[3][3];
        for (int k = 0; k < 3; ++k)
            for (int i = 0; i < 3; ++i) D[i][k] = X[3 * v[k + 1] + i] - X[3 * v[0] + i];
        const double c00 = D[1][1] * D[2][2] - D[1][2] * D[2][1], c01 = D[1][2] * D[2][0] - D[1][0] * D[2][2],
                     c02 = D[1][0] * D[2][1] - D[1][1] * D[2][0];
        const double det = D[0][0] * c00 + D[0][1] * c01 + D[0][2] * c02;
        const double inv[9] = {c00 / det, (D[0][2] * D[2][1] - D[0][1] * D[2][2]) / det,
                               (D[0][1] * D[1][2] - D[0][2] * D[1][1]) / det, c01 / det,
                               (D[0][0] * D[2][2] - D[0][2] * D[2][0]) / det,
                               (D[0][2] * D[1][0] - D[0][0] * D[1][2]) / det, c02 / det,
                               (D[0][1] * D[2][0] - D[0][0] * D[2][1]) / det,
                               (D[0][0] * D[1][1] - D[0][1] * D[1][0]) / det};
        S.tet.insert(S.tet.end(), v, v + 4);
        S.tDinv.insert(S.tDinv.end(), inv, inv + 9);
        S.tvol.push_back(det / 6);
        const double mp = det / 6 * rho / 4;
        for (int k = 0; k < 4; ++k) {
            S.mass[v[k]] += mp;
            for (int d = 0; d < 3; ++d) S.b[3 * v[k] + d] += mp * gravity[d];
        }
    }
}

extern "C" double orc_sl_elem(const double* x9, const double* P, double kh, const double* s, const double* s_hat,
                               const double* kappa_s, int project, double* g, double* H, int* valid);
extern "C" double orc_sl_strain(const double* x9, const double* P);

// strain-limiting barrier over the triangles (INEXT.h:120-466); *valid cleared by
// an infeasible triangle
static double strain_terms(const Shell& S, const double* x, double h, double* g, Asm* A, bool* valid)
{
    if (!(S.sl_kappa[0] > 0)) return 0;
    double E = 0;
    const int nt = (int)S.vol.size();
    for (int t = 0; t < nt; ++t) {
        const int* v = &S.tri[3 * t];
        if (all_dbc(S, v, 3)) continue;
        double xe[9], ge[9], H[81];
        gather(x, v, 3, xe);
        int ok = 1;
        E += orc_sl_elem(xe, &S.P[3 * t], h * h * S.vol[t], S.sl_s, S.sl_shat, S.sl_kappa, 1, g ? ge : nullptr,
                         A ? H : nullptr, &ok);
        if (!ok && valid) *valid = false;
        if (g) scatter_add(g, v, 3, ge);
        if (A) A->add_block(v, 3, H);
    }
    return E;
}

// largest stretch per triangle, 1 where all vertices are Dirichlet
// (Compute_Inextensibility, INEXT.h:72-118)
static void strains(const Shell& S, const double* x, std::vector<double>& out)
{
    const int nt = (int)S.vol.size();
    out.assign(nt, 1.0);
    for (int t = 0; t < nt; ++t) {
        const int* v = &S.tri[3 * t];
        if (all_dbc(S, v, 3)) continue;
        double xe[9];
        gather(x, v, 3, xe);
        out[t] = orc_sl_strain(xe, &S.P[3 * t]);
    }
}

static double elastic_energy(const Shell& S, const double* x, double h)
{
    double E = 0;
    int nt = (int)S.vol.size();
    for (int t = 0; t < nt; ++t) {
        const int* v = &S.tri[3 * t];
        if (all_dbc(S, v, 3)) continue;
        double xe[9];
        gather(x, v, 3, xe);
        E += membrane_energy(xe, &S.P[3 * t], h * h * S.vol[t], S.lam, S.mu, S.nh_model);
    }
    if (S.kbend) {
        int nh = (int)S.hinfo.size() / 3;
        for (int e = 0; e < nh; ++e) {
            const int* v = &S.hinge[4 * e];
            if (all_dbc(S, v, 4)) continue;
            double xe[12];
            gather(x, v, 4, xe);
            double th = dihedral_value(ld3(xe), ld3(xe + 3), ld3(xe + 6), ld3(xe + 9));
            const double* hi = &S.hinfo[3 * e];
            E += h * h * S.kbend * (th - hi[0]) * (th - hi[0]) * hi[1] / hi[2];
        }
    }
    E += rod_terms(S, x, h, nullptr, nullptr);
    return E;
}

static void elastic_grad_hess(const Shell& S, const double* x, double h, double* g, Asm* A)
{
    rod_terms(S, x, h, g, A);
    int nt = (int)S.vol.size();
    for (int t = 0; t < nt; ++t) {
        const int* v = &S.tri[3 * t];
        if (all_dbc(S, v, 3)) continue;
        double xe[9];
        gather(x, v, 3, xe);
        const double* P = &S.P[3 * t];
        double coef = h * h * S.vol[t];
        auto gf = [&](const Du* xd, Du* gd) { membrane_grad<Du>(xd, P, coef, S.lam, S.mu, S.nh_model, gd); };
        if (g) {
            Du xd[9], gd[9];
            for (int k = 0; k < 9; ++k) xd[k] = dc(xe[k]);
            gf(xd, gd);
            double gv[9];
            for (int k = 0; k < 9; ++k) gv[k] = gd[k].v;
            scatter_add(g, v, 3, gv);
        }
        if (A) {
            double H[81];
            hess_from_grad<9>(xe, gf, H);
            make_pd(9, H);
            A->add_block(v, 3, H);
        }
    }
    if (!S.kbend) return;
    int nh = (int)S.hinfo.size() / 3;
    for (int e = 0; e < nh; ++e) {
        const int* v = &S.hinge[4 * e];
        if (all_dbc(S, v, 4)) continue;
        double xe[12];
        gather(x, v, 4, xe);
        const double* hi = &S.hinfo[3 * e];
        double c = h * h * S.kbend * hi[1] / hi[2];
        if (g) {
            double gv[12];
            bending_grad_d(xe, hi[0], c, gv);
            scatter_add(g, v, 4, gv);
        }
        if (A) {
            double H[144];
            auto gf = [&](const Du* xd, Du* gd) { bending_grad<Du>(xd, hi[0], c, gd); };
            hess_from_grad<12>(xe, gf, H);
            make_pd(12, H);
            A->add_block(v, 4, H);
        }
    }
}

// ---------------------------------------------------------------------------
// Uniform grid for candidate enumeration (plays the role of Grid/SPATIAL_HASH.h:
// only candidates come from it; every predicate that decides membership is the
// reference's own AABB test and distance classification).
// ---------------------------------------------------------------------------
struct Grid {
    double inv = 1;
    V3 lo{0, 0, 0};
    std::map<int64_t, std::vector<int>> cells;
    static int64_t key(int64_t i, int64_t j, int64_t k) { return ((i + 1048576) << 42) | ((j + 1048576) << 21) | (k + 1048576); }
    void cell(V3 p, int64_t* c) const
    {
        c[0] = (int64_t)std::floor((p.x - lo.x) * inv);
        c[1] = (int64_t)std::floor((p.y - lo.y) * inv);
        c[2] = (int64_t)std::floor((p.z - lo.z) * inv);
    }
    void insert(int id, V3 bmin, V3 bmax)
    {
        int64_t a[3], b[3];
        cell(bmin, a);
        cell(bmax, b);
        for (int64_t i = a[0]; i <= b[0]; ++i)
            for (int64_t j = a[1]; j <= b[1]; ++j)
                for (int64_t k = a[2]; k <= b[2]; ++k) cells[key(i, j, k)].push_back(id);
    }
    void query(V3 bmin, V3 bmax, std::vector<int>& out) const
    {
        out.clear();
        int64_t a[3], b[3];
        cell(bmin, a);
        cell(bmax, b);
        for (int64_t i = a[0]; i <= b[0]; ++i)
            for (int64_t j = a[1]; j <= b[1]; ++j)
                for (int64_t k = a[2]; k <= b[2]; ++k) {
                    auto f = cells.find(key(i, j, k));
                    if (f != cells.end()) out.insert(out.end(), f->second.begin(), f->second.end());
                }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
};

static inline V3 vmin(V3 a, V3 b) { return V3{std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
static inline V3 vmax(V3 a, V3 b) { return V3{std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
static inline V3 vadd(V3 a, double s) { return V3{a.x + s, a.y + s, a.z + s}; }
static inline bool any_gt(V3 a, double d) { return a.x > d || a.y > d || a.z > d; }

static double mean_edge_length(const Shell& S, const double* x)
{
    int ne = (int)S.bedge.size() / 2;
    double s = 0;
    for (int e = 0; e < ne; ++e) s += std::sqrt(norm2(ld3(x + 3 * S.bedge[2 * e]) - ld3(x + 3 * S.bedge[2 * e + 1])));
    return ne ? s / ne : 1.0;
}

static void grid_setup(Grid& G, const Shell& S, const double* x, const double* x2)
{
    V3 lo{1e300, 1e300, 1e300};
    for (int i = 0; i < S.nv; ++i) {
        lo = vmin(lo, ld3(x + 3 * i));
        if (x2) lo = vmin(lo, ld3(x2 + 3 * i));
    }
    G.lo = lo;
    G.inv = 1.0 / mean_edge_length(S, x);
    G.cells.clear();
}

// ---------------------------------------------------------------------------
// Constraint set — IPC.h:19-740 (3D, shell = false, no codimensional nodes).
// Activation: classified d^2 < (sqrt(dHat2) + xi)^2 (IPC.h:53-54).  PP / PE
// constraints that are not mollified are merged with a multiplicity
// (IPC.h:571-661); everything else is kept as is.
// ---------------------------------------------------------------------------
static void constraint_set(const Shell& S, const double* x, double dHat2, double xi, std::vector<Con>& cs)
{
    cs.clear();
    const double dHat = std::sqrt(dHat2) + xi;
    const double dh2 = dHat * dHat;
    std::map<std::vector<int>, int> merge;  // (kind, v0, v1, v2) -> count
    std::vector<std::vector<int>> order;
    auto add_merge = [&](int k, int a, int b, int c) {
        std::vector<int> key{k, a, b, c};
        if (merge[key]++ == 0) order.push_back(key);
    };
    Grid G;
    grid_setup(G, S, x, nullptr);
    int ntr = (int)S.btri.size() / 3;
    for (int t = 0; t < ntr; ++t) {
        const int* v = &S.btri[3 * t];
        V3 a = ld3(x + 3 * v[0]), b = ld3(x + 3 * v[1]), c = ld3(x + 3 * v[2]);
        G.insert(t, vmin(vmin(a, b), c), vmax(vmax(a, b), c));
    }
    std::vector<int> cand;
    for (int vI : S.bnode) {
        V3 p = ld3(x + 3 * vI);
        G.query(vadd(p, -dHat), vadd(p, dHat), cand);
        for (int t : cand) {
            const int* tv = &S.btri[3 * t];
            if (vI == tv[0] || vI == tv[1] || vI == tv[2]) continue;
            if (S.dbc[vI] && S.dbc[tv[0]] && S.dbc[tv[1]] && S.dbc[tv[2]]) continue;
            V3 t0 = ld3(x + 3 * tv[0]), t1 = ld3(x + 3 * tv[1]), t2 = ld3(x + 3 * tv[2]);
            V3 mx = vmax(vmax(t0, t1), t2), mn = vmin(vmin(t0, t1), t2);
            if (any_gt(p - mx, dHat) || any_gt(mn - p, dHat)) continue;  // CCD.h:149-165
            switch (pt_type(p, t0, t1, t2)) {
                case 0: if (pp_d2(p, t0) < dh2) add_merge(kPP, vI, tv[0], -1); break;
                case 1: if (pp_d2(p, t1) < dh2) add_merge(kPP, vI, tv[1], -1); break;
                case 2: if (pp_d2(p, t2) < dh2) add_merge(kPP, vI, tv[2], -1); break;
                case 3: if (pe_d2(p, t0, t1) < dh2) add_merge(kPE, vI, tv[0], tv[1]); break;
                case 4: if (pe_d2(p, t1, t2) < dh2) add_merge(kPE, vI, tv[1], tv[2]); break;
                case 5: if (pe_d2(p, t2, t0) < dh2) add_merge(kPE, vI, tv[2], tv[0]); break;
                case 6: if (pt_d2(p, t0, t1, t2) < dh2) cs.push_back(Con{kPT, {vI, tv[0], tv[1], tv[2]}, 1}); break;
            }
        }
    }
    // edge-edge
    G.cells.clear();
    int ne = (int)S.bedge.size() / 2;
    for (int e = 0; e < ne; ++e) {
        V3 a = ld3(x + 3 * S.bedge[2 * e]), b = ld3(x + 3 * S.bedge[2 * e + 1]);
        G.insert(e, vmin(a, b), vmax(a, b));
    }
    for (int eI = 0; eI < ne; ++eI) {
        int a0 = S.bedge[2 * eI], a1 = S.bedge[2 * eI + 1];
        V3 ea0 = ld3(x + 3 * a0), ea1 = ld3(x + 3 * a1);
        V3 mna = vmin(ea0, ea1), mxa = vmax(ea0, ea1);
        G.query(vadd(mna, -dHat), vadd(mxa, dHat), cand);
        for (int eJ : cand) {
            if (eJ <= eI) continue;
            int b0 = S.bedge[2 * eJ], b1 = S.bedge[2 * eJ + 1];
            if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) continue;
            if (S.dbc[a0] && S.dbc[a1] && S.dbc[b0] && S.dbc[b1]) continue;
            V3 eb0 = ld3(x + 3 * b0), eb1 = ld3(x + 3 * b1);
            V3 mnb = vmin(eb0, eb1), mxb = vmax(eb0, eb1);
            if (any_gt(mna - mxb, dHat) || any_gt(mnb - mxa, dHat)) continue;  // CCD.h:167-185
            double eps_x = mollifier_threshold(ld3(&S.X0[3 * a0]), ld3(&S.X0[3 * a1]), ld3(&S.X0[3 * b0]),
                                               ld3(&S.X0[3 * b1]));
            bool moll = ee_cross_n2(ea0, ea1, eb0, eb1) < eps_x;
            switch (ee_type(ea0, ea1, eb0, eb1)) {
                case 0:
                    if (pp_d2(ea0, eb0) < dh2) {
                        if (moll) cs.push_back(Con{kPPM, {a0, a1, b0, b1}, 1});
                        else add_merge(kPP, a0, b0, -1);
                    }
                    break;
                case 1:
                    if (pp_d2(ea0, eb1) < dh2) {
                        if (moll) cs.push_back(Con{kPPM, {a0, a1, b1, b0}, 1});
                        else add_merge(kPP, a0, b1, -1);
                    }
                    break;
                case 2:
                    if (pe_d2(ea0, eb0, eb1) < dh2) {
                        if (moll) cs.push_back(Con{kPEM, {a0, a1, b0, b1}, 1});
                        else add_merge(kPE, a0, b0, b1);
                    }
                    break;
                case 3:
                    if (pp_d2(ea1, eb0) < dh2) {
                        if (moll) cs.push_back(Con{kPPM, {a1, a0, b0, b1}, 1});
                        else add_merge(kPP, a1, b0, -1);
                    }
                    break;
                case 4:
                    if (pp_d2(ea1, eb1) < dh2) {
                        if (moll) cs.push_back(Con{kPPM, {a1, a0, b1, b0}, 1});
                        else add_merge(kPP, a1, b1, -1);
                    }
                    break;
                case 5:
                    if (pe_d2(ea1, eb0, eb1) < dh2) {
                        if (moll) cs.push_back(Con{kPEM, {a1, a0, b0, b1}, 1});
                        else add_merge(kPE, a1, b0, b1);
                    }
                    break;
                case 6:
                    if (pe_d2(eb0, ea0, ea1) < dh2) {
                        if (moll) cs.push_back(Con{kPEM, {b0, b1, a0, a1}, 1});
                        else add_merge(kPE, b0, a0, a1);
                    }
                    break;
                case 7:
                    if (pe_d2(eb1, ea0, ea1) < dh2) {
                        if (moll) cs.push_back(Con{kPEM, {b1, b0, a0, a1}, 1});
                        else add_merge(kPE, b1, a0, a1);
                    }
                    break;
                case 8:
                    if (ee_d2(ea0, ea1, eb0, eb1) < dh2) {
                        if (moll) cs.push_back(Con{kEEM, {a0, a1, b0, b1}, 1});
                        else cs.push_back(Con{kEE, {a0, a1, b0, b1}, 1});
                    }
                    break;
            }
        }
    }
    // codimensional nodes (IPC.h:271-350): rod and particle nodes against rod
    // segments (point-edge classification), particles against later boundary nodes
    const int nbn = (int)S.bnode.size();
    if (S.nrod_e > 0 && nbn > S.codim0) {
        const int e_begin = ne - S.nrod_e;
        G.cells.clear();
        for (int e = e_begin; e < ne; ++e) {
            V3 a = ld3(x + 3 * S.bedge[2 * e]), b = ld3(x + 3 * S.bedge[2 * e + 1]);
            G.insert(e, vmin(a, b), vmax(a, b));
        }
        for (int sv = S.codim0; sv < nbn; ++sv) {
            const int vI = S.bnode[sv];
            V3 p = ld3(x + 3 * vI);
            G.query(vadd(p, -dHat), vadd(p, dHat), cand);
            for (int eI : cand) {
                const int e0 = S.bedge[2 * eI], e1 = S.bedge[2 * eI + 1];
                if (vI == e0 || vI == e1) continue;
                if (S.dbc[vI] && S.dbc[e0] && S.dbc[e1]) continue;
                V3 x0 = ld3(x + 3 * e0), x1 = ld3(x + 3 * e1);
                if (any_gt(p - vmax(x0, x1), dHat) || any_gt(vmin(x0, x1) - p, dHat)) continue;  // CCD.h:16-30
                switch (pe_type(p, x0, x1)) {
                    case 0: if (pp_d2(p, x0) < dh2) add_merge(kPP, vI, e0, -1); break;
                    case 1: if (pp_d2(p, x1) < dh2) add_merge(kPP, vI, e1, -1); break;
                    default: if (pe_d2(p, x0, x1) < dh2) add_merge(kPE, vI, e0, e1); break;
                }
            }
        }
    }
    for (int sv = S.codim1; sv < nbn; ++sv) {
        const int vI = S.bnode[sv];
        V3 p = ld3(x + 3 * vI);
        for (int svJ = sv + 1; svJ < nbn; ++svJ) {
            const int vJ = S.bnode[svJ];
            if (S.dbc[vI] && S.dbc[vJ]) continue;
            if (pp_d2(p, ld3(x + 3 * vJ)) < dh2) add_merge(kPP, vI, vJ, -1);
        }
    }
    for (auto& k : order) cs.push_back(Con{k[0], {k[1], k[2], k[3], -1}, merge[k]});
}

static int con_nv(int k) { return k == kPP ? 2 : (k == kPE ? 3 : 4); }

// classified squared distance of a constraint
static double con_d2(const Con& c, const double* x)
{
    V3 a = ld3(x + 3 * c.v[0]), b = ld3(x + 3 * c.v[1]);
    switch (c.k) {
        case kPP: return pp_d2(a, b);
        case kPE: return pe_d2(a, b, ld3(x + 3 * c.v[2]));
        case kPT: return pt_d2(a, b, ld3(x + 3 * c.v[2]), ld3(x + 3 * c.v[3]));
        case kEE:
        case kEEM: return ee_d2(a, b, ld3(x + 3 * c.v[2]), ld3(x + 3 * c.v[3]));
        case kPEM: return pe_d2(a, ld3(x + 3 * c.v[2]), ld3(x + 3 * c.v[3]));
        default: return pp_d2(a, ld3(x + 3 * c.v[2]));
    }
}

// ---------------------------------------------------------------------------
// Barrier over the constraint set — IPC.h:742-1731 (weights 1).
// Returns false if some constraint has d^2 - xi^2 <= 0 (the reference exits).
// ---------------------------------------------------------------------------
static bool barrier_terms(const Shell& S, const double* x, const std::vector<Con>& cs, double dHat2, double xi,
                          double kappa, double* E, double* g, Asm* A)
{
    const double xi2 = xi * xi, shat = dHat2 + 2 * std::sqrt(dHat2) * xi;
    for (const Con& c : cs) {
        int nvc = con_nv(c.k);
        double xe[12];
        gather(x, c.v, nvc, xe);
        double s = con_d2(c, x) - xi2;
        if (!(s > 0)) return false;
        double bv, bg, bh;
        barrier3(s, shat, kappa, &bv, &bg, &bh);
        int m = 3 * nvc;
        double gr[12] = {0}, H[144] = {0};
        if (c.k <= kEE) {
            double gd[12], Hd[144];
            d2_grad_hess(c.k == kPP ? 0 : (c.k == kPE ? 1 : (c.k == kPT ? 2 : 3)), xe, gd, Hd);
            if (E) *E += c.mult * bv;
            for (int i = 0; i < m; ++i) gr[i] = c.mult * bg * gd[i];
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < m; ++j) H[i * m + j] = c.mult * (bh * gd[i] * gd[j] + bg * Hd[i * m + j]);
        } else {
            // mollified: distance over a subset of the 4 vertices, mollifier over all 4
            int sub[3], ns;
            int kind;
            if (c.k == kEEM) { ns = 4; kind = 3; }
            else if (c.k == kPEM) { ns = 3; kind = 1; sub[0] = 0; sub[1] = 2; sub[2] = 3; }
            else { ns = 2; kind = 0; sub[0] = 0; sub[1] = 2; }
            double xs[12], gs[12], Hs[144];
            int ms = 3 * ns;
            if (c.k == kEEM) std::memcpy(xs, xe, sizeof(xs));
            else
                for (int a = 0; a < ns; ++a)
                    for (int d = 0; d < 3; ++d) xs[3 * a + d] = xe[3 * sub[a] + d];
            d2_grad_hess(kind, xs, gs, Hs);
            double gd[12] = {0}, Hd[144] = {0};
            for (int a = 0; a < ns; ++a) {
                int va = c.k == kEEM ? a : sub[a];
                for (int d = 0; d < 3; ++d) {
                    gd[3 * va + d] = gs[3 * a + d];
                    for (int bb = 0; bb < ns; ++bb) {
                        int vb = c.k == kEEM ? bb : sub[bb];
                        for (int d2 = 0; d2 < 3; ++d2) Hd[(3 * va + d) * 12 + 3 * vb + d2] = Hs[(3 * a + d) * ms + 3 * bb + d2];
                    }
                }
            }
            double eps_x = mollifier_threshold(ld3(&S.X0[3 * c.v[0]]), ld3(&S.X0[3 * c.v[1]]), ld3(&S.X0[3 * c.v[2]]),
                                               ld3(&S.X0[3 * c.v[3]]));
            double ge[12], He[144];
            double e = mollifier(xe, eps_x, ge, He);
            if (E) *E += e * bv;
            for (int i = 0; i < 12; ++i) gr[i] = e * bg * gd[i] + bv * ge[i];
            for (int i = 0; i < 12; ++i)
                for (int j = 0; j < 12; ++j)
                    H[i * 12 + j] = bg * gd[i] * ge[j] + ge[i] * bg * gd[j] + bv * He[i * 12 + j] +
                                    e * bh * gd[i] * gd[j] + e * bg * Hd[i * 12 + j];
        }
        if (g) scatter_add(g, c.v, nvc, gr);
        if (A) {
            make_pd(m, H);
            A->add_block(c.v, nvc, H);
        }
    }
    return true;
}

// minimum of d^2 - xi^2 over a constraint list (IPC.h:2246-2388); per-constraint values in out
static double min_dist2(const std::vector<Con>& cs, const double* x, double xi, std::vector<double>* out)
{
    double m = 1e300;
    if (out) out->resize(cs.size());
    for (size_t i = 0; i < cs.size(); ++i) {
        double d = con_d2(cs[i], x) - xi * xi;
        if (out) (*out)[i] = d;
        m = std::min(m, d);
    }
    return m;
}

// ---------------------------------------------------------------------------
// Lagged friction — FRICTION.h:16-660, FRICTION_UTILS.h:9-289.
// ---------------------------------------------------------------------------
struct Fric {
    Con c;
    double w[4];   // relative-displacement weights per vertex: relDX = sum_i w_i dx_i
    double T[6];   // tangent basis, columns T0 = T[0..2], T1 = T[3..5]
    double lam;    // normal force
};

static V3 normalized(V3 a) { return scale(a, 1.0 / std::sqrt(norm2(a))); }

static void friction_basis(const double* x, const std::vector<Con>& cs, double dHat2, double xi, double kappa,
                           std::vector<Fric>& out)
{
    out.clear();
    const double xi2 = xi * xi, shat = dHat2 + 2 * std::sqrt(dHat2) * xi;
    for (const Con& c : cs) {
        if (c.k >= kEEM) continue;  // mollified constraints carry no friction (FRICTION.h:32-37)
        Fric f;
        f.c = c;
        V3 v0 = ld3(x + 3 * c.v[0]), v1 = ld3(x + 3 * c.v[1]);
        V3 T0, T1;
        double d2 = 0;
        for (double& w : f.w) w = 0;
        if (c.k == kEE) {
            V3 v2 = ld3(x + 3 * c.v[2]), v3 = ld3(x + 3 * c.v[3]);
            // Edge_Edge_Closest_Point: solve for (gamma1, gamma2)
            V3 e20 = v0 - v2, e01 = v1 - v0, e23 = v3 - v2;
            double g1, g2;
            double a00 = norm2(e01), a01 = -dot(e23, e01), a11 = norm2(e23);
            double r0 = -dot(e20, e01), r1 = dot(e20, e23);
            // symmetric 2x2 LDL^T (pivoted) as in Eigen
            {
                bool sw = std::fabs(a11) > std::fabs(a00);
                double d0 = sw ? a11 : a00, m11 = sw ? a00 : a11, b0 = sw ? r1 : r0, b1 = sw ? r0 : r1;
                if (d0 == 0) { g1 = g2 = 0; }
                else {
                    double l = a01 / d0, d1 = m11 - l * (d0 * l);
                    double z0 = b0, z1 = b1 - l * z0;
                    z0 = std::fabs(d0) > 2.2250738585072014e-308 ? z0 / d0 : 0;
                    z1 = std::fabs(d1) > 2.2250738585072014e-308 ? z1 / d1 : 0;
                    z0 = z0 - l * z1;
                    g1 = sw ? z1 : z0;
                    g2 = sw ? z0 : z1;
                }
            }
            f.w[0] = 1 - g1; f.w[1] = g1; f.w[2] = g2 - 1; f.w[3] = -g2;
            T0 = normalized(e01);
            T1 = normalized(cross(cross(e01, e23), e01));
            d2 = ee_d2(v0, v1, v2, v3);
        } else if (c.k == kPP) {
            V3 v01 = v1 - v0;
            V3 xc = cross(V3{1, 0, 0}, v01), yc = cross(V3{0, 1, 0}, v01);
            if (norm2(xc) > norm2(yc)) {
                T0 = normalized(xc);
                T1 = normalized(cross(v01, xc));
            } else {
                T0 = normalized(yc);
                T1 = normalized(cross(v01, yc));
            }
            f.w[0] = 1; f.w[1] = -1;
            d2 = pp_d2(v0, v1);
        } else if (c.k == kPE) {
            V3 v2 = ld3(x + 3 * c.v[2]);
            V3 e12 = v2 - v1;
            double yita = dot(v0 - v1, e12) / norm2(e12);
            f.w[0] = 1; f.w[1] = yita - 1; f.w[2] = -yita;
            T0 = normalized(e12);
            T1 = normalized(cross(e12, v0 - v1));
            d2 = pe_d2(v0, v1, v2);
        } else {
            V3 v2 = ld3(x + 3 * c.v[2]), v3 = ld3(x + 3 * c.v[3]);
            V3 r0 = v2 - v1, r1 = v3 - v1, q = v0 - v1;
            double b1, b2;
            double a00 = norm2(r0), a01 = dot(r1, r0), a11 = norm2(r1);
            double bb0 = dot(r0, q), bb1 = dot(r1, q);
            {
                bool sw = std::fabs(a11) > std::fabs(a00);
                double d0 = sw ? a11 : a00, m11 = sw ? a00 : a11, c0 = sw ? bb1 : bb0, c1 = sw ? bb0 : bb1;
                if (d0 == 0) { b1 = b2 = 0; }
                else {
                    double l = a01 / d0, d1 = m11 - l * (d0 * l);
                    double z0 = c0, z1 = c1 - l * z0;
                    z0 = std::fabs(d0) > 2.2250738585072014e-308 ? z0 / d0 : 0;
                    z1 = std::fabs(d1) > 2.2250738585072014e-308 ? z1 / d1 : 0;
                    z0 = z0 - l * z1;
                    b1 = sw ? z1 : z0;
                    b2 = sw ? z0 : z1;
                }
            }
            f.w[0] = 1; f.w[1] = -1 + b1 + b2; f.w[2] = -b1; f.w[3] = -b2;
            T0 = normalized(r0);
            T1 = normalized(cross(cross(r0, r1), r0));
            d2 = pt_d2(v0, v1, v2, v3);
        }
        f.T[0] = T0.x; f.T[1] = T0.y; f.T[2] = T0.z;
        f.T[3] = T1.x; f.T[4] = T1.y; f.T[5] = T1.z;
        double bg;
        barrier3(d2 - xi2, shat, kappa, nullptr, &bg, nullptr);
        f.lam = -bg * 2 * std::sqrt(d2);
        out.push_back(f);
    }
}

// f0 (FRICTION_UTILS.h:9-17), f1 / |u| (:19-28), f2 term (:30-34)
static double f0_sf(double x2, double eh)
{
    if (x2 >= eh * eh) return std::sqrt(x2);
    return x2 * (-std::sqrt(x2) / 3.0 + eh) / (eh * eh) + eh / 3.0;
}
static double f1_div(double x2, double eh)
{
    if (x2 >= eh * eh) return 1 / std::sqrt(x2);
    return (-std::sqrt(x2) + 2.0 * eh) / (eh * eh);
}
// the three friction mollifier scalars for the golden-vector checks:
// out = (f0, f1 / |u|, f2 term) at squared relative slip x2, eh = epsv h
extern "C" void orc_friction_scalars(double x2, double eh, double* out)
{
    out[0] = f0_sf(x2, eh);
    out[1] = f1_div(x2, eh);
    out[2] = -1 / (eh * eh);
}

static void friction_terms(const std::vector<Fric>& F, const double* x, const double* xn, double epsvh2, double mu,
                           double* E, double* g, Asm* A)
{
    const double eh = std::sqrt(epsvh2);
    for (const Fric& f : F) {
        int nvc = con_nv(f.c.k);
        V3 r{0, 0, 0};
        for (int a = 0; a < nvc; ++a) r = r + scale(ld3(x + 3 * f.c.v[a]) - ld3(xn + 3 * f.c.v[a]), f.w[a]);
        V3 T0 = ld3(f.T), T1 = ld3(f.T + 3);
        double u0 = dot(T0, r), u1 = dot(T1, r);
        double u2 = u0 * u0 + u1 * u1;
        double ml = mu * f.lam * f.c.mult;
        if (E) *E += ml * f0_sf(u2, eh);
        double f1 = f1_div(u2, eh);
        if (g) {
            V3 tu = scale(T0, u0 * f1 * ml) + scale(T1, u1 * f1 * ml);
            for (int a = 0; a < nvc; ++a) {
                g[3 * f.c.v[a]] += f.w[a] * tu.x;
                g[3 * f.c.v[a] + 1] += f.w[a] * tu.y;
                g[3 * f.c.v[a] + 2] += f.w[a] * tu.z;
            }
        }
        if (A) {
            // inner 2x2 matrix (FRICTION.h:446-466)
            double M[4];
            double un = std::sqrt(u2);
            if (u2 >= epsvh2) {
                double s = ml * f1 / u2;
                double ub0 = -u1, ub1 = u0;
                M[0] = s * ub0 * ub0; M[1] = s * ub0 * ub1; M[2] = M[1]; M[3] = s * ub1 * ub1;
            } else if (un == 0) {
                M[0] = ml * f1; M[1] = M[2] = 0; M[3] = ml * f1;
            } else {
                double f2 = -1 / (eh * eh);
                double inner[4] = {f2 / un * u0 * u0 + f1, f2 / un * u0 * u1, f2 / un * u1 * u0, f2 / un * u1 * u1 + f1};
                make_pd(2, inner);
                for (int k = 0; k < 4; ++k) M[k] = inner[k] * ml;
            }
            // H = TT^T M TT with TT = [w_a T^T] blocks
            int m = 3 * nvc;
            double H[144];
            for (int a = 0; a < nvc; ++a)
                for (int b = 0; b < nvc; ++b)
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) {
                            double ti[2] = {f.T[i], f.T[3 + i]}, tj[2] = {f.T[j], f.T[3 + j]};
                            double s = 0;
                            for (int p = 0; p < 2; ++p)
                                for (int q = 0; q < 2; ++q) s += ti[p] * M[2 * p + q] * tj[q];
                            H[(3 * a + i) * m + 3 * b + j] = f.w[a] * f.w[b] * s;
                        }
            A->add_block(f.c.v, nvc, H);
        }
    }
}

// ---------------------------------------------------------------------------
// Intersection-free step size — IPC.h:1879-2244 (3D, surface primitives only) with
// the span-size cap of SPATIAL_HASH.h:477-482.  Candidates come from swept boxes
// of the capped step; each candidate is filtered by the reference's swept-AABB
// test with the full direction (CCD.h:187-277) before ACCD (eta = 0.1).
// ---------------------------------------------------------------------------
static double ccd_step_size(const Shell& S, const double* x, const double* p, double alpha, double xi)
{
    // span-size cap
    double pSize = 0;
    for (int vI : S.bnode)
        for (int d = 0; d < 3; ++d) pSize += std::fabs(p[3 * vI + d]);
    pSize /= S.bnode.size() * 3;
    double voxel = mean_edge_length(S, x);
    double span = alpha * pSize / voxel;
    if (span > 1) alpha /= span;
    std::vector<double> xe(3 * S.nv);
    for (int i = 0; i < 3 * S.nv; ++i) xe[i] = x[i] + alpha * p[i];
    Grid G;
    grid_setup(G, S, x, xe.data());
    auto sbox = [&](int v, V3& mn, V3& mx) {
        V3 a = ld3(x + 3 * v), b = ld3(&xe[3 * v]);
        mn = vmin(mn, vmin(a, b));
        mx = vmax(mx, vmax(a, b));
    };
    int ntr = (int)S.btri.size() / 3;
    for (int t = 0; t < ntr; ++t) {
        V3 mn{1e300, 1e300, 1e300}, mx{-1e300, -1e300, -1e300};
        for (int k = 0; k < 3; ++k) sbox(S.btri[3 * t + k], mn, mx);
        G.insert(t, vadd(mn, -xi), vadd(mx, xi));
    }
    double stepSize = alpha;
    std::vector<int> cand;
    const int64_t cap = 1 << 20;
    for (int vI : S.bnode) {
        V3 mn{1e300, 1e300, 1e300}, mx{-1e300, -1e300, -1e300};
        sbox(vI, mn, mx);
        G.query(mn, mx, cand);
        V3 pp = ld3(x + 3 * vI), dp = ld3(p + 3 * vI);
        for (int t : cand) {
            const int* tv = &S.btri[3 * t];
            if (vI == tv[0] || vI == tv[1] || vI == tv[2]) continue;
            if (S.dbc[vI] && S.dbc[tv[0]] && S.dbc[tv[1]] && S.dbc[tv[2]]) continue;
            V3 t0 = ld3(x + 3 * tv[0]), t1 = ld3(x + 3 * tv[1]), t2 = ld3(x + 3 * tv[2]);
            V3 d0 = ld3(p + 3 * tv[0]), d1 = ld3(p + 3 * tv[1]), d2 = ld3(p + 3 * tv[2]);
            V3 mxp = vmax(pp, pp + dp), mnp = vmin(pp, pp + dp);
            V3 mxt = vmax(vmax(vmax(t0, t1), t2), vmax(vmax(t0 + d0, t1 + d1), t2 + d2));
            V3 mnt = vmin(vmin(vmin(t0, t1), t2), vmin(vmin(t0 + d0, t1 + d1), t2 + d2));
            if (any_gt(mnp - mxt, xi) || any_gt(mnt - mxp, xi)) continue;
            double toc = stepSize;
            int64_t it;
            if (accd_pt(pp, t0, t1, t2, dp, d0, d1, d2, 0.1, xi, &toc, cap, &it) == 1 && toc < stepSize) stepSize = toc;
        }
    }
    G.cells.clear();
    int ne = (int)S.bedge.size() / 2;
    for (int e = 0; e < ne; ++e) {
        V3 mn{1e300, 1e300, 1e300}, mx{-1e300, -1e300, -1e300};
        sbox(S.bedge[2 * e], mn, mx);
        sbox(S.bedge[2 * e + 1], mn, mx);
        G.insert(e, vadd(mn, -xi), vadd(mx, xi));
    }
    for (int eI = 0; eI < ne; ++eI) {
        int a0 = S.bedge[2 * eI], a1 = S.bedge[2 * eI + 1];
        V3 mn{1e300, 1e300, 1e300}, mx{-1e300, -1e300, -1e300};
        sbox(a0, mn, mx);
        sbox(a1, mn, mx);
        G.query(mn, mx, cand);
        V3 ea0 = ld3(x + 3 * a0), ea1 = ld3(x + 3 * a1), da0 = ld3(p + 3 * a0), da1 = ld3(p + 3 * a1);
        for (int eJ : cand) {
            if (eJ <= eI) continue;
            int b0 = S.bedge[2 * eJ], b1 = S.bedge[2 * eJ + 1];
            if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) continue;
            if (S.dbc[a0] && S.dbc[a1] && S.dbc[b0] && S.dbc[b1]) continue;
            V3 eb0 = ld3(x + 3 * b0), eb1 = ld3(x + 3 * b1), db0 = ld3(p + 3 * b0), db1 = ld3(p + 3 * b1);
            V3 mxa = vmax(vmax(ea0, ea1), vmax(ea0 + da0, ea1 + da1)), mna = vmin(vmin(ea0, ea1), vmin(ea0 + da0, ea1 + da1));
            V3 mxb = vmax(vmax(eb0, eb1), vmax(eb0 + db0, eb1 + db1)), mnb = vmin(vmin(eb0, eb1), vmin(eb0 + db0, eb1 + db1));
            if (any_gt(mna - mxb, xi) || any_gt(mnb - mxa, xi)) continue;
            double toc = stepSize;
            int64_t it;
            if (accd_ee(ea0, ea1, eb0, eb1, da0, da1, db0, db1, 0.1, xi, &toc, cap, &it) == 1 && toc < stepSize)
                stepSize = toc;
        }
    }
    // codimensional pairs (IPC.h:2087-2165): particles against rod segments and
    // against later boundary nodes
    const int nbn = (int)S.bnode.size();
    for (int sv = S.codim1; sv < nbn; ++sv) {
        const int vI = S.bnode[sv];
        V3 pp = ld3(x + 3 * vI), dp = ld3(p + 3 * vI);
        V3 mxp = vmax(pp, pp + dp), mnp = vmin(pp, pp + dp);
        for (int eI = ne - S.nrod_e; eI < ne; ++eI) {
            const int e0 = S.bedge[2 * eI], e1 = S.bedge[2 * eI + 1];
            if (vI == e0 || vI == e1) continue;
            if (S.dbc[vI] && S.dbc[e0] && S.dbc[e1]) continue;
            V3 x0 = ld3(x + 3 * e0), x1 = ld3(x + 3 * e1), d0 = ld3(p + 3 * e0), d1 = ld3(p + 3 * e1);
            V3 mxe = vmax(vmax(x0, x1), vmax(x0 + d0, x1 + d1)), mne = vmin(vmin(x0, x1), vmin(x0 + d0, x1 + d1));
            if (any_gt(mnp - mxe, xi) || any_gt(mne - mxp, xi)) continue;
            double toc = stepSize;
            int64_t it;
            if (accd_pe(pp, x0, x1, dp, d0, d1, 0.1, xi, &toc, cap, &it) == 1 && toc < stepSize) stepSize = toc;
        }
        for (int svJ = sv + 1; svJ < nbn; ++svJ) {
            const int vJ = S.bnode[svJ];
            if (S.dbc[vI] && S.dbc[vJ]) continue;
            V3 q = ld3(x + 3 * vJ), dq = ld3(p + 3 * vJ);
            V3 mxq = vmax(q, q + dq), mnq = vmin(q, q + dq);
            if (any_gt(mnp - mxq, xi) || any_gt(mnq - mxp, xi)) continue;
            double toc = stepSize;
            int64_t it;
            if (accd_pp(pp, q, dp, dq, 0.1, xi, &toc, cap, &it) == 1 && toc < stepSize) stepSize = toc;
        }
    }
    return stepSize;
}

// ---------------------------------------------------------------------------
// Skyline LDL^T on a reverse Cuthill-McKee ordering of the vertex graph.
// ---------------------------------------------------------------------------
static bool skyline_solve(int n, std::vector<Trip>& T, const double* rhs, double* sol)
{
    int nb = n / 3;
    // vertex graph
    std::vector<std::vector<int>> adj(nb);
    for (auto& t : T) {
        int a = t.r / 3, b = t.c / 3;
        if (a != b) adj[a].push_back(b);
    }
    std::vector<int> deg(nb);
    for (int i = 0; i < nb; ++i) {
        std::sort(adj[i].begin(), adj[i].end());
        adj[i].erase(std::unique(adj[i].begin(), adj[i].end()), adj[i].end());
        deg[i] = (int)adj[i].size();
    }
    // RCM
    std::vector<int> order;
    order.reserve(nb);
    std::vector<char> seen(nb, 0);
    std::vector<int> byDeg(nb);
    for (int i = 0; i < nb; ++i) byDeg[i] = i;
    std::stable_sort(byDeg.begin(), byDeg.end(), [&](int a, int b) { return deg[a] < deg[b]; });
    for (int s : byDeg) {
        if (seen[s]) continue;
        size_t head = order.size();
        order.push_back(s);
        seen[s] = 1;
        while (head < order.size()) {
            int u = order[head++];
            std::vector<int> nb2;
            for (int w : adj[u])
                if (!seen[w]) {
                    seen[w] = 1;
                    nb2.push_back(w);
                }
            std::stable_sort(nb2.begin(), nb2.end(), [&](int a, int b) { return deg[a] < deg[b]; });
            order.insert(order.end(), nb2.begin(), nb2.end());
        }
    }
    std::reverse(order.begin(), order.end());
    std::vector<int> perm(nb);  // vertex -> new index
    for (int i = 0; i < nb; ++i) perm[order[i]] = i;
    auto P = [&](int dof) { return 3 * perm[dof / 3] + dof % 3; };
    std::vector<int> first(n);
    for (int i = 0; i < n; ++i) first[i] = i;
    for (auto& t : T) {
        int r = P(t.r), c = P(t.c);
        if (c < r) first[r] = std::min(first[r], c);
        else first[c] = std::min(first[c], r);
    }
    std::vector<size_t> off(n + 1, 0);
    for (int i = 0; i < n; ++i) off[i + 1] = off[i] + (i - first[i] + 1);
    std::vector<double> L(off[n], 0.0);
    auto at = [&](int i, int j) -> double& { return L[off[i] + (j - first[i])]; };  // j in [first[i], i]
    for (auto& t : T) {
        int r = P(t.r), c = P(t.c);
        if (c <= r) at(r, c) += t.v;
    }
    std::vector<double> D(n);
    for (int i = 0; i < n; ++i) {
        for (int j = first[i]; j < i; ++j) {
            double s = at(i, j);
            int k0 = std::max(first[i], first[j]);
            for (int k = k0; k < j; ++k) s -= at(i, k) * D[k] * at(j, k);
            at(i, j) = s / D[j];
        }
        double d = at(i, i);
        for (int k = first[i]; k < i; ++k) d -= at(i, k) * at(i, k) * D[k];
        if (!(d > 0)) return false;
        D[i] = d;
    }
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i) y[P(i)] = rhs[i];
    for (int i = 0; i < n; ++i) {
        double s = y[i];
        for (int k = first[i]; k < i; ++k) s -= at(i, k) * y[k];
        y[i] = s;
    }
    for (int i = 0; i < n; ++i) y[i] /= D[i];
    for (int i = n - 1; i >= 0; --i) {
        double yi = y[i];
        for (int k = first[i]; k < i; ++k) y[k] -= at(i, k) * yi;
    }
    for (int i = 0; i < n; ++i) sol[i] = y[P(i)];
    return true;
}

// ---------------------------------------------------------------------------
// One implicit-Euler step — IMPLICIT_EULER.h:151-902 restated (no strain
// limiting, no tets/rods/stitches, DBC handled by projection when the DBC step is
// intersection-free).
// ---------------------------------------------------------------------------
struct StepOut {
    int pn_iters = 0;
    int n_constraints = 0;
    double min_dist2 = 0;
    int gd_iters = 0;
    int status = 0;  // 0 ok, -1 iteration cap, -2 DBC step blocked by contact, -3 negative distance
};

struct Ctx {
    Shell* S;
    StepParams P;
    const double* xtilde;
    const double* xn;
    double kappa;
    // augmented-Lagrangian Dirichlet penalty (Shell/DIRICHLET.h), off when stiff == 0
    double stiff = 0;
    const int* dbc_idx = nullptr;
    const double* dbc_tgt = nullptr;
    int ndbc = 0;
    std::vector<char> proj;  // rows / columns projected out of the Newton system
    bool slp = false;        // split stepper projection: no membrane, bending, rods, tets
};

static double dbc_dist2(const Ctx& C, const double* x)
{
    double s = 0;
    for (int k = 0; k < C.ndbc; ++k)
        for (int d = 0; d < 3; ++d) {
            double dd = C.dbc_tgt[3 * k + d] - x[3 * C.dbc_idx[k] + d];
            s += dd * dd;
        }
    return s;
}

static double total_energy(const Ctx& C, const double* x, const std::vector<Con>& cs, const std::vector<Fric>& F,
                           bool* ok)
{
    const Shell& S = *C.S;
    double E = C.slp ? 0.0 : elastic_energy(S, x, C.P.h);
    double ine = 0;
    for (int i = 0; i < S.nv; ++i)
        for (int d = 0; d < 3; ++d) {
            double dd = x[3 * i + d] - C.xtilde[3 * i + d];
            ine += S.mass[i] * dd * dd;
        }
    E += 0.5 * ine;
    if (C.stiff != 0) {
        double pen = 0;
        for (int k = 0; k < C.ndbc; ++k) {
            double p = 0;
            for (int d = 0; d < 3; ++d) {
                double dd = C.dbc_tgt[3 * k + d] - x[3 * C.dbc_idx[k] + d];
                p += dd * dd;
            }
            pen += p * S.mass[C.dbc_idx[k]];
        }
        E += 0.5 * C.stiff * pen;
    }
    bool good = true;
    E += strain_terms(S, x, C.P.h, nullptr, nullptr, &good);
    if (!C.slp) E += tet_terms(S, x, C.P.h, nullptr, nullptr, &good);
    if (C.P.withCollision) good = barrier_terms(S, x, cs, C.P.dHat2, C.P.xi, C.kappa, &E, nullptr, nullptr) && good;
    if (C.P.withCollision && C.P.mu > 0) friction_terms(F, x, C.xn, C.P.epsv2 * C.P.h * C.P.h, C.P.mu, &E, nullptr, nullptr);
    if (ok) *ok = good;
    return E;
}

static void total_grad(const Ctx& C, const double* x, const std::vector<Con>& cs, const std::vector<Fric>& F,
                       double* g, Asm* A)
{
    const Shell& S = *C.S;
    int n = 3 * S.nv;
    for (int i = 0; i < n; ++i) g[i] = 0;
    if (!C.slp) elastic_grad_hess(S, x, C.P.h, g, A);
    strain_terms(S, x, C.P.h, g, A, nullptr);
    if (!C.slp) tet_terms(S, x, C.P.h, g, A, nullptr);
    for (int i = 0; i < S.nv; ++i)
        for (int d = 0; d < 3; ++d) g[3 * i + d] += S.mass[i] * (x[3 * i + d] - C.xtilde[3 * i + d]);
    const std::vector<char>& proj = C.proj.empty() ? S.dbc : C.proj;
    if (A)
        for (int i = 0; i < S.nv; ++i)
            if (!proj[i])
                for (int d = 0; d < 3; ++d) A->t.push_back({3 * i + d, 3 * i + d, S.mass[i]});
    if (C.stiff != 0)
        for (int k = 0; k < C.ndbc; ++k) {
            const int v = C.dbc_idx[k];
            for (int d = 0; d < 3; ++d) {
                g[3 * v + d] += C.stiff * S.mass[v] * (x[3 * v + d] - C.dbc_tgt[3 * k + d]);
                if (A && !proj[v]) A->t.push_back({3 * v + d, 3 * v + d, C.stiff * S.mass[v]});
            }
        }
    if (C.P.withCollision) barrier_terms(S, x, cs, C.P.dHat2, C.P.xi, C.kappa, nullptr, g, A);
    if (C.P.withCollision && C.P.mu > 0) friction_terms(F, x, C.xn, C.P.epsv2 * C.P.h * C.P.h, C.P.mu, nullptr, g, A);
    for (int i = 0; i < S.nv; ++i)
        if (proj[i]) {
            g[3 * i] = g[3 * i + 1] = g[3 * i + 2] = 0;
            if (A)
                for (int d = 0; d < 3; ++d) A->t.push_back({3 * i + d, 3 * i + d, 1.0});
        }
}

static void shell_step(Shell& S, const StepParams& P_in, double* x, double* v, double* kappa, const int* dbc_idx,
                       const double* dbc_tgt, int ndbc, StepOut& out)
{
    StepParams P = P_in;
    if (P.elastic) P.xi = 0;  // IPC.h:49-51, 752-754, FRICTION.h:28-30
    // the elastic barrier -k (d/dh - 1)^2 ln(d/dh) on squared distances is the
    // offset form with k / dh^2 (Math/BARRIER.h:9-62)
    auto bkappa = [&]() { return P.elastic ? kappa[0] / (P.dHat2 * P.dHat2) : kappa[0]; };
    const int nv = S.nv, n = 3 * nv;
    S.dbc.assign(nv, 0);
    for (int k = 0; k < ndbc; ++k) S.dbc[dbc_idx[k]] = 1;
    std::vector<double> xn(x, x + n), xt(n);
    for (int i = 0; i < nv; ++i)
        for (int d = 0; d < 3; ++d) {
            double a = S.mass[i] > 0 ? S.b[3 * i + d] / S.mass[i] : 0.0;
            xt[3 * i + d] = x[3 * i + d] + P.h * v[3 * i + d] + P.h * P.h * a;
        }
    // DBC step (IMPLICIT_EULER.h:304-401)
    std::vector<double> disp(n, 0.0);
    for (int k = 0; k < ndbc; ++k)
        for (int d = 0; d < 3; ++d) disp[3 * dbc_idx[k] + d] = dbc_tgt[3 * k + d] - x[3 * dbc_idx[k] + d];
    double dbcAlpha = 1;
    if (P.withCollision) dbcAlpha = ccd_step_size(S, x, disp.data(), 1.0, P.xi);
    Ctx C{&S, P, xt.data(), xn.data(), bkappa()};
    C.dbc_idx = dbc_idx;
    C.dbc_tgt = dbc_tgt;
    C.ndbc = ndbc;
    C.proj = S.dbc;
    double dbcPenaltyXn = 0;
    if (dbcAlpha == 1) {
        for (int k = 0; k < ndbc; ++k)
            for (int d = 0; d < 3; ++d) x[3 * dbc_idx[k] + d] = dbc_tgt[3 * k + d];
    } else {
        // augmented Lagrangian: Dirichlet vertices stay at x^n, pulled by a penalty;
        // only those with zero displacement stay projected (IMPLICIT_EULER.h:380-401)
        C.stiff = 1e6;
        dbcPenaltyXn = dbc_dist2(C, xn.data());
        C.proj.assign(nv, 0);
        for (int k = 0; k < ndbc; ++k) {
            const int v = dbc_idx[k];
            C.proj[v] = (disp[3 * v] == 0 && disp[3 * v + 1] == 0 && disp[3 * v + 2] == 0) ? 1 : 0;
        }
    }
    std::vector<Con> cs, cs_prev;
    std::vector<Fric> F;
    std::vector<double> dist2_prev, strain_prev;
    if (P.withCollision) {
        constraint_set(S, x, P.dHat2, P.xi, cs);
        if (P.mu > 0) friction_basis(x, cs, P.dHat2, P.xi, C.kappa, F);
    }
    double Eprev = total_energy(C, x, cs, F, nullptr);
    std::deque<double> res;
    int fricIterI = 0;
    bool useGD = false;
    std::vector<double> g(n), sol(n), rhs(n), xprev(n);
    int it = 0;
    double L2 = 0;
    do {
        if (it >= P.maxIter) {
            out.status = -1;
            break;
        }
        Asm A;
        A.dbc = &C.proj;
        total_grad(C, x, cs, F, g.data(), useGD ? nullptr : &A);
        for (int i = 0; i < n; ++i) rhs[i] = -g[i];
        if (useGD) sol = rhs;
        else if (!skyline_solve(n, A.t, rhs.data(), sol.data())) {
            useGD = true;
            sol = rhs;
            ++out.gd_iters;
        }
        // line search (IMPLICIT_EULER.h:9-149)
        xprev.assign(x, x + n);
        double alpha = 1.0;
        if (S.sl_kappa[0] > 0 || !S.tvol.empty()) {
            // elastic feasibility first (IMPLICIT_EULER.h:74-94)
            for (;;) {
                for (int i = 0; i < n; ++i) x[i] = xprev[i] + alpha * sol[i];
                bool feas = true;
                strain_terms(S, x, P.h, nullptr, nullptr, &feas);
                tet_terms(S, x, P.h, nullptr, nullptr, &feas);
                if (feas) break;
                alpha /= 2;
            }
            for (int i = 0; i < n; ++i) x[i] = xprev[i];
        }
        if (P.withCollision) alpha = ccd_step_size(S, xprev.data(), sol.data(), alpha, P.xi);
        double feasible = alpha, E;
        bool ok;
        do {
            for (int i = 0; i < n; ++i) x[i] = xprev[i] + alpha * sol[i];
            if (P.withCollision) {
                constraint_set(S, x, P.dHat2, P.xi, cs);
                if (!cs.empty() && min_dist2(cs, x, P.xi, nullptr) <= 0) {
                    alpha /= 2;
                    E = Eprev + 1;
                    ok = true;
                    continue;
                }
            }
            E = total_energy(C, x, cs, F, &ok);
            alpha /= 2;
        } while (E > Eprev || !ok);
        Eprev = E;
        // barrier stiffness update (IMPLICIT_EULER.h:566-595; offset IPC only)
        if (!cs_prev.empty() && !P.elastic) {
            std::vector<double> cur;
            min_dist2(cs_prev, x, P.xi, &cur);
            bool up = false;
            for (size_t i = 0; i < cur.size(); ++i)
                if (dist2_prev[i] < 1e-18 && cur[i] < dist2_prev[i]) {
                    up = true;
                    break;
                }
            if (up && kappa[0] < kappa[1]) {
                kappa[0] *= 2;
                C.kappa = kappa[0];
                Eprev = total_energy(C, x, cs, F, nullptr);
            }
        }
        dist2_prev.clear();
        if (!cs.empty()) min_dist2(cs, x, P.xi, &dist2_prev);
        cs_prev = cs;
        // strain-limit stiffness update (IMPLICIT_EULER.h:606-645)
        if (S.sl_kappa[0] > 0) {
            std::vector<double> st;
            strains(S, x, st);
            const double thr = 1.0e-4 * (S.sl_s[0] - S.sl_shat[0]);
            bool up = false;
            for (size_t i = 0; i < strain_prev.size() && !up; ++i)
                up = S.sl_s[0] - strain_prev[i] < thr && S.sl_s[0] - st[i] < thr;
            if (up && S.sl_kappa[0] < 1e5) {
                S.sl_kappa[0] *= 2;
                Eprev = total_energy(C, x, cs, F, nullptr);
            }
            strain_prev = st;
        }
        // convergence (IMPLICIT_EULER.h:647-710)
        double ss = 0;
        for (int i = 0; i < n; ++i) ss += sol[i] * sol[i];
        L2 = std::sqrt(ss / (nv - ndbc)) / P.h;
        ++it;
        res.push_back(L2);
        if (res.size() > 3) res.pop_front();
        double cur = L2;
        L2 = *std::max_element(res.begin(), res.end());
        if (useGD) L2 = P.tol * 10;
        if (alpha * 2 < 1e-8 && feasible > 1e-8) {
            if (!useGD) {
                if (cur < P.tol) res.assign(3, cur);
                else useGD = true;
            }
        } else {
            useGD = false;
        }
        // Dirichlet progress of the augmented-Lagrangian path (IMPLICIT_EULER.h:713-764)
        if (C.stiff != 0) {
            const double progress = 1 - std::sqrt(dbc_dist2(C, x) / dbcPenaltyXn);
            if (progress < 0.99) {
                if (L2 < P.tol * 10 && C.stiff < 1e8) {
                    C.stiff *= 2;
                    Eprev = total_energy(C, x, cs, F, nullptr);
                }
                L2 = P.tol * 10;
            } else {
                C.stiff = 0;
                C.proj = S.dbc;
                Eprev = total_energy(C, x, cs, F, nullptr);
            }
        }
        if (res.size() == 3 && L2 <= P.tol) {
            ++fricIterI;
            if ((fricIterI < P.fricIterAmt || P.fricIterAmt <= 0) && P.withCollision && P.mu > 0) {
                friction_basis(x, cs, P.dHat2, P.xi, C.kappa, F);
                Asm A2;
                A2.dbc = &C.proj;
                total_grad(C, x, cs, F, g.data(), &A2);
                for (int i = 0; i < n; ++i) rhs[i] = -g[i];
                if (!skyline_solve(n, A2.t, rhs.data(), sol.data())) {
                    out.status = -4;
                    break;
                }
                double s2 = 0;
                for (int i = 0; i < n; ++i) s2 += sol[i] * sol[i];
                L2 = std::sqrt(s2 / (nv - ndbc)) / P.h;
                if (L2 > P.tol) Eprev = total_energy(C, x, cs, F, nullptr);
            }
        }
    } while (res.size() < 3 || L2 > P.tol);
    for (int i = 0; i < n; ++i) v[i] = (x[i] - xn[i]) / P.h;
    out.pn_iters = it;
    out.n_constraints = (int)cs.size();
    out.min_dist2 = cs.empty() ? 0 : min_dist2(cs, x, P.xi, nullptr);
}

// Split stepper (Advance_One_Step_SIE_Discrete_Shell, SPLITTING_IE.h:362-729):
// implicit-Euler substep without contact and strain limiting (x'), then from x^n
// the projection minimising 1/2 |x - x'|_M^2 + strain barrier + contact barrier +
// friction (+ Dirichlet penalty, Compute_SLP_Energy :7-69), with DBC_Info_Init
// (:218-301) and DBC_Dual_Update (:303-360).
static void shell_step_split(Shell& S, const StepParams& P_in, double* x, double* v, double* kappa,
                             const int* dbc_idx, const double* dbc_tgt, int ndbc, StepOut& out)
{
    const int nv = S.nv, n = 3 * nv;
    std::vector<double> xs(x, x + n);
    StepOut o1;
    {
        StepParams P1 = P_in;
        P1.withCollision = 0;
        const double k0 = S.sl_kappa[0], k1 = S.sl_kappa[1];
        S.sl_kappa[0] = S.sl_kappa[1] = 0;
        shell_step(S, P1, x, v, kappa, dbc_idx, dbc_tgt, ndbc, o1);
        S.sl_kappa[0] = k0;
        S.sl_kappa[1] = k1;
    }
    StepParams P = P_in;
    if (P.elastic) P.xi = 0;
    std::vector<double> xprim(x, x + n);
    for (int i = 0; i < n; ++i) x[i] = xs[i];
    const double bk = P.elastic ? kappa[0] / (P.dHat2 * P.dHat2) : kappa[0];
    Ctx C{&S, P, xprim.data(), xs.data(), bk};
    C.slp = true;
    C.dbc_idx = dbc_idx;
    C.dbc_tgt = dbc_tgt;
    C.ndbc = ndbc;
    C.proj = S.dbc;
    std::vector<double> disp(n, 0.0);
    for (int k = 0; k < ndbc; ++k)
        for (int d = 0; d < 3; ++d) disp[3 * dbc_idx[k] + d] = dbc_tgt[3 * k + d] - x[3 * dbc_idx[k] + d];
    double dbcAlpha = 1, penaltyXn = 0;
    if (S.sl_kappa[0] > 0) {
        std::vector<double> xt(n);
        for (;;) {
            for (int i = 0; i < n; ++i) xt[i] = xs[i] + dbcAlpha * disp[i];
            bool feas = true;
            strain_terms(S, xt.data(), P.h, nullptr, nullptr, &feas);
            if (feas) break;
            dbcAlpha /= 2;
        }
    }
    if (dbcAlpha == 1) {
        for (int k = 0; k < ndbc; ++k)
            for (int d = 0; d < 3; ++d) x[3 * dbc_idx[k] + d] = dbc_tgt[3 * k + d];
    } else {
        C.stiff = 1e8;
        penaltyXn = dbc_dist2(C, xs.data());
        C.proj.assign(nv, 0);
        for (int k = 0; k < ndbc; ++k) {
            const int vv = dbc_idx[k];
            C.proj[vv] = (disp[3 * vv] == 0 && disp[3 * vv + 1] == 0 && disp[3 * vv + 2] == 0) ? 1 : 0;
        }
    }
    std::vector<Con> cs;
    std::vector<Fric> F;
    if (P.withCollision) {
        constraint_set(S, x, P.dHat2, P.xi, cs);
        if (P.mu > 0) friction_basis(x, cs, P.dHat2, P.xi, C.kappa, F);
    }
    bool ok;
    double Eprev = total_energy(C, x, cs, F, &ok);
    if (!ok) {
        out.status = -3;
        return;
    }
    std::deque<double> res;
    bool useGD = false;
    std::vector<double> g(n), sol(n), rhs(n), xprev(n);
    int it = 0;
    double L2 = 0;
    do {
        if (it >= P.maxIter) {
            out.status = -1;
            break;
        }
        Asm A;
        A.dbc = &C.proj;
        total_grad(C, x, cs, F, g.data(), useGD ? nullptr : &A);
        for (int i = 0; i < n; ++i) rhs[i] = -g[i];
        if (useGD) sol = rhs;
        else if (!skyline_solve(n, A.t, rhs.data(), sol.data())) {
            useGD = true;
            sol = rhs;
            ++out.gd_iters;
        }
        xprev.assign(x, x + n);
        double alpha = 1.0, feasible = 0, E = Eprev;
        if (P.withCollision) alpha = ccd_step_size(S, xprev.data(), sol.data(), 1.0, P.xi);
        bool valid = true;
        int trials = 0;
        do {
            if (++trials > 200) {
                out.status = -3;
                return;
            }
            for (int i = 0; i < n; ++i) x[i] = xprev[i] + alpha * sol[i];
            valid = true;
            strain_terms(S, x, P.h, nullptr, nullptr, &valid);
            if (valid) {
                if (feasible == 0) feasible = alpha;
                if (P.withCollision) {
                    constraint_set(S, x, P.dHat2, P.xi, cs);
                    if (!cs.empty() && min_dist2(cs, x, P.xi, nullptr) <= 0) {
                        alpha /= 2;
                        valid = false;
                        feasible = 0;
                        continue;
                    }
                }
                bool eok;
                E = total_energy(C, x, cs, F, &eok);
                valid = valid && eok;
            }
            alpha /= 2;
        } while (E > Eprev || !valid);
        Eprev = E;
        double ss = 0;
        for (int i = 0; i < n; ++i) ss += sol[i] * sol[i];
        L2 = std::sqrt(ss / (nv - ndbc)) / P.h;
        ++it;
        res.push_back(L2);
        if (res.size() > 3) res.pop_front();
        L2 = *std::max_element(res.begin(), res.end());
        if (useGD) L2 = P.tol * 10;
        useGD = alpha * 2 < 1e-6 && feasible > 1e-6;
        if (C.stiff != 0) {
            const double progress = 1 - std::sqrt(dbc_dist2(C, x) / penaltyXn);
            if (progress < 0.99) {
                if (L2 < P.tol * 10 && C.stiff < 1e10) {
                    C.stiff *= 2;
                    Eprev = total_energy(C, x, cs, F, nullptr);
                }
                L2 = P.tol * 10;
            } else {
                C.stiff = 0;
                C.proj = S.dbc;
                Eprev = total_energy(C, x, cs, F, nullptr);
            }
        }
    } while (res.size() < 3 || L2 > P.tol);
    for (int i = 0; i < n; ++i) v[i] = (x[i] - xs[i]) / P.h;
    out.pn_iters = o1.pn_iters + it;
    out.n_constraints = (int)cs.size();
    out.min_dist2 = cs.empty() ? 0 : min_dist2(cs, x, P.xi, nullptr);
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C entry points for ctypes
// ---------------------------------------------------------------------------
using namespace orc;

extern "C" {

void* orc_shell_create(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                       double thickness, const double* gravity, double bendMult, int nh_model)
{
    Shell* S = new Shell();
    shell_init(*S, nv, X, nt, tri, rho, E, nu, thickness, gravity, bendMult, nh_model);
    return S;
}

// shell scene plus rods and particles; codim = (rodE, rodRho, rodT, rodBendMult, partRho, partT)
void* orc_shell_create_codim(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                             double thickness, const double* gravity, double bendMult, int nh_model, int nseg,
                             const int* seg, int npart, const int* part, const double* codim)
{
    Shell* S = new Shell();
    shell_init(*S, nv, X, nt, tri, rho, E, nu, thickness, gravity, bendMult, nh_model);
    codim_init(*S, X, nseg, seg, codim[0], codim[1], codim[2], codim[3], npart, part, codim[4], codim[5], gravity);
    return S;
}

// shell + optional codimensional parts (codim null: none) + tetrahedra with
// material tetmat = (E, nu, rho)
void* orc_shell_create_full(int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                            double thickness, const double* gravity, double bendMult, int nh_model, int nseg,
                            const int* seg, int npart, const int* part, const double* codim, int ntet,
                            const int* tets, const double* tetmat)
{
    Shell* S = new Shell();
    shell_init(*S, nv, X, nt, tri, rho, E, nu, thickness, gravity, bendMult, nh_model, ntet, tets);
    if (codim) codim_init(*S, X, nseg, seg, codim[0], codim[1], codim[2], codim[3], npart, part, codim[4], codim[5], gravity);
    if (ntet) tet_init(*S, X, ntet, tets, tetmat[0], tetmat[1], tetmat[2], gravity);
    return S;
}

void orc_shell_destroy(void* h) { delete (Shell*)h; }

// counts: nt, nh, n_bnode, n_bedge, n_btri
void orc_shell_counts(void* h, int* c)
{
    Shell* S = (Shell*)h;
    c[0] = (int)S->vol.size();
    c[1] = (int)S->hinfo.size() / 3;
    c[2] = (int)S->bnode.size();
    c[3] = (int)S->bedge.size() / 2;
    c[4] = (int)S->btri.size() / 3;
}

// copies the setup arrays (sizes from orc_shell_counts); scal = (lam, mu, kbend)
void orc_shell_arrays(void* h, int* tri, double* P, double* vol, int* hinge, double* hinfo, double* mass, double* b,
                      int* bnode, int* bedge, double* scal)
{
    Shell* S = (Shell*)h;
    std::copy(S->tri.begin(), S->tri.end(), tri);
    std::copy(S->P.begin(), S->P.end(), P);
    std::copy(S->vol.begin(), S->vol.end(), vol);
    std::copy(S->hinge.begin(), S->hinge.end(), hinge);
    std::copy(S->hinfo.begin(), S->hinfo.end(), hinfo);
    std::copy(S->mass.begin(), S->mass.end(), mass);
    std::copy(S->b.begin(), S->b.end(), b);
    std::copy(S->bnode.begin(), S->bnode.end(), bnode);
    std::copy(S->bedge.begin(), S->bedge.end(), bedge);
    scal[0] = S->lam;
    scal[1] = S->mu;
    scal[2] = S->kbend;
}

double orc_shell_oipc(void* h, double dhat, double stiffMult, double* kappa2)
{
    return shell_oipc_kappa(*(Shell*)h, dhat, stiffMult, kappa2);
}

void orc_shell_set_strain_limit(void* h, const double* s, const double* s_hat, const double* kappa_s)
{
    Shell* S = (Shell*)h;
    for (int k = 0; k < 2; ++k) {
        S->sl_s[k] = s[k];
        S->sl_shat[k] = s_hat[k];
        S->sl_kappa[k] = kappa_s[k];
    }
}

void orc_shell_get_strain_limit(void* h, double* kappa_s)
{
    const Shell* S = (const Shell*)h;
    kappa_s[0] = S->sl_kappa[0];
    kappa_s[1] = S->sl_kappa[1];
}

static void set_dbc(Shell* S, const int* idx, int n)
{
    S->dbc.assign(S->nv, 0);
    for (int k = 0; k < n; ++k) S->dbc[idx[k]] = 1;
}

// constraint set at x: out rows of (kind, v0, v1, v2, v3, mult); returns the count
// (rows beyond cap are not written)
int orc_shell_constraints(void* h, const double* x, const int* dbc_idx, int ndbc, double dHat2, double xi, int* out,
                          int cap)
{
    Shell* S = (Shell*)h;
    set_dbc(S, dbc_idx, ndbc);
    std::vector<Con> cs;
    constraint_set(*S, x, dHat2, xi, cs);
    for (int i = 0; i < (int)cs.size() && i < cap; ++i) {
        out[6 * i] = cs[i].k;
        for (int k = 0; k < 4; ++k) out[6 * i + 1 + k] = cs[i].v[k];
        out[6 * i + 5] = cs[i].mult;
    }
    return (int)cs.size();
}

// incremental potential and its gradient at x (constraint set and, when
// xbasis != NULL, friction basis computed at xbasis with displacement from xn);
// params = (h, dHat2, xi, kappa, mu, epsv2, withCollision); returns E, or NaN on
// a non-positive distance.  DBC rows of g are zeroed.
double orc_shell_eval(void* h, const double* x, const double* xtilde, const double* xbasis, const double* xn,
                      const int* dbc_idx, int ndbc, const double* params, double* g)
{
    Shell* S = (Shell*)h;
    set_dbc(S, dbc_idx, ndbc);
    StepParams P{params[0], params[1], params[2], params[4], params[5], 1, 0, (int)params[6], 100};
    Ctx C{S, P, xtilde, xn, params[3]};
    std::vector<Con> cs;
    std::vector<Fric> F;
    if (P.withCollision) {
        constraint_set(*S, x, P.dHat2, P.xi, cs);
        if (P.mu > 0 && xbasis) {
            std::vector<Con> cb;
            constraint_set(*S, xbasis, P.dHat2, P.xi, cb);
            friction_basis(xbasis, cb, P.dHat2, P.xi, C.kappa, F);
        }
    }
    if (!(P.mu > 0 && xbasis)) P.mu = 0, C.P.mu = 0;
    bool ok;
    double E = total_energy(C, x, cs, F, &ok);
    if (!ok) return NAN;
    if (g) total_grad(C, x, cs, F, g, nullptr);
    return E;
}

// intersection-free step size along p from alpha (span cap + ACCD)
double orc_shell_ccd(void* h, const double* x, const double* p, double alpha, double xi, const int* dbc_idx, int ndbc)
{
    Shell* S = (Shell*)h;
    set_dbc(S, dbc_idx, ndbc);
    return ccd_step_size(*S, x, p, alpha, xi);
}

// one time step; params = (h, dHat2, xi, mu, epsv2, fricIterAmt, tol, withCollision, maxIter);
// kappa2 = (kappa, kappa_max) in/out; stats = (pn_iters, n_constraints, min_dist2, gd_iters)
int orc_shell_step(void* h, const double* params, double* x, double* v, double* kappa2, const int* dbc_idx,
                   const double* dbc_tgt, int ndbc, double* stats)
{
    Shell* S = (Shell*)h;
    StepParams P{params[0], params[1], params[2], params[3], params[4], (int)params[5], params[6], (int)params[7],
                 (int)params[8], (int)params[9]};
    StepOut o;
    shell_step(*S, P, x, v, kappa2, dbc_idx, dbc_tgt, ndbc, o);
    if (stats) {
        stats[0] = o.pn_iters;
        stats[1] = o.n_constraints;
        stats[2] = o.min_dist2;
        stats[3] = o.gd_iters;
    }
    return o.status;
}

int orc_shell_step_split(void* h, const double* params, double* x, double* v, double* kappa2, const int* dbc_idx,
                   const double* dbc_tgt, int ndbc, double* stats)
{
    Shell* S = (Shell*)h;
    StepParams P{params[0], params[1], params[2], params[3], params[4], (int)params[5], params[6], (int)params[7],
                 (int)params[8], (int)params[9]};
    StepOut o;
    shell_step_split(*S, P, x, v, kappa2, dbc_idx, dbc_tgt, ndbc, o);
    if (stats) {
        stats[0] = o.pn_iters;
        stats[1] = o.n_constraints;
        stats[2] = o.min_dist2;
        stats[3] = o.gd_iters;
    }
    return o.status;
}

}  // extern "C"

extern "C" {
// single-element checks: energy, gradient, Hessian (project = 1 applies makePD)
double orc_membrane_elem(const double* x9, const double* P, double k, double lam, double mu, int nh, int project,
                         double* g, double* H)
{
    Du xd[9], gd[9];
    for (int i = 0; i < 9; ++i) xd[i] = dc(x9[i]);
    membrane_grad<Du>(xd, P, k, lam, mu, nh, gd);
    for (int i = 0; i < 9; ++i) g[i] = gd[i].v;
    auto gf = [&](const Du* xx, Du* gg) { membrane_grad<Du>(xx, P, k, lam, mu, nh, gg); };
    hess_from_grad<9>(x9, gf, H);
    if (project) make_pd(9, H);
    return membrane_energy(x9, P, k, lam, mu, nh);
}

// gradient and Hessian of the dihedral angle itself (the bending element's
// building block), for the golden-vector checks
void orc_dihedral_derivs(const double* x12, double* g, double* H)
{
    dihedral_grad<double>(x12, g);
    auto gf = [&](const Du* xx, Du* gg) { dihedral_grad<Du>(xx, gg); };
    hess_from_grad<12>(x12, gf, H);
}

double orc_bending_elem(const double* x12, double thetabar, double c, int project, double* g, double* H)
{
    bending_grad_d(x12, thetabar, c, g);
    auto gf = [&](const Du* xx, Du* gg) { bending_grad<Du>(xx, thetabar, c, gg); };
    hess_from_grad<12>(x12, gf, H);
    if (project) make_pd(12, H);
    double th = dihedral_value(ld3(x12), ld3(x12 + 3), ld3(x12 + 6), ld3(x12 + 9));
    return c * (th - thetabar) * (th - thetabar);
}
}
