// Host-side scene construction for shells and its upload to the device.
//
// Restates the reference's shell initialization (Library/FEM/Shell/DISCRETE_SHELL.h
// Initialize_Discrete_Shell :218-357 and Compute_Discrete_Shell_Inv_Basis :131-216,
// Library/Utils/MESHIO.h Find_Surface_Primitives :728-767): degenerate triangles are
// dropped, surface edges keep the orientation of their first occurrence and are
// ordered like a std::set of index pairs, each interior edge becomes a hinge
// (x0, x1, x2, x3) with rest angle, rest length and h = (|n1| + |n2|) / (6 |e|),
// masses are lumped (area * thickness * rho / 3 per corner), the membrane uses
// plane-stress Lame parameters and the hinge stiffness E t^3 / (24 (1 - nu^2)).
// On top of that it builds the block-sparsity pattern of the elastic Hessian
// (vertex pairs sharing a triangle or a hinge) with per-element slot maps, which
// is the sort-reduce of the reference's triplet assembly done once per mesh.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <map>
#include <set>
#include <vector>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "sim.h"
#include "sim_host.h"

namespace cipc {

static inline void v3sub(const double* a, const double* b, double* o)
{
    o[0] = a[0] - b[0];
    o[1] = a[1] - b[1];
    o[2] = a[2] - b[2];
}
static inline double v3dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void v3cross(const double* a, const double* b, double* o)
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double v3norm(const double* a) { return std::sqrt(v3dot(a, a)); }

static double rest_dihedral(const double* X0, const double* X1, const double* X2, const double* X3)
{
    double a[3], b[3], n1[3], n2[3], c[3], d[3];
    v3sub(X1, X0, a);
    v3sub(X2, X0, b);
    v3cross(a, b, n1);
    v3sub(X2, X3, a);
    v3sub(X1, X3, b);
    v3cross(a, b, n2);
    double cs = v3dot(n1, n2) / std::sqrt(v3dot(n1, n1) * v3dot(n2, n2));
    double th = std::acos(std::max(-1.0, std::min(1.0, cs)));
    v3cross(n2, n1, c);
    v3sub(X1, X2, d);
    if (v3dot(c, d) < 0) th = -th;
    return th;
}

// surface triangles of a tetrahedral mesh (Find_Surface_TriMesh, MESHIO.h:486-544):
// the four outward faces (0,2,1), (0,3,2), (0,1,3), (1,2,3) of every tetrahedron
// keyed as given; a face is on the surface if no rotation of its reverse is a key;
// output in key order
static void tet_surface(int ntet, const int* tet, std::vector<int>& out)
{
    std::set<std::array<int, 3>> keys;
    for (int t = 0; t < ntet; ++t) {
        const int* v = tet + 4 * t;
        keys.insert({v[0], v[2], v[1]});
        keys.insert({v[0], v[3], v[2]});
        keys.insert({v[0], v[1], v[3]});
        keys.insert({v[1], v[2], v[3]});
    }
    for (const auto& k : keys) {
        if (keys.count({k[2], k[1], k[0]}) || keys.count({k[1], k[0], k[2]}) || keys.count({k[0], k[2], k[1]})) continue;
        out.insert(out.end(), k.begin(), k.end());
    }
}

int build_host_scene(HostScene& S, int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                     double thickness, const double* gravity, double bendMult, int nh_model, const CodimDesc* cd,
                     const TetDesc* td)
{
    if (td && td->ntet) {
        if (td->ntet < 0 || !td->tet || !(td->rho > 0) || !(td->E > 0) || !(td->nu > -1 && td->nu < 0.5))
            return set_error(CIPC_ERR_INVALID_ARG, "tet setup: null arrays or bad material");
        for (int i = 0; i < 4 * td->ntet; ++i)
            if (td->tet[i] < 0 || td->tet[i] >= nv) return set_error(CIPC_ERR_INDEX_RANGE, "tet setup: vertex index out of range");
    }
    if (cd) {
        if (cd->nseg < 0 || cd->npart < 0 || (cd->nseg && !cd->seg) || (cd->npart && !cd->part))
            return set_error(CIPC_ERR_INVALID_ARG, "codim setup: null arrays or negative counts");
        for (int i = 0; i < 2 * cd->nseg; ++i)
            if (cd->seg[i] < 0 || cd->seg[i] >= nv) return set_error(CIPC_ERR_INDEX_RANGE, "codim setup: segment index out of range");
        for (int i = 0; i < cd->nseg; ++i)
            if (cd->seg[2 * i] == cd->seg[2 * i + 1]) return set_error(CIPC_ERR_INVALID_ARG, "codim setup: degenerate segment");
        for (int i = 0; i < cd->npart; ++i)
            if (cd->part[i] < 0 || cd->part[i] >= nv) return set_error(CIPC_ERR_INDEX_RANGE, "codim setup: particle index out of range");
        if (cd->nseg && !(cd->rod_thickness > 0 && cd->rod_rho > 0))
            return set_error(CIPC_ERR_INVALID_ARG, "codim setup: rods need thickness > 0 and density > 0");
        if (cd->npart && !(cd->part_thickness > 0 && cd->part_rho > 0))
            return set_error(CIPC_ERR_INVALID_ARG, "codim setup: particles need thickness > 0 and density > 0");
    }
    if (nv <= 0 || nt < 0 || !X || (nt && !tri))
        return set_error(CIPC_ERR_INVALID_ARG, "shell setup: empty mesh or null arrays");
    for (int i = 0; i < 3 * nt; ++i)
        if (tri[i] < 0 || tri[i] >= nv) return set_error(CIPC_ERR_INDEX_RANGE, "shell setup: triangle index out of range");
    S = HostScene();
    S.nv = nv;
    S.nh_model = nh_model;
    S.X0.assign(X, X + 3 * nv);
    for (int t = 0; t < nt; ++t) {
        const double *x1 = X + 3 * tri[3 * t], *x2 = X + 3 * tri[3 * t + 1], *x3 = X + 3 * tri[3 * t + 2];
        double e1[3], e2[3];
        v3sub(x2, x1, e1);
        v3sub(x3, x1, e2);
        double a00 = v3dot(e1, e1), a01 = v3dot(e1, e2), a11 = v3dot(e2, e2);
        if (a00 * a11 - a01 * a01 != 0) S.tri.insert(S.tri.end(), tri + 3 * t, tri + 3 * t + 3);
    }
    nt = (int)S.tri.size() / 3;
    // contact triangles: tetrahedral surface first, then the shell (IMPLICIT_EULER.h:235-241)
    std::vector<int> ctri;
    if (td && td->ntet) tet_surface(td->ntet, td->tet, ctri);
    ctri.insert(ctri.end(), S.tri.begin(), S.tri.end());
    const int nct = (int)ctri.size() / 3;
    std::map<std::pair<int, int>, int> e2t;
    for (int t = 0; t < nt; ++t) {
        const int* v = &S.tri[3 * t];
        for (int k = 0; k < 3; ++k) e2t[{v[k], v[(k + 1) % 3]}] = t;
    }
    std::set<std::pair<int, int>> es;
    std::vector<char> isb(nv, 0);
    for (int t = 0; t < nct; ++t) {
        const int* v = &ctri[3 * t];
        for (int k = 0; k < 3; ++k) {
            int a = v[k], b = v[(k + 1) % 3];
            if (!es.count({b, a})) es.insert({a, b});
            isb[a] = 1;
        }
    }
    for (auto& e : es) {
        S.bedge.push_back(e.first);
        S.bedge.push_back(e.second);
    }
    for (int i = 0; i < nv; ++i)
        if (isb[i]) S.bnode.push_back(i);
    S.btri = ctri;
    S.P.resize(3 * nt);
    S.vol.resize(nt);
    S.mass.assign(nv, 0.0);
    S.b.assign(3 * nv, 0.0);
    for (int t = 0; t < nt; ++t) {
        const double *x1 = X + 3 * S.tri[3 * t], *x2 = X + 3 * S.tri[3 * t + 1], *x3 = X + 3 * S.tri[3 * t + 2];
        double e1[3], e2[3], n[3];
        v3sub(x2, x1, e1);
        v3sub(x3, x1, e2);
        double a00 = v3dot(e1, e1), a01 = v3dot(e1, e2), a11 = v3dot(e2, e2);
        double det = a00 * a11 - a01 * a01;
        S.P[3 * t] = a11 / det;
        S.P[3 * t + 1] = -a01 / det;
        S.P[3 * t + 2] = a00 / det;
        v3cross(e1, e2, n);
        double area = v3norm(n) / 2;
        S.vol[t] = area * thickness;
        double mp = area * thickness * rho / 3;
        for (int k = 0; k < 3; ++k) {
            int vv = S.tri[3 * t + k];
            S.mass[vv] += mp;
            for (int d = 0; d < 3; ++d) S.b[3 * vv + d] += mp * gravity[d];
        }
    }
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
        const double *X0v = X + 3 * v0, *X1v = X + 3 * v1, *X2v = X + 3 * v2, *X3v = X + 3 * v3;
        double el3[3], a[3], b[3], n1[3], n2[3];
        v3sub(X1v, X2v, el3);
        double el = v3norm(el3);
        v3sub(X1v, X0v, a);
        v3sub(X2v, X0v, b);
        v3cross(a, b, n1);
        v3sub(X2v, X3v, a);
        v3sub(X1v, X3v, b);
        v3cross(a, b, n2);
        S.hinfo.insert(S.hinfo.end(), {rest_dihedral(X0v, X1v, X2v, X3v), el, (v3norm(n1) + v3norm(n2)) / (el * 6)});
    }
    // tetrahedra (DEFORMATION_GRADIENT.h:39-76): Dm = [X1-X0, X2-X0, X3-X0],
    // vol = det(Dm) / 6, Dm^-1; mass vol rho / 4 per corner
    if (td && td->ntet) {
        S.tlam = td->E * td->nu / ((1 + td->nu) * (1 - 2 * td->nu));
        S.tmu = td->E / (2 * (1 + td->nu));
        for (int t = 0; t < td->ntet; ++t) {
            const int* v = td->tet + 4 * t;
            double D[3][3];
            for (int k = 0; k < 3; ++k)
                for (int i = 0; i < 3; ++i) D[i][k] = X[3 * v[k + 1] + i] - X[3 * v[0] + i];
            const double c00 = D[1][1] * D[2][2] - D[1][2] * D[2][1], c01 = D[1][2] * D[2][0] - D[1][0] * D[2][2],
                         c02 = D[1][0] * D[2][1] - D[1][1] * D[2][0];
            const double det = D[0][0] * c00 + D[0][1] * c01 + D[0][2] * c02;
            if (!(det > 0)) return set_error(CIPC_ERR_INVALID_ARG, "tet setup: tetrahedron %d is degenerate or inverted", t);
            const double inv[9] = {c00 / det,
                                   (D[0][2] * D[2][1] - D[0][1] * D[2][2]) / det,
                                   (D[0][1] * D[1][2] - D[0][2] * D[1][1]) / det,
                                   c01 / det,
                                   (D[0][0] * D[2][2] - D[0][2] * D[2][0]) / det,
                                   (D[0][2] * D[1][0] - D[0][0] * D[1][2]) / det,
                                   c02 / det,
                                   (D[0][1] * D[2][0] - D[0][0] * D[2][1]) / det,
                                   (D[0][0] * D[1][1] - D[0][1] * D[1][0]) / det};
            S.tet.insert(S.tet.end(), v, v + 4);
            S.tDinv.insert(S.tDinv.end(), inv, inv + 9);
            const double vol = det / 6;
            S.tvol.push_back(vol);
            const double mp = vol * td->rho / 4;
            for (int k = 0; k < 4; ++k) {
                S.mass[v[k]] += mp;
                for (int d = 0; d < 3; ++d) S.b[3 * v[k] + d] += mp * gravity[d];
            }
        }
    }
    S.lam = E * nu / (1 - nu * nu);
    S.mu = E / (2 * (1 + nu));
    S.kbend = bendMult * (E * std::pow(thickness, 3) / (24 * (1 - nu * nu)));
    // rods (DISCRETE_ROD.h:100-150): lumped segment mass, hinges between every pair
    // of segments meeting at a vertex (vertex-ordered), rest data
    S.codim0 = S.codim1 = (int)S.bnode.size();
    if (cd && cd->nseg) {
        std::map<int, std::vector<int>> nb;
        std::map<int, double> rod_node;
        for (int i = 0; i < cd->nseg; ++i) {
            const int a = cd->seg[2 * i], b = cd->seg[2 * i + 1];
            nb[a].push_back(b);
            nb[b].push_back(a);
            double d[3];
            v3sub(X + 3 * a, X + 3 * b, d);
            const double L = v3norm(d);
            S.rseg.insert(S.rseg.end(), {a, b});
            S.rinfo.insert(S.rinfo.end(), {cd->rod_E, L, cd->rod_thickness});
            const double mp = L * M_PI * cd->rod_thickness * cd->rod_thickness / 4 * cd->rod_rho / 2;
            for (int v : {a, b}) {
                S.mass[v] += mp;
                for (int k = 0; k < 3; ++k) S.b[3 * v + k] += mp * gravity[k];
                rod_node[v] += 0;
            }
            S.bedge.insert(S.bedge.end(), {a, b});
        }
        for (auto& kv : nb)
            if (kv.second.size() >= 2)
                for (size_t i = 0; i < kv.second.size(); ++i)
                    for (size_t j = i + 1; j < kv.second.size(); ++j) {
                        const int x0 = kv.second[i], x1 = kv.first, x2 = kv.second[j];
                        double d0[3], d1[3];
                        v3sub(X + 3 * x1, X + 3 * x0, d0);
                        v3sub(X + 3 * x2, X + 3 * x1, d1);
                        S.rhinge.insert(S.rhinge.end(), {x0, x1, x2});
                        S.rhinfo.insert(S.rhinfo.end(), {cd->rod_E * cd->rod_bend_mult, v3norm(d0) + v3norm(d1),
                                                         cd->rod_thickness});
                    }
        for (auto& kv : rod_node) S.bnode.push_back(kv.first);
        S.nrod_e = cd->nseg;
    }
    S.codim1 = (int)S.bnode.size();
    // particles (DISCRETE_PARTICLE.h:60-69): mass 4/3 pi t^3 / 8 rho
    if (cd && cd->npart) {
        const double m = 4.0 / 3.0 * M_PI * std::pow(cd->part_thickness, 3) / 8 * cd->part_rho;
        for (int i = 0; i < cd->npart; ++i) {
            const int v = cd->part[i];
            S.mass[v] += m;
            for (int k = 0; k < 3; ++k) S.b[3 * v + k] += m * gravity[k];
            S.bnode.push_back(v);
        }
    }
    // broad-phase cell: mean rest edge length
    double el = 0;
    int ne = (int)S.bedge.size() / 2;
    for (int e = 0; e < ne; ++e) {
        double d[3];
        v3sub(X + 3 * S.bedge[2 * e], X + 3 * S.bedge[2 * e + 1], d);
        el += v3norm(d);
    }
    S.cell = ne ? el / ne : 1.0;
    // block-sparsity pattern of the elastic Hessian
    std::vector<std::vector<int>> adj(nv);
    for (int i = 0; i < nv; ++i) adj[i].push_back(i);
    for (int t = 0; t < nt; ++t)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) adj[S.tri[3 * t + a]].push_back(S.tri[3 * t + b]);
    int nh = (int)S.hinge.size() / 4;
    for (int e = 0; e < nh; ++e)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) adj[S.hinge[4 * e + a]].push_back(S.hinge[4 * e + b]);
    const int nrs = (int)S.rseg.size() / 2, nrh = (int)S.rhinge.size() / 3;
    for (int e = 0; e < nrs; ++e)
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) adj[S.rseg[2 * e + a]].push_back(S.rseg[2 * e + b]);
    for (int e = 0; e < nrh; ++e)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) adj[S.rhinge[3 * e + a]].push_back(S.rhinge[3 * e + b]);
    const int ntet = (int)S.tet.size() / 4;
    for (int e = 0; e < ntet; ++e)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) adj[S.tet[4 * e + a]].push_back(S.tet[4 * e + b]);
    int K = 1;
    for (int i = 0; i < nv; ++i) {
        std::sort(adj[i].begin(), adj[i].end());
        adj[i].erase(std::unique(adj[i].begin(), adj[i].end()), adj[i].end());
        K = std::max(K, (int)adj[i].size());
    }
    if ((long long)K * nv >= (1ll << 31) / 9) return set_error(CIPC_ERR_INVALID_ARG, "mesh too large for the block pattern");
    // ELL layout: block k of row i at k * nv + i, so that consecutive rows'
    // k-th blocks are contiguous in memory
    S.ell_k = K;
    S.col.assign((size_t)K * nv, 0);
    S.diag.resize(nv);
    S.rowlen.resize(nv);
    for (int i = 0; i < nv; ++i) S.rowlen[i] = (int)adj[i].size();
    for (int i = 0; i < nv; ++i)
        for (int k = 0; k < K; ++k) {
            S.col[(size_t)k * nv + i] = k < (int)adj[i].size() ? adj[i][k] : i;
            if (k < (int)adj[i].size() && adj[i][k] == i) S.diag[i] = k * nv + i;
        }
    auto slot = [&](int r, int c) {
        const int k = (int)(std::lower_bound(adj[r].begin(), adj[r].end(), c) - adj[r].begin());
        return k * nv + r;
    };
    S.tri_slot.resize(9 * nt);
    for (int t = 0; t < nt; ++t)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) S.tri_slot[9 * t + 3 * a + b] = slot(S.tri[3 * t + a], S.tri[3 * t + b]);
    S.hinge_slot.resize(16 * nh);
    for (int e = 0; e < nh; ++e)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) S.hinge_slot[16 * e + 4 * a + b] = slot(S.hinge[4 * e + a], S.hinge[4 * e + b]);
    S.rseg_slot.resize(4 * nrs);
    for (int e = 0; e < nrs; ++e)
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) S.rseg_slot[4 * e + 2 * a + b] = slot(S.rseg[2 * e + a], S.rseg[2 * e + b]);
    S.rhinge_slot.resize(9 * nrh);
    for (int e = 0; e < nrh; ++e)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) S.rhinge_slot[9 * e + 3 * a + b] = slot(S.rhinge[3 * e + a], S.rhinge[3 * e + b]);
    S.tet_slot.resize(16 * ntet);
    for (int e = 0; e < ntet; ++e)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) S.tet_slot[16 * e + 4 * a + b] = slot(S.tet[4 * e + a], S.tet[4 * e + b]);
    return CIPC_OK;
}

// offset-IPC barrier stiffness (DISCRETE_SHELL.h:555-577, elasticIPC = false):
// kappa = mult * 1e11 * mean(diag M) * 3 / (4e-16 * b''(1e-16; dhat^2, kappa = 1)), kappa_max = 100 kappa
double oipc_kappa(const std::vector<double>& mass, double dhat, double stiffMult, double* kappa2)
{
    const double dHat2 = dhat * dhat;
    const double d = 1.0e-16, t2 = d - dHat2;
    const double Hb = (std::log(d / dHat2) * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2);
    double msum = 0;
    for (double m : mass) msum += 3 * m;
    const double mmean = mass.empty() ? 0.0 : msum / (3.0 * mass.size());
    kappa2[0] = stiffMult * 1.0e11 * mmean * 3 / (4.0e-16 * Hb);
    kappa2[1] = 100 * kappa2[0];
    return dHat2;
}

template <typename T>
static cudaError_t up(DBuf<T>& d, const std::vector<T>& h)
{
    cudaError_t e = d.alloc(h.size());
    if (e != cudaSuccess || h.empty()) return e;
    return cudaMemcpy(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

int sim_upload(Sim* s, const HostScene& S)
{
    s->nv = S.nv;
    s->nt = (int)S.vol.size();
    s->nh = (int)S.hinfo.size() / 3;
    s->nbn = (int)S.bnode.size();
    s->nbe = (int)S.bedge.size() / 2;
    s->nbt = (int)S.btri.size() / 3;
    s->nh_model = S.nh_model;
    s->lam = S.lam;
    s->mu = S.mu;
    s->kbend = S.kbend;
    s->cell = S.cell;
    s->nnzb = (int)S.col.size();
    s->ell_k = S.ell_k;
    {
        long long real = 0;
        for (int L : S.rowlen) real += L;
        s->rows_uniform = 10 * real >= 9 * (long long)S.ell_k * S.nv;
    }
    cudaError_t e = cudaSuccess;
#define UP(a, b)                       \
    if (e == cudaSuccess) e = up(a, b);
    UP(s->tri, S.tri) UP(s->hinge, S.hinge) UP(s->bnode, S.bnode) UP(s->bedge, S.bedge) UP(s->btri, S.btri)
    UP(s->P, S.P) UP(s->vol, S.vol) UP(s->hinfo, S.hinfo) UP(s->mass, S.mass) UP(s->b, S.b) UP(s->X0, S.X0)
    UP(s->col, S.col) UP(s->diag, S.diag) UP(s->rowlen, S.rowlen) UP(s->tri_slot, S.tri_slot)
    UP(s->hinge_slot, S.hinge_slot)
    UP(s->rseg, S.rseg) UP(s->rhinge, S.rhinge) UP(s->rseg_slot, S.rseg_slot) UP(s->rhinge_slot, S.rhinge_slot)
    UP(s->rinfo, S.rinfo) UP(s->rhinfo, S.rhinfo)
    UP(s->tet, S.tet) UP(s->tet_slot, S.tet_slot) UP(s->tDinv, S.tDinv) UP(s->tvol, S.tvol)
#undef UP
    s->ntet = (int)S.tvol.size();
    s->tlam = S.tlam;
    s->tmu = S.tmu;
    s->nrs = (int)S.rseg.size() / 2;
    s->nrh = (int)S.rhinge.size() / 3;
    s->codim0 = S.codim0;
    s->codim1 = S.codim1;
    s->nrod_e = S.nrod_e;
    const size_t n3 = 3 * (size_t)S.nv;
    for (DBuf<double>* d : {&s->x, &s->xn, &s->xt, &s->v, &s->g, &s->dir, &s->xprev, &s->rhs, &s->disp})
        if (e == cudaSuccess) e = d->alloc(n3);
    for (DBuf<uint8_t>* m : {&s->dbc, &s->proj, &s->dbc_fixed}) {
        if (e == cudaSuccess) e = m->alloc(S.nv);
        if (e == cudaSuccess) e = cudaMemset(m->p, 0, S.nv);
    }
    if (e == cudaSuccess) e = s->x.alloc(n3);
    if (e == cudaSuccess) e = cudaMemcpy(s->x.p, S.X0.data(), n3 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(s->v.p, 0, n3 * sizeof(double));
    if (e == cudaSuccess) e = s->pdiag.alloc(9 * (size_t)S.nv);
    if (e == cudaSuccess) e = s->pinv.alloc(9 * sizeof(double) * (size_t)S.nv);
    if (e == cudaSuccess) e = s->hval.alloc(9 * sizeof(double) * (size_t)s->nnzb);
    if (e == cudaSuccess) e = s->red.alloc(1 << 16);
    if (e == cudaSuccess) e = s->cnt.alloc(64);
    if (e != cudaSuccess) return set_cuda_error(e, "sim upload");
    return CIPC_OK;
}

int sim_create(Sim** out, int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
               double thickness, const double* gravity, double bendMult, int nh_model, const CodimDesc* cd,
               const TetDesc* td)
{
    HostScene S;
    int rc = build_host_scene(S, nv, X, nt, tri, rho, E, nu, thickness, gravity, bendMult, nh_model, cd, td);
    if (rc != CIPC_OK) return rc;
    rc = ensure_device();
    if (rc != CIPC_OK) return rc;
    Sim* s = new Sim();
    s->trace = std::getenv("CIPC_TRACE") != nullptr;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return set_error(CIPC_ERR_CUDA, "sim: stream creation failed");
    }
    rc = sim_upload(s, S);
    if (rc != CIPC_OK) {
        sim_destroy(s);
        return rc;
    }
    s->host_mass = S.mass;
    *out = s;
    return CIPC_OK;
}

}  // namespace cipc
