// Host-side shell scene (built once per mesh, then uploaded).
#pragma once
#include <vector>

namespace cipc {

struct Sim;

// Codimensional parts of a scene: discrete rods (Initialize_Discrete_Rod,
// Library/FEM/Shell/Rod/DISCRETE_ROD.h:85-150) and particles
// (Initialize_Discrete_Particle, Library/FEM/Shell/DISCRETE_PARTICLE.h:52-75).
struct CodimDesc {
    int nseg = 0;
    const int* seg = nullptr;  // 2 vertex indices per rod segment
    double rod_E = 0, rod_rho = 0, rod_thickness = 0, rod_bend_mult = 1;
    int npart = 0;
    const int* part = nullptr;  // particle vertex indices
    double part_rho = 0, part_thickness = 0;
};

// Volumetric tetrahedra (the drivers' add_object_3D: FEM.Compute_Vol_And_Inv_Basis,
// Library/FEM/DEFORMATION_GRADIENT.h:39-76; lumped mass; Neo-Hookean material with
// lambda = E nu / ((1 + nu)(1 - 2 nu)), mu = E / (2 (1 + nu))).
struct TetDesc {
    int ntet = 0;
    const int* tet = nullptr;  // 4 vertex indices per tetrahedron
    double E = 0, nu = 0, rho = 0;
};

struct HostScene {
    int nv = 0, nh_model = 1;
    std::vector<double> X0, P, vol, hinfo, mass, b;
    std::vector<int> tri, hinge, bnode, bedge, btri;
    double lam = 0, mu = 0, kbend = 0, cell = 1;
    // elastic block pattern in ELL form: row i's k-th block (k < ell_k) is block
    // k * nv + i, column col[k * nv + i]; rows shorter than ell_k are padded with
    // their own column and zero blocks
    int ell_k = 0;
    std::vector<int> col, diag, tri_slot, hinge_slot;
    std::vector<int> rowlen;  // real blocks of each row (the rest of the row is zero padding)
    // rods: segments (2 each) with (E, L, t), hinges (3 each) with (E bendMult, lsum, t)
    std::vector<int> rseg, rhinge, rseg_slot, rhinge_slot;
    std::vector<double> rinfo, rhinfo;
    // boundary layout of the codimensional primitives (IMPLICIT_EULER.h:242-277):
    // bnode = [shell nodes | rod nodes | particles], bedge = [shell edges | rod segments]
    int codim0 = 0, codim1 = 0, nrod_e = 0;
    // tetrahedra: vertices (4), rest inverse basis Dm^-1 (9, row-major), volume,
    // ELL slots (16); their surface triangles lead the contact triangles
    std::vector<int> tet, tet_slot;
    std::vector<double> tDinv, tvol;
    double tlam = 0, tmu = 0;
};

int build_host_scene(HostScene& S, int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                     double thickness, const double* gravity, double bendMult, int nh_model,
                     const CodimDesc* cd = nullptr, const TetDesc* td = nullptr);
double oipc_kappa(const std::vector<double>& mass, double dhat, double stiffMult, double* kappa2);
int sim_upload(Sim* s, const HostScene& S);

}  // namespace cipc
