// Host-side shell scene (built once per mesh, then uploaded).
#pragma once
#include <vector>

namespace cipc {

struct Sim;

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
};

int build_host_scene(HostScene& S, int nv, const double* X, int nt, const int* tri, double rho, double E, double nu,
                     double thickness, const double* gravity, double bendMult, int nh_model);
double oipc_kappa(const std::vector<double>& mass, double dhat, double stiffMult, double* kappa2);
int sim_upload(Sim* s, const HostScene& S);

}  // namespace cipc
