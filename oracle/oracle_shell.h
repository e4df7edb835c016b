// CPU ORACLE — test infrastructure only.  Shell scene, contact set and one
// implicit-Euler step, restated from the reference (see oracle_shell.cpp).
#pragma once
#include <cstdint>
#include <vector>

namespace orc {

// constraint kinds (mollified kinds carry the 4 vertices of the two edges)
enum ConKind { kPP = 0, kPE = 1, kPT = 2, kEE = 3, kEEM = 4, kPEM = 5, kPPM = 6 };

struct Con {
    int k;     // ConKind
    int v[4];  // PP (p0,p1) PE (p,e0,e1) PT (p,t0,t1,t2) EE (ea0,ea1,eb0,eb1)
               // EEM (ea0,ea1,eb0,eb1) PEM (p,p',e0,e1) PPM (p,p',q,q'): primed = edge partner
    int mult;  // PP/PE multiplicity after merging duplicates (1 otherwise)
};

struct Shell {
    int nv = 0;
    std::vector<double> X0;           // rest positions (nv*3), nodeAttr.x0
    std::vector<int> tri;             // nt*3 (degenerate triangles removed)
    std::vector<double> P;            // nt*3 inverse rest first fundamental form (p00,p01,p11)
    std::vector<double> vol;          // nt area * thickness
    double lam = 0, mu = 0;           // plane-stress Lame parameters
    std::vector<int> hinge;           // nh*4 (x0, x1, x2, x3), hinge edge x1-x2
    std::vector<double> hinfo;        // nh*3 (thetabar, |ebar|, hbar)
    double kbend = 0;                 // bendingStiffMult * E t^3 / (24 (1 - nu^2))
    std::vector<double> mass;         // nv lumped
    std::vector<double> b;            // nv*3 body force
    std::vector<int> bnode, bedge, btri;  // contact primitives
    std::vector<char> dbc;            // nv mask
    int nh_model = 1;                 // membrane: 1 Neo-Hookean (reference default), 0 StVK
    // discrete rods: segments (2) with (E, L, t), hinges (3) with (E bendMult, lsum, t)
    std::vector<int> rseg, rhinge;
    std::vector<double> rinfo, rhinfo;
    // bnode = [shell nodes | rod nodes from codim0 | particles from codim1];
    // the last nrod_e boundary edges are the rod segments
    int codim0 = 0, codim1 = 0, nrod_e = 0;
    // isotropic strain limiting (INEXT.h): the reference's s, sHat, kappa_s pairs;
    // off while sl_kappa[0] == 0
    double sl_s[2] = {1.01, 0}, sl_shat[2] = {1, 1}, sl_kappa[2] = {0, 0};
    // volumetric Neo-Hookean tetrahedra: vertices (4), Dm^-1 (9, row-major), volume
    std::vector<int> tet;
    std::vector<double> tDinv, tvol;
    double tlam = 0, tmu = 0;
};

struct StepParams {
    double h, dHat2, xi;  // time step, dhat^2, offset (thickness)
    double mu, epsv2;     // friction coefficient, epsv^2
    int fricIterAmt;
    double tol;           // Newton tolerance (velocity units: RMS step / h)
    int withCollision;
    int maxIter;          // safety cap on Newton iterations
    int elastic = 0;      // 1: elastic IPC (Advance_One_Step_IE_Hinge_EIPC): no offset, barrier / dhat^4, kappa fixed
};

}  // namespace orc
