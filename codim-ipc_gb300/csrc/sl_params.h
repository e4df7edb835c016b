// Parameters of the isotropic strain-limiting barrier (Library/FEM/Shell/INEXT.h;
// the reference's s, sHat and kappa_s pairs).
#pragma once

namespace cipc {

struct SlParams {
    double s0 = 1.01, s1 = 0;    // limits (upper, lower)
    double sh0 = 1, sh1 = 1;     // activation (upper, lower)
    double k0 = 0, k1 = 0;       // kappa_s (upper: 0 = strain limiting off; lower: 0 = off)
};

}  // namespace cipc
