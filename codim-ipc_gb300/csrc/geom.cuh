// Device geometry for contact pairs: distance-type classification, squared
// distances and additive-CCD state, in FP64.
//
// Arithmetic rule (shared with the CPU checker so FP64 decisions agree bit for
// bit): dot products are fma chains  dot(a,b) = fma(a.z,b.z, fma(a.x,b.x, a.y*b.y)),
// cross products use one fma per component, position updates x + t*d are a single
// fma, and everything else is evaluated left to right.  On the device every other
// FP64 operation here is an explicit-rounding intrinsic (__dadd_rn, __dmul_rn,
// __ddiv_rn, ...), which the compiler never contracts, so the rule holds in any
// translation unit whatever its -fmad setting.
#pragma once
#include <cmath>
#include <cstdint>

#ifndef CIPC_HD
#define CIPC_HD __host__ __device__ __forceinline__
#endif

namespace cipc {

#ifdef __CUDA_ARCH__
#define G_ADD(a, b) __dadd_rn((a), (b))
#define G_SUB(a, b) __dsub_rn((a), (b))
#define G_MUL(a, b) __dmul_rn((a), (b))
#define G_DIV(a, b) __ddiv_rn((a), (b))
#else
#define G_ADD(a, b) ((a) + (b))
#define G_SUB(a, b) ((a) - (b))
#define G_MUL(a, b) ((a) * (b))
#define G_DIV(a, b) ((a) / (b))
#endif

struct d3 {
    double x, y, z;
};

CIPC_HD d3 mk(double a, double b, double c) { return d3{a, b, c}; }
CIPC_HD d3 operator-(d3 a, d3 b) { return d3{G_SUB(a.x, b.x), G_SUB(a.y, b.y), G_SUB(a.z, b.z)}; }
CIPC_HD d3 operator+(d3 a, d3 b) { return d3{G_ADD(a.x, b.x), G_ADD(a.y, b.y), G_ADD(a.z, b.z)}; }
CIPC_HD d3 scl(d3 a, double s) { return d3{G_MUL(a.x, s), G_MUL(a.y, s), G_MUL(a.z, s)}; }
CIPC_HD d3 dvs(d3 a, double s) { return d3{G_DIV(a.x, s), G_DIV(a.y, s), G_DIV(a.z, s)}; }
CIPC_HD double dot(d3 a, d3 b) { return fma(a.z, b.z, fma(a.x, b.x, G_MUL(a.y, b.y))); }
CIPC_HD double n2(d3 a) { return dot(a, a); }
CIPC_HD d3 cross(d3 a, d3 b)
{
    return d3{fma(a.y, b.z, -G_MUL(a.z, b.y)), fma(a.z, b.x, -G_MUL(a.x, b.z)), fma(a.x, b.y, -G_MUL(a.y, b.x))};
}
CIPC_HD d3 axpy(double t, d3 d, d3 x)
{
    return d3{fma(t, d.x, x.x), fma(t, d.y, x.y), fma(t, d.z, x.z)};
}
CIPC_HD d3 ld(const double* __restrict__ p, int64_t i)
{
#ifdef __CUDA_ARCH__
    return d3{__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2)};
#else
    return d3{p[3 * i], p[3 * i + 1], p[3 * i + 2]};
#endif
}

// Eigen-style pivoted LDL^T solve of a symmetric 2x2 system; the pivot is the
// larger |diagonal| (first on ties), zero pivots give zero, |D| <= DBL_MIN entries
// are pseudo-inverted to zero.
CIPC_HD void ldlt2(double a00, double a10, double a11, double b0, double b1,
                                      double& y0, double& y1)
{
    const bool sw = fabs(a11) > fabs(a00);
    const double d0 = sw ? a11 : a00;
    const double m11 = sw ? a00 : a11;
    if (sw) {
        double t = b0;
        b0 = b1;
        b1 = t;
    }
    if (d0 == 0.0) {
        y0 = 0.0;
        y1 = 0.0;
        return;
    }
    const double l10 = G_DIV(a10, d0);
    const double d1 = fma(-l10, G_MUL(d0, l10), m11);
    double z0 = b0;
    double z1 = fma(-l10, z0, b1);
    z0 = (fabs(d0) > 2.2250738585072014e-308) ? G_DIV(z0, d0) : 0.0;
    z1 = (fabs(d1) > 2.2250738585072014e-308) ? G_DIV(z1, d1) : 0.0;
    z0 = fma(-l10, z1, z0);
    if (sw) {
        y0 = z1;
        y1 = z0;
    } else {
        y0 = z0;
        y1 = z1;
    }
}

CIPC_HD void pt_param(d3 r0, d3 n, d3 v, double& s, double& q)
{
    const d3 r1 = cross(r0, n);
    ldlt2(dot(r0, r0), dot(r1, r0), dot(r1, r1), dot(r0, v), dot(r1, v), s, q);
}

// Point-triangle distance type: 0-2 PP(t0,t1,t2), 3-5 PE(t0t1,t1t2,t2t0), 6 PT.
CIPC_HD int pt_type(d3 p, d3 t0, d3 t1, d3 t2)
{
    const d3 n = cross(t1 - t0, t2 - t0);
    double s0, q0, s1, q1, s2, q2;
    pt_param(t1 - t0, n, p - t0, s0, q0);
    if (s0 > 0.0 && s0 < 1.0 && q0 >= 0.0) return 3;
    pt_param(t2 - t1, n, p - t1, s1, q1);
    if (s1 > 0.0 && s1 < 1.0 && q1 >= 0.0) return 4;
    pt_param(t0 - t2, n, p - t2, s2, q2);
    if (s2 > 0.0 && s2 < 1.0 && q2 >= 0.0) return 5;
    if (s0 <= 0.0 && s2 >= 1.0) return 0;
    if (s1 <= 0.0 && s0 >= 1.0) return 1;
    if (s2 <= 0.0 && s1 >= 1.0) return 2;
    return 6;
}

// Edge-edge distance type: 0 PP(a0,b0) 1 PP(a0,b1) 2 PE(a0,b) 3 PP(a1,b0) 4 PP(a1,b1)
// 5 PE(a1,b) 6 PE(b0,a) 7 PE(b1,a) 8 EE; nearly parallel pairs fall back to PE.
CIPC_HD int ee_type(d3 ea0, d3 ea1, d3 eb0, d3 eb1)
{
    const d3 u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0;
    const double a = dot(u, u), b = dot(u, v), c = dot(v, v), d = dot(u, w), e = dot(v, w);
    const double D = fma(a, c, -G_MUL(b, b));
    double tD = D, tN;
    int dc = 8;
    const double sN = fma(b, e, -G_MUL(c, d));
    if (sN <= 0.0) {
        tN = e;
        tD = c;
        dc = 2;
    } else if (sN >= D) {
        tN = G_ADD(e, b);
        tD = c;
        dc = 5;
    } else {
        tN = fma(a, e, -G_MUL(b, d));
        if (tN > 0.0 && tN < tD) {
            const d3 uxv = cross(u, v);
            if (dot(uxv, w) == 0.0 || n2(uxv) < G_MUL(G_MUL(1.0e-20, a), c)) {
                if (sN < G_DIV(D, 2.0)) {
                    tN = e;
                    tD = c;
                    dc = 2;
                } else {
                    tN = G_ADD(e, b);
                    tD = c;
                    dc = 5;
                }
            }
        }
    }
    if (tN <= 0.0) {
        if (-d <= 0.0) return 0;
        if (-d >= a) return 3;
        return 6;
    } else if (tN >= tD) {
        if (G_ADD(-d, b) <= 0.0) return 1;
        if (G_ADD(-d, b) >= a) return 4;
        return 7;
    }
    return dc;
}

CIPC_HD double pp_d2(d3 a, d3 b) { return n2(a - b); }
CIPC_HD double pe_d2(d3 p, d3 e0, d3 e1) { return G_DIV(n2(cross(e0 - p, e1 - p)), n2(e1 - e0)); }

// DISTANCE_TYPE.h:11-27, point-edge: 0 point-e0, 1 point-e1, 2 interior
CIPC_HD int pe_type(d3 p, d3 e0, d3 e1)
{
    const d3 e = e1 - e0;
    const double ratio = G_DIV(dot(e, p - e0), n2(e));
    return ratio < 0 ? 0 : (ratio > 1 ? 1 : 2);
}
CIPC_HD double pt_d2(d3 p, d3 t0, d3 t1, d3 t2)
{
    const d3 b = cross(t1 - t0, t2 - t0);
    const double aTb = dot(p - t0, b);
    return G_DIV(G_MUL(aTb, aTb), n2(b));
}
CIPC_HD double ee_d2(d3 ea0, d3 ea1, d3 eb0, d3 eb1)
{
    const d3 b = cross(ea1 - ea0, eb1 - eb0);
    const double aTb = dot(eb0 - ea0, b);
    return G_DIV(G_MUL(aTb, aTb), n2(b));
}
CIPC_HD double ee_cross_n2(d3 ea0, d3 ea1, d3 eb0, d3 eb1)
{
    return n2(cross(ea1 - ea0, eb1 - eb0));
}

CIPC_HD double pt_d2_any(d3 p, d3 t0, d3 t1, d3 t2)
{
    switch (pt_type(p, t0, t1, t2)) {
        case 0: return pp_d2(p, t0);
        case 1: return pp_d2(p, t1);
        case 2: return pp_d2(p, t2);
        case 3: return pe_d2(p, t0, t1);
        case 4: return pe_d2(p, t1, t2);
        case 5: return pe_d2(p, t2, t0);
        default: return pt_d2(p, t0, t1, t2);
    }
}

CIPC_HD double ee_d2_any(d3 ea0, d3 ea1, d3 eb0, d3 eb1)
{
    switch (ee_type(ea0, ea1, eb0, eb1)) {
        case 0: return pp_d2(ea0, eb0);
        case 1: return pp_d2(ea0, eb1);
        case 2: return pe_d2(ea0, eb0, eb1);
        case 3: return pp_d2(ea1, eb0);
        case 4: return pp_d2(ea1, eb1);
        case 5: return pe_d2(ea1, eb0, eb1);
        case 6: return pe_d2(eb0, ea0, ea1);
        case 7: return pe_d2(eb1, ea0, ea1);
        default: return ee_d2(ea0, ea1, eb0, eb1);
    }
}

// projection form used by the unclassified point-edge CCD distance
CIPC_HD double pe_d2_any(d3 p, d3 e0, d3 e1)
{
    const d3 v = e1 - e0, w = p - e0;
    const double c1 = dot(w, v);
    if (c1 <= 0.0) return pp_d2(p, e0);
    const double c2 = dot(v, v);
    if (c2 <= c1) return pp_d2(p, e1);
    return pp_d2(p, axpy(G_DIV(c1, c2), v, e0));
}

// Pair types used throughout: PP=0, PE=1, PT=2, EE=3 (vertex counts 2,3,4,4).
enum PairType : int { kPP = 0, kPE = 1, kPT = 2, kEE = 3 };

}  // namespace cipc
