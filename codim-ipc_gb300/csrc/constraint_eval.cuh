// Barrier energy, FP64 gradient and PSD-projected Hessian of one contact
// constraint of the time step (IPC.h Compute_Barrier / _Gradient / _Hessian,
// :742-1731), for every constraint kind of the reference's encoding:
//   PP, PE, PT, EE                  b(s) times the PP/PE multiplicity
//   EEM, PEM, PPM (mollified)       e(x) b(s), e the edge-edge mollifier over the
//                                   two edges, the distance over a subset of them
// All kinds are written in the reduced (translation-free) variables of their
// vertex set: PP d = p0 - p1; PE (a, b) = (e0 - p, e1 - p); PT/EE/mollified
// (a, e1, e2) as in derivs.cuh, with the mollified point-edge distance taken as
// the PE function of (a, a + e2) and the mollified point-point distance |a|^2.
#pragma once
#include "derivs.cuh"

namespace cipc {

enum : int { kc_PP = 0, kc_PE = 1, kc_PT = 2, kc_EE = 3, kc_EEM = 4, kc_PEM = 5, kc_PPM = 6 };

CIPC_HD int con_nv(int k) { return k == kc_PP ? 2 : (k == kc_PE ? 3 : 4); }

// classified squared distance of a constraint (FP64, same formulas as the
// constraint-set test)
CIPC_HD double con_d2(int k, const d3 (&v)[4])
{
    switch (k) {
        case kc_PP: return pp_d2(v[0], v[1]);
        case kc_PE: return pe_d2(v[0], v[1], v[2]);
        case kc_PT: return pt_d2(v[0], v[1], v[2], v[3]);
        case kc_EE:
        case kc_EEM: return ee_d2(v[0], v[1], v[2], v[3]);
        case kc_PEM: return pe_d2(v[0], v[2], v[3]);
        default: return pp_d2(v[0], v[2]);
    }
}

// incidence of the reduced variables per kind
CIPC_HD int con_inc(int k, int r, int v)
{
    if (k == kc_PP) return v == 0 ? 1 : (v == 1 ? -1 : 0);
    if (k == kc_PE) return (v == 0) ? -1 : ((v == r + 1) ? 1 : 0);
    if (k == kc_PT) {  // a = p - t0, e1 = t1 - t0, e2 = t2 - t0
        if (r == 0) return v == 0 ? 1 : (v == 1 ? -1 : 0);
        if (r == 1) return v == 2 ? 1 : (v == 1 ? -1 : 0);
        return v == 3 ? 1 : (v == 1 ? -1 : 0);
    }
    // EE family: a = v2 - v0, e1 = v1 - v0, e2 = v3 - v2
    if (r == 0) return v == 2 ? 1 : (v == 0 ? -1 : 0);
    if (r == 1) return v == 1 ? 1 : (v == 0 ? -1 : 0);
    return v == 3 ? 1 : (v == 2 ? -1 : 0);
}

template <typename HT, int NV>
struct ConOut {
    double E;
    double g[3 * NV];
    HT H[3 * NV][3 * NV];
};

// Evaluates constraint kind K with vertices v (positions) and rest positions vr
// (mollified kinds).  s = d^2 - xi^2 must be > 0 (checked by the caller).
template <typename HT, int K>
CIPC_HD void con_eval(const d3 (&v)[4], const d3 (&vr)[4], double s, double shat, double kappa, double mult,
                      bool want_h, ConOut<HT, (K == kc_PP ? 2 : (K == kc_PE ? 3 : 4))>& o)
{
    constexpr int NV = (K == kc_PP ? 2 : (K == kc_PE ? 3 : 4));
    constexpr int NR = NV - 1;
    constexpr int M3 = 3 * NR;
    constexpr bool MOLL = (K >= kc_EEM);
    double bv, bg, bh;
    barrier3(s, shat, kappa, bv, bg, bh);
    d3 rv[3];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        d3 acc = mk(0, 0, 0);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const int c = con_inc(K, r, q);
            if (c == 1) acc = acc + v[q];
            if (c == -1) acc = acc - v[q];
        }
        rv[r] = acc;
    }
    // ---- FP64 gradient of d^2 in reduced variables (+ FP64 intermediates for HT)
    double gd[M3];
#pragma unroll
    for (int k = 0; k < M3; ++k) gd[k] = 0;
    d3 nref = mk(0, 0, 0);
    double rref = 0;
    if constexpr (K == kc_PP) {
        gd[0] = 2 * rv[0].x; gd[1] = 2 * rv[0].y; gd[2] = 2 * rv[0].z;
    } else if constexpr (K == kc_PE) {
        double g6[6];
        pe_grad(rv[0], rv[1], g6);
#pragma unroll
        for (int k = 0; k < 6; ++k) gd[k] = g6[k];
        nref = cross(rv[0], rv[1]);
        const d3 ba = rv[1] - rv[0];
        rref = dot(nref, nref) / dot(ba, ba);
    } else if constexpr (K == kc_PT || K == kc_EE || K == kc_EEM) {
        double g9[9];
        u2w_grad(rv[0], rv[1], rv[2], g9);
#pragma unroll
        for (int k = 0; k < 9; ++k) gd[k] = g9[k];
        nref = cross(rv[1], rv[2]);
        rref = dot(rv[0], nref) / dot(nref, nref);
    } else if constexpr (K == kc_PEM) {
        // PE over (a', b') = (a, a + e2)
        const d3 bp = rv[0] + rv[2];
        double g6[6];
        pe_grad(rv[0], bp, g6);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            gd[c] = g6[c] + g6[3 + c];
            gd[6 + c] = g6[3 + c];
        }
        nref = cross(rv[0], bp);
        const d3 ba = bp - rv[0];
        rref = dot(nref, nref) / dot(ba, ba);
    } else {  // PPM: |a|^2
        gd[0] = 2 * rv[0].x; gd[1] = 2 * rv[0].y; gd[2] = 2 * rv[0].z;
    }
    // ---- mollifier (reduced e1, e2 = variables 1, 2)
    double e = 1.0, qg = 0.0, qH = 0.0;
    double ge[M3];
#pragma unroll
    for (int k = 0; k < M3; ++k) ge[k] = 0;
    d3 ncr = mk(0, 0, 0);
    if constexpr (MOLL) {
        const double eps_x = 1.0e-3 * n2(vr[0] - vr[1]) * n2(vr[2] - vr[3]);
        ncr = cross(rv[1], rv[2]);
        const double c = n2(ncr);
        if (c < eps_x) {
            const double rr = c / eps_x;
            e = (-rr + 2.0) * rr;
            const double one = 1.0 / eps_x;
            qg = 2.0 * one * (-one * c + 1.0);
            qH = -2.0 / (eps_x * eps_x);
            const d3 g1 = cross(rv[2], ncr), g2 = cross(ncr, rv[1]);
            ge[3] = qg * 2 * g1.x; ge[4] = qg * 2 * g1.y; ge[5] = qg * 2 * g1.z;
            ge[6] = qg * 2 * g2.x; ge[7] = qg * 2 * g2.y; ge[8] = qg * 2 * g2.z;
        }
    }
    o.E = mult * e * bv;
    double gr[M3];
#pragma unroll
    for (int k = 0; k < M3; ++k) gr[k] = mult * (e * bg * gd[k] + bv * ge[k]);
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double acc = 0;
#pragma unroll
            for (int r = 0; r < NR; ++r) acc += con_inc(K, r, q) * gr[3 * r + c];
            o.g[3 * q + c] = acc;
        }
    if (!want_h) return;
    // ---- reduced Hessian in HT
    HT H[M3][M3];
#pragma unroll
    for (int p = 0; p < M3; ++p)
#pragma unroll
        for (int q = 0; q < M3; ++q) H[p][q] = 0;
    if constexpr (K == kc_PP || K == kc_PPM) {
#pragma unroll
        for (int p = 0; p < 3; ++p) H[p][p] = HT(2);
    } else if constexpr (K == kc_PE) {
        HT g6[6];
        pe_derivs<HT>(tv<HT>(rv[0]), tv<HT>(rv[1]), tv<HT>(nref), (HT)rref, g6, H);
    } else if constexpr (K == kc_PEM) {
        HT g6[6], Hp[6][6];
        pe_derivs<HT>(tv<HT>(rv[0]), tv<HT>(rv[0] + rv[2]), tv<HT>(nref), (HT)rref, g6, Hp);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const HT aa = Hp[i][j], ab = Hp[i][3 + j], ba = Hp[3 + i][j], bb = Hp[3 + i][3 + j];
                H[i][j] = aa + ab + ba + bb;
                H[i][6 + j] = ab + bb;
                H[6 + i][j] = ba + bb;
                H[6 + i][6 + j] = bb;
            }
    } else {
        HT g9[9];
        u2w_derivs<HT>(tv<HT>(rv[0]), tv<HT>(rv[1]), tv<HT>(rv[2]), tv<HT>(nref), (HT)rref, g9, H);
    }
    {
        const HT cb = (HT)(mult * e * bg), ch = (HT)(mult * e * bh);
        HT gdh[M3];
#pragma unroll
        for (int k = 0; k < M3; ++k) gdh[k] = (HT)gd[k];
#pragma unroll
        for (int p = 0; p < M3; ++p)
#pragma unroll
            for (int q = 0; q < M3; ++q) H[p][q] = cb * H[p][q] + ch * gdh[p] * gdh[q];
        if constexpr (MOLL) {
            if (qg != 0.0) {
                HT gc[9], Hc[9][9];
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    gc[k] = 0;
#pragma unroll
                    for (int l = 0; l < 9; ++l) Hc[k][l] = 0;
                }
                crossn2_add<HT, 9>(tv<HT>(rv[1]), tv<HT>(rv[2]), tv<HT>(ncr), 1, 2, HT(1), gc, Hc);
                const HT hbgqg = (HT)(bg * qg), hbqg = (HT)(bv * qg), hbqH = (HT)(bv * qH);
#pragma unroll
                for (int p = 0; p < 9; ++p)
#pragma unroll
                    for (int q = 0; q < 9; ++q)
                        H[p][q] += hbgqg * (gdh[p] * gc[q] + gc[p] * gdh[q]) + hbqg * Hc[p][q] + hbqH * gc[p] * gc[q];
            }
        }
    }
    // ---- to the translation-free basis (M = C Q^T), PSD projection, back to vertices
    HT Kt[M3][M3];
    {
        double Mm[NR][NR];
#pragma unroll
        for (int r = 0; r < NR; ++r)
#pragma unroll
            for (int q = 0; q < NR; ++q) {
                double acc = 0;
#pragma unroll
                for (int w = 0; w < NV; ++w) {
                    const double hq = (NV == 2) ? (w == 0 ? 0.70710678118654752440 : -0.70710678118654752440)
                                                : (q == 0 ? (w == 0 ? 0.70710678118654752440 : (w == 1 ? -0.70710678118654752440 : 0.0))
                                                          : (q == 1 ? (w < 2 ? 0.40824829046386301637 : (w == 2 ? -0.81649658092772603273 : 0.0))
                                                                    : (w < 3 ? 0.28867513459481288225 : -0.86602540378443864676)));
                    acc += con_inc(K, r, w) * hq;
                }
                Mm[r][q] = acc;
            }
#pragma unroll
        for (int bi = 0; bi < NR; ++bi)
#pragma unroll
            for (int bj = 0; bj < NR; ++bj)
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int c2 = 0; c2 < 3; ++c2) {
                        HT acc = 0;
#pragma unroll
                        for (int r = 0; r < NR; ++r)
#pragma unroll
                            for (int r2 = 0; r2 < NR; ++r2)
                                if (Mm[r][bi] != 0.0 && Mm[r2][bj] != 0.0)
                                    acc += (HT)(Mm[r][bi] * Mm[r2][bj]) * H[3 * r + c][3 * r2 + c2];
                        Kt[3 * bi + c][3 * bj + c2] = acc;
                    }
    }
    jacobi_psd<HT, M3>(Kt);
#pragma unroll
    for (int p = 0; p < 3 * NV; ++p)
#pragma unroll
        for (int q = p; q < 3 * NV; ++q) {
            const int va = p / 3, c = p % 3, vb = q / 3, c2 = q % 3;
            HT acc = 0;
#pragma unroll
            for (int bi = 0; bi < NR; ++bi)
#pragma unroll
                for (int bj = 0; bj < NR; ++bj) {
                    const double qa = (NV == 2) ? (va == 0 ? 0.70710678118654752440 : -0.70710678118654752440)
                                                : (bi == 0 ? (va == 0 ? 0.70710678118654752440 : (va == 1 ? -0.70710678118654752440 : 0.0))
                                                           : (bi == 1 ? (va < 2 ? 0.40824829046386301637 : (va == 2 ? -0.81649658092772603273 : 0.0))
                                                                      : (va < 3 ? 0.28867513459481288225 : -0.86602540378443864676)));
                    const double qb = (NV == 2) ? (vb == 0 ? 0.70710678118654752440 : -0.70710678118654752440)
                                                : (bj == 0 ? (vb == 0 ? 0.70710678118654752440 : (vb == 1 ? -0.70710678118654752440 : 0.0))
                                                           : (bj == 1 ? (vb < 2 ? 0.40824829046386301637 : (vb == 2 ? -0.81649658092772603273 : 0.0))
                                                                      : (vb < 3 ? 0.28867513459481288225 : -0.86602540378443864676)));
                    acc += (HT)(qa * qb) * Kt[3 * bi + c][3 * bj + c2];
                }
            o.H[p][q] = acc;
            o.H[q][p] = acc;
        }
}

}  // namespace cipc
