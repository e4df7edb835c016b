// Per-pair barrier evaluation shared by the CUDA kernel and host-side checks.
// See barrier.cu for the formulas and the precision split.
#pragma once
#include "derivs.cuh"

namespace cipc {

// Helmert bases of the translation complement (rows orthonormal, orthogonal to 1)
CIPC_HD double Qb(int nv, int i, int v)
{
    constexpr double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637,
                     r12 = 0.28867513459481288225;
    if (nv == 2) return v == 0 ? r2 : -r2;
    if (i == 0) return v == 0 ? r2 : (v == 1 ? -r2 : 0.0);
    if (i == 1) return v < 2 ? r6 : (v == 2 ? -2 * r6 : 0.0);
    return v < 3 ? r12 : -3 * r12;
}

// incidence matrices: reduced variable r = sum_v C[r][v] x_v
CIPC_HD int Cinc(int tp, int r, int v)
{
    // PP: d = p0 - p1
    // PE: a = e0 - p, b = e1 - p
    // PT: a = p - t0, e1 = t1 - t0, e2 = t2 - t0
    // EE: a = eb0 - ea0, e1 = ea1 - ea0, e2 = eb1 - eb0
    constexpr int pp[1][4] = {{1, -1, 0, 0}};
    constexpr int pe[2][4] = {{-1, 1, 0, 0}, {-1, 0, 1, 0}};
    constexpr int pt[3][4] = {{1, -1, 0, 0}, {0, -1, 1, 0}, {0, -1, 0, 1}};
    constexpr int ee[3][4] = {{-1, 0, 1, 0}, {-1, 1, 0, 0}, {0, 0, -1, 1}};
    switch (tp) {
        case kPP: return pp[0][v];
        case kPE: return pe[r][v];
        case kPT: return pt[r][v];
        default: return ee[r][v];
    }
}

struct BarrierArgs {
    int64_t n;
    const uint8_t* type;
    const int4* idx;
    const double* x;
    const double* x_rest;
    double xi2, shat, kappa;
    int project;
    int64_t nv;
    double* E;
    double* grad;   // [n][12]
    void* hess;     // [n][78] of HT
    unsigned long long* bad;  // [0] s <= 0, [1] invalid pairs
};

template <typename HT, int TP>
CIPC_HD void pair_body(const BarrierArgs& a, int64_t i, const d3 (&xv)[4], double bv, double bg,
                                          double bh, double* __restrict__ gout, HT* __restrict__ hout)
{
    constexpr int NV = TP == kPP ? 2 : (TP == kPE ? 3 : 4);
    constexpr int NR = NV - 1;
    constexpr int M3 = 3 * NR;
    constexpr int MX = 3 * NV;
    // reduced variables (FP64 differences)
    d3 rv[3];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        d3 s = mk(0, 0, 0);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const int c = Cinc(TP, r, v);
            if (c == 1) s = s + xv[v];
            if (c == -1) s = s - xv[v];
        }
        rv[r] = s;
    }
    // ---- FP64 gradient of d^2 in reduced variables, and the cancellation-prone
    // intermediates the HT Hessian needs (n, u/w or f), also in FP64
    double gd[M3];
    d3 nref = mk(0, 0, 0);
    double rref = 0;
    if constexpr (TP == kPP) {
        gd[0] = 2 * rv[0].x;
        gd[1] = 2 * rv[0].y;
        gd[2] = 2 * rv[0].z;
    } else if constexpr (TP == kPE) {
        double g6[6];
        pe_grad(rv[0], rv[1], g6);
#pragma unroll
        for (int k = 0; k < 6; ++k) gd[k] = g6[k];
        nref = cross(rv[0], rv[1]);
        const d3 ba = rv[1] - rv[0];
        rref = dot(nref, nref) / dot(ba, ba);
    } else {
        double g9[9];
        u2w_grad(rv[0], rv[1], rv[2], g9);
#pragma unroll
        for (int k = 0; k < 9; ++k) gd[k] = g9[k];
        nref = cross(rv[1], rv[2]);
        rref = dot(rv[0], nref) / dot(nref, nref);
    }
    // ---- mollifier (EE only)
    bool moll = false;
    double e = 1.0, qg = 0.0, qH = 0.0;
    if constexpr (TP == kEE) {
        const int4 id = a.idx[i];
        const d3 r0 = ld(a.x_rest, id.x), r1 = ld(a.x_rest, id.y), r2 = ld(a.x_rest, id.z), r3 = ld(a.x_rest, id.w);
        const double eps_x = 1.0e-3 * n2(r0 - r1) * n2(r2 - r3);
        const double c = ee_cross_n2(xv[0], xv[1], xv[2], xv[3]);
        if (c < eps_x) {
            moll = true;
            const double rr = c / eps_x;
            e = (-rr + 2.0) * rr;
            const double one = 1.0 / eps_x;
            qg = 2.0 * one * (-one * c + 1.0);
            qH = -2.0 / (eps_x * eps_x);
        }
    }
    // gradient of the mollifier (FP64), reduced (e1, e2) blocks = variables 1,2
    double ge[M3];
#pragma unroll
    for (int k = 0; k < M3; ++k) ge[k] = 0;
    if constexpr (TP == kEE) {
        if (moll) {
            const d3 n = cross(rv[1], rv[2]);
            const d3 g1 = cross(rv[2], n), g2 = cross(n, rv[1]);
            ge[3] = qg * 2 * g1.x;
            ge[4] = qg * 2 * g1.y;
            ge[5] = qg * 2 * g1.z;
            ge[6] = qg * 2 * g2.x;
            ge[7] = qg * 2 * g2.y;
            ge[8] = qg * 2 * g2.z;
        }
    }
    // energy and vertex gradient
    double gr[M3];
#pragma unroll
    for (int k = 0; k < M3; ++k) gr[k] = moll ? (e * bg * gd[k] + bv * ge[k]) : bg * gd[k];
    a.E[i] = moll ? e * bv : bv;
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double s = 0;
#pragma unroll
            for (int r = 0; r < NR; ++r) s += Cinc(TP, r, v) * gr[3 * r + c];
            gout[3 * v + c] = s;
        }
    // ---- Hessian in HT, reduced variables
    HT H[M3][M3];
    {
        HT gdh[M3];
#pragma unroll
        for (int k = 0; k < M3; ++k) gdh[k] = (HT)gd[k];
        if constexpr (TP == kPP) {
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int q = 0; q < 3; ++q) H[p][q] = (p == q) ? HT(2) : HT(0);
        } else if constexpr (TP == kPE) {
            HT g6[6];
            pe_derivs<HT>(tv<HT>(rv[0]), tv<HT>(rv[1]), tv<HT>(nref), (HT)rref, g6, H);
        } else {
            HT g9[9];
            u2w_derivs<HT>(tv<HT>(rv[0]), tv<HT>(rv[1]), tv<HT>(rv[2]), tv<HT>(nref), (HT)rref, g9, H);
        }
        const HT cb = (HT)((moll ? e : 1.0) * bg), ch = (HT)((moll ? e : 1.0) * bh);
#pragma unroll
        for (int p = 0; p < M3; ++p)
#pragma unroll
            for (int q = 0; q < M3; ++q) H[p][q] = cb * H[p][q] + ch * gdh[p] * gdh[q];
        if constexpr (TP == kEE) {
            if (moll) {
                // + bg (gd ge^T + ge gd^T) + b (qg hess c + qH grad c grad c^T)
                HT gc[9], Hc[9][9];
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    gc[k] = 0;
#pragma unroll
                    for (int l = 0; l < 9; ++l) Hc[k][l] = 0;
                }
                crossn2_add<HT, 9>(tv<HT>(rv[1]), tv<HT>(rv[2]), tv<HT>(nref), 1, 2, HT(1), gc, Hc);
                const HT hbg = (HT)bg, hqg = (HT)qg, hb = (HT)bv, hbqg = (HT)(bv * qg), hbqH = (HT)(bv * qH);
#pragma unroll
                for (int p = 0; p < 9; ++p)
#pragma unroll
                    for (int q = 0; q < 9; ++q)
                        H[p][q] += hbg * hqg * (gdh[p] * gc[q] + gc[p] * gdh[q]) + hbqg * Hc[p][q] +
                                   hbqH * gc[p] * gc[q];
                (void)hb;
            }
        }
    }
    // ---- K = M^T H M with M = C Q^T (constant), PSD projection, back to vertices
    HT K[M3][M3];
    {
        HT Mm[NR][NR];
#pragma unroll
        for (int r = 0; r < NR; ++r)
#pragma unroll
            for (int q = 0; q < NR; ++q) {
                double s = 0;
#pragma unroll
                for (int v = 0; v < NV; ++v) s += Cinc(TP, r, v) * Qb(NV, q, v);
                Mm[r][q] = (HT)s;
            }
#pragma unroll
        for (int bi = 0; bi < NR; ++bi)
#pragma unroll
            for (int bj = 0; bj < NR; ++bj)
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int c2 = 0; c2 < 3; ++c2) {
                        HT s = 0;
#pragma unroll
                        for (int r = 0; r < NR; ++r)
#pragma unroll
                            for (int r2 = 0; r2 < NR; ++r2)
                                if (Mm[r][bi] != HT(0) && Mm[r2][bj] != HT(0))
                                    s += Mm[r][bi] * Mm[r2][bj] * H[3 * r + c][3 * r2 + c2];
                        K[3 * bi + c][3 * bj + c2] = s;
                    }
    }
    if (a.project) jacobi_psd<HT, M3>(K);
    int o = 0;
#pragma unroll
    for (int p = 0; p < MX; ++p)
#pragma unroll
        for (int q = p; q < MX; ++q) {
            const int v = p / 3, c = p % 3, v2 = q / 3, c2 = q % 3;
            HT s = 0;
#pragma unroll
            for (int bi = 0; bi < NR; ++bi)
#pragma unroll
                for (int bj = 0; bj < NR; ++bj)
                    s += (HT)(Qb(NV, bi, v) * Qb(NV, bj, v2)) * K[3 * bi + c][3 * bj + c2];
            hout[o++] = s;
        }
}


// Evaluates pair i: returns 0 (evaluated or inactive), 1 (s <= 0: reported, zero
// outputs), 2 (bad type or index: reported, never dereferenced).
template <typename HT>
CIPC_HD int barrier_one(const BarrierArgs& a, int64_t i)
{
    const int tp = a.type[i];
    const int4 id = a.idx[i];
    const int nv = tp == kPP ? 2 : (tp == kPE ? 3 : 4);
    double* gout = a.grad + 12 * i;
    HT* hout = reinterpret_cast<HT*>(a.hess) + 78 * i;
    bool ok = tp <= kEE && id.x >= 0 && id.x < a.nv && id.y >= 0 && id.y < a.nv;
    if (nv > 2) ok = ok && id.z >= 0 && id.z < a.nv;
    if (nv > 3) ok = ok && id.w >= 0 && id.w < a.nv;
    if (!ok) {
        a.E[i] = 0;
        for (int k = 0; k < 12; ++k) gout[k] = 0;
        for (int k = 0; k < 78; ++k) hout[k] = 0;
        return 2;
    }
    d3 xv[4];
    xv[0] = ld(a.x, id.x);
    xv[1] = ld(a.x, id.y);
    xv[2] = nv > 2 ? ld(a.x, id.z) : mk(0, 0, 0);
    xv[3] = nv > 3 ? ld(a.x, id.w) : mk(0, 0, 0);
    double d2;
    switch (tp) {
        case kPP: d2 = pp_d2(xv[0], xv[1]); break;
        case kPE: d2 = pe_d2(xv[0], xv[1], xv[2]); break;
        case kPT: d2 = pt_d2(xv[0], xv[1], xv[2], xv[3]); break;
        default: d2 = ee_d2(xv[0], xv[1], xv[2], xv[3]); break;
    }
    const double s = d2 - a.xi2;
    if (!(s > 0) || s >= a.shat) {
        a.E[i] = 0;
        for (int k = 0; k < 12; ++k) gout[k] = 0;
        for (int k = 0; k < 78; ++k) hout[k] = 0;
        return (s > 0) ? 0 : 1;
    }
    double bv, bg, bh;
    barrier3(s, a.shat, a.kappa, bv, bg, bh);
    for (int k = 3 * nv; k < 12; ++k) gout[k] = 0;
    for (int k = 3 * nv * (3 * nv + 1) / 2; k < 78; ++k) hout[k] = 0;  // unused tail of PP / PE records
    switch (tp) {
        case kPP: pair_body<HT, kPP>(a, i, xv, bv, bg, bh, gout, hout); break;
        case kPE: pair_body<HT, kPE>(a, i, xv, bv, bg, bh, gout, hout); break;
        case kPT: pair_body<HT, kPT>(a, i, xv, bv, bg, bh, gout, hout); break;
        default: pair_body<HT, kEE>(a, i, xv, bv, bg, bh, gout, hout); break;
    }
    return 0;
}

}  // namespace cipc
