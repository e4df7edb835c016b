// Certified FP32 evaluation of the FP64 distance-type decisions.
//
// The distance-type classifications pt_type / ee_type (geom.cuh, restating
// DISTANCE_TYPE.h:30-164) return only a branch: which of the 7 / 9 regions the
// closest points lie in.  On this part the FP64 pipe issues 2 operations per SM
// per clock against 128 for FP32, and the classification is most of the FP64
// work of an ACCD step (point-triangle: three 2x2 LDL^T solves, ~200 FP64
// operations and 9 divisions).  Here the same operation sequence runs in FP32
// midpoint-radius arithmetic whose every interval encloses the value the FP64
// sequence computes (not the exact real value: each FP64 rounding is part of the
// enclosure).  A comparison is decided when the enclosure lies entirely on one
// side of its threshold; otherwise the classification is "uncertain" (-1) and the
// caller runs the FP64 classifier.  A decided type is therefore the type the FP64
// code returns, bit for bit, and the distances are then computed in FP64 as before.
//
// Enclosure rules (a = [ma +- ra], b = [mb +- rb] enclose FP64 values a64, b64;
// u32 = 2^-24, u64 = 2^-53):
//   add:  m = RN32(ma + mb), r >= ra + rb + 2^-23 (|ma| + |mb|)
//   mul:  m = RN32(ma mb),   r >= |ma| rb + |mb| ra + ra rb + 2^-23 |m|
//   fma:  m = RN32(ma mb + mc) (one rounding), r >= |ma| rb + |mb| ra + ra rb + rc
//                                                   + 2^-23 (|ma mb| + |mc|)
//   div:  m = RN32(ma / mb), r >= (|ma| rb + |mb| ra) / (|mb| (|mb| - rb)) + 2^-23 |m|
// The 2^-23 term covers the FP32 rounding of the midpoint (<= 2^-24 of the
// magnitudes) and the FP64 rounding of the value itself (<= 2^-53 of them, plus
// 2^-53 of the propagated radius, covered by the factor below).  Each radius is
// computed with round-to-nearest FP32 operations (at most 7 per rule, each low by
// at most 2^-24 relative), so it is multiplied by kInflate = 1 + 2^-20, and kTiny =
// 2^-120 is added to absorb underflow (FP32 gradual underflow loses at most 2^-149
// per operation; FP64 underflow in the unscaled problem maps to far less, below).
//
// Scaling.  Inputs are FP64 coordinate differences of one pair.  They are scaled
// by 2^-E (E = the largest binary exponent among them) while being converted, so
// the FP32 values stay in [2^-126, 1) or round to zero.  Every decision quantity
// is a homogeneous polynomial (or ratio) of the differences, and an FP64 operation
// on values scaled by a power of two gives the scaled result exactly, so the
// scaled FP64 sequence takes the same branches as the unscaled one; underflow
// and overflow of the unscaled FP64 sequence are excluded by requiring |E| <= 60
// (degree <= 6: magnitudes stay within 2^+-400 of the scaled ones) and by
// deciding "nonzero" only when a value exceeds twice its radius (>= 2^-120).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "geom.cuh"

namespace cipc {

#ifdef __CUDA_ARCH__
#define CF_ADD(a, b) __fadd_rn((a), (b))
#define CF_SUB(a, b) __fsub_rn((a), (b))
#define CF_MUL(a, b) __fmul_rn((a), (b))
#define CF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define CF_DIV(a, b) __fdiv_rn((a), (b))
#else
// host build (tests): every operation rounded once to FP32
inline float cf_add(float a, float b) { volatile float r = a + b; return r; }
inline float cf_sub(float a, float b) { volatile float r = a - b; return r; }
inline float cf_mul(float a, float b) { volatile float r = a * b; return r; }
inline float cf_div(float a, float b) { volatile float r = a / b; return r; }
#define CF_ADD(a, b) cf_add((a), (b))
#define CF_SUB(a, b) cf_sub((a), (b))
#define CF_MUL(a, b) cf_mul((a), (b))
#define CF_FMA(a, b, c) std::fmaf((a), (b), (c))
#define CF_DIV(a, b) cf_div((a), (b))
#endif

constexpr float kCertU = 0x1p-23f;         // per-operation rounding allowance
constexpr float kInflate = 1.0f + 0x1p-20f;  // rounding of the radius computation
constexpr float kTiny = 0x1p-120f;          // underflow allowance
constexpr float kShrink = 1.0f - 0x1p-22f;  // for decisions: margin of the difference

// |v - m| <= r for the FP64 value v it stands for
struct iv {
    float m, r;
};
struct iv3 {
    iv x, y, z;
};

CIPC_HD iv iv_exact(float m) { return iv{m, 0.0f}; }
CIPC_HD iv iv_neg(iv a) { return iv{-a.m, a.r}; }
CIPC_HD float cert_fin(float r) { return CF_FMA(r, kInflate, kTiny); }

CIPC_HD iv iv_add(iv a, iv b)
{
    const float m = CF_ADD(a.m, b.m);
    const float r = CF_FMA(kCertU, CF_ADD(fabsf(a.m), fabsf(b.m)), CF_ADD(a.r, b.r));
    return iv{m, cert_fin(r)};
}
CIPC_HD iv iv_sub(iv a, iv b) { return iv_add(a, iv_neg(b)); }
CIPC_HD iv iv_mul(iv a, iv b)
{
    const float m = CF_MUL(a.m, b.m);
    const float am = fabsf(a.m), bm = fabsf(b.m);
    float r = CF_FMA(am, b.r, CF_FMA(bm, a.r, CF_MUL(a.r, b.r)));
    r = CF_FMA(kCertU, fabsf(m), r);
    return iv{m, cert_fin(r)};
}
// FP64 fma(a, b, c) = RN(a b + c)
CIPC_HD iv iv_fma(iv a, iv b, iv c)
{
    const float m = CF_FMA(a.m, b.m, c.m);
    const float am = fabsf(a.m), bm = fabsf(b.m);
    float r = CF_FMA(am, b.r, CF_FMA(bm, a.r, CF_FMA(a.r, b.r, c.r)));
    r = CF_FMA(kCertU, CF_ADD(CF_MUL(am, bm), fabsf(c.m)), r);
    return iv{m, cert_fin(r)};
}
// FP64 a / b; false when b's enclosure reaches zero
CIPC_HD bool iv_div(iv a, iv b, iv& out)
{
    const float bm = fabsf(b.m);
    const float den = CF_MUL(CF_SUB(bm, b.r), kShrink);  // lower bound of |b|
    if (!(den > 0.0f)) return false;
    const float m = CF_DIV(a.m, b.m);
    const float num = CF_FMA(fabsf(a.m), b.r, CF_MUL(bm, a.r));
    float r = CF_DIV(num, CF_MUL(bm, den));
    r = CF_FMA(kCertU, fabsf(m), r);
    out = iv{m, cert_fin(r)};
    return true;
}
// exact multiplication by a power of two (the radius keeps its underflow allowance)
CIPC_HD iv iv_scale2(iv a, float p2) { return iv{CF_MUL(a.m, p2), CF_FMA(a.r, p2, kTiny)}; }

// +1: v > c for every v in the enclosure; -1: v < c for every v; 0: undecided.
// c must be exactly representable in FP32 and FP64 (0, 1).
CIPC_HD int iv_cmp(iv a, float c)
{
    const float d = CF_SUB(a.m, c);
    if (CF_MUL(d, kShrink) > a.r) return 1;
    if (CF_MUL(-d, kShrink) > a.r) return -1;
    return 0;
}
// sign of a - b (FP64 comparison a > b / a < b; the difference is not an FP64 operation)
CIPC_HD int iv_cmp2(iv a, iv b) { return iv_cmp(iv_sub(a, b), 0.0f); }
// the FP64 value is certainly nonzero and at least 2^-120 in magnitude
CIPC_HD bool iv_big(iv a) { return CF_MUL(fabsf(a.m), kShrink) > CF_MUL(a.r, 2.0f); }

// three-valued truth: kT, kF, kU (undecided)
enum : int { kF = 0, kT = 1, kUnd = 2 };
CIPC_HD int tri_and(int a, int b) { return (a == kF || b == kF) ? kF : ((a == kT && b == kT) ? kT : kUnd); }
CIPC_HD int tri_or(int a, int b) { return (a == kT || b == kT) ? kT : ((a == kF && b == kF) ? kF : kUnd); }
CIPC_HD int tri_gt(iv a, float c) { const int s = iv_cmp(a, c); return s > 0 ? kT : (s < 0 ? kF : kUnd); }  // a > c, a >= c
CIPC_HD int tri_lt(iv a, float c) { const int s = iv_cmp(a, c); return s < 0 ? kT : (s > 0 ? kF : kUnd); }  // a < c, a <= c
CIPC_HD int tri_gt2(iv a, iv b) { const int s = iv_cmp2(a, b); return s > 0 ? kT : (s < 0 ? kF : kUnd); }
CIPC_HD int tri_lt2(iv a, iv b) { const int s = iv_cmp2(a, b); return s < 0 ? kT : (s > 0 ? kF : kUnd); }

CIPC_HD iv3 iv3_sub(iv3 a, iv3 b) { return iv3{iv_sub(a.x, b.x), iv_sub(a.y, b.y), iv_sub(a.z, b.z)}; }
CIPC_HD iv3 iv3_neg(iv3 a) { return iv3{iv_neg(a.x), iv_neg(a.y), iv_neg(a.z)}; }
// dot(a,b) = fma(az,bz, fma(ax,bx, ay*by))  (the FP64 rule of geom.cuh)
CIPC_HD iv iv3_dot(iv3 a, iv3 b) { return iv_fma(a.z, b.z, iv_fma(a.x, b.x, iv_mul(a.y, b.y))); }
// cross: fma(a.y, b.z, -(a.z * b.y)), ...
CIPC_HD iv3 iv3_cross(iv3 a, iv3 b)
{
    return iv3{iv_fma(a.y, b.z, iv_neg(iv_mul(a.z, b.y))), iv_fma(a.z, b.x, iv_neg(iv_mul(a.x, b.z))),
               iv_fma(a.x, b.y, iv_neg(iv_mul(a.y, b.x)))};
}

// ---------------------------------------------------------------------------
// FP64 -> scaled FP32 enclosure by integer operations on the bit pattern
// ---------------------------------------------------------------------------
CIPC_HD uint64_t cert_bits(double d)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
#endif
}
CIPC_HD float cert_f32(uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, 4);
    return f;
#endif
}
CIPC_HD int cert_bexp(double d) { return (int)((cert_bits(d) >> 52) & 0x7ffu); }

// d * 2^-E (E given as a biased FP64 exponent shift `sh` = E) truncated to 24
// significant bits, with radius 2^-23 |m| (truncation); values that scale below
// 2^-126 become 0 with radius 2^-125.
CIPC_HD iv cert_iv_scaled(double d, int sh)
{
    const uint64_t b = cert_bits(d);
    const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
    const int e = (int)((hw >> 20) & 0x7ffu);
    const int fe = e - sh - 896;  // FP32 biased exponent of the scaled value
    if (e == 0 || fe <= 0) return iv{0.0f, 0x1p-125f};
    const uint32_t sg = hw & 0x80000000u;
    const uint32_t m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
    const float m = cert_f32(sg | ((uint32_t)fe << 23) | m23);
    return iv{m, CF_MUL(fabsf(m), 0x1p-23f)};
}

// largest biased exponent among the components; returns the shift E (unbiased
// exponent + 1, so scaled magnitudes are < 1), or a sentinel outside [-60, 60]
// when the inputs are all zero / subnormal / too far from 1
CIPC_HD int cert_shift3(const d3* v, int n)
{
    int mx = 0;
    for (int k = 0; k < n; ++k) {
        const int a = cert_bexp(v[k].x), b = cert_bexp(v[k].y), c = cert_bexp(v[k].z);
        mx = mx > a ? mx : a;
        mx = mx > b ? mx : b;
        mx = mx > c ? mx : c;
    }
    if (mx == 0) return 1000;
    return mx - 1023 + 1;
}
CIPC_HD iv3 cert_iv3(d3 v, int E) { return iv3{cert_iv_scaled(v.x, E), cert_iv_scaled(v.y, E), cert_iv_scaled(v.z, E)}; }

// ---------------------------------------------------------------------------
// Certified restatements of geom.cuh's classifiers
// ---------------------------------------------------------------------------

// ldlt2 (geom.cuh) on enclosures; false when a branch inside is undecided
CIPC_HD bool iv_ldlt2(iv a00, iv a10, iv a11, iv b0, iv b1, iv& y0, iv& y1)
{
    const int swc = tri_gt2(iv{fabsf(a11.m), a11.r}, iv{fabsf(a00.m), a00.r});  // |a11| > |a00|
    if (swc == kUnd) return false;
    const bool sw = swc == kT;
    const iv d0 = sw ? a11 : a00;
    const iv m11 = sw ? a00 : a11;
    if (sw) {
        const iv t = b0;
        b0 = b1;
        b1 = t;
    }
    if (!iv_big(d0)) return false;  // d0 == 0 (or below DBL_MIN unscaled) not decided here
    iv l10;
    if (!iv_div(a10, d0, l10)) return false;
    const iv d1 = iv_fma(iv_neg(l10), iv_mul(d0, l10), m11);
    iv z0 = b0;
    iv z1 = iv_fma(iv_neg(l10), z0, b1);
    if (!iv_div(z0, d0, z0)) return false;
    if (!iv_big(d1)) return false;
    if (!iv_div(z1, d1, z1)) return false;
    z0 = iv_fma(iv_neg(l10), z1, z0);
    if (sw) {
        y0 = z1;
        y1 = z0;
    } else {
        y0 = z0;
        y1 = z1;
    }
    return true;
}

CIPC_HD bool iv_pt_param(iv3 r0, iv3 n, iv3 v, iv& s, iv& q)
{
    const iv3 r1 = iv3_cross(r0, n);
    return iv_ldlt2(iv3_dot(r0, r0), iv3_dot(r1, r0), iv3_dot(r1, r1), iv3_dot(r0, v), iv3_dot(r1, v), s, q);
}

// pt_type from e1 = t1 - t0, e2 = t2 - t0, w = p - t0 (FP64 differences, as the
// FP64 code forms them); the other differences the FP64 code forms from absolute
// positions (t2 - t1, p - t1, p - t2) are enclosed as e2 - e1, w - e1, w - e2:
// they differ from those FP64 values by at most 2^-51 (|e1| + |e2|) (resp. with
// w), far inside the subtraction's 2^-23 allowance; t0 - t2 is exactly -e2.
// Returns the type (0..6) or -1 when a decision is not certain.
CIPC_HD int pt_type_cert(d3 w, d3 e1, d3 e2)
{
    const d3 in[3] = {w, e1, e2};
    const int E = cert_shift3(in, 3);
    if (E < -60 || E > 60) return -1;
    const iv3 W = cert_iv3(w, E), A = cert_iv3(e1, E), B = cert_iv3(e2, E);
    const iv3 n = iv3_cross(A, B);
    iv s0, q0, s1, q1, s2, q2;
    if (!iv_pt_param(A, n, W, s0, q0)) return -1;
    int c = tri_and(tri_and(tri_gt(s0, 0.0f), tri_lt(s0, 1.0f)), tri_gt(q0, 0.0f));
    if (c == kT) return 3;
    if (c == kUnd) return -1;
    if (!iv_pt_param(iv3_sub(B, A), n, iv3_sub(W, A), s1, q1)) return -1;
    c = tri_and(tri_and(tri_gt(s1, 0.0f), tri_lt(s1, 1.0f)), tri_gt(q1, 0.0f));
    if (c == kT) return 4;
    if (c == kUnd) return -1;
    if (!iv_pt_param(iv3_neg(B), n, iv3_sub(W, B), s2, q2)) return -1;
    c = tri_and(tri_and(tri_gt(s2, 0.0f), tri_lt(s2, 1.0f)), tri_gt(q2, 0.0f));
    if (c == kT) return 5;
    if (c == kUnd) return -1;
    c = tri_and(tri_lt(s0, 0.0f), tri_gt(s2, 1.0f));
    if (c == kT) return 0;
    if (c == kUnd) return -1;
    c = tri_and(tri_lt(s1, 0.0f), tri_gt(s0, 1.0f));
    if (c == kT) return 1;
    if (c == kUnd) return -1;
    c = tri_and(tri_lt(s2, 0.0f), tri_gt(s1, 1.0f));
    if (c == kT) return 2;
    if (c == kUnd) return -1;
    return 6;
}

// ee_type from u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0 (FP64 differences, the
// ones the FP64 code forms).  Returns the type (0..8) or -1.
CIPC_HD int ee_type_cert(d3 u64, d3 v64, d3 w64)
{
    const d3 in[3] = {u64, v64, w64};
    const int E = cert_shift3(in, 3);
    if (E < -60 || E > 60) return -1;
    const iv3 u = cert_iv3(u64, E), v = cert_iv3(v64, E), w = cert_iv3(w64, E);
    const iv a = iv3_dot(u, u), b = iv3_dot(u, v), c = iv3_dot(v, v), d = iv3_dot(u, w), e = iv3_dot(v, w);
    const iv D = iv_fma(a, c, iv_neg(iv_mul(b, b)));
    iv tD = D, tN = iv_exact(0.0f);
    int dc = 8;
    const iv sN = iv_fma(b, e, iv_neg(iv_mul(c, d)));
    const int s_le0 = tri_lt(sN, 0.0f);
    if (s_le0 == kUnd) return -1;
    if (s_le0 == kT) {
        tN = e;
        tD = c;
        dc = 2;
    } else {
        const int s_geD = tri_gt2(sN, D);
        if (s_geD == kUnd) return -1;
        if (s_geD == kT) {
            tN = iv_add(e, b);
            tD = c;
            dc = 5;
        } else {
            tN = iv_fma(a, e, iv_neg(iv_mul(b, d)));
            const int inner = tri_and(tri_gt(tN, 0.0f), tri_lt2(tN, tD));
            if (inner == kUnd) return -1;
            if (inner == kT) {
                const iv3 uxv = iv3_cross(u, v);
                // dot(uxv, w) == 0 is decided only as "nonzero"
                const iv dw = iv3_dot(uxv, w);
                if (!iv_big(dw)) return -1;
                const iv lim = iv_mul(iv_mul(iv{1.0e-20f, 1.0e-20f * 0x1p-22f}, a), c);
                const int par = tri_lt2(iv3_dot(uxv, uxv), lim);
                if (par == kUnd) return -1;
                if (par == kT) {
                    const int half = tri_lt2(sN, iv_mul(D, iv_exact(0.5f)));
                    if (half == kUnd) return -1;
                    if (half == kT) {
                        tN = e;
                        tD = c;
                        dc = 2;
                    } else {
                        tN = iv_add(e, b);
                        tD = c;
                        dc = 5;
                    }
                }
            }
        }
    }
    const int t_le0 = tri_lt(tN, 0.0f);
    if (t_le0 == kUnd) return -1;
    if (t_le0 == kT) {
        const iv md = iv_neg(d);
        const int c0 = tri_lt(md, 0.0f);
        if (c0 == kUnd) return -1;
        if (c0 == kT) return 0;
        const int c1 = tri_gt2(md, a);
        if (c1 == kUnd) return -1;
        return c1 == kT ? 3 : 6;
    }
    const int t_geD = tri_gt2(tN, tD);
    if (t_geD == kUnd) return -1;
    if (t_geD == kT) {
        const iv mdb = iv_add(iv_neg(d), b);
        const int c0 = tri_lt(mdb, 0.0f);
        if (c0 == kUnd) return -1;
        if (c0 == kT) return 1;
        const int c1 = tri_gt2(mdb, a);
        if (c1 == kUnd) return -1;
        return c1 == kT ? 4 : 7;
    }
    return dc;
}

// FP64 RN(f / den) < gap, decided in FP32 when certain (f, den, gap are FP64
// values known exactly; only the FP64 division is enclosed).  -1 when undecided.
CIPC_HD int gap_less_cert(double f, double den, double gap)
{
    const int ef = cert_bexp(f), ed = cert_bexp(den), eg = cert_bexp(gap);
    // all three within [2^-100, 2^100): FP32 normal range with room for the quotient
    if (ef < 923 || ef > 1122 || ed < 923 || ed > 1122 || eg < 923 || eg > 1122) return -1;
    const iv F = cert_iv_scaled(f, 0), Dn = cert_iv_scaled(den, 0), G = cert_iv_scaled(gap, 0);
    iv q;
    if (!iv_div(F, Dn, q)) return -1;
    const int s = iv_cmp2(q, G);
    return s < 0 ? 1 : (s > 0 ? 0 : -1);
}

// ---------------------------------------------------------------------------
// FP64 squared distances with the type decided by the certified classifier
// (the FP64 classifier when undecided).  The distance of the decided type is
// computed by exactly the FP64 operations of pt_d2_any / ee_d2_any (geom.cuh),
// so results are bit-identical to them; the interior cases reuse the
// differences already formed for the classification (RN(t0 - p) = -RN(p - t0)
// and RN(eb0 - ea0) = -RN(ea0 - eb0) exactly).
// ---------------------------------------------------------------------------
// type with the FP64 classifier as the fallback (inputs as the FP64 code forms them)
CIPC_HD int pt_type_fast(d3 p, d3 t0, d3 t1, d3 t2, d3 w, d3 e1, d3 e2)
{
    const int ty = pt_type_cert(w, e1, e2);
    return ty >= 0 ? ty : pt_type(p, t0, t1, t2);
}
CIPC_HD int ee_type_fast(d3 ea0, d3 ea1, d3 eb0, d3 eb1, d3 u, d3 v, d3 w)
{
    const int ty = ee_type_cert(u, v, w);
    return ty >= 0 ? ty : ee_type(ea0, ea1, eb0, eb1);
}
// pt_d2 / ee_d2 of geom.cuh from the differences already formed
CIPC_HD double pt_d2_w(d3 w, d3 e1, d3 e2)
{
    const d3 b = cross(e1, e2);
    const double aTb = dot(w, b);
    return G_DIV(G_MUL(aTb, aTb), n2(b));
}
CIPC_HD double ee_d2_w(d3 u, d3 v, d3 w)
{
    const d3 b = cross(u, v);
    const double aTb = dot(mk(-w.x, -w.y, -w.z), b);
    return G_DIV(G_MUL(aTb, aTb), n2(b));
}

CIPC_HD double pt_d2_cert(d3 p, d3 t0, d3 t1, d3 t2)
{
    const d3 e1 = t1 - t0, e2 = t2 - t0, w = p - t0;
    int ty = pt_type_cert(w, e1, e2);
    if (ty < 0) ty = pt_type(p, t0, t1, t2);
    switch (ty) {
        case 0: return n2(w);
        case 1: return pp_d2(p, t1);
        case 2: return pp_d2(p, t2);
        case 3: return pe_d2(p, t0, t1);
        case 4: return pe_d2(p, t1, t2);
        case 5: return pe_d2(p, t2, t0);
        default: {
            const d3 b = cross(e1, e2);
            const double aTb = dot(w, b);
            return G_DIV(G_MUL(aTb, aTb), n2(b));
        }
    }
}

CIPC_HD double ee_d2_cert(d3 ea0, d3 ea1, d3 eb0, d3 eb1)
{
    const d3 u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0;
    int ty = ee_type_cert(u, v, w);
    if (ty < 0) ty = ee_type(ea0, ea1, eb0, eb1);
    switch (ty) {
        case 0: return n2(w);
        case 1: return pp_d2(ea0, eb1);
        case 2: return pe_d2(ea0, eb0, eb1);
        case 3: return pp_d2(ea1, eb0);
        case 4: return pp_d2(ea1, eb1);
        case 5: return pe_d2(ea1, eb0, eb1);
        case 6: return pe_d2(eb0, ea0, ea1);
        case 7: return pe_d2(eb1, ea0, ea1);
        default: {
            const d3 b = cross(u, v);
            const double aTb = dot(mk(-w.x, -w.y, -w.z), b);
            return G_DIV(G_MUL(aTb, aTb), n2(b));
        }
    }
}

}  // namespace cipc
