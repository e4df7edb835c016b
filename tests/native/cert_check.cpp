// Host check of the certified FP32 classifiers of codim-ipc_gb300/csrc/cert.cuh
// against the FP64 classifiers of geom.cuh (both compiled here with
// -ffp-contract=off, the FP64 arithmetic rule of the device code).  Whenever the
// certified version decides a type it must be the FP64 type; "undecided" (-1) is
// allowed and counted.  Cases: random configurations over 16 orders of magnitude
// of size and 6 of translation, and constructed boundary cases (projections on
// edges and vertices, collinear and degenerate triangles, parallel and touching
// edges, exact ties of the gap test).
// Prints "name value bound" lines; exits 1 on any wrong certain decision.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#define CIPC_HD inline
#include "../../codim-ipc_gb300/csrc/cert.cuh"

using namespace cipc;

static std::mt19937_64 rng(20240607);
static double U(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }
static d3 rv(double s) { return mk(U(-s, s), U(-s, s), U(-s, s)); }
static d3 add(d3 a, d3 b) { return a + b; }
static d3 mul(d3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static d3 lerp(d3 a, d3 b, double t) { return mk(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z)); }

struct Count {
    long long n = 0, und = 0, wrong = 0;
};

static void check_pt(Count& c, d3 p, d3 t0, d3 t1, d3 t2)
{
    const int ref = pt_type(p, t0, t1, t2);
    const int got = pt_type_cert(p - t0, t1 - t0, t2 - t0);
    ++c.n;
    if (got < 0)
        ++c.und;
    else if (got != ref) {
        ++c.wrong;
        if (c.wrong < 5) std::fprintf(stderr, "PT wrong: ref %d cert %d\n", ref, got);
    }
}

static void check_ee(Count& c, d3 a0, d3 a1, d3 b0, d3 b1)
{
    const int ref = ee_type(a0, a1, b0, b1);
    const int got = ee_type_cert(a1 - a0, b1 - b0, a0 - b0);
    ++c.n;
    if (got < 0)
        ++c.und;
    else if (got != ref) {
        ++c.wrong;
        if (c.wrong < 5) std::fprintf(stderr, "EE wrong: ref %d cert %d\n", ref, got);
    }
}

int main()
{
    Count pt_rand, pt_adv, ee_rand, ee_adv, gap;
    // random point-triangle configurations at many scales and offsets
    for (int i = 0; i < 400000; ++i) {
        const double s = std::pow(10.0, U(-8, 2)), off = std::pow(10.0, U(-3, 3));
        const d3 o = rv(off);
        const d3 t0 = add(o, rv(s)), t1 = add(o, rv(s)), t2 = add(o, rv(s));
        const double a = U(-0.5, 1.5), b = U(-0.5, 1.5);
        const d3 n = cross(t1 - t0, t2 - t0);
        const double nn = std::sqrt(n2(n));
        d3 p = add(t0, add(mul(t1 - t0, a), mul(t2 - t0, b)));
        if (nn > 0) p = add(p, mul(n, std::pow(10.0, U(-12, 0)) * s / nn * (U(0, 1) < 0.5 ? -1 : 1)));
        check_pt(pt_rand, p, t0, t1, t2);
    }
    // boundary cases: projections exactly on edge lines, vertices, extensions,
    // degenerate and sliver triangles
    for (int i = 0; i < 200000; ++i) {
        const double s = std::pow(10.0, U(-6, 1));
        const d3 o = rv(std::pow(10.0, U(-2, 2)));
        d3 t0 = add(o, rv(s)), t1 = add(o, rv(s)), t2 = add(o, rv(s));
        const int k = i % 8;
        if (k == 6) t2 = lerp(t0, t1, U(-1, 2));                 // collinear
        if (k == 7) t2 = add(lerp(t0, t1, 0.5), rv(s * 1e-9));   // sliver
        d3 p;
        const double t = (k < 3) ? (double)(i % 3) * 0.5 : U(-0.2, 1.2);
        switch (k % 6) {
            case 0: p = lerp(t0, t1, t); break;      // on edge t0t1 (0, 0.5, 1)
            case 1: p = lerp(t1, t2, t); break;
            case 2: p = lerp(t2, t0, t); break;
            case 3: p = t0; break;
            case 4: p = lerp(t0, t1, (i & 1) ? 0.0 : 1.0); break;
            default: p = add(lerp(t0, t2, t), rv(s * 1e-15)); break;
        }
        check_pt(pt_adv, p, t0, t1, t2);
    }
    // random edge pairs
    for (int i = 0; i < 400000; ++i) {
        const double s = std::pow(10.0, U(-8, 2)), off = std::pow(10.0, U(-3, 3));
        const d3 o = rv(off);
        const d3 a0 = add(o, rv(s)), a1 = add(o, rv(s));
        d3 b0 = add(o, rv(s)), b1 = add(o, rv(s));
        if (i % 4 == 0) {  // near-parallel
            const d3 dir = (a1 - a0);
            const d3 base = add(o, rv(s));
            b0 = base;
            b1 = add(add(base, mul(dir, U(0.3, 2.0))), rv(s * std::pow(10.0, U(-14, -1))));
        }
        check_ee(ee_rand, a0, a1, b0, b1);
    }
    // boundary edge pairs: shared or touching endpoints, exact parallels, crossing at endpoints
    for (int i = 0; i < 200000; ++i) {
        const double s = std::pow(10.0, U(-6, 1));
        const d3 o = rv(std::pow(10.0, U(-2, 2)));
        const d3 a0 = add(o, rv(s)), a1 = add(o, rv(s));
        d3 b0, b1;
        switch (i % 6) {
            case 0: b0 = a0; b1 = add(o, rv(s)); break;                   // shared endpoint
            case 1: b0 = lerp(a0, a1, 0.5); b1 = add(o, rv(s)); break;    // touching interior
            case 2: b0 = add(a0, rv(s)); b1 = add(b0, a1 - a0); break;    // parallel (same direction)
            case 3: b0 = lerp(a0, a1, 1.0); b1 = lerp(a0, a1, 2.0); break;  // collinear continuation
            case 4: b0 = add(o, rv(s)); b1 = b0; break;                   // degenerate edge
            default: b0 = a1; b1 = add(a1, a1 - a0); break;
        }
        check_ee(ee_adv, a0, a1, b0, b1);
    }
    // gap test RN(f/den) < gap, including exact ties and neighbours
    for (int i = 0; i < 400000; ++i) {
        const double f = std::pow(10.0, U(-25, 2)) * (U(0, 1) < 0.1 ? -1 : 1);
        const double den = std::pow(10.0, U(-12, 1));
        double g = f / den;
        const int k = i % 4;
        if (k == 1) g = std::nextafter(g, 1e300);
        if (k == 2) g = std::nextafter(g, -1e300);
        if (k == 3) g = g * U(0.5, 2.0);
        const int ref = (f / den < g) ? 1 : 0;
        const int got = gap_less_cert(f, den, g);
        ++gap.n;
        if (got < 0)
            ++gap.und;
        else if (got != ref)
            ++gap.wrong;
    }
    const Count* all[5] = {&pt_rand, &pt_adv, &ee_rand, &ee_adv, &gap};
    const char* names[5] = {"pt_random", "pt_boundary", "ee_random", "ee_boundary", "gap"};
    long long wrong = 0;
    for (int k = 0; k < 5; ++k) {
        std::printf("%s_wrong %lld 0\n", names[k], all[k]->wrong);
        std::printf("%s_undecided_frac %.6g 1\n", names[k], (double)all[k]->und / (double)all[k]->n);
        wrong += all[k]->wrong;
    }
    // the random (non-constructed) cases must almost always be decided
    std::printf("pt_random_undecided_bound %.6g %.6g\n", (double)pt_rand.und / pt_rand.n, 0.01);
    std::printf("ee_random_undecided_bound %.6g %.6g\n", (double)ee_rand.und / ee_rand.n, 0.3);
    return wrong ? 1 : 0;
}
