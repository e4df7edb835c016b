// Host check of the float-float helpers of codim-ipc_gb300/csrc/ff.cuh: the
// device intrinsics are mapped to IEEE single-precision host operations (each
// result forced through a float store, FMA from the C library), and the split of
// FP64 values and the basic operations are compared with long double results.
// Prints one line per check, "name value bound", and exits 1 if any value
// exceeds its bound.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#define __device__
#define __forceinline__ inline
#define __noinline__
static inline float __fadd_rn(float a, float b) { volatile float r = a + b; return r; }
static inline float __fsub_rn(float a, float b) { volatile float r = a - b; return r; }
static inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline long long __double_as_longlong(double d) { long long r; std::memcpy(&r, &d, 8); return r; }
static inline float __uint_as_float(unsigned u) { float r; std::memcpy(&r, &u, 4); return r; }
static inline unsigned __float_as_uint(float f) { unsigned r; std::memcpy(&r, &f, 4); return r; }
#include "../../codim-ipc_gb300/csrc/ff.cuh"

using cipc::ff;
static long double val(ff x) { return (long double)x.hi + (long double)x.lo; }

int main()
{
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    double split = 0, add = 0, mul = 0, fma = 0;
    for (int i = 0; i < 1000000; ++i) {
        const double d = u(g) * std::ldexp(1.0, (int)(g() % 160) - 80);
        const ff f = cipc::ff_from_double(d);
        split = std::fmax(split, (double)fabsl((val(f) - d) / d));
        const double a = u(g), b = u(g) * 3.0, c = u(g) * 0.5;
        const ff fa = cipc::ff_from_double(a), fb = cipc::ff_from_double(b), fc = cipc::ff_from_double(c);
        const long double A = val(fa), B = val(fb), Cc = val(fc);
        add = std::fmax(add, (double)(fabsl(val(cipc::ff_sub(fa, fb)) - (A - B)) / (fabsl(A) + fabsl(B))));
        mul = std::fmax(mul, (double)(fabsl(val(cipc::ff_mul(fa, fb)) - A * B) / fabsl(A * B)));
        fma = std::fmax(fma, (double)(fabsl(val(cipc::ff_fma(fa, fb, fc)) - (A * B + Cc)) / (fabsl(A * B) + fabsl(Cc))));
    }
    // zero, FP64 subnormals and out-of-range magnitudes
    int special = 0;
    const double sp[] = {0.0, -0.0, 5e-324, -1e-310, 1e-35, 3e38, -1e-31};
    for (double d : sp) {
        const ff f = cipc::ff_from_double(d);
        const bool ok = (std::fabs(d) < 1e-300) ? (f.hi == 0.f && f.lo == 0.f)
                                                 : fabsl((val(f) - d) / d) < 1e-7L;
        special += ok ? 0 : 1;
    }
    const struct { const char* name; double v, bound; } rows[] = {
        {"split_rel", split, std::ldexp(1.0, -46)},
        {"sub_abs_over_magnitudes", add, std::ldexp(1.0, -45)},
        {"mul_rel", mul, std::ldexp(1.0, -44)},
        {"fma_abs_over_magnitudes", fma, std::ldexp(1.0, -44)},
        {"special_value_failures", (double)special, 0.0},
    };
    int bad = 0;
    for (const auto& r : rows) {
        std::printf("%s %.3e %.3e\n", r.name, r.v, r.bound);
        bad += r.v > r.bound;
    }
    return bad ? 1 : 0;
}
