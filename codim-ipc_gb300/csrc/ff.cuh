// Float-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers with |lo| <= ulp(hi)/2, carrying ~48 significant bits.
//
// Built from the error-free transformations TwoSum (Knuth, TAOCP vol. 2, 4.2.2),
// FastTwoSum (Dekker 1971) and the FMA form of TwoProduct (p = a*b, e = fma(a, b,
// -p)).  Additions are the "sloppy" form (one TwoSum on the high parts, the low
// parts added in FP32): their absolute error is O(2^-47 (|x| + |y|)), the same
// form as an FP64 operation's error on inputs that carry rounding error
// themselves, 2^5 larger.  Every operation uses the explicit-rounding intrinsics,
// so the compiler contracts nothing and results do not depend on -fmad.
//
// Why: on this part the FP64 pipe issues 2 operations per SM per clock against
// 128 for FP32, so the 10-16 FP32 operations of a float-float operation cost a
// fraction of one FP64 operation.
#pragma once
#include <cstdint>

namespace cipc {

struct ff {
    float hi, lo;
};
struct ff3 {
    ff x, y, z;
};

__device__ __forceinline__ ff fast_two_sum(float a, float b)  // exact when exponent(a) >= exponent(b)
{
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float v = __fsub_rn(s, a);
    return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}
__device__ __forceinline__ ff ffv(float a) { return ff{a, 0.f}; }
__device__ __forceinline__ ff ff_neg(ff x) { return ff{-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_add(ff x, ff y)
{
    const ff s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }
__device__ __forceinline__ ff ff_add_f(ff x, float b)
{
    const ff s = two_sum(x.hi, b);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}
__device__ __forceinline__ ff ff_mul(ff x, ff y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return fast_two_sum(p, e);
}
// x * y + z
__device__ __forceinline__ ff ff_fma(ff x, ff y, ff z)
{
    const float p = __fmul_rn(x.hi, y.hi);
    const float e = __fmaf_rn(x.hi, y.hi, -p);
    const ff s = two_sum(p, z.hi);
    float t = __fadd_rn(s.lo, e);
    t = __fmaf_rn(x.hi, y.lo, t);
    t = __fmaf_rn(x.lo, y.hi, t);
    t = __fadd_rn(t, z.lo);
    return fast_two_sum(s.hi, t);
}
// exact scaling by a power of two (barring overflow and underflow)
__device__ __forceinline__ ff ff_scale(ff x, float p2) { return ff{__fmul_rn(x.hi, p2), __fmul_rn(x.lo, p2)}; }
__device__ __forceinline__ bool ff_gt(ff a, ff b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }

// FP64 conversion, kept out of line so that the compiler cannot evaluate it
// speculatively on the common path (it would occupy the FP64 pipe for every value)
__device__ __noinline__ ff ff_from_double_rare(double d)
{
    const float h = (float)d;
    return ff{h, (float)(d - (double)h)};
}

// double -> float-float by integer operations on the bit pattern (no FP64
// instruction): hi = d truncated to 24 significant bits, lo = the next 23 bits,
// exactly (the lowest 6 of the 52 stored bits are dropped: relative error below
// 2^-46).  The pair is not renormalised (0 <= |lo| < ulp(hi), same sign), which
// the sums and products above accept.  Zero and FP64 subnormals map to zero
// (tested on the exponent field: a test of d itself compiles to an FP64
// comparison); other magnitudes outside [2^-103, 2^127) take the FP64 conversion.
__device__ __forceinline__ ff ff_from_double(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const unsigned e = (hw >> 20) & 0x7ffu;
    if (e == 0u) return ff{0.f, 0.f};
    if (e < 920u || e > 1150u) return ff_from_double_rare(d);
    const unsigned sg = hw & 0x80000000u;
    const unsigned m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
    const float h = __uint_as_float(sg | ((e - 896u) << 23) | m23);
    const unsigned el = (e - 919u) << 23;  // 2^(e - 1023 - 23) as a float
    const float l = __fsub_rn(__uint_as_float(el | ((lw & 0x1fffffffu) >> 6)), __uint_as_float(el));
    return ff{h, __uint_as_float(__float_as_uint(l) | sg)};
}
__device__ __forceinline__ double ff_to_double(ff x) { return (double)x.hi + (double)x.lo; }

__device__ __forceinline__ ff3 ff3_sub(ff3 a, ff3 b) { return ff3{ff_sub(a.x, b.x), ff_sub(a.y, b.y), ff_sub(a.z, b.z)}; }
__device__ __forceinline__ ff3 ff3_add(ff3 a, ff3 b) { return ff3{ff_add(a.x, b.x), ff_add(a.y, b.y), ff_add(a.z, b.z)}; }
__device__ __forceinline__ ff3 ff3_axpy(ff s, ff3 d, ff3 x)
{
    return ff3{ff_fma(s, d.x, x.x), ff_fma(s, d.y, x.y), ff_fma(s, d.z, x.z)};
}
__device__ __forceinline__ ff ff3_dot(ff3 a, ff3 b) { return ff_fma(a.z, b.z, ff_fma(a.y, b.y, ff_mul(a.x, b.x))); }
__device__ __forceinline__ ff ff3_n2(ff3 a) { return ff3_dot(a, a); }
__device__ __forceinline__ ff3 ff3_cross(ff3 a, ff3 b)
{
    return ff3{ff_fma(a.y, b.z, ff_neg(ff_mul(a.z, b.y))), ff_fma(a.z, b.x, ff_neg(ff_mul(a.x, b.z))),
               ff_fma(a.x, b.y, ff_neg(ff_mul(a.y, b.x)))};
}
__device__ __forceinline__ ff3 ff3_scale(ff3 a, float p2)
{
    return ff3{ff_scale(a.x, p2), ff_scale(a.y, p2), ff_scale(a.z, p2)};
}

}  // namespace cipc
