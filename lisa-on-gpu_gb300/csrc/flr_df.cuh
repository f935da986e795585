// Double-float ("df") arithmetic: a value is the unevaluated sum hi + lo of
// two FP32 numbers, giving about 48 significand bits on the FP32 pipe (which
// on GB300 issues ~70x more operations per clock than the FP64 pipe).
//
// Built from the classical error-free transformations:
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + e = a + b exactly, 6 flops;
//   FastTwoSum (Dekker 1971): the same in 3 flops when |a| >= |b|;
//   TwoProduct with FMA: p + e = a * b exactly, 2 flops;
// and the compensated dot product of Ogita, Rump and Oishi ("Accurate sum and
// dot product", SIAM J. Sci. Comput. 26, 2005), Dot2: products split exactly,
// high parts summed with TwoSum, all error terms gathered in a float.
//
// Translation units using this header are compiled with --fmad=false, so the
// compiler cannot fuse the separate multiplies and adds these algorithms rely
// on; every FMA below is explicit.
#pragma once

namespace flr {
namespace df {

struct f2 {
    float hi, lo;
};

__device__ __forceinline__ f2 two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

// Requires |a| >= |b| (or a == 0).
__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
    float s = a + b;
    float e = b - (s - a);
    return {s, e};
}

__device__ __forceinline__ f2 two_prod(float a, float b) {
    float p = a * b;
    return {p, __fmaf_rn(a, b, -p)};
}

// Split an FP64 value into hi + lo (|lo| <= ulp(hi)/2; exact to ~2^-48).
__device__ __forceinline__ f2 from_double(double x) {
    float hi = __double2float_rn(x);
    float lo = __double2float_rn(x - (double)hi);
    return {hi, lo};
}

__device__ __forceinline__ double to_double(f2 a) { return (double)a.hi + (double)a.lo; }

// x * 2^shift as a df value, from the bits of x with integer operations only
// (no FP64-pipe conversion; on GB300 that pipe is the scarce one): hi = the
// top 24 significant bits of x, lo = the next 24 (the remaining 5 dropped),
// so hi + lo is x to ~2^-48, |lo| < ulp(hi).  Values whose scaled exponent
// leaves [-100, 100] (zero, tiny, huge, not finite) take the conversion route.
__device__ __forceinline__ f2 from_double_bits(double x, int shift = 0) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ffu) - 1023 + shift;
    if (e < -100 || e > 100) {
        const double y = ldexp(x, shift);
        const float hi = __double2float_rn(y);
        return {hi, __double2float_rn(y - (double)hi)};
    }
    const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) |
                                     (unsigned)((b >> 29) & 0x7fffffu));
    const unsigned m = (unsigned)(b & 0x1fffffffu);  // the 29 bits below hi
    if (m == 0u) return {hi, 0.f};
    const int lz = __clz(m) - 3;                      // leading zeros within the 29 bits
    const unsigned mant = ((m << (lz + 3)) >> 8) & 0x7fffffu;
    return {hi, __uint_as_float(sign | ((unsigned)(e - 24 - lz + 127) << 23) | mant)};
}

// (hi + lo) * 2^shift as a double: both floats widened from their bits (integer
// operations), one FP64 addition.  Zero and subnormal parts count as zero.
__device__ __forceinline__ double float_bits_to_double(float v, int shift) {
    const unsigned u = __float_as_uint(v);
    const unsigned ef = (u >> 23) & 0xffu;
    if (ef == 0u) return 0.0;
    if (ef == 0xffu) return ldexp((double)v, shift);
    const unsigned long long bits = ((unsigned long long)(u & 0x80000000u) << 32) |
                                    ((unsigned long long)(ef - 127 + 1023 + shift) << 52) |
                                    ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double to_double_bits(f2 a, int shift) {
    return float_bits_to_double(a.hi, shift) + float_bits_to_double(a.lo, shift);
}

__device__ __forceinline__ f2 renorm(f2 a) { return fast_two_sum(a.hi, a.lo); }

// a + b, result normalised.
__device__ __forceinline__ f2 add(f2 a, f2 b) {
    f2 s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

// a + b without the final renormalisation: for operands that cannot cancel
// (|lo| of the result stays within a few ulp of hi).
__device__ __forceinline__ f2 add_raw(f2 a, f2 b) {
    f2 s = two_sum(a.hi, b.hi);
    return {s.hi, s.lo + (a.lo + b.lo)};
}
// a - b, result normalised.
__device__ __forceinline__ f2 sub(f2 a, f2 b) {
    f2 s = two_sum(a.hi, -b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo - b.lo));
}

// 1 - a for 0 <= a.hi <= 1 (FastTwoSum applies); not normalised.
__device__ __forceinline__ f2 one_minus(f2 a) {
    f2 s = fast_two_sum(1.0f, -a.hi);
    return {s.hi, s.lo - a.lo};
}
// a * b with the lo*lo term dropped (relative error ~2^-46); not normalised
// (|lo| is a few ulp of hi at most), which the consumers below accept.
__device__ __forceinline__ f2 mul_raw(f2 a, f2 b) {
    f2 p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    return p;
}

__device__ __forceinline__ f2 mul(f2 a, f2 b) { return renorm(mul_raw(a, b)); }

// float + df, for |j| >= |a| (the Lagrange denominators j + eps, j >= 1).
__device__ __forceinline__ f2 add_big_float(float j, f2 a) {
    f2 s = fast_two_sum(j, a.hi);
    s.lo += a.lo;
    return s;
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// 1 / b for |b.hi| a normal float (the projection's 1 - k.n; 1/b must not
// overflow): hardware approximation refined by one Newton step carried out on
// the df residual, r = r0 + r0 * (1 - b r0); relative error about 1e-14.  Not
// normalised.
__device__ __forceinline__ f2 rcp(f2 b) {
    float r0 = rcp_approx(b.hi);
    float t = __fmaf_rn(-b.hi, r0, 1.0f);
    t = __fmaf_rn(-b.lo, r0, t);
    return {r0, r0 * t};
}

// a / b for b in [1, 64): q0 = a.hi / b.hi from the hardware reciprocal,
// corrected once by the df residual, q = q0 + r0 (a - q0 b); relative error
// about 1e-13.  Not normalised.
__device__ __forceinline__ f2 div_raw(f2 a, f2 b) {
    const float r0 = rcp_approx(b.hi);
    const float q0 = a.hi * r0;
    float res = __fmaf_rn(-q0, b.hi, a.hi);
    res = __fmaf_rn(-q0, b.lo, res);
    res = res + a.lo;
    return {q0, r0 * res};
}
// Dot2 accumulator (Ogita-Rump-Oishi): sum of df products.
struct Acc {
    float s;    // running FP32 sum of the high parts
    float c;    // gathered error terms and low parts
};

__device__ __forceinline__ void acc_init(Acc &a) {
    a.s = 0.f;
    a.c = 0.f;
}

// a += w * x for df w and df x.
__device__ __forceinline__ void acc_fma(Acc &a, f2 w, f2 x) {
    f2 p = two_prod(w.hi, x.hi);
    float cross = __fmaf_rn(w.hi, x.lo, __fmaf_rn(w.lo, x.hi, p.lo));
    f2 s = two_sum(a.s, p.hi);
    a.s = s.hi;
    a.c += s.lo + cross;
}

// a += v for a df value v.
__device__ __forceinline__ void acc_add(Acc &a, f2 v) {
    f2 s = two_sum(a.s, v.hi);
    a.s = s.hi;
    a.c += s.lo + v.lo;
}

__device__ __forceinline__ f2 acc_value(const Acc &a) { return fast_two_sum(a.s, a.c); }

}  // namespace df
}  // namespace flr
