// df64.cuh — double-FP32 ("df64") arithmetic: a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi) / 2, about 48 significant bits.
//
// GB300 issues FP32 at 64 times its FP64 rate, so FP64-accurate work that
// does not need FP64's exponent range can run in pairs of FP32 operations
// instead.  The error-free transformations are the classical ones: Knuth's
// two-sum and Dekker's fast two-sum for addition, a fused multiply-add for the
// exact product error.  Every operation uses explicitly rounded intrinsics
// (__fadd_rn, __fmul_rn, __fmaf_rn), which the compiler never contracts or
// reassociates, so the transformations stay exact.  The exponent range is
// FP32's: callers scale their data by powers of two (exact) first.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace ipcg {

// the FP64 / FP32 math functions stay visible beside the df64 overloads below
using ::fabs;
using ::fma;
using ::hypot;
using ::rsqrt;
using ::sqrt;

// double -> df64: hi = x rounded to FP32; x - hi is exact in FP64 (at most 29
// significant bits) and rounded once more, so hi + lo carries x to about 48
// bits (x must lie in FP32's normal range).  Constants and small integers
// convert implicitly, so generic code reads the same for double and dd.
struct alignas(8) dd {
    float hi, lo;
    dd() = default;
    __device__ __forceinline__ constexpr dd(float h, float l) : hi(h), lo(l) { }
    __device__ __forceinline__ dd(double x)
    {
        hi = __double2float_rn(x);
        lo = __double2float_rn(x - (double)hi);
    }
    __device__ __forceinline__ constexpr dd(int x) : hi((float)x), lo(0.f) { }
};

__device__ __forceinline__ dd dd_from_double(double x) { return dd(x); }
__device__ __forceinline__ double dd_to_double(dd a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dd two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return dd { s, e };
}
__device__ __forceinline__ dd fast_two_sum(float a, float b) // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return dd { s, __fsub_rn(b, __fsub_rn(s, a)) };
}
// a + b with the error of the leading parts kept exactly and the trailing
// parts added in FP32: the error is below about 2^-47 (|a| + |b|) -- the
// bound a backward-stable matrix algorithm needs (not relative to a + b when
// it cancels) -- at about half the cost of the fully accurate sum.
__device__ __forceinline__ dd operator+(dd a, dd b)
{
    const dd s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dd operator-(dd a) { return dd { -a.hi, -a.lo }; }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
// a / b: three quotient digits, each from the remainder times an
// approximate reciprocal of b.hi (about 22 correct bits); the remainders are
// exact to df64 precision, so every digit adds ~22 bits and the result is
// correct to df64 precision although the reciprocal is not.
__device__ __forceinline__ dd operator/(dd a, dd b)
{
    const float inv = __fdividef(1.f, b.hi);
    const float q1 = __fmul_rn(a.hi, inv);
    dd r = a - dd { q1, 0.f } * b;
    const float q2 = __fmul_rn(r.hi, inv);
    r = r - dd { q2, 0.f } * b;
    const float q3 = __fmul_rn(r.hi, inv);
    return fast_two_sum(q1, q2) + dd { q3, 0.f };
}
__device__ __forceinline__ dd& operator+=(dd& a, dd b) { return a = a + b; }
__device__ __forceinline__ dd& operator-=(dd& a, dd b) { return a = a - b; }
__device__ __forceinline__ dd& operator*=(dd& a, dd b) { return a = a * b; }
__device__ __forceinline__ bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dd a, dd b) { return b < a; }
__device__ __forceinline__ bool operator<=(dd a, dd b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dd a, dd b) { return !(a < b); }
__device__ __forceinline__ bool operator==(dd a, dd b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(dd a, dd b) { return !(a == b); }
__device__ __forceinline__ dd fabs(dd a) { return a.hi < 0.f ? -a : a; }
// sqrt and 1/sqrt: an approximate FP32 reciprocal square root (about 22
// correct bits) refined by one Newton step whose residual is formed in
// df64, which doubles the correct bits (about 44).
__device__ __forceinline__ dd sqrt(dd a)
{
    if (!(a.hi > 0.f)) return dd { 0.f, 0.f };
    const float rs = rsqrtf(a.hi);
    const float y = __fmul_rn(a.hi, rs);
    const dd r = a - dd { y, 0.f } * dd { y, 0.f };
    return fast_two_sum(y, __fmul_rn(r.hi, __fmul_rn(0.5f, rs)));
}
__device__ __forceinline__ dd rsqrt(dd a)
{
    const float y = rsqrtf(a.hi);
    const dd yy = dd { y, 0.f } * dd { y, 0.f };
    const dd d = dd { 1.f, 0.f } - a * yy; // 1 - a y^2, small
    return fast_two_sum(y, __fmul_rn(__fmul_rn(0.5f, y), d.hi));
}
__device__ __forceinline__ dd hypot(dd a, dd b) { return sqrt(a * a + b * b); }
__device__ __forceinline__ dd fma(dd a, dd b, dd c) { return a * b + c; }
// power-of-two exponent of |a| (frexp convention: |a.hi| = m 2^e with m in
// [1/2, 1); from the exponent bits; 0 for zero) and exact scaling by 2^e
// (a multiplication by a power of two built from its bits, in two steps when
// 2^e is outside FP32's normal range)
__device__ __forceinline__ int pow2_exp(dd a)
{
    const int bits = (__float_as_int(a.hi) >> 23) & 0xff;
    return bits == 0 ? 0 : bits - 126;
}
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); } // e in [-126, 127]
__device__ __forceinline__ dd scale2(dd a, int e)
{
    if (e >= -126 && e <= 127) {
        const float p = pow2f(e);
        return dd { __fmul_rn(a.hi, p), __fmul_rn(a.lo, p) };
    }
    const int e1 = e / 2, e2 = e - e1;
    const float p1 = pow2f(e1), p2 = pow2f(e2);
    return dd { __fmul_rn(__fmul_rn(a.hi, p1), p2), __fmul_rn(__fmul_rn(a.lo, p1), p2) };
}
__device__ __forceinline__ dd dmax(dd a, dd b) { return a < b ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return fmax(a, b); }

} // namespace ipcg
