// Double-float ("df64") arithmetic: a value held as an unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant
// bits. GB300 runs FP32 on its CUDA cores some sixty times faster than FP64,
// so FFT stages in double-float arithmetic (about eleven FP32 operations for
// an FP64 operation) give FP64-class accuracy (relative errors near 1e-14)
// faster than FP64 stages. The exponent range is FP32's (values between
// about 1e-38 and 3e38).
//
// Published algorithms (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2): the
// error-free sum (two_sum: s + e = a + b exactly), the fast sum for
// |a| >= |b| (quick_two_sum), and the exact product through a fused
// multiply-add (two_prod: p + e = a * b exactly). Addition is the
// "sloppy" double-float sum (one error-free sum of the high parts, the low
// parts added in FP32): its error is bounded by about 2^-47 (|a| + |b|),
// which is what a normwise FFT error bound needs. Every operation is written
// with explicit round-to-nearest intrinsics so that no product and sum are
// contracted into a fused multiply-add behind the algorithm's back.
#pragma once
#include <cuda_runtime.h>

namespace ps {

struct __align__(8) dfloat {
    float hi, lo;
    dfloat() = default;
    __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
    // exact for integers below 2^24 (wavenumber indices)
    __host__ __device__ constexpr dfloat(int v) : hi((float)v), lo(0.0f) {}
    // the double rounded to about 48 bits: hi = fl(d), lo = fl(d - hi)
    __host__ __device__ constexpr dfloat(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

struct __align__(16) dfloat2 {
    dfloat x, y;
};

// read-only cached loads, as for the built-in vector types (beside, not
// hiding, the built-in overloads)
using ::__ldg;
__device__ __forceinline__ dfloat2 __ldg(const dfloat2 *p)
{
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    return dfloat2{dfloat(v.x, v.y), dfloat(v.z, v.w)};
}
__device__ __forceinline__ dfloat __ldg(const dfloat *p)
{
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return dfloat(v.x, v.y);
}

namespace dfa {
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void quick_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
}  // namespace dfa

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b)
{
    float s, e;
    dfa::two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    dfloat r;
    dfa::quick_two_sum(s, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);  // p + e = a.hi b.hi exactly
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    dfloat r;
    dfa::quick_two_sum(p, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat &operator-=(dfloat &a, dfloat b) { return a = a - b; }
__device__ __forceinline__ dfloat &operator*=(dfloat &a, dfloat b) { return a = a * b; }

}  // namespace ps
