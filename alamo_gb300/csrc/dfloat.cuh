// Double-float numbers ("df32"): the unevaluated sum hi + lo of two FP32
// values, |lo| <= ulp(hi) / 2, about 48 significant bits, computed with FP32
// instructions only.  Sum by Knuth's TwoSum and Dekker's FastTwoSum, product
// by Dekker's TwoProduct written with the fused multiply-add (the error-free
// transformations of Ogita, Rump and Oishi, "Accurate sum and dot product",
// 2005); the additions are the "sloppy" double-float sum, whose error is
// bounded by about 2^-46 (|a| + |b|).  The operator's stencil code is
// templated on its number type, so instantiating it on dfloat evaluates the
// FP64 operator on the FP32 pipe (GB300 runs FP32 at 64 times its FP64 rate).
#pragma once
#include <cuda_runtime.h>

namespace agb {

struct dfloat {
    float hi, lo;
    __host__ __device__ dfloat() : hi(0.f), lo(0.f) {}
    __host__ __device__ dfloat(int a) : hi((float)a), lo(0.f) {}
    __host__ __device__ dfloat(float a) : hi(a), lo(0.f) {}
    // split of a double: hi its FP32 rounding, lo the rounded remainder
    __host__ __device__ dfloat(double a) : hi((float)a), lo((float)(a - (double)(float)a)) {}
    __host__ __device__ dfloat(float h, float l, int) : hi(h), lo(l) {}
};

__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return dfloat(s, e, 0);
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {
    const float s = a + b;
    return dfloat(s, b - (s - a), 0);
}

// The sum renormalises its pair (FastTwoSum): after cancellation of the hi
// parts an unnormalised lo would be as large as hi, and a later product
// would round it in single precision (measured: the 257^3 solve stalled
// above 1e-8 without it).  The product leaves its pair unnormalised, |lo| a
// few ulp(hi) at most, which the next operation absorbs.
__device__ __forceinline__ dfloat operator+(const dfloat& a, const dfloat& b) {
    const dfloat s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ dfloat operator-(const dfloat& a) { return dfloat(-a.hi, -a.lo, 0); }
__device__ __forceinline__ dfloat operator-(const dfloat& a, const dfloat& b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(const dfloat& a, const dfloat& b) {
    const float p = a.hi * b.hi;
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return dfloat(p, e, 0);
}
// the pair's value rounded to FP32 / FP64
__device__ __forceinline__ float df_float(const dfloat& a) { return a.hi + a.lo; }
__device__ __forceinline__ double df_double(const dfloat& a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfloat& operator+=(dfloat& a, const dfloat& b) { return a = a + b; }
__device__ __forceinline__ dfloat& operator-=(dfloat& a, const dfloat& b) { return a = a - b; }
__device__ __forceinline__ dfloat& operator*=(dfloat& a, const dfloat& b) { return a = a * b; }

}  // namespace agb
