// Double-single ("float-float") arithmetic for the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits (relative rounding ~4e-15), with float's exponent
// range.  Sums use Knuth's two-sum and products Dekker's exact product
// through a fused multiply-add, renormalised by a quick two-sum: the
// "sloppy" double-single operations of D. H. Bailey's DSFUN package.  Every
// step is an explicitly rounded intrinsic, so the compiler neither contracts
// nor reassociates them.  On GB300 a double-single multiply-add costs about
// ten FP32 instructions, several times cheaper than an FP64 one.
#pragma once
#include <cuda_runtime.h>

struct dsf {
  float hi, lo;
  __device__ __forceinline__ dsf() {}
  __device__ __forceinline__ dsf(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ dsf(int v) : hi((float)v), lo(0.f) {}
};

__device__ __forceinline__ dsf dsf_from(double d) {
  const float h = __double2float_rn(d);
  return dsf(h, __double2float_rn(d - (double)h));
}

__device__ __forceinline__ double dsf_to(dsf a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dsf dsf_quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dsf(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dsf operator+(dsf a, dsf b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return dsf_quick_two_sum(s, e);
}

__device__ __forceinline__ dsf operator-(dsf a) { return dsf(-a.hi, -a.lo); }
__device__ __forceinline__ dsf operator-(dsf a, dsf b) { return a + (-b); }

__device__ __forceinline__ dsf operator*(dsf a, dsf b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return dsf_quick_two_sum(p, e);
}

// small integer constants (exact in float)
__device__ __forceinline__ dsf operator*(int k, dsf b) {
  const float kf = (float)k;
  const float p = __fmul_rn(kf, b.hi);
  const float e = __fmaf_rn(kf, b.lo, __fmaf_rn(kf, b.hi, -p));
  return dsf_quick_two_sum(p, e);
}
__device__ __forceinline__ dsf operator*(dsf b, int k) { return k * b; }

__device__ __forceinline__ dsf& operator+=(dsf& a, dsf b) {
  a = a + b;
  return a;
}

__device__ __forceinline__ dsf fma(dsf a, dsf b, dsf c) { return a * b + c; }
