// Double-float arithmetic: a value is an unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits.  Built
// from error-free transformations (Knuth's TwoSum, and TwoProd through one
// fused multiply-add) so that every operation runs on the FP32 pipes,
// which on GB300 issue 64 times as fast as FP64.  The compensated dot
// product is Ogita, Rump and Oishi's Dot2 (SIAM J. Sci. Comput. 26, 2005):
// the result is as accurate as if the sum had been formed in twice the
// working precision and then rounded.  Products and sums use the _rn
// intrinsics, which the compiler never contracts into a multiply-add: a
// contraction would break the exactness the transformations rely on.
#pragma once

#include <cuda_runtime.h>

namespace adp {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_from_double(double x) {
  const float h = (float)x;
  return ff{h, (float)(x - (double)h)};
}

__device__ __forceinline__ double ff_to_double(ff x) { return (double)x.hi + (double)x.lo; }

// Double-float arrays are stored as float2 (hi, lo) pairs: one 8-byte
// access per value instead of two 4-byte ones.
__device__ __forceinline__ ff ld_ff(const float2* p) {
  const float2 v = *p;
  return ff{v.x, v.y};
}
__device__ __forceinline__ void st_ff(float2* p, ff v) { *p = make_float2(v.hi, v.lo); }

__device__ __forceinline__ ff ff_norm(float s, float e) {   // FastTwoSum, |s| >= |e|
  const float t = __fadd_rn(s, e);
  return ff{t, __fsub_rn(e, __fsub_rn(t, s))};
}

// TwoSum: s + err == a + b exactly
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}

__device__ __forceinline__ ff ff_add(ff x, ff y) {
  float e;
  const float s = two_sum(x.hi, y.hi, e);
  e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
  return ff_norm(s, e);
}

__device__ __forceinline__ ff ff_add_f(ff x, float y) {
  float e;
  const float s = two_sum(x.hi, y, e);
  return ff_norm(s, __fadd_rn(e, x.lo));
}

__device__ __forceinline__ ff ff_mul(ff x, ff y) {   // drops lo*lo (2^-48 relative)
  const float p = __fmul_rn(x.hi, y.hi);
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return ff_norm(p, e);
}

// x - y as a single float (the difference of two nearby double-floats).
__device__ __forceinline__ float ff_diff(ff x, ff y) {
  return __fadd_rn(__fsub_rn(x.hi, y.hi), __fsub_rn(x.lo, y.lo));
}

// Dot2 accumulator: sum + err, terms a*x added with TwoProd and TwoSum.
struct Dot2 {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(ff a, ff x) {
    const float h = __fmul_rn(a.hi, x.hi);
    float r = fmaf(a.hi, x.hi, -h);
    r = fmaf(a.hi, x.lo, r);
    r = fmaf(a.lo, x.hi, r);
    float q;
    s = two_sum(s, h, q);
    c = __fadd_rn(c, __fadd_rn(q, r));
  }
  __device__ __forceinline__ void sub(ff a, ff x) { add(ff{-a.hi, -a.lo}, x); }
  __device__ __forceinline__ ff value() const { return ff_norm(s, c); }
};

}  // namespace adp
