// Double-word FP32 arithmetic ("double-float"): a value is the unevaluated sum hi + lo
// of two floats with |lo| <= ulp(hi)/2, about 48 significant bits.  GB300 runs FP32 at
// many times its FP64 rate, so element integrals that need more than FP32 accuracy
// (the residual of the mixed-precision Newton step) run on the FP32 pipes in this type.
//
// Building blocks, all with explicit round-to-nearest intrinsics so that no operation
// is contracted or reordered:
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + e = a + b exactly;
//   FastTwoSum (Dekker 1971, |a| >= |b|): the same with three operations;
//   TwoProd with a fused multiply-add: p + e = a * b exactly.
// Addition follows "SloppyDWPlusDW" and multiplication "DWTimesDW3" of Joldes,
// Muller and Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017 (u = 2^-24).  The sloppy sum is exact
// in its high parts (TwoSum) and rounds only the low-order terms, so its error is
// below about 3 u^2 (|x| + |y|): relative to the operands, not to the (possibly
// cancelled) sum, which is the accuracy an assembled residual needs (its terms cancel
// between elements anyway).  Its relative error is below 3 u^2 when x and y have the
// same sign.  The multiplication's relative error is below 4 u^2.  Division and square
// root take an FP32 first approximation and one correction from the double-word
// remainder (Newton's method), which leaves a relative error of a few u^2.
#pragma once

#include <cuda_runtime.h>

namespace svgpu {
namespace dwf {

struct dw {
  float hi, lo;
  dw() = default;
  __host__ __device__ constexpr dw(float h, float l) : hi(h), lo(l) {}
  __device__ dw(int v) : hi((float)v), lo(0.f) {}
  __device__ dw(float v) : hi(v), lo(0.f) {}
  __device__ dw(double v) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
  }
  __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dw operator+(const dw& x, const dw& y) {
  float sh, sl;
  two_sum(x.hi, y.hi, sh, sl);
  const float w = __fadd_rn(sl, __fadd_rn(x.lo, y.lo));
  dw z;
  fast_two_sum(sh, w, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dw operator-(const dw& x) { return dw(-x.hi, -x.lo); }
__device__ __forceinline__ dw operator-(const dw& x, const dw& y) { return x + (-y); }

__device__ __forceinline__ dw operator*(const dw& x, const dw& y) {
  const float ch = __fmul_rn(x.hi, y.hi);
  const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
  const float tl0 = __fmul_rn(x.lo, y.lo);
  const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  const float cl3 = __fadd_rn(cl1, cl2);
  dw z;
  fast_two_sum(ch, cl3, z.hi, z.lo);
  return z;
}

// x - q y for a float q, as a double word (the remainder of a division step)
__device__ __forceinline__ dw remainder_of(const dw& x, const dw& y, float q) {
  const float ph = __fmul_rn(y.hi, q);
  float pl = __fmaf_rn(y.hi, q, -ph);
  pl = __fmaf_rn(y.lo, q, pl);
  return x - dw(ph, pl);
}

__device__ __forceinline__ dw operator/(const dw& x, const dw& y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  const dw r = remainder_of(x, y, q1);
  const float q2 = __fdiv_rn(r.hi, y.hi);
  dw z;
  fast_two_sum(q1, q2, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dw sqrt(const dw& x) {
  if (!(x.hi > 0.f)) return dw(__fsqrt_rn(x.hi), 0.f);  // 0, or NaN for a negative value
  const float s = __fsqrt_rn(x.hi);
  const dw r = remainder_of(x, dw(s, 0.f), s);  // x - s^2
  const float c = __fdiv_rn(r.hi, __fmul_rn(2.f, s));
  dw z;
  fast_two_sum(s, c, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dw fabs(const dw& x) { return x.hi < 0.f ? -x : x; }
__device__ __forceinline__ bool operator<(const dw& a, const dw& b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ dw& operator+=(dw& a, const dw& b) { return a = a + b; }
__device__ __forceinline__ dw& operator-=(dw& a, const dw& b) { return a = a - b; }
__device__ __forceinline__ dw& operator*=(dw& a, const dw& b) { return a = a * b; }

}  // namespace dwf
}  // namespace svgpu
