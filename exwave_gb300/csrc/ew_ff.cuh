// ew_ff.cuh -- float-float arithmetic for the compensated operator.
//
// An FF value is the unevaluated sum hi + lo of two floats.  Products use the
// exact FMA residual of hi*hi (Dekker's product with a fused multiply-add),
// sums use Knuth's error-free two-sum; results are renormalised with a fast
// two-sum so that |lo| <= ulp(hi)/2.  About 44 significant bits: enough that
// the rounding of the operator's sums and coefficients no longer shows in
// the discretisation error, while the data stay FP32.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "ew_device.cuh"

namespace ew {

struct FF;
// compute types of the operator arithmetic: FP64, FP32 or float-float (FF)
template <typename R>
constexpr bool is_f64_v = std::is_same<R, double>::value;
template <typename R>
constexpr bool is_ff_v = std::is_same<R, FF>::value;

struct FF {
  float hi, lo;
  FF() = default;
  __host__ __device__ constexpr FF(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr FF(float v) : hi(v), lo(0.f) {}
  // split of a double into its nearest float and the float nearest the rest
  __host__ __device__ static FF from_double(double d) {
    const float h = (float)d;
    return FF(h, (float)(d - (double)h));
  }
  __host__ __device__ double to_double() const { return (double)hi + (double)lo; }
};

// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
}

// s + e = a + b exactly, for |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ FF operator+(FF a, FF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  FF r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ FF operator-(FF a) { return FF(-a.hi, -a.lo); }
__device__ __forceinline__ FF operator-(FF a, FF b) { return a + (-b); }

__device__ __forceinline__ FF operator*(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  FF r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ FF operator*(FF a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  FF r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ FF operator*(float a, FF b) { return b * a; }
__device__ __forceinline__ FF& operator+=(FF& a, FF b) { return a = a + b; }
__device__ __forceinline__ FF& operator-=(FF& a, FF b) { return a = a - b; }
__device__ __forceinline__ FF& operator*=(FF& a, FF b) { return a = a * b; }

// a / b by long division: quotient digits a.hi / b.hi, each followed by the
// exact remainder in float-float (about 44 bits)
__device__ __forceinline__ FF operator/(FF a, FF b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const FF r1 = a - b * q1;
  const float q2 = __fdiv_rn(r1.hi, b.hi);
  const FF r2 = r1 - b * q2;
  const float q3 = __fdiv_rn(r2.hi, b.hi);
  FF q;
  fast_two_sum(q1, q2, q.hi, q.lo);
  return q + FF(q3);
}
__device__ __forceinline__ FF& operator/=(FF& a, FF b) { return a = a / b; }

// square root: the float root and one Newton correction from the exact
// residual (a >= 0)
__device__ __forceinline__ FF ff_sqrt(FF a) {
  if (!(a.hi > 0.f)) return FF(0.f);
  const float s = __fsqrt_rn(a.hi);
  const FF r = a - FF(s) * FF(s);
  FF q;
  fast_two_sum(s, __fdiv_rn(r.hi, 2.f * s), q.hi, q.lo);
  return q;
}
__device__ __forceinline__ FF ff_fabs(FF a) { return a.hi < 0.f ? -a : a; }

// square root and absolute value in the compute type
template <typename R>
__device__ __forceinline__ R real_sqrt(R v) {
  if constexpr (is_ff_v<R>)
    return ff_sqrt(v);
  else
    return sqrt(v);
}
template <typename R>
__device__ __forceinline__ R real_fabs(R v) {
  if constexpr (is_ff_v<R>)
    return ff_fabs(v);
  else
    return fabs(v);
}

// acc + a * b inside a sum: one exact product and one two-sum, the result
// left unnormalised (its lo part collects the errors of the chain, which
// ff_norm folds in once at the end)
__device__ __forceinline__ FF ff_mac(FF acc, FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float s, t;
  two_sum(acc.hi, p, s, t);
  return FF(s, __fadd_rn(t, __fadd_rn(acc.lo, e)));
}
__device__ __forceinline__ FF ff_norm(FF v) {
  FF r;
  two_sum(v.hi, v.lo, r.hi, r.lo);
  return r;
}

// ---- unnormalised pair arithmetic -------------------------------------------
// Sums and products whose lo part is left as computed (no renormalisation).
// Every error stays below about 2^-48 times the operands' magnitude, which is
// what the operator needs: its accuracy is measured against the size of the
// values on a line, not against each intermediate result.
__device__ __forceinline__ FF ffu_add(FF a, FF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return FF(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ FF ffu_sub(FF a, FF b) { return ffu_add(a, FF(-b.hi, -b.lo)); }
__device__ __forceinline__ FF ffu_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return FF(p, e);
}
__device__ __forceinline__ FF ffu_norm(FF v) {
  FF r;
  fast_two_sum(v.hi, v.lo, r.hi, r.lo);
  return r;
}

// ---- anchored sums of products ----------------------------------------------
// A dot product sum_j c_j x_j of float pairs, accumulated on top of an anchor
// S, a power of two with S >= 2 sum_j |c_j x_j| (so every partial sum plus S
// stays in [S/2, 3S/2]).  With acc' = fma(c, x, acc) the increment actually
// taken, t = acc' - acc, is exact (both lie on the grid of S 2^-24 and differ
// by less than S), and r = fma(c, x, -t) is the part of the exact product
// c x that acc' missed, |r| <= S 2^-24, rounded once.  r and the cross terms
// of the pairs' lo parts go to a plain float sum lo.  The result
// (acc - S) + lo, an unevaluated pair, carries an error of about
// n^2 2^-48 S: the same size as a float-float dot product's, at half of its
// instructions (6 per term against the two-sum's 12).  Two sums on the same
// anchor also add exactly: (acc_a - S) + (acc_b - S) is a float.
struct AAcc {
  float a, l;
};
__device__ __forceinline__ AAcc aa_init(float S) { return AAcc{S, 0.f}; }
__device__ __forceinline__ void aa_add(AAcc& s, FF c, FF x) {
  const float a1 = __fmaf_rn(c.hi, x.hi, s.a);
  const float t = __fsub_rn(a1, s.a);
  const float r = __fmaf_rn(c.hi, x.hi, -t);
  float l = __fadd_rn(s.l, r);
  l = __fmaf_rn(c.lo, x.hi, l);
  l = __fmaf_rn(c.hi, x.lo, l);
  s.a = a1;
  s.l = l;
}
// the sum as a pair (acc - S is exact)
__device__ __forceinline__ FF aa_value(const AAcc& s, float S) { return FF(__fsub_rn(s.a, S), s.l); }
// y_i = a_i + b_i and y_{n-1-i} = b_i - a_i of two sums on the same anchor:
// exact in the hi parts
__device__ __forceinline__ void aa_pm(const AAcc& a, const AAcc& b, float S, FF& plus, FF& minus) {
  const float ha = __fsub_rn(a.a, S), hb = __fsub_rn(b.a, S);
  plus = FF(__fadd_rn(hb, ha), __fadd_rn(b.l, a.l));
  minus = FF(__fsub_rn(hb, ha), __fsub_rn(b.l, a.l));
}
// the smallest power of two >= 2 (1 + 2^-20) bound, for bound >= 0 (0 for 0)
__device__ __forceinline__ float anchor_for(float bound) {
  const float b = __fmul_rn(bound, 2.000002f);
  return __uint_as_float((__float_as_uint(b) + 0x007fffffu) & 0xff800000u);
}

// read-only load of a pair (8-byte aligned: arrays of FF)
template <>
__device__ __forceinline__ FF load_nc<FF>(const FF* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return FF(v.x, v.y);
}

}  // namespace ew
