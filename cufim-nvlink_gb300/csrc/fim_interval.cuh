// fim_interval.cuh -- FP32 interval enclosures of the reference's FP64
// local-solver arithmetic (cuda_fim.h:1256-1360), used to decide cheaply
// which candidates can be the minimum of a vertex update, so that only
// those are evaluated in (slow, on GB300) FP64.
//
// Soundness: every interval below encloses the value that the FP64
// expression of the reference takes, not only the exact real value.  Each
// binary operation is evaluated with directed rounding (__f*_rd/__f*_ru),
// which encloses the exact result for every operand pair in the input
// intervals, and is then widened by one FP32 step in each direction.  One
// FP32 step is at least 2^-24 relative (or 2^-149 absolute near zero),
// which covers the <= 2^-53 relative (or 2^-1075 absolute) rounding of the
// corresponding FP64 operation, so by induction the enclosure holds through
// the whole expression.  Float casts of the reference (its triangle
// solver's float intermediates) round to the nearest float of a value that
// lies between two float bounds, so they stay inside the interval.  A
// non-finite bound or a divisor interval containing 0 yields the whole real
// line, which makes every decision "uncertain" and sends the candidate to
// the exact FP64 path.
#pragma once

#include <cfloat>
#include <cstdint>

namespace fimgb {

struct Iv {
  float lo, hi;
};

#define FIM_TINYF 1.40129846e-45f  // smallest subnormal float

__device__ __forceinline__ Iv iv_make(float lo, float hi) { Iv r; r.lo = lo; r.hi = hi; return r; }
__device__ __forceinline__ Iv iv_all() { return iv_make(-INFINITY, INFINITY); }
__device__ __forceinline__ Iv iv_d(double x) { return iv_make(__double2float_rd(x), __double2float_ru(x)); }
__device__ __forceinline__ bool iv_finite(Iv a) { return isfinite(a.lo) && isfinite(a.hi); }
// one float step outward: covers the FP64 rounding of the modelled operation
__device__ __forceinline__ Iv iv_widen(Iv a) { return iv_make(__fsub_rd(a.lo, FIM_TINYF), __fadd_ru(a.hi, FIM_TINYF)); }

__device__ __forceinline__ Iv iv_add(Iv a, Iv b)
{
  return iv_widen(iv_make(__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)));
}
__device__ __forceinline__ Iv iv_sub(Iv a, Iv b)
{
  return iv_widen(iv_make(__fsub_rd(a.lo, b.hi), __fsub_ru(a.hi, b.lo)));
}
__device__ __forceinline__ Iv iv_neg(Iv a) { return iv_make(-a.hi, -a.lo); }
__device__ __forceinline__ Iv iv_mul(Iv a, Iv b)
{
  if (!iv_finite(a) || !iv_finite(b)) return iv_all();
  const float l0 = __fmul_rd(a.lo, b.lo), l1 = __fmul_rd(a.lo, b.hi), l2 = __fmul_rd(a.hi, b.lo), l3 = __fmul_rd(a.hi, b.hi);
  const float h0 = __fmul_ru(a.lo, b.lo), h1 = __fmul_ru(a.lo, b.hi), h2 = __fmul_ru(a.hi, b.lo), h3 = __fmul_ru(a.hi, b.hi);
  return iv_widen(iv_make(fminf(fminf(l0, l1), fminf(l2, l3)), fmaxf(fmaxf(h0, h1), fmaxf(h2, h3))));
}
// multiplication by an exact power of two (2, 0.5, -0.5, 2^m): exact in FP64
// unless it underflows, directed and widened here for FP32 range limits
__device__ __forceinline__ Iv iv_scale(Iv a, float k)
{
  if (k > 0.f) return iv_widen(iv_make(__fmul_rd(a.lo, k), __fmul_ru(a.hi, k)));
  return iv_widen(iv_make(__fmul_rd(a.hi, k), __fmul_ru(a.lo, k)));
}
// multiplication by 2^m (|m| <= 126)
__device__ __forceinline__ Iv iv_pow2(Iv a, int m)
{
  if (m > 126 || m < -126) return iv_all();
  return iv_scale(a, __int_as_float((m + 127) << 23));
}
// x*x of one FP64 value (tighter than a product of independent intervals)
__device__ __forceinline__ Iv iv_sqr(Iv a)
{
  if (!iv_finite(a)) return iv_all();
  if (a.lo >= 0.f) return iv_widen(iv_make(__fmul_rd(a.lo, a.lo), __fmul_ru(a.hi, a.hi)));
  if (a.hi <= 0.f) return iv_widen(iv_make(__fmul_rd(a.hi, a.hi), __fmul_ru(a.lo, a.lo)));
  const float m = fmaxf(-a.lo, a.hi);
  return iv_widen(iv_make(0.f, __fmul_ru(m, m)));
}
__device__ __forceinline__ Iv iv_div(Iv a, Iv b)
{
  if (!iv_finite(a) || !iv_finite(b) || (b.lo <= 0.f && b.hi >= 0.f)) return iv_all();
  const float l0 = __fdiv_rd(a.lo, b.lo), l1 = __fdiv_rd(a.lo, b.hi), l2 = __fdiv_rd(a.hi, b.lo), l3 = __fdiv_rd(a.hi, b.hi);
  const float h0 = __fdiv_ru(a.lo, b.lo), h1 = __fdiv_ru(a.lo, b.hi), h2 = __fdiv_ru(a.hi, b.lo), h3 = __fdiv_ru(a.hi, b.hi);
  return iv_widen(iv_make(fminf(fminf(l0, l1), fminf(l2, l3)), fmaxf(fmaxf(h0, h1), fmaxf(h2, h3))));
}
// square root of the part of the interval that is >= 0 (the caller decides
// separately what a negative argument means: the reference gets NaN there)
__device__ __forceinline__ Iv iv_sqrt(Iv a)
{
  const float lo = a.lo > 0.f ? a.lo : 0.f;
  if (!(a.hi >= 0.f)) return iv_all();
  return iv_widen(iv_make(__fsqrt_rd(lo), __fsqrt_ru(a.hi)));
}
// Outcome of a filtered candidate.  Candidates that certainly contribute
// nothing (rejected root, NaN value) are NONE; otherwise lb is a lower
// bound of every value the candidate can take and ub an upper bound when its
// value is certain to exist (else +inf).
enum : int { CAND_NONE = 0, CAND_SOME = 1 };

}  // namespace fimgb
