// fim_filter.cuh -- FP32 screens of the reference's triangle and tet local
// solves (solve_tri_cu, cuda_fim.h:1256-1300; solve_tet_cu, :1302-1360).
//
// Each screen evaluates the reference's FP64 expression operation by
// operation, in the same order, on FP32 values that carry a rigorous error
// bound ("running error analysis"): a value is (v, e) with the guarantee
// |v - x| <= e, where x is the value the reference's FP64 code computes for
// that subexpression (not only the exact real value).  Per operation the
// bound grows by the propagated input errors plus |v| * 2^-22, which covers
// the FP32 rounding of v (2^-24), the FP64 rounding of the reference
// (2^-53) and the float casts of the reference's triangle solve (2^-24), and
// by an absolute 1e-44 for subnormal rounding.  The error terms themselves
// are rounded, so every decision inflates them by (1 + 2^-14).  A screen
// answers: can the solve return a value at all, a lower bound of every value
// it can return, and an upper bound when a value is certain.  Only solves
// that can still be a vertex's minimum are then run in FP64.
//
// Inputs are float copies of the FP64 operands (round-to-nearest, relative
// error <= 2^-24): the squared edge norms scaled by 2^-k (k even, chosen per
// tet corner so that they are O(1)) and the times.  Scaling every edge norm
// by 2^-k and every time difference by 2^-k/2 scales each homogeneous
// intermediate of the reference by an exact power of two; the scale is
// removed exactly where the reference mixes degrees.
#pragma once

#include <cfloat>
#include <cstdint>

namespace fimgb {

struct Re {
  float v, e;
};

#define FIM_RE_U 0x1p-22f       // per-operation relative bound
#define FIM_RE_TINY 1e-44f      // absolute bound of a subnormal rounding
#define FIM_RE_SAFE 1.00006103515625f  // 1 + 2^-14: rounding of the bounds themselves

__device__ __forceinline__ Re re_make(float v, float e) { Re r; r.v = v; r.e = e; return r; }
// float copy of an FP64 operand (round to nearest)
__device__ __forceinline__ Re re_in(float v) { return re_make(v, fmaf(fabsf(v), 0x1p-24f, FIM_RE_TINY)); }
// float edge length (sqrtf of the scaled float norm times 2^(k/2)): within
// 1.5 * 2^-24 relative of the FP64 sqrt of the FP64 norm, plus an absolute
// 2^-48 for norms that the scaling pushes into the subnormal range
__device__ __forceinline__ Re re_len(float v) { return re_make(v, fmaf(fabsf(v), 0x1p-23f, 0x1p-48f)); }
__device__ __forceinline__ Re operator+(Re a, Re b)
{
  const float v = a.v + b.v;
  return re_make(v, fmaf(fabsf(v), FIM_RE_U, a.e + b.e + FIM_RE_TINY));
}
__device__ __forceinline__ Re operator-(Re a, Re b)
{
  const float v = a.v - b.v;
  return re_make(v, fmaf(fabsf(v), FIM_RE_U, a.e + b.e + FIM_RE_TINY));
}
__device__ __forceinline__ Re operator-(Re a) { return re_make(-a.v, a.e); }
__device__ __forceinline__ Re operator*(Re a, Re b)
{
  const float v = a.v * b.v;
  const float e = fmaf(fabsf(a.v), b.e, fmaf(fabsf(b.v), a.e, fmaf(a.e, b.e, fmaf(fabsf(v), FIM_RE_U, FIM_RE_TINY))));
  return re_make(v, e);
}
// exact multiplication by a power of two (2, 0.5, -0.5, 2^m)
__device__ __forceinline__ Re re_scale(Re a, float k) { return re_make(a.v * k, fmaf(a.e, fabsf(k), FIM_RE_TINY)); }
__device__ __forceinline__ float re_pow2f(int m) { return (m > 126 || m < -126) ? INFINITY : __int_as_float((m + 127) << 23); }
__device__ __forceinline__ Re re_div(Re a, Re b)
{
  const float d = fabsf(b.v) - b.e * FIM_RE_SAFE;
  if (!(d > 0.f)) return re_make(0.f, INFINITY);
  const float v = a.v / b.v;
  return re_make(v, fmaf(fabsf(v), FIM_RE_U, (a.e + fabsf(v) * b.e) / d + FIM_RE_TINY));
}
// square root of the non-negative part (the caller decides what a possibly
// negative argument means: the reference gets NaN there)
__device__ __forceinline__ Re re_sqrt(Re a)
{
  const float v = sqrtf(fmaxf(a.v, 0.f));
  const float ea = a.e * FIM_RE_SAFE;
  const float e = v > 0.f ? fminf(ea / v, sqrtf(ea)) : sqrtf(ea);
  return re_make(v, fmaf(v, FIM_RE_U, e + FIM_RE_TINY));
}
__device__ __forceinline__ float re_err(Re a) { return fmaf(a.e, FIM_RE_SAFE, fabsf(a.v) * 0x1p-22f); }
__device__ __forceinline__ float re_lo(Re a) { return a.v - re_err(a); }
__device__ __forceinline__ float re_hi(Re a) { return a.v + re_err(a); }

enum : int { CAND_NONE = 0, CAND_SOME = 1 };

struct CandBound {
  int some;   // CAND_NONE: the solve certainly returns no value (INF or NaN)
  float lb;   // every value it can return is >= lb (NaN: no bound)
  float ub;   // it certainly returns a value <= ub (+inf when not certain)
};

// solve_tri_cu(e12, e13, e23, p1, p2) in true units (the reference's float
// intermediates make float range part of its semantics, so no rescaling: a
// bound that leaves the float range becomes an undecided case).
__device__ __forceinline__ CandBound tri_screen(Re e12, Re e13, Re e23, Re p1, Re p2)
{
  CandBound r;
  r.some = CAND_SOME;
  r.lb = INFINITY;
  r.ub = INFINITY;
  const Re P12 = p2 - p1;
  const Re A = e23, C = e12;
  const Re B = re_scale((e12 + e23) - e13, -0.5f);
  const Re DV = P12 * P12 - C;                    // float divident
  const Re SV = DV * (B * B - A * C);              // float sqrt_val
  if (re_hi(SV) < 0.f) { r.some = CAND_NONE; return r; }
  const bool cond_certain = (re_lo(DV) > 0.f || re_hi(DV) < 0.f) && re_lo(SV) >= 0.f;
  const Re DV2 = C * DV;
  const Re ST = re_sqrt(SV);                       // float sqrtTmp
  const Re BPC = (B * P12) * P12 - B * C;
  const Re SP = ST * P12;
  const Re L[2] = {re_div(-(BPC - SP), DV2), re_div(-(BPC + SP), DV2)};
  bool any = false, nan_lb = false;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const Re l = L[k];
    if (re_hi(l) < 0.f || re_lo(l) > 1.f) continue;      // rejected root
    const bool acc = re_lo(l) >= 0.f && re_hi(l) <= 1.f;
    const Re Q = (A + re_scale(l, 2.f) * B) + (l * l) * C;
    if (re_hi(Q) < 0.f) continue;                         // NaN value: dropped by fminf
    const Re V = (p2 - l * P12) + re_sqrt(Q);
    any = true;
    r.lb = fminf(r.lb, re_lo(V));
    if (cond_certain && acc && re_lo(Q) >= 0.f) r.ub = fminf(r.ub, re_hi(V));
    if (isnan(re_lo(V))) nan_lb = true;  // an overflowed bound of either root: no bound at all
  }
  if (nan_lb) r.lb = NAN;
  if (!any) r.some = CAND_NONE;
  return r;
}

// Branch-free division and square root (hardware approximations, no
// operand-range branches): __fdividef is within 2 ulp for divisors of
// magnitude in [2^-126, 2^126] (elsewhere the result gets no bound: e = inf);
// x rsqrtf(x) within 2.5 ulp for x >= 2^-126 (smaller x: value 0, error
// 2^-63 = sqrt(2^-126)).  The extra error is covered by |v| 2^-21; the error
// terms are raised by 2^-20 to stay upper bounds.
#define FIM_RE_APPROX 0x1p-21f
#define FIM_RE_UP 1.00000095367431640625f  // 1 + 2^-20
__device__ __forceinline__ Re re_div_bf(Re a, Re b)
{
  const float ay = fabsf(b.v);
  const float d = ay - b.e * FIM_RE_SAFE;
  const float v = __fdividef(a.v, b.v);
  const float prop = __fdividef(a.e + fabsf(v) * b.e, fmaxf(d, 0x1p-126f)) * FIM_RE_UP;
  const float e = fmaf(fabsf(v), FIM_RE_U + FIM_RE_APPROX, prop + FIM_RE_TINY);
  const bool ok = d > 0.f && ay >= 0x1p-126f && ay <= 0x1p126f;
  return re_make(ok ? v : 0.f, ok ? e : INFINITY);
}
__device__ __forceinline__ float sqrt_up_bf(float x)  // an upper bound of sqrt(x), x >= 0
{
  const float y = fmaxf(x, 0x1p-126f);
  return y * rsqrtf(y) * FIM_RE_UP * (1.f + 0x1p-21f);
}
__device__ __forceinline__ Re re_sqrt_bf(Re a)
{
  const float x = fmaxf(a.v, 0.f);
  const bool big = x >= 0x1p-126f;
  const float r = rsqrtf(fmaxf(x, 0x1p-126f));
  const float v = big ? x * r : 0.f;
  const float ea = a.e * FIM_RE_SAFE;
  const float e = fminf(big ? ea * r * FIM_RE_UP * (1.f + 0x1p-21f) : INFINITY, sqrt_up_bf(ea)) + (big ? 0.f : 0x1p-63f);
  return re_make(v, fmaf(v, FIM_RE_U + FIM_RE_APPROX, e + FIM_RE_TINY));
}

// tri_screen without branches (the same decisions, the two roots as
// independent chains), for lanes that screen two pairs at once.
__device__ __forceinline__ CandBound tri_screen_bf(Re e12, Re e13, Re e23, Re p1, Re p2)
{
  CandBound r;
  const Re P12 = p2 - p1;
  const Re A = e23, C = e12;
  const Re B = re_scale((e12 + e23) - e13, -0.5f);
  const Re DV = P12 * P12 - C;
  const Re SV = DV * (B * B - A * C);
  const bool none_sv = re_hi(SV) < 0.f;
  const bool cond_certain = (re_lo(DV) > 0.f || re_hi(DV) < 0.f) && re_lo(SV) >= 0.f;
  const Re DV2 = C * DV;
  const Re ST = re_sqrt_bf(SV);
  const Re BPC = (B * P12) * P12 - B * C;
  const Re SP = ST * P12;
  const Re L0 = re_div_bf(-(BPC - SP), DV2), L1 = re_div_bf(-(BPC + SP), DV2);
  bool any = false, nan_lb = false;
  float lb = INFINITY, ub = INFINITY;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const Re l = k == 0 ? L0 : L1;
    const Re Q = (A + re_scale(l, 2.f) * B) + (l * l) * C;
    const Re V = (p2 - l * P12) + re_sqrt_bf(Q);
    const bool use = !(re_hi(l) < 0.f || re_lo(l) > 1.f) && !(re_hi(Q) < 0.f);
    const bool acc = re_lo(l) >= 0.f && re_hi(l) <= 1.f;
    const float vl = re_lo(V);
    any = any || use;
    nan_lb = nan_lb || (use && isnan(vl));
    lb = use ? fminf(lb, vl) : lb;
    ub = (use && cond_certain && acc && re_lo(Q) >= 0.f) ? fminf(ub, re_hi(V)) : ub;
  }
  r.some = (none_sv || !any) ? CAND_NONE : CAND_SOME;
  r.lb = nan_lb ? NAN : lb;
  r.ub = none_sv ? INFINITY : ub;
  return r;
}

// solve_tet_cu with scaled edge norms gv = e13, e23, e34, e12, e14, e24
// (each times 2^-k, float copies), the float copies of the times p1..p3 and
// k.  kBf: the two roots as independent branch-free chains (re_div_bf,
// re_sqrt_bf; the same decisions), so that they interleave.
template <bool kBf>
__device__ __forceinline__ CandBound tet_screen_t(const float *gv, float p1f, float p2f, float p3f, int k, int *why)
{
  const Re g[6] = {re_in(gv[0]), re_in(gv[1]), re_in(gv[2]), re_in(gv[3]), re_in(gv[4]), re_in(gv[5])};
  const Re p1 = re_in(p1f), p2 = re_in(p2f), p3 = re_in(p3f);
  CandBound r;
  r.some = CAND_SOME;
  r.lb = NAN;
  r.ub = INFINITY;
  const float sq = re_pow2f(-k / 2);
  const Re Q13 = re_scale(p3 - p1, sq), Q23 = re_scale(p3 - p2, sq);
  const Re A = g[0];
  const Re B = re_scale((g[1] + g[0]) - g[3], 0.5f);
  const Re C = re_scale((g[2] + g[0]) - g[4], -0.5f);
  const Re D = g[1];
  const Re E = re_scale((g[2] + g[1]) - g[5], -0.5f);
  const Re F = g[2];

  const Re B2 = B * B, E2 = E * E;
  const Re AC = A * C, EC = E * C, BD = B * D, AD = A * D;
  const Re B2mAC = B2 - AC;
  const Re E2C = E2 * C;
  const Re ADD = AD * D, ADDD = ADD * D;
  const Re B2C = B2 * C, ACC = AC * C;
  const Re ECD = EC * D, ECDD = ECD * D;
  const Re BDD = BD * D, BDDD = BDD * D;
  const Re ECC = EC * C, BCD = (B * C) * D;
  const Re E2CC = E2C * C;
  const Re E2x = re_scale(E, 2.f);
  const Re ECCmBCD = ECC - BCD;

  const Re T0 = ((-E2C) * D) * D;
  const Re T1 = ADDD * D;
  const Re T2 = ((B2C - ACC) * F) * F;
  const Re K1 = (B2mAC * F) * F - ((E2C - ADD) - re_scale(EC - BD, 2.f) * E) * F;
  const Re K2 = re_scale(((E2C * D - ((E2x * B) * D) * D) + ADDD) + (B2mAC * D) * F, 2.f);
  const Re K3 = ((E2CC - ((E2x * B) * C) * D) + (AC * D) * D) + (B2C - ACC) * F;
  const Re T6 = re_scale(ECDD - BDDD, 2.f) * E;
  const Re T7 = ((E2CC + ((B2 - re_scale(A, 2.f) * C) * D) * D) - re_scale(ECCmBCD, 2.f) * E) * F;
  const Re S = (((((((T0 + T1) - T2) + (K1 * Q13) * Q13) - (K2 * Q13) * Q23) + (K3 * Q23) * Q23) + T6) + T7);
  if (re_hi(S) < 0.f) { r.some = CAND_NONE; if (why) *why = 0; return r; }  // sqt < 0: INF
  if (!(re_lo(S) >= 0.f)) { if (why) *why = 1; return r; }                 // undecided: FP64

  const Re PA = (((((ECDD - BDDD) + (((EC - BD) * F) * Q13) * Q13) - (re_scale(ECD - BDD, 2.f) * Q13) * Q23) +
                  (ECCmBCD * Q23) * Q23) - ECCmBCD * F);
  const Re D2 = D * D, DDD = D2 * D, CD = C * D, CF = C * F, C2 = C * C;
  const Re PB = (((((DDD * D - ((re_scale(C, 2.f) * D) * D) * F) + (C2 * F) * F) + ((D2 * F - CF * F) * Q13) * Q13) -
                  (re_scale(DDD - CD * F, 2.f) * Q13) * Q23) + ((CD * D - C2 * F) * Q23) * Q23);
  const Re X = D * Q13 - C * Q23;
  const Re SX = re_scale(S * X, re_pow2f(5 * k / 2));  // sqt*X without its extra 2^(-2.5k)
  const Re ONE = re_make(1.f, 0.f);
  const float sk = re_pow2f(k / 2);

  float lb = INFINITY, ub = INFINITY;
  bool any = false, nan_lb = false;
  if constexpr (kBf) {
#pragma unroll
    for (int root = 0; root < 2; ++root) {
      const Re L2 = re_div_bf(root == 0 ? PA + SX : PA - SX, PB);
      const Re L1 = re_div_bf(-((F * L2 + E) * Q13 - (D * L2 + B) * Q23), X);
      const Re L3 = (ONE - L1) - L2;
      const Re L1x2 = re_scale(L1, 2.f);
      const Re Qs = ((((A + L1x2 * B) + (L1 * L1) * C) + (L1x2 * L2) * D) + re_scale(L2, 2.f) * E) + (L2 * L2) * F;
      const Re V = ((L1 * p1 + L2 * p2) + L3 * p3) + re_scale(re_sqrt_bf(Qs), sk);
      const bool use = !(re_hi(L2) <= 0.f || re_lo(L2) >= 1.f) && !(re_hi(L1) <= 0.f || re_lo(L1) >= 1.f) &&
                       !(re_hi(L3) <= 0.f) && !(re_hi(Qs) < 0.f);
      const bool acc = re_lo(L1) > 0.f && re_hi(L1) < 1.f && re_lo(L2) > 0.f && re_hi(L2) < 1.f && re_lo(L3) > 0.f;
      const float vl = re_lo(V);
      any = any || use;
      nan_lb = nan_lb || (use && isnan(vl));
      lb = use ? fminf(lb, vl) : lb;
      ub = (use && acc && re_lo(Qs) >= 0.f) ? fminf(ub, re_hi(V)) : ub;
    }
  } else {
#pragma unroll
    for (int root = 0; root < 2; ++root) {
      const Re L2 = re_div(root == 0 ? PA + SX : PA - SX, PB);
      if (re_hi(L2) <= 0.f || re_lo(L2) >= 1.f) continue;
      const Re L1 = re_div(-((F * L2 + E) * Q13 - (D * L2 + B) * Q23), X);
      if (re_hi(L1) <= 0.f || re_lo(L1) >= 1.f) continue;
      const Re L3 = (ONE - L1) - L2;
      if (re_hi(L3) <= 0.f) continue;
      const bool acc = re_lo(L1) > 0.f && re_hi(L1) < 1.f && re_lo(L2) > 0.f && re_hi(L2) < 1.f && re_lo(L3) > 0.f;
      const Re L1x2 = re_scale(L1, 2.f);
      const Re Qs = ((((A + L1x2 * B) + (L1 * L1) * C) + (L1x2 * L2) * D) + re_scale(L2, 2.f) * E) + (L2 * L2) * F;
      if (re_hi(Qs) < 0.f) continue;  // NaN value, dropped by fmin
      const Re V = ((L1 * p1 + L2 * p2) + L3 * p3) + re_scale(re_sqrt(Qs), sk);
      any = true;
      const float vl = re_lo(V);
      if (isnan(vl)) nan_lb = true;
      lb = fminf(lb, vl);
      if (acc && re_lo(Qs) >= 0.f) ub = fminf(ub, re_hi(V));
    }
  }
  if (!any) { r.some = CAND_NONE; if (why) *why = 2; return r; }
  if (why) *why = 3;
  r.lb = nan_lb ? NAN : lb;
  r.ub = ub;
  return r;
}
__device__ __forceinline__ CandBound tet_screen(const float *gv, float p1f, float p2f, float p3f, int k,
                                                int *why = nullptr)
{
  return tet_screen_t<false>(gv, p1f, p2f, p3f, k, why);
}
__device__ __forceinline__ CandBound tet_screen_bf(const float *gv, float p1f, float p2f, float p3f, int k,
                                                   int *why = nullptr)
{
  return tet_screen_t<true>(gv, p1f, p2f, p3f, k, why);
}

// Per-corner lower bounds, in true units, of the square-root term of the
// reference's local solves, from the scaled squared edge norms
// g = e13, e23, e34, e12, e14, e24 (times 2^-k, k even):
//  * triangle pair (1,2), (2,3), (1,3): solve_tri_cu's root term is the
//    metric distance from the target "4" to the point l x_a + (1-l) x_b of
//    the pair's segment (its a + 2 l b + l^2 c is that squared distance), so
//    the distance from "4" to the segment bounds it: foot
//    lambda* = (Sb - (Sa + Sb - B)/2) / B; inside (0,1) the line distance
//    h^2 = (Sa Sb - ((Sa + Sb - B)/2)^2) / B, else min(Sa, Sb);
//  * tet: solve_tet_cu's root term is sqrt(Q(l1, l2)) with the reference's
//    Q = a + 2 l1 b + l1^2 c + 2 l1 l2 d + 2 l2 e + l2^2 f (cuda_fim.h:1302-1360;
//    not a distance), at an accepted root (l1, l2, 1 - l1 - l2 > 0), so the
//    minimum of Q over the closed triangle l1, l2 >= 0, l1 + l2 <= 1 bounds
//    it: the minimum over the three edges (1D quadratics) and, when the
//    Hessian is certainly positive definite, the unconstrained minimum.
// A solve's value is a convex combination of its times plus that term, so
// min(times) + bound is below every value it returns (up to roundings the
// caller adds).  Undecidable or degenerate cases give 0 (no bound).
__device__ __forceinline__ float root_lo(Re q, float emax, float tk)
{
  // the solves' own rounding of the squared term is absolute and below
  // 2^-23 emax (the triangle solve squares its float l: 2^-24 e12; FP64
  // roundings: below 2^-45 emax); then the rounding of the square root
  const float lo = re_lo(q) - 0x1p-22f * emax;
  if (!(lo > 0.f)) return 0.f;
  const float h = sqrtf(lo) * (1.f - 0x1p-22f);
  const float r = h * tk;
  return isfinite(r) ? r : 0.f;
}

__device__ __forceinline__ float segment_lo(Re B, Re Sa, Re Sb, float emax, float tk)
{
  const Re uw = re_scale((Sa + Sb) - B, 0.5f);
  const Re lam = re_div(Sb - uw, B);
  if (re_hi(lam) <= 0.f) return root_lo(Sb, emax, tk);
  if (re_lo(lam) >= 1.f) return root_lo(Sa, emax, tk);
  return root_lo(re_div(Sa * Sb - uw * uw, B), emax, tk);  // line distance <= segment distance
}

// re_lo, with NaN (an overflowed bound) turned into -inf, so that a minimum
// over candidates never drops it
__device__ __forceinline__ float safe_lo(Re a)
{
  const float l = re_lo(a);
  return l == l ? l : -INFINITY;
}

// Lower bound of the minimum over s in [0,1] of al + 2 be s + ga s^2.
__device__ __forceinline__ float quad01_lo(Re al, Re be, Re ga)
{
  const float ends = fminf(safe_lo(al), safe_lo((al + re_scale(be, 2.f)) + ga));
  if (re_hi(ga) <= 0.f) return ends;         // concave or linear: the minimum is at an end
  if (!(re_lo(ga) > 0.f)) return -INFINITY;  // curvature sign undecided: no bound
  const Re s = re_div(-be, ga);              // vertex of the parabola
  if (re_hi(s) <= 0.f || re_lo(s) >= 1.f) return ends;
  return fminf(ends, safe_lo(al - re_div(be * be, ga)));
}

__device__ __forceinline__ void corner_bounds(const float *gs, int k, float *h)
{
  const Re e13 = re_in(gs[0]), e23 = re_in(gs[1]), e34 = re_in(gs[2]);
  const Re e12 = re_in(gs[3]), e14 = re_in(gs[4]), e24 = re_in(gs[5]);
  float emax = 0.f;
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 6; ++i) { emax = fmaxf(emax, gs[i]); finite = finite && isfinite(gs[i]); }
  const float tk = re_pow2f(k / 2);
  h[0] = h[1] = h[2] = h[3] = 0.f;
  if (!finite || !(emax > 0.f) || !isfinite(tk)) return;
  h[0] = segment_lo(e12, e14, e24, emax, tk);   // pair (1,2)
  h[1] = segment_lo(e23, e24, e34, emax, tk);   // pair (2,3)
  h[2] = segment_lo(e13, e14, e34, emax, tk);   // pair (1,3)
  // the tet's Q with the reference's coefficients
  const Re A = e13;
  const Re B = re_scale((e23 + e13) - e12, 0.5f);
  const Re C = re_scale((e34 + e13) - e14, -0.5f);
  const Re D = e23;
  const Re E = re_scale((e34 + e23) - e24, -0.5f);
  const Re F = e34;
  float qmin = quad01_lo(A, B, C);                                   // l2 = 0
  qmin = fminf(qmin, quad01_lo(A, E, F));                            // l1 = 0
  qmin = fminf(qmin, quad01_lo((A + re_scale(B, 2.f)) + C,           // l1 = 1 - s, l2 = s
                               ((D + E) - B) - C, (C - re_scale(D, 2.f)) + F));
  // an interior minimum needs a positive definite Hessian (c > 0, cf - d^2 > 0);
  // unless that is excluded, the unconstrained minimum
  // a - (f b^2 - 2 d b e + c e^2) / (cf - d^2) joins the candidates (-inf when
  // the determinant's sign is undecided)
  const Re det = C * F - D * D;
  if (!(re_hi(C) <= 0.f || re_hi(det) <= 0.f)) {
    const Re num = ((F * B) * B - re_scale((D * B) * E, 2.f)) + (C * E) * E;
    qmin = fminf(qmin, safe_lo(A - re_div(num, det)));
  }
  h[3] = root_lo(re_make(qmin, 0.f), emax, tk);
}

// Lower bound of every value a triangle or tet solve can return, given the
// float lower bound m_lo of the minimum and an upper bound m_hi of the
// maximum of its times and the distance bound h: covers the float rounding
// of the sum and of the reference's float-typed triangle result and the FP64
// roundings of both solves.
__device__ __forceinline__ float solve_lo(float m_lo, float m_hi, float h)
{
  const float x = m_lo + h;
  return x - 0x1p-21f * (fabsf(m_lo) + fabsf(m_hi) + h);
}

}  // namespace fimgb
