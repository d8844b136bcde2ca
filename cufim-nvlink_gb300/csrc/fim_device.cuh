// fim_device.cuh -- device arithmetic shared by the kernels of the GB300 FIM
// solver: exact float/double conversions, the reference's local solvers in
// FP64 (solve_tri_cu / solve_tet_cu, cuda_fim.h:1256-1360) and the tet prefix
// program, the corner relabelling, fp16 bound packing and the bounded grid
// barrier.  Included by every CUDA translation unit of the solver; all of
// them are compiled with -fmad=false (see fim_kernels.cu).
#pragma once

#include "fim_internal.h"
#include "fim_filter.cuh"

#include <cfloat>
#include <cstdint>
#include <cuda_fp16.h>

namespace fimgb {

#define FIM_INF DBL_MAX
#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------------------
// local solver, FP64 with the reference's float-typed triangle intermediates

// Exact float <-> double conversions and FP64 sign tests from the bit
// patterns (IEEE 754 binary32 / binary64), on the integer pipes: on GB300 a
// conversion or an FP64 comparison occupies the FP64 pipe like an FP64
// multiply.  Operands outside the normal range take the hardware
// instruction.

// (double)f, exact
__device__ __forceinline__ double f2d(float f)
{
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e - 1u < 254u)  // normal: rebias the exponent, widen the fraction
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                            ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
  return (double)f;  // zero, subnormal, infinity, NaN
}

// (float)x, round to nearest, ties to even
__device__ __forceinline__ float d2f(double x)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e - 897u < 254u) {  // the float is normal, or rounds up to infinity
    const uint32_t frac = (uint32_t)(b >> 29) & 0x7fffffu;
    const uint32_t rest = (uint32_t)b & 0x1fffffffu;  // the 29 bits dropped
    uint32_t r = ((e - 896u) << 23) | frac;
    r += (rest > 0x10000000u || (rest == 0x10000000u && (frac & 1u))) ? 1u : 0u;  // carries into the exponent
    return __uint_as_float(r | ((uint32_t)(b >> 32) & 0x80000000u));
  }
  return (float)x;  // zero, subnormal result, infinity, NaN
}

// (float)(x * 2^-s) for |s| <= 60, round to nearest, ties to even: the
// scaling is an exponent change, exact whenever the scaled double is normal
__device__ __forceinline__ float d2f_pow2(double x, int s)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ffu);
  const int es = e - s;  // biased exponent of x * 2^-s
  if (e != 0 && e != 0x7ff && (uint32_t)(es - 897) < 254u) {
    const uint32_t frac = (uint32_t)(b >> 29) & 0x7fffffu;
    const uint32_t rest = (uint32_t)b & 0x1fffffffu;
    uint32_t r = ((uint32_t)(es - 896) << 23) | frac;
    r += (rest > 0x10000000u || (rest == 0x10000000u && (frac & 1u))) ? 1u : 0u;
    return __uint_as_float(r | ((uint32_t)(b >> 32) & 0x80000000u));
  }
  return (float)(x * ldexp(1.0, -s));
}

// x > 0 (false for zeros and NaN)
__device__ __forceinline__ bool dgt0(double x)
{
  return (unsigned long long)__double_as_longlong(x) - 1ull < 0x7ff0000000000000ull;
}
// 0 < x < 1
__device__ __forceinline__ bool din01(double x)
{
  return (unsigned long long)__double_as_longlong(x) - 1ull < 0x3fefffffffffffffull;
}
// 0 < x < inf (false for NaN)
__device__ __forceinline__ bool dpos_finite(double x)
{
  return (unsigned long long)__double_as_longlong(x) - 1ull < 0x7fefffffffffffffull;
}
// x finite (not inf, not NaN)
__device__ __forceinline__ bool dfinite(double x)
{
  return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}
// x < 0 (false for zeros and NaN)
__device__ __forceinline__ bool dlt0(double x)
{
  return (unsigned long long)__double_as_longlong(x) - 0x8000000000000001ull < 0x7ff0000000000000ull;
}

// solve_tri_cu, cuda_fim.h:1256-1300
__device__ __forceinline__ double tri_ref(double e12, double e13, double e23, double p1, double p2)
{
  const double a = e23;
  const double b = -0.5 * (e12 + e23 - e13);
  const double c = e12;
  const double p12 = p2 - p1;
  // the reference's float casts as d2f / f2d (same values)
  float dv = d2f(p12 * p12 - c);
  const float sv = d2f(f2d(dv) * (b * b - a * c));
  // the reference compares the float intermediates after widening them to
  // double; comparing the floats themselves gives the same answers (NaN too)
  // without the FP64 conversions
  if (dv != 0.f && sv >= 0.f) {
    dv = d2f(c * f2d(dv));
    const float st = sqrtf(sv);
    const double dst = f2d(st), ddv = f2d(dv);
    const float l1 = d2f(-(b * p12 * p12 - b * c - dst * p12) / ddv);
    const float l2 = d2f(-(b * p12 * p12 - b * c + dst * p12) / ddv);
    const double dl1 = f2d(l1), dl2 = f2d(l2);
    float r1 = d2f(p2 - dl1 * p12 + sqrt(a + 2.0 * dl1 * b + f2d(l1 * l1) * c));
    if (!((l1 >= 0.f) && (l1 <= 1.f))) r1 = (float)FIM_INF;
    float r2 = d2f(p2 - dl2 * p12 + sqrt(a + 2.0 * dl2 * b + f2d(l2 * l2) * c));
    if (!((l2 >= 0.f) && (l2 <= 1.f))) r2 = (float)FIM_INF;
    return f2d(fminf(r1, r2));
  }
  return FIM_INF;
}

// solve_tet_cu, cuda_fim.h:1302-1360 (the reference's closed form, term for term)
__device__ __forceinline__ double tet_ref(double e13, double e23, double e34, double e12, double e14,
                                          double e24, double p1, double p2, double p3)
{
  const double a = e13;
  const double b = 0.5 * (e23 + e13 - e12);
  const double c = -0.5 * (e34 + e13 - e14);
  const double d = e23;
  const double e = -0.5 * (e34 + e23 - e24);
  const double f = e34;
  const double q13 = p3 - p1;
  const double q23 = p3 - p2;

  const double sqt =
    -e*e*c*d*d + a*d*d*d*d - (b*b*c - a*c*c)*f*f + ((b*b - a*c)*f*f -
    (e*e*c - a*d*d - 2.*(e*c - b*d)*e)*f)*q13*q13 - 2.*(e*e*c*d -
    2.*e*b*d*d + a*d*d*d + (b*b - a*c)*d*f)*q13*q23 + (e*e*c*c -
    2.*e*b*c*d + a*c*d*d + (b*b*c - a*c*c)*f)*q23*q23 + 2.*(e*c*d*d -
    b*d*d*d)*e + (e*e*c*c + (b*b - 2.*a*c)*d*d - 2.*(e*c*c - b*c*d)*e)*f;

  if (sqt < 0.) return FIM_INF;

  const double pa = e*c*d*d - b*d*d*d + (e*c - b*d)*f*q13*q13 - 2.*(e*c*d - b*d*d)*q13*q23 +
                    (e*c*c - b*c*d)*q23*q23 - (e*c*c - b*c*d)*f;
  const double pb = (d*d*d*d - 2.*c*d*d*f + c*c*f*f + (d*d*f - c*f*f)*q13*q13 -
                     2.*(d*d*d - c*d*f)*q13*q23 + (c*d*d - c*c*f)*q23*q23);

  const double la2 = (pa + sqt*(d*q13 - c*q23))/pb;
  const double lb2 = (pa - sqt*(d*q13 - c*q23))/pb;
  const double la1 = -((f*la2 + e)*q13 - (d*la2 + b)*q23)/(d*q13 - c*q23);
  const double lb1 = -((f*lb2 + e)*q13 - (d*lb2 + b)*q23)/(d*q13 - c*q23);

  double l3 = 1 - la1 - la2, ra = FIM_INF, rb = FIM_INF;
  if ((la1 > 0. && la1 < 1.) && (la2 > 0. && la2 < 1.) && l3 > 0.)
    ra = la1*p1 + la2*p2 + l3*p3 + sqrt(a + 2.*la1*b + la1*la1*c + 2.*la1*la2*d + 2.*la2*e + la2*la2*f);
  l3 = 1 - lb1 - lb2;
  if ((lb1 > 0. && lb1 < 1.) && (lb2 > 0. && lb2 < 1.) && l3 > 0.)
    rb = lb1*p1 + lb2*p2 + l3*p3 + sqrt(a + 2.*lb1*b + lb1*lb1*c + 2.*lb1*lb2*d + 2.*lb2*e + lb2*lb2*f);
  return fmin(ra, rb);
}

// The same tet solve with its long FP64 prefix (b, c, e, q13, q23, sqt, pa,
// pb, sqt*X) spread over a group of kDagLanes lanes: the generated level
// program (gen_tet_dag.py) gives each lane one DFMA per level on operands in
// the group's scratch S, so the prefix costs kDagLevels dependent FP64
// instructions instead of one per node.  The results are bit-identical to
// tet_ref (every node is one correctly rounded operation of the source's own
// expression tree).
#include "tet_dag.inc"

__device__ __forceinline__ double flip_sign(double x, uint32_t flip)
{
  return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)(flip != 0u) << 63));
}

// Runs the level program on scratch S (leaves already stored); gl is the
// lane's index in its group.  All lanes of the warp take part.
__device__ __forceinline__ void tet_dag_prefix(double *S, int gl)
{
#pragma unroll
  for (int lv = 0; lv < kDagLevels; ++lv) {
    const uint32_t w = kTetDagProg[lv][gl];
    const double A = flip_sign(S[w & 255u], w & (1u << 24));
    const double B = flip_sign(S[(w >> 8) & 255u], w & (1u << 25));
    const double C = flip_sign(S[(w >> 16) & 255u], w & (1u << 26));
    S[kDagLeaves + lv * kDagLanes + gl] = fma(A, B, C);
    __syncwarp();
  }
}

// One root of tet_ref from the prefix in S: second = false gives its "a"
// value (pa + sqt X), true its "b" value (pa - sqt X, written as
// pa + (-(sqt X)), which IEEE arithmetic rounds identically), so two lanes
// run one instruction stream and tet_ref's result is the fmin of their
// values.  The sign tests run on the integer pipes (dlt0, din01, dgt0).
__device__ __forceinline__ double tet_root_tail(const double *S, bool second)
{
  const double a = S[kDagLeafE13], d = S[kDagLeafE13 + 1], f = S[kDagLeafE13 + 2];
  const double b = S[kDagOut_b], c = S[kDagOut_c], e = S[kDagOut_e];
  const double p1 = S[kDagLeafP1], p2 = S[kDagLeafP1 + 1], p3 = S[kDagLeafP1 + 2];
  const double q13 = S[kDagOut_q13], q23 = S[kDagOut_q23];
  const double sqt = S[kDagOut_sqt];
  if (dlt0(sqt)) return FIM_INF;
  const double pa = S[kDagOut_pa], pb = S[kDagOut_pb], sx = S[kDagOut_sx], X = S[kDagOut_X];
  const double l2 = (pa + (second ? -sx : sx))/pb;
  const double l1 = -((f*l2 + e)*q13 - (d*l2 + b)*q23)/X;
  const double l3 = 1 - l1 - l2;
  double r = FIM_INF;
  if (din01(l1) && din01(l2) && dgt0(l3))
    r = l1*p1 + l2*p2 + l3*p3 + sqrt(a + 2.*l1*b + l1*l1*c + 2.*l1*l2*d + 2.*l2*e + l2*l2*f);
  return r;
}


// ---------------------------------------------------------------------------
// corner relabelling and bound packing (metric kernel and solve)

// Edge numbering of a tet with slots 0..3: (0,1) (0,2) (1,2) (0,3) (1,3) (2,3)
// (types.cpp:240-245).
__host__ __device__ constexpr int edge_index(int i, int j)
{
  return (i > j) ? edge_index(j, i) : (j == 1 ? 0 : (j == 2 ? (i == 0 ? 1 : 2) : 3 + i));
}
// For target slot t the other slots are relabelled "1","2","3" =
// (t+1)%4, (t+2)%4, (t+3)%4 (the reference's gray-code mapping,
// cuda_fim.h:41-48).  sel_of(t, k) is the edge index of the k-th relabelled
// edge e13, e23, e34, e12, e14, e24.
__host__ __device__ constexpr int sel_of(int t, int k)
{
  return k == 0 ? edge_index((t + 1) & 3, (t + 3) & 3)
       : k == 1 ? edge_index((t + 2) & 3, (t + 3) & 3)
       : k == 2 ? edge_index((t + 3) & 3, t)
       : k == 3 ? edge_index((t + 1) & 3, (t + 2) & 3)
       : k == 4 ? edge_index((t + 1) & 3, t)
       :          edge_index((t + 2) & 3, t);
}

// Two non-negative lower bounds as fp16 rounded towards -inf (so they stay
// lower bounds), packed low | high << 16.
__device__ __forceinline__ uint32_t half_pair_rd(float lo, float hi)
{
  return (uint32_t)__half_as_ushort(__float2half_rd(lo)) | ((uint32_t)__half_as_ushort(__float2half_rd(hi)) << 16);
}
__device__ __forceinline__ float half_lo(uint32_t w) { return __half2float(__ushort_as_half((unsigned short)(w & 0xffffu))); }
__device__ __forceinline__ float half_hi(uint32_t w) { return __half2float(__ushort_as_half((unsigned short)(w >> 16))); }

// ---------------------------------------------------------------------------
// bounded grid barrier

__device__ __forceinline__ uint64_t global_timer()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p)
{
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile_i32(const int32_t *p)
{
  return *(const volatile int32_t *)p;
}

// All blocks of the (co-resident) grid meet here.  One arrival word: block 0
// adds 2^31 - (nblocks - 1), every other block adds 1, so the top bit flips
// exactly when the last block arrives (and the low bits return to zero);
// everyone waits for the flip.  A block cannot be two flips behind, since the
// next flip needs its own arrival.  Every wait is bounded by timeout_ns of
// %globaltimer and by a spin cap; on expiry the block records KERR_TIMEOUT
// and the phase, and every block leaves the kernel at its next barrier.
// Returns false when the caller must return.
static __device__ bool grid_sync(FimCtl *ctl, uint32_t nblocks, uint64_t timeout_ns, int where)
{
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const uint32_t inc = blockIdx.x == 0 ? 0x80000000u - (nblocks - 1u) : 1u;
    __threadfence();
    const uint32_t old = atomicAdd(&ctl->bar_count, inc);
    const uint64_t t0 = global_timer();
    uint32_t spins = 0;
    while (((ld_acquire_u32(&ctl->bar_count) ^ old) & 0x80000000u) == 0u) {
      ++spins;
      if ((spins & 255u) == 0u) {
        if (ld_volatile_i32(&ctl->error) != KERR_NONE) { ok = 0; break; }
        if (global_timer() - t0 > timeout_ns || spins > (1u << 30)) {
          if (atomicCAS(&ctl->error, KERR_NONE, KERR_TIMEOUT) == KERR_NONE) ctl->error_where = where;
          ok = 0;
          break;
        }
      }
    }
    if (ok && ld_volatile_i32(&ctl->error) != KERR_NONE) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Order-preserving map of doubles to unsigned integers, so that the minimum
// of a vertex's candidates can be formed with integer atomicMin.
__device__ __forceinline__ unsigned long long dkey(double x)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(unsigned long long k)
{
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

}  // namespace fimgb
