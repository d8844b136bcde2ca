// fim_kernels.cu -- sm_103a kernels of the GB300 FIM eikonal solver.
//
// This translation unit is compiled with -fmad=false and without fast-math:
// every FP64 expression below is evaluated in the order written, with IEEE
// round-to-nearest division and square root and no fused multiply-adds, so
// the solver reproduces the reference's FP64 source semantics bit for bit
// (the reference's results are chaotic in the last bits: a 1e-6 relative
// change of the inputs moves single vertices by 1e-3 of max(t), so nothing
// weaker than bit-exact arithmetic can match it to 1e-4).
//
// Kernels
//  * fim_metric_kernel -- FP64 per-tet metric and squared edge norms
//    (compute_velocity_tensor_f3 + compute_geo, types.h:173-188,
//    types.cpp:227-257), written straight into the four corner records of
//    the tet in the relabelled order the local solver reads
//    (gray-code tables, cuda_fim.h:41-48), plus the three edge lengths.
//  * fim_solve_kernel -- one persistent cooperative launch for the whole
//    solve: reset + seeding (reset_states_gpu / update_events_gpu,
//    cuda_fim.cu:479-542, 632-683), per window update_states
//    (cuda_fim.cu:1790-1845), then FIM iterations with the phases of
//    compute_step (cuda_fim.cu:1992-2334) as global Jacobi steps over
//    compacted lists (narrow list, vertices frozen this iteration,
//    neighbours to re-solve), separated by a bounded grid barrier: four
//    phases per iteration with windows, two with one endless window.
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
// metric kernel

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

__global__ void fim_metric_kernel(const int32_t *__restrict__ tslots, const int64_t *__restrict__ cidx,
                                  const double *__restrict__ xyz, const double *__restrict__ fib,
                                  const double *__restrict__ cf, const double *__restrict__ ct,
                                  int64_t e0, int64_t e1, double *__restrict__ cgeo, float *__restrict__ cgf,
                                  uint4 *__restrict__ crec, unsigned long long *__restrict__ bad)
{
  // The speed terms 1/cf/cf and 1/ct/ct cost four FP64 divisions, and an
  // FP64 warp instruction costs the same for one active lane as for 32.  So
  // thread 0 of the block evaluates them for its own tet, and every warp
  // whose tets all have the same speeds (bit for bit) takes that result
  // instead of dividing: with piecewise-constant conduction most warps do.
  __shared__ double s_sp[4];  // thread 0's cf, ct and their 1/cf/cf, 1/ct/ct
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t eb = e0 + blockIdx.x * (int64_t)blockDim.x; eb < e1; eb += stride) {  // block-uniform
    const int64_t e = eb + threadIdx.x;
    const bool in = e < e1;
    const double cfe = in ? cf[e] : 0.0, cte = in ? ct[e] : 0.0;
    if (threadIdx.x == 0) {  // eb < e1: thread 0 is in range
      s_sp[0] = cfe; s_sp[1] = cte;
      s_sp[2] = 1. / cfe / cfe; s_sp[3] = 1. / cte / cte;
    }
    __syncthreads();
    const bool same = !in || (__double_as_longlong(cfe) == __double_as_longlong(s_sp[0]) &&
                              __double_as_longlong(cte) == __double_as_longlong(s_sp[1]));
    double vf, vs;
    if (__all_sync(0xffffffffu, same)) {
      vf = s_sp[2]; vs = s_sp[3];
    } else {
      vf = 1. / cfe / cfe; vs = 1. / cte / cte;
    }
    __syncthreads();  // s_sp is rewritten by the next round
    if (!in) continue;
    const double f0 = fib[3 * e + 0], f1 = fib[3 * e + 1], f2 = fib[3 * e + 2];
    // the input check of fim_set_conduction: positive finite speeds, finite
    // fibre; the first offending tet is reported
    // (sign and exponent tests on the integer pipes: the FP64 pipe is this
    // kernel's bound)
    if (!(dpos_finite(cfe) && dpos_finite(cte) && dfinite(f0) && dfinite(f1) && dfinite(f2)))
      atomicMin(bad, (unsigned long long)e);
    // compute_velocity_tensor_f3 (types.h:173-188)
    const double fa = f0*f0, fb = f0*f1, fc = f0*f2, fd = f1*f1, fe = f1*f2, ff = f2*f2;
    const double M0 = vf*fa + vs*(1. - fa);
    const double M1 = (vf - vs)*fb;
    const double M2 = (vf - vs)*fc;
    const double M3 = vf*fd + vs*(1. - fd);
    const double M4 = (vf - vs)*fe;
    const double M5 = vf*ff + vs*(1. - ff);
    const int32_t v0 = tslots[4 * e + 0], v1 = tslots[4 * e + 1];
    const int32_t v2 = tslots[4 * e + 2], v3 = tslots[4 * e + 3];
    const int32_t va[6] = {v0, v0, v1, v0, v1, v2};
    const int32_t vb[6] = {v1, v2, v2, v3, v3, v3};
    double g[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      // load_edge(a, b) = x_a - x_b (types.h:210-216); aMb_sym (types.h:165-171)
      const double ex = xyz[3 * (int64_t)va[k] + 0] - xyz[3 * (int64_t)vb[k] + 0];
      const double ey = xyz[3 * (int64_t)va[k] + 1] - xyz[3 * (int64_t)vb[k] + 1];
      const double ez = xyz[3 * (int64_t)va[k] + 2] - xyz[3 * (int64_t)vb[k] + 2];
      g[k] = (M0*ex + M1*ey + M2*ez)*ex + (M1*ex + M3*ey + M4*ez)*ey + (M2*ex + M4*ey + M5*ez)*ez;
    }
    // scale 2^-k (k even) of the float screen record: edge norms O(1).  The
    // largest norm by its bit pattern (the order of non-negative doubles;
    // a negative or NaN norm only turns the scaling off), its binary
    // exponent from the exponent field (a subnormal maximum is out of range
    // either way), all on the integer pipes
    long long gbits = __double_as_longlong(g[0]);
#pragma unroll
    for (int kk = 1; kk < 6; ++kk) gbits = max(gbits, __double_as_longlong(g[kk]));
    const double gmax = __longlong_as_double(gbits);
    const int ex = (int)((gbits >> 52) & 0x7ff) - 1022;  // frexp's exponent for a normal gmax
    int ks = ex & ~1;
    const bool ok = dpos_finite(gmax) && ks <= 50 && ks >= -50;
    if (!ok) ks = 0;
    const float tk = ldexpf(1.f, ks / 2);
    // FP32 copies of the edge norms (scaled) and of the three edge lengths
    // towards each corner: sqrtf of the scaled norm times 2^(k/2), within
    // 1.5 * 2^-24 of the FP64 sqrt the reference adds (the FP64 lengths
    // themselves are taken where an edge candidate is evaluated exactly)
    float gsc[6], len[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      gsc[k] = d2f_pow2(g[k], ks);  // (float)(g * 2^-ks)
      len[k] = sqrtf(gsc[k]) * tk;
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int64_t c = cidx[4 * e + t];
      double2 *o = reinterpret_cast<double2 *>(cgeo + kCgeoStride * c);
      o[0] = make_double2(g[sel_of(t, 0)], g[sel_of(t, 1)]);
      o[1] = make_double2(g[sel_of(t, 2)], g[sel_of(t, 3)]);
      o[2] = make_double2(g[sel_of(t, 4)], g[sel_of(t, 5)]);
      float4 *of = reinterpret_cast<float4 *>(cgf + kCgfStride * c);
      const float gs[6] = {gsc[sel_of(t, 0)], gsc[sel_of(t, 1)], gsc[sel_of(t, 2)],
                           gsc[sel_of(t, 3)], gsc[sel_of(t, 4)], gsc[sel_of(t, 5)]};
      float hb[4];
      corner_bounds(gs, ok ? ks : 0, hb);
      if (!ok) hb[0] = hb[1] = hb[2] = hb[3] = 0.f;
      of[0] = make_float4(gs[0], gs[1], gs[2], gs[3]);
      of[1] = make_float4(gs[4], gs[5], (float)ks, 0.f);
      // first-read record: the lengths and the bounds (fp16, rounded down, so
      // still lower bounds); its ids were written at mesh staging
      uint4 *rc = crec + kCrecWords * c;
      rc[0].w = half_pair_rd(hb[0], hb[1]);
      rc[1] = make_uint4(__float_as_uint(len[sel_of(t, 4)]), __float_as_uint(len[sel_of(t, 5)]),
                         __float_as_uint(len[sel_of(t, 2)]), half_pair_rd(hb[2], hb[3]));
    }
  }
}

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
__device__ bool grid_sync(FimCtl *ctl, uint32_t nblocks, uint64_t timeout_ns, int where)
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

// ---------------------------------------------------------------------------
// persistent solve

// Phase-time instrumentation (builds with -DFIM_PROBE only): thread 0 of
// every block adds the time since its previous mark to accumulator k of its
// block; the marks sit right after block barriers.
#ifdef FIM_PROBE
__device__ __forceinline__ void probe_mark(const FimDev &d, int k)
{
  __shared__ unsigned long long s_probe_t;
  if (threadIdx.x == 0) {
    const unsigned long long t = global_timer();
    if (k >= 0) d.probe[blockIdx.x * kProbeSlots + k] += t - s_probe_t;
    s_probe_t = t;
  }
}
__device__ __forceinline__ void probe_count(const FimDev &d, int k)
{
  if (threadIdx.x == 0) d.probe[blockIdx.x * kProbeSlots + k] += 1;
}
#define PROBE(k) probe_mark(d, (k))
#define PROBE_COUNT(k) probe_count(d, (k))
#else
#define PROBE(k) ((void)0)
#define PROBE_COUNT(k) ((void)0)
#endif
// accumulators
enum : int { kPrSetup = 0, kPrA, kPrB, kPrS, kPrD, kPrE, kPrMark, kPrBarrier, kPrLight, kPrBatches,
             kPrPhases };

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

// One block of 16 warps per SM: the FP64 solves of a batch are packed into
// as few warps as possible, and those warps sit on different SM
// sub-partitions (an FP64 warp instruction occupies its sub-partition's
// FP64 pipe for 64 cycles whatever its active lanes, so two blocks per SM
// would stack their FP64 warps on the same sub-partitions).
constexpr int kThreads = kSolveThreads;  // threads per block of the solve kernel
constexpr int kMarkLanes = 16;           // threads per frozen vertex in the neighbour marking
static_assert(kThreads % kMarkLanes == 0, "marking groups must tile the grid");
constexpr int kSlots = 160;         // vertices per batch (at most)
constexpr int kCornerCap = 3072;    // corners per batch
constexpr int kTriCap = kCornerCap * 6 / 5;  // triangle screens per batch (more are screened on the spot)
constexpr int kTetCap = kCornerCap; // tet screens per batch: never full
constexpr int kQcap = 768;          // exact solves queued per kind and batch (more run on the spot)
// Phase D runs the queued tets on at most kDagWarps warps, one group of
// kDagLanes lanes per tet (scratch: kDagGroups * kDagSlots doubles).
constexpr int kDagWarps = 10;
constexpr int kDagGroups = kDagWarps * 32 / kDagLanes;

// Update phases.  With windows (finite dt) an iteration runs the reference's
// four steps as four grid-synchronised phases: kNarrow4 (update the narrow
// list), the apply + neighbour marking, kMarked4 (re-solve the marked
// neighbours), the apply + next list.  With one endless window no vertex
// can leave the narrow list for "next" inside the window, so an iteration
// needs only two: kNarrow2 updates the narrow list and marks the downwind
// neighbours of the vertices it freezes, kMarked2 re-solves them, applies
// everything and builds the next list.
enum : int { kNarrow4 = 0, kMarked4 = 1, kNarrow2 = 2, kMarked2 = 3 };
__host__ __device__ constexpr bool is_marked_mode(int m) { return m == kMarked4 || m == kMarked2; }

// Order-preserving map of floats to unsigned integers (for atomicMin).
__device__ __forceinline__ unsigned int fkey(float x)
{
  const unsigned int b = __float_as_uint(x);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float funkey(unsigned int k)
{
  return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k);
}

// The state word of a vertex copy: state in the low 8 bits, the stamp of the
// iteration that last marked it for re-solving in the upper 24.
__device__ __forceinline__ uint32_t sw_state(uint32_t w) { return w & 0xffu; }
__device__ __forceinline__ uint32_t sw_stamp(uint32_t w) { return w >> 8; }
__device__ __forceinline__ uint32_t sw_make(uint32_t state, uint32_t stamp) { return state | (stamp << 8); }
// The state a re-solve phase sees: a vertex marked in this iteration counts
// as "neig" (cuda_fim.cu:2196-2204), whatever its word still says.
__device__ __forceinline__ uint32_t sw_seen(uint32_t w, bool marked_mode, uint32_t stamp)
{
  return (marked_mode && sw_stamp(w) == stamp) ? (uint32_t)ST_NEIG : sw_state(w);
}

// Shared memory of one batch of vertex updates.  Phase A loads everything a
// corner's screens and decisions need once; the later phases read it from
// here and go to global memory only for the FP64 operands of the solves
// that survive the screens (and their vertex ids, from the corner record
// phase A has read: not keeping 12 bytes of ids per corner here makes room
// for 3072 corners a batch).
struct BatchSh {
  int32_t vtx[kSlots];
  int32_t cnt[kSlots];              // corners of each vertex
  int64_t c0[kSlots];
  int32_t cp[kSlots + 1];           // corner prefix over the batch's vertices
  double old[kSlots];
  unsigned long long res[kSlots];   // dkey of the running minimum (exact values)
  unsigned int bhi[kSlots];         // fkey of a float upper bound of the new time
  int64_t n0[kSlots];               // kNarrow2: neighbourhood range of each vertex (marking)
  int32_t ncnt[kSlots];
  uint8_t tsv[kSlots];              // kMarked2: tmp_state of each vertex
  int32_t fz[kSlots];               // kNarrow2: slots frozen in this batch
  // per corner of the batch
  union {
    struct {
      float pf[kCornerCap][3];      // their float times
      float sf[kCornerCap][3];      // float edge lengths sqrt(e14), sqrt(e24), sqrt(e34)
    };
    double dag[kDagGroups][kDagSlots];  // phase D (where pf and sf are dead): scratch of the tet prefix groups
  };
  uint32_t hb[kCornerCap][2];       // root-term bounds of pairs (1,2), (2,3) | (1,3), tet: fp16 pairs rounded down
  uint8_t vm[kCornerCap];           // validity bits of the three neighbours
  uint8_t cs[kCornerCap];           // slot of the corner's vertex
  // compacted screen lists: item (corner j | pair k << 16)
  uint32_t tri[kTriCap];
  uint32_t tet[kTetCap];
  uint32_t q[3][kQcap];             // queued exact solves: [0] tets, [1] triangles, [2] edges
  float qlb[3][kQcap];              // their lower bounds (rechecked against the final bhi)
  int ntri, ntet, nq[3];
  int next_item;                    // next unclaimed screen item (phase S)
  int nslot;                        // vertices of the current batch
  int nfz;                          // kNarrow2: frozen slots of the batch
};

static_assert(sizeof(double) * kDagGroups * kDagSlots <= sizeof(float) * kCornerCap * 6,
              "the tet prefix scratch must fit in the arrays it overlays");

// Queue item: slot (8 bits) | kind (2 bits) | corner index in the batch (22 bits).
// kind: triangle pair 0..2 or 3 (tet) in queues 0 and 1, edge 0..2 in queue 2.
static_assert(kSlots <= 256 && kCornerCap <= (1 << 22), "queue item fields");
__device__ __forceinline__ uint32_t make_item(int slot, int kind, int j)
{
  return (uint32_t)slot | ((uint32_t)kind << 8) | ((uint32_t)j << 10);
}
__device__ __forceinline__ int item_slot(uint32_t it) { return (int)(it & 255u); }
__device__ __forceinline__ int item_kind(uint32_t it) { return (int)((it >> 8) & 3u); }
__device__ __forceinline__ int item_corner(uint32_t it) { return (int)(it >> 10); }

// Appends one item per lane with `need` to a list (warp-ballot compaction;
// every lane of the warp takes part).  Returns the item's position, or -1.
__device__ __forceinline__ int warp_append(int *counter, bool need, int lane)
{
  const unsigned mask = __ballot_sync(FULL_MASK, need);
  if (mask == 0) return -1;
  int base = 0;
  if (lane == 0) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(FULL_MASK, base, 0);
  return need ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

// One FP64 local solve of corner c with neighbours nb, on the times ph:
// kind 0..2 are the triangle solves (1,2), (2,3), (1,3) and kind 3 the tet solve.
__device__ __forceinline__ double exact_solve(const FimDev &d, const double *ph, int64_t c, int kind,
                                              const int32_t *nb)
{
  const double p1 = __ldcg(ph + nb[0]), p2 = __ldcg(ph + nb[1]), p3 = __ldcg(ph + nb[2]);
  const double2 *gp = reinterpret_cast<const double2 *>(d.cgeo + kCgeoStride * c);
  const double2 t0 = __ldg(gp), t1 = __ldg(gp + 1), t2 = __ldg(gp + 2);
  if (kind == 3) return tet_ref(t0.x, t0.y, t1.x, t1.y, t2.x, t2.y, p1, p2, p3);
  // the pair's operands are selected first, so that a warp whose lanes hold
  // different pairs runs one triangle solve, not one per pair:
  // (1,2): tri(e12, e14, e24, p1, p2); (2,3): tri(e23, e24, e34, p2, p3);
  // (1,3): tri(e13, e14, e34, p1, p3)
  const double e12 = kind == 0 ? t1.y : (kind == 1 ? t0.y : t0.x);
  const double e13 = kind == 1 ? t2.y : t2.x;
  const double e23 = kind == 0 ? t2.y : t1.x;
  const double pa = kind == 1 ? p2 : p1;
  const double pb = kind == 0 ? p2 : p3;
  return tri_ref(e12, e13, e23, pa, pb);
}

// FP64 triangle solve kind 0..2 of corner c (exact_solve without its tet
// branch, for the warps that run only triangle solves).
__device__ __forceinline__ double exact_tri(const FimDev &d, const double *ph, int64_t c, int kind,
                                            const int32_t *nb)
{
  const double pa = __ldcg(ph + (kind == 1 ? nb[1] : nb[0])), pb = __ldcg(ph + (kind == 0 ? nb[1] : nb[2]));
  const double2 *gp = reinterpret_cast<const double2 *>(d.cgeo + kCgeoStride * c);
  const double2 t0 = __ldg(gp), t1 = __ldg(gp + 1), t2 = __ldg(gp + 2);
  const double e12 = kind == 0 ? t1.y : (kind == 1 ? t0.y : t0.x);
  const double e13 = kind == 1 ? t2.y : t2.x;
  const double e23 = kind == 0 ? t2.y : t1.x;
  return tri_ref(e12, e13, e23, pa, pb);
}

// Position of e14, e24, e34 (the edges from neighbour 0, 1, 2 to the corner's
// vertex) in a corner record.
__device__ __forceinline__ int edge_slot(int i) { return i == 0 ? 4 : (i == 1 ? 5 : 2); }

// Edge candidate i (time of neighbour i + its FP64 edge length) of corner c.
__device__ __forceinline__ double exact_edge(const FimDev &d, const double *ph, int64_t c, int i, int32_t nbi)
{
  return __ldcg(ph + nbi) + sqrt(__ldg(d.cgeo + kCgeoStride * c + edge_slot(i)));
}

// The other three vertices of corner c (from its first-read record, which
// phase A has just read: a cache hit).
__device__ __forceinline__ void corner_nb(const FimDev &d, int64_t c, int32_t *nb)
{
  const uint4 id = __ldg(d.crec + kCrecWords * c);
  nb[0] = (int32_t)id.x; nb[1] = (int32_t)id.y; nb[2] = (int32_t)id.z;
}
// nb[i] by selects (a runtime index would put nb in local memory)
__device__ __forceinline__ int32_t pick3(const int32_t *nb, int i) { return i == 0 ? nb[0] : (i == 1 ? nb[1] : nb[2]); }

// Evaluates queued item `it` (queue qi) in FP64 and folds it into the minimum.
__device__ __noinline__ void run_item(const FimDev &d, const double *ph, BatchSh &sh, int qi, uint32_t it)
{
  const int slot = item_slot(it), kind = item_kind(it), j = item_corner(it);
  const int64_t c = sh.c0[slot] + (j - sh.cp[slot]);
  int32_t nb[3];
  corner_nb(d, c, nb);
  const double val = qi == 2 ? exact_edge(d, ph, c, kind, pick3(nb, kind)) : exact_solve(d, ph, c, kind, nb);
  if (val < FIM_INF) atomicMin(&sh.res[slot], dkey(val));
}

// Queues an exact solve with lower bound lb (or runs it on the spot when the
// queue is full).  qi must be the same on every lane of the warp; the item's
// kind may differ.
__device__ __forceinline__ void queue_exact(const FimDev &d, const double *ph, BatchSh &sh, bool need, int qi,
                                            int kind, int slot, int j, float lb, int lane)
{
  const int pos = warp_append(&sh.nq[qi], need, lane);
  if (pos < 0) return;
  const uint32_t it = make_item(slot, kind, j);
  if (pos < kQcap) { sh.q[qi][pos] = it; sh.qlb[qi][pos] = lb; }
  else run_item(d, ph, sh, qi, it);
}

// FP32 screen record of batch corner j: e13, e23, e34, e12, e14, e24 times
// 2^-k and k (phase A has just read the record, so this hits the caches).
__device__ __forceinline__ void screen_record(const FimDev &d, const BatchSh &sh, int j, float *g)
{
  const int slot = sh.cs[j];
  const float4 *rp = reinterpret_cast<const float4 *>(d.cgf + kCgfStride * (sh.c0[slot] + (j - sh.cp[slot])));
  const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
  g[0] = r0.x; g[1] = r0.y; g[2] = r0.z; g[3] = r0.w; g[4] = r1.x; g[5] = r1.y; g[6] = r1.z;
}

// FP32 screens of triangle pair k (0: (1,2), 1: (2,3), 2: (1,3)) and of the
// tet of batch corner j.
__device__ __forceinline__ CandBound tri_screen_sm(const FimDev &d, const BatchSh &sh, int j, int k)
{
  float g[7];
  screen_record(d, sh, j, g);
  const float tk = re_pow2f((int)g[6]);
  // roles e12, e13, e23 of the pair's triangle solve (selects, no indexing)
  const float g12 = k == 0 ? g[3] : (k == 1 ? g[1] : g[0]);
  const float g13 = k == 1 ? g[5] : g[4];
  const float g23 = k == 0 ? g[5] : g[2];
  const float pa = k == 1 ? sh.pf[j][1] : sh.pf[j][0];
  const float pb = k == 0 ? sh.pf[j][1] : sh.pf[j][2];
  return tri_screen(re_scale(re_in(g12), tk), re_scale(re_in(g13), tk), re_scale(re_in(g23), tk), re_in(pa),
                    re_in(pb));
}

__device__ __forceinline__ CandBound tet_screen_sm(const FimDev &d, const BatchSh &sh, int j)
{
  float g[7];
  screen_record(d, sh, j, g);
  const Re gs[6] = {re_in(g[0]), re_in(g[1]), re_in(g[2]), re_in(g[3]), re_in(g[4]), re_in(g[5])};
  return tet_screen(gs, re_in(sh.pf[j][0]), re_in(sh.pf[j][1]), re_in(sh.pf[j][2]), (int)g[6]);
}

// A triangle pair that finds the screen list full: screened (and solved)
// on the spot; out of line, since it is rare and large.
__device__ __noinline__ void tri_list_full(const FimDev &d, const double *ph, BatchSh &sh, int j, int k, int slot,
                                           float bhi, bool exact_all)
{
  CandBound cb;
  if (exact_all) { cb.some = CAND_SOME; cb.lb = NAN; cb.ub = INFINITY; }
  else cb = tri_screen_sm(d, sh, j, k);
  if (cb.some && !(cb.lb > bhi)) run_item(d, ph, sh, 1, make_item(slot, k, j));
}

// The corners of a batch beyond kCornerCap (only a batch of one vertex, in
// slot 0, has them): every solve of them in FP64, the reference's validity
// on the FP64 times.  Returns the corners with a valid neighbour.
__device__ __noinline__ int64_t excess_corners(const FimDev &d, const double *ph, BatchSh &sh, int kept, int total,
                                               double lower, bool marked_mode, uint32_t stamp)
{
  int64_t n_valid = 0;
  for (int j = kept + (int)threadIdx.x; j < total; j += kThreads) {
    const int slot = 0;
    const int64_t c = sh.c0[slot] + (j - sh.cp[slot]);
    const uint4 id = __ldg(d.crec + kCrecWords * c);
    const int32_t nb[3] = {(int32_t)id.x, (int32_t)id.y, (int32_t)id.z};
    uint32_t m = 0;
    for (int i = 0; i < 3; ++i) {
      const double p = __ldcg(ph + nb[i]);
      if (sw_seen(__ldcg(d.sw + nb[i]), marked_mode, stamp) >= ST_NARROW && p > lower) {
        m |= 1u << i;
        atomicMin(&sh.res[slot], dkey(p + sqrt(__ldg(d.cgeo + kCgeoStride * c + edge_slot(i)))));
      }
    }
    if (m) ++n_valid;
    for (int k = 0; k < 4; ++k) {
      const bool use = k == 3 ? m == 7u : (((m >> (k == 1 ? 1 : 0)) & 1u) && ((m >> (k == 0 ? 1 : 2)) & 1u));
      if (!use) continue;
      const double val = exact_solve(d, ph, c, k, nb);
      if (val < FIM_INF) atomicMin(&sh.res[slot], dkey(val));
    }
  }
  return n_valid;
}

// Writes a time and its float copy.
__device__ __forceinline__ void set_phi(const FimDev &d, int64_t v, double x)
{
  d.phi[v] = x;
  d.phi_f[v] = (float)x;
}
// Writes a time into both time buffers and their float copies.
__device__ __forceinline__ void set_phi_both(const FimDev &d, int64_t v, double x)
{
  const float f = (float)x;
  d.phi[v] = x; d.phi_f[v] = f;
  d.phi2[v] = x; d.phi2_f[v] = f;
}

// Where an update phase appends the vertices of the next narrow list, and
// the counters of this iteration's lists.
struct ListOut {
  int32_t *next;      // next iteration's narrow list
  int32_t *n_next;    // its length
  int32_t *n_frozen;  // kNarrow4: vertices frozen now (lfrozen)
  int32_t *n_marked;  // kNarrow2: neighbours marked now (lmarked)
};

// One update phase over a vertex list.  Every block takes a contiguous part
// of the list and processes it in batches of up to kSlots vertices / up to
// kCornerCap corners, the corners of a batch spread over all threads:
//  A -- load every corner's first-read record once (neighbour ids, float
//       edge lengths, fp16 root-term bounds) and its neighbours' states and
//       float times; validity of the neighbours (state >= narrow and
//       phi > phi_start - front_width, on the float copies when conclusive,
//       else on the FP64 times), float edge bounds -> per-vertex upper
//       bound bhi of the new time;
//  B -- triangle and tet solves whose lower bound min(neighbour times) +
//       root-term bound does not exceed bhi are appended to compacted
//       screen lists (warp ballots);
//  S -- the FP32 screens run over the lists in chunks claimed by whichever
//       warp is free (tets, then triangles, then the edge checks); certain
//       upper bounds tighten bhi; a solve whose lower bound does not exceed
//       the current bhi is queued at once, and so are the edges that can
//       still be the minimum;
//  D -- the queued solves whose lower bound does not exceed the final bhi run
//       in FP64 (tet prefixes on 8-lane groups and their roots packed from
//       thread 0; triangles and edges each from a warp boundary);
//  E -- the reference's per-vertex decision on the exact minimum
//       (narrow vertices: window test (next), freeze test,
//       cuda_fim.cu:2125-2163; re-solved neighbours: keep or restore the
//       state, cuda_fim.cu:2255-2317), per MODE:
//   kNarrow4 -- new time into phi2, next / frozen-now;
//   kMarked4 -- new time into phi2, the decided state into dec;
//   kNarrow2 -- new time into phi2; the vertices frozen now mark their
//               downwind neighbours (cuda_fim.cu:2172-2205) at once: the
//               mark is the iteration stamp in the state word, which the
//               narrow updates running at the same time ignore;
//   kMarked2 -- new time into both buffers, the state decided and the
//               vertex appended to the next narrow list.
// Times are read from phi (narrow modes) or phi2 (kMarked2: the narrow
// list's new times live there until the phase applies them).  The minimum
// over everything equals the reference's update_per_element minimum over
// all corners (cuda_fim.h:1362-1411).
template <int MODE>
__device__ void update_phase(const FimDev &d, BatchSh &sh, const int32_t *list, int32_t n, double lower,
                             float lower_lo, float lower_hi, double phi_start, double dt, bool exact_all,
                             uint32_t stamp, const ListOut &lo_, int64_t &n_filtered, int64_t &n_exact)
{
  constexpr bool kMarkedMode = is_marked_mode(MODE);
  const double *ph = MODE == kMarked2 ? d.phi2 : d.phi;      // times this phase reads
  const float *phf = MODE == kMarked2 ? d.phi2_f : d.phi_f;
  constexpr int kPer = 3;  // corners per thread and group in phase A
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t per_block = ((int64_t)n + gridDim.x - 1) / gridDim.x;
  const int64_t lbeg = min((int64_t)n, (int64_t)blockIdx.x * per_block);
  const int64_t lend = min((int64_t)n, lbeg + per_block);
  int64_t pos = lbeg;
  while (pos < lend) {
    PROBE_COUNT(kPrBatches);
    // batch: the longest run of vertices with <= kCornerCap corners (>= 1 vertex)
    const int cand = (int)min((int64_t)kSlots, lend - pos);
    if (tid < cand) {
      const int32_t v = __ldcg(list + pos + tid);
      const double old = __ldcg(ph + v);
      sh.vtx[tid] = v;
      sh.c0[tid] = d.cptr[v];
      sh.cnt[tid] = (int32_t)(d.cptr[v + 1] - d.cptr[v]);
      sh.old[tid] = old;
      sh.res[tid] = dkey(old);
      sh.bhi[tid] = fkey(exact_all ? INFINITY : re_hi(re_in(__ldcg(phf + v))));
      if (MODE == kNarrow2) {
        const int64_t a = d.nptr[v];
        sh.n0[tid] = a;
        sh.ncnt[tid] = (int32_t)(d.nptr[v + 1] - a);
      }
      if (MODE == kMarked2) sh.tsv[tid] = __ldcg(d.tst + v);
    }
    if (tid == 0) {
      sh.cp[0] = 0;
      sh.ntri = 0; sh.ntet = 0; sh.nq[0] = 0; sh.nq[1] = 0; sh.nq[2] = 0; sh.next_item = 0; sh.nfz = 0;
    }
    __syncthreads();
    if (tid < 32) {
      // inclusive prefix of the corner counts (slot lane + 32 r in round r)
      // and the longest run of slots with <= kCornerCap corners, at least one
      int carry = 0, fit = 0;
#pragma unroll
      for (int r = 0; r < kSlots / 32; ++r) {
        const int sl = tid + 32 * r;
        int a = sl < cand ? sh.cnt[sl] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int u = __shfl_up_sync(FULL_MASK, a, o);
          if (tid >= o) a += u;
        }
        a += carry;
        sh.cp[sl + 1] = a;
        fit += __popc(__ballot_sync(FULL_MASK, sl < cand && a <= kCornerCap));
        carry = __shfl_sync(FULL_MASK, a, 31);
      }
      if (tid == 0) sh.nslot = max(1, fit);
    }
    __syncthreads();
    PROBE(kPrSetup);
    const int nslot = sh.nslot;
    const int total = sh.cp[nslot];     // may exceed kCornerCap for a single huge vertex
    const int kept = min(total, kCornerCap);

    // A: load, validity, float edge bounds.  Pass 1 loads every corner's
    // first-read record (ids, float lengths, fp16 bounds), pass 2 the
    // neighbours' states and float times; within a pass the loads of a
    // thread's corners are independent, so they are all in flight together.
    for (int jb = 0; jb < kept; jb += kPer * kThreads) {
      // all of a thread's record loads first, then the neighbour loads that
      // need their ids, then the stores: every load of a pass is in flight
      // at once
      int slot[kPer];
      uint4 h0[kPer], h1[kPer];
#pragma unroll
      for (int r = 0; r < kPer; ++r) {
        const int j = jb + tid + r * kThreads;
        slot[r] = 0;
        h0[r] = make_uint4(0u, 0u, 0u, 0u);
        h1[r] = h0[r];
        if (j < kept) {
          int lo = 0, hi = nslot - 1;  // last slot with cp[slot] <= j
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sh.cp[mid] <= j) lo = mid; else hi = mid - 1;
          }
          slot[r] = lo;
          const int64_t c = sh.c0[lo] + (j - sh.cp[lo]);
          h0[r] = __ldg(d.crec + kCrecWords * c);
          h1[r] = __ldg(d.crec + kCrecWords * c + 1);
        }
      }
      float pf[kPer][3];
      uint8_t stn[kPer][3];
#pragma unroll
      for (int r = 0; r < kPer; ++r) {
        const int j = jb + tid + r * kThreads;
        if (j < kept) {
          const int32_t nbs[3] = {(int32_t)h0[r].x, (int32_t)h0[r].y, (int32_t)h0[r].z};
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            pf[r][i] = __ldcg(phf + nbs[i]);
            stn[r][i] = (uint8_t)sw_seen(__ldcg(d.sw + nbs[i]), kMarkedMode, stamp);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < kPer; ++r) {
        const int j = jb + tid + r * kThreads;
        if (j < kept) {
          sh.hb[j][0] = h0[r].w;
          sh.hb[j][1] = h1[r].w;
          sh.sf[j][0] = __uint_as_float(h1[r].x); sh.sf[j][1] = __uint_as_float(h1[r].y);
          sh.sf[j][2] = __uint_as_float(h1[r].z);
          sh.cs[j] = (uint8_t)slot[r];
        }
      }
#pragma unroll
      for (int r = 0; r < kPer; ++r) {
        const int j = jb + tid + r * kThreads;
        if (j >= kept) continue;
        uint32_t m = 0;
        float ub = INFINITY;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const Re P = re_in(pf[r][i]);
          bool ok = stn[r][i] >= ST_NARROW;
          if (ok) {
            if (re_lo(P) > lower_hi) ok = true;
            else if (re_hi(P) <= lower_lo) ok = false;
            else {  // rare: the FP64 time decides
              int32_t nb[3];
              corner_nb(d, sh.c0[slot[r]] + (j - sh.cp[slot[r]]), nb);
              ok = __ldcg(ph + pick3(nb, i)) > lower;
            }
          }
          if (ok) {
            m |= 1u << i;
            ub = fminf(ub, re_hi(P + re_len(sh.sf[j][i])));
          }
          sh.pf[j][i] = pf[r][i];
        }
        if (m) ++n_filtered;
        if (!exact_all && ub < INFINITY) atomicMin(&sh.bhi[slot[r]], fkey(ub));
        sh.vm[j] = (uint8_t)m;
      }
    }
    // corners beyond kCornerCap (a single vertex with very many corners):
    // every solve of them goes to FP64
    if (total > kept) n_filtered += excess_corners(d, ph, sh, kept, total, lower, kMarkedMode, stamp);
    __syncthreads();
    PROBE(kPrA);

    // B: screen lists
    for (int jb = 0; jb < kept; jb += kThreads) {
      const int j = jb + tid;
      const bool in = j < kept;
      int slot = 0;
      uint32_t m = 0;
      float bhi = 0.f, lb[4] = {0.f, 0.f, 0.f, 0.f};
      if (in) {
        slot = sh.cs[j];
        m = sh.vm[j];
        bhi = funkey(sh.bhi[slot]);
        // lower bounds of the triangle pairs and the tet: min(times) + root-term bound
        float lo[3], hi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const Re P = re_in(sh.pf[j][i]);
          lo[i] = re_lo(P);
          hi[i] = re_hi(P);
        }
        const uint32_t w0 = sh.hb[j][0], w1 = sh.hb[j][1];
        lb[0] = solve_lo(fminf(lo[0], lo[1]), fmaxf(hi[0], hi[1]), half_lo(w0));
        lb[1] = solve_lo(fminf(lo[1], lo[2]), fmaxf(hi[1], hi[2]), half_hi(w0));
        lb[2] = solve_lo(fminf(lo[0], lo[2]), fmaxf(hi[0], hi[2]), half_lo(w1));
        lb[3] = solve_lo(fminf(lo[0], fminf(lo[1], lo[2])), fmaxf(hi[0], fmaxf(hi[1], hi[2])), half_hi(w1));
      }
      // triangle pairs (1,2), (2,3), (1,3), appended together (one atomic
      // per warp for the three), then the tet
      bool need[3];
      unsigned msk[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int a = k == 1 ? 1 : 0, b = k == 0 ? 1 : 2;
        need[k] = in && ((m >> a) & 1u) && ((m >> b) & 1u) && !(lb[k] > bhi);
        msk[k] = __ballot_sync(FULL_MASK, need[k]);
      }
      const int n0 = __popc(msk[0]), n1 = __popc(msk[1]), n2 = __popc(msk[2]);
      if (n0 + n1 + n2 > 0) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&sh.ntri, n0 + n1 + n2);
        base = __shfl_sync(FULL_MASK, base, 0);
        const unsigned below = (1u << lane) - 1u;
        const int first[3] = {base, base + n0, base + n0 + n1};  // the warp's pair-0 items, then 1, then 2
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (!need[k]) continue;
          const int p = first[k] + __popc(msk[k] & below);
          if (p < kTriCap) {
            sh.tri[p] = (uint32_t)j | ((uint32_t)k << 16);
          } else {  // list full: screen here
            tri_list_full(d, ph, sh, j, k, slot, bhi, exact_all);
          }
        }
      }
      {
        const bool need = in && m == 7u && !(lb[3] > bhi);
        const int p = warp_append(&sh.ntet, need, lane);
        if (p >= 0) sh.tet[p] = (uint32_t)j;  // kTetCap == kCornerCap: never full
      }
    }
    __syncthreads();
    PROBE(kPrB);

    // S: screens over the compacted lists, handed out in chunks to whichever
    // warp is free -- tets first (32 per chunk, one per lane), then triangles
    // from the next chunk boundary (64 per chunk: each lane screens two with
    // the branch-free tri_screen_bf, so that the two chains interleave), so
    // that every chunk holds one kind, and last the edges of 32 corners per
    // chunk; a solve whose lower bound does not exceed the current bhi is
    // queued at once (bhi only decreases: phase D rechecks against the final
    // bound)
    {
      const int ntet = min(sh.ntet, kTetCap), ntri = min(sh.ntri, kTriCap);
      const int tri0 = (ntet + 31) & ~31;
      const int edge_c0 = tri0 + ((ntri + 63) / 64) * 32;  // claim index of the first edge chunk
      const int nclaim = edge_c0 + ((kept + 31) & ~31);
      for (;;) {
        // claims of 32: tet chunks, then triangle chunks of 64 (two per
        // lane), then edge chunks of 32 corners
        int cl = 0;
        if (lane == 0) cl = atomicAdd(&sh.next_item, 32);
        cl = __shfl_sync(FULL_MASK, cl, 0);
        if (cl >= nclaim) break;
        if (cl >= edge_c0) {
          // the edges that can still be the minimum
          const int j = cl - edge_c0 + lane;
          const bool in = j < kept;
          int slot = 0;
          uint32_t m = 0;
          float bhi = 0.f;
          if (in) { slot = sh.cs[j]; m = sh.vm[j]; bhi = funkey(sh.bhi[slot]); }
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const float le = in ? re_lo(re_in(sh.pf[j][i]) + re_len(sh.sf[j][i])) : 0.f;
            const bool need = in && ((m >> i) & 1u) && !(le > bhi);
            queue_exact(d, ph, sh, need, 2, i, slot, j, le, lane);
          }
          continue;
        }
        const int ib = cl < tri0 ? cl : tri0 + 2 * (cl - tri0);  // 32 claimed in the triangle range stand for 64
        if (ib < tri0) {
          const int i = ib + lane;
          bool need = false;
          int slot = 0, j = 0;
          float lb = 0.f;
          if (i < ntet) {
            j = (int)sh.tet[i];
            slot = sh.cs[j];
            CandBound cb;
            if (exact_all) { cb.some = CAND_SOME; cb.lb = NAN; cb.ub = INFINITY; }
            else cb = tet_screen_sm(d, sh, j);
            if (!exact_all && cb.some && cb.ub < INFINITY) atomicMin(&sh.bhi[slot], fkey(cb.ub));
            lb = isnan(cb.lb) ? -INFINITY : cb.lb;
            need = cb.some && !(lb > funkey(sh.bhi[slot]));
          }
          queue_exact(d, ph, sh, need, 0, 3, slot, j, lb, lane);
        } else {
          int jj[2], kk[2], sl[2];
          bool in[2];
          CandBound cb[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int i = ib + 32 * h + lane;
            in[h] = i < tri0 + ntri;
            const uint32_t it = in[h] ? sh.tri[i - tri0] : 0u;
            jj[h] = (int)(it & 0xffffu);
            kk[h] = (int)(it >> 16);
            sl[h] = sh.cs[jj[h]];
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            float g[7];
            screen_record(d, sh, jj[h], g);
            const float tk = re_pow2f((int)g[6]);
            const int k = kk[h], j = jj[h];
            const float g12 = k == 0 ? g[3] : (k == 1 ? g[1] : g[0]);
            const float g13 = k == 1 ? g[5] : g[4];
            const float g23 = k == 0 ? g[5] : g[2];
            const float pa = k == 1 ? sh.pf[j][1] : sh.pf[j][0];
            const float pb = k == 0 ? sh.pf[j][1] : sh.pf[j][2];
            cb[h] = tri_screen_bf(re_scale(re_in(g12), tk), re_scale(re_in(g13), tk), re_scale(re_in(g23), tk),
                                  re_in(pa), re_in(pb));
            if (exact_all) { cb[h].some = CAND_SOME; cb[h].lb = NAN; cb[h].ub = INFINITY; }
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            bool need = false;
            float lb = 0.f;
            if (in[h]) {
              if (!exact_all && cb[h].some && cb[h].ub < INFINITY) atomicMin(&sh.bhi[sl[h]], fkey(cb[h].ub));
              lb = isnan(cb[h].lb) ? -INFINITY : cb[h].lb;
              need = cb[h].some && !(lb > funkey(sh.bhi[sl[h]]));
            }
            queue_exact(d, ph, sh, need, 1, kk[h], sl[h], jj[h], lb, lane);
          }
        }
      }
    }
    __syncthreads();
    PROBE(kPrS);

    // D: exact solves; tets (a lane group each) from thread 0, triangles and
    // edges each from the next warp boundary
    {
      const int ntet = min(sh.nq[0], kQcap), ntri = min(sh.nq[1], kQcap), nedge = min(sh.nq[2], kQcap);
      // tets: one group of kDagLanes lanes per tet runs the prefix
      // (tet_dag_prefix); then the roots, two per tet, on consecutive
      // threads from thread 0, so that they fill as few warps as possible
      // (an FP64 warp instruction costs the same for any number of active
      // lanes); groups of kDagWarps warps at most, a loop uniform over the
      // tet warps, which meet at named barrier 1 between prefix and roots
      const int tet_warps = min(kDagWarps, (ntet * kDagLanes + 31) / 32);
      const int tri0 = 32 * tet_warps;
      if (tid < tri0) {
        const int grp = tid / kDagLanes, gl = tid % kDagLanes;
        double *S = sh.dag[grp];
        const int ngrp = tri0 / kDagLanes;
        for (int base = 0; base < ntet; base += ngrp) {
          const int pos = base + grp;
          int slot = 0;
          bool run = false;
          if (pos < ntet) {
            const uint32_t it = sh.q[0][pos];
            slot = item_slot(it);
            run = !(sh.qlb[0][pos] > funkey(sh.bhi[slot]));  // else overtaken by a later bound
            if (run) {
              const int jj = item_corner(it);
              const int64_t c = sh.c0[slot] + (jj - sh.cp[slot]);
              // leaves: e13 e23 e34 e12 e14 e24 p1 p2 (lanes 0..7), p3, 0.5 2.0 1.0 -0.0
              int32_t nb[3];
              corner_nb(d, c, nb);
              S[gl] = gl < 6 ? __ldg(d.cgeo + kCgeoStride * c + gl) : __ldcg(ph + (gl == 6 ? nb[0] : nb[1]));
              if (gl == 0) S[kDagLeafP1 + 2] = __ldcg(ph + nb[2]);
              else if (gl <= 4) S[kDagLeafConst + gl - 1] = gl == 1 ? 0.5 : (gl == 2 ? 2.0 : (gl == 3 ? 1.0 : -0.0));
            }
          }
          __syncwarp();
          tet_dag_prefix(S, gl);
          asm volatile("bar.sync 1, %0;" ::"r"(tri0) : "memory");
          const int rpos = base + (tid >> 1);  // root (tid & 1) of tet rpos
          if (tid < 2 * ngrp && rpos < ntet) {
            const uint32_t it = sh.q[0][rpos];
            const int rslot = item_slot(it);
            if (!(sh.qlb[0][rpos] > funkey(sh.bhi[rslot]))) {
              const double v = tet_root_tail(sh.dag[tid >> 1], (tid & 1) != 0);
              if ((tid & 1) == 0) ++n_exact;
              if (v < FIM_INF) atomicMin(&sh.res[rslot], dkey(v));
            }
          }
          asm volatile("bar.sync 1, %0;" ::"r"(tri0) : "memory");  // the next pass overwrites the scratch
        }
      }
      const int edge0 = tri0 + ((ntri + 31) & ~31);
      for (int j = tid; j < edge0 + nedge; j += kThreads) {  // threads past the tets' warps: concurrently
        int qi, pos;
        if (j < tri0) continue;
        else if (j < tri0 + ntri) { qi = 1; pos = j - tri0; }
        else if (j >= edge0) { qi = 2; pos = j - edge0; }
        else continue;
        const uint32_t it = sh.q[qi][pos];
        if (sh.qlb[qi][pos] > funkey(sh.bhi[item_slot(it)])) continue;  // overtaken by a later bound
        const int slot = item_slot(it), kind = item_kind(it), jj = item_corner(it);
        const int64_t c = sh.c0[slot] + (jj - sh.cp[slot]);
        int32_t nb[3];
        corner_nb(d, c, nb);
        const double val = qi == 2 ? exact_edge(d, ph, c, kind, pick3(nb, kind)) : exact_tri(d, ph, c, kind, nb);
        if (val < FIM_INF) atomicMin(&sh.res[slot], dkey(val));
        if (qi < 2) ++n_exact;
      }
    }
    __syncthreads();
    PROBE(kPrD);

    // E: decisions
    if (MODE == kNarrow4 || MODE == kMarked4) {
      if (tid < nslot) {
        const int slot = tid;
        const int32_t v = sh.vtx[slot];
        const double old = sh.old[slot];
        const double nw = dunkey(sh.res[slot]);
        d.phi2[v] = nw;
        if (MODE == kNarrow4) {
          d.tst[v] = ST_FAR;
          if (nw - phi_start > dt) {
            d.sw[v] = ST_NEXT;
          } else if (fabs(old - nw) < (1e-6 * (1 + (old + nw) * .5))) {
            d.tst[v] = ST_FROZEN;
            d.lfrozen[atomicAdd(lo_.n_frozen, 1)] = v;
          }
        } else {
          d.dec[pos + slot] = (nw < old) ? (uint8_t)ST_NARROW : __ldcg(d.tst + v);
        }
      }
    } else if (MODE == kNarrow2) {
      // the window test never fires (endless window)
      if (tid < nslot) {
        const int slot = tid;
        const int32_t v = sh.vtx[slot];
        const double old = sh.old[slot];
        const double nw = dunkey(sh.res[slot]);
        d.phi2[v] = nw;
        d.phi2_f[v] = (float)nw;
        uint8_t t = ST_FAR;
        if (fabs(old - nw) < (1e-6 * (1 + (old + nw) * .5))) {
          t = ST_FROZEN;
          sh.fz[atomicAdd(&sh.nfz, 1)] = slot;
        }
        d.tst[v] = t;
      }
      __syncthreads();
      PROBE(kPrE);
      // the downwind neighbours of the vertices frozen now (not narrow, later
      // time): stamped in their state word, first stamp wins; a group of
      // kMarkLanes threads per frozen vertex
      const int nfz = sh.nfz;
      for (int g = tid / kMarkLanes; g < nfz; g += kThreads / kMarkLanes) {
        const int slot = sh.fz[g];
        const double pn = dunkey(sh.res[slot]);
        const int64_t k0 = sh.n0[slot], k1 = k0 + sh.ncnt[slot];
        for (int64_t k = k0 + tid % kMarkLanes; k < k1; k += kMarkLanes) {
          const int32_t v = __ldg(d.nbr + k);
          const uint32_t w = __ldcg(d.sw + v);
          const double pv = __ldcg(d.phi2 + v);
          if (sw_state(w) != ST_NARROW && sw_stamp(w) != stamp && pn < pv) {
            if (atomicCAS(d.sw + v, w, sw_make(sw_state(w), stamp)) == w) {
              d.tst[v] = (uint8_t)sw_state(w);
              d.lmarked[atomicAdd(lo_.n_marked, 1)] = v;
            }
          }
        }
      }
    } else {  // kMarked2
      if (tid < kSlots) {  // whole warps: the next-list appends are warp-aggregated
        const int slot = tid;
        const bool in = slot < nslot;
        bool push = false;
        if (in) {
          const int32_t v = sh.vtx[slot];
          const double old = sh.old[slot];
          const double nw = dunkey(sh.res[slot]);
          const uint8_t tv = sh.tsv[slot];
          uint8_t sv = (nw < old) ? (uint8_t)ST_NARROW : tv;
          if (sv == ST_NARROW) {
            if (tv == ST_FROZEN) sv = ST_FROZEN;
            else push = true;
          }
          d.sw[v] = sw_make(sv, stamp);  // still marked for the re-solves running now
          set_phi_both(d, v, nw);
        }
        const int p = warp_append(lo_.n_next, push, lane);
        if (p >= 0) lo_.next[p] = sh.vtx[slot];
      }
    }
    __syncthreads();
    PROBE(MODE == kNarrow2 ? kPrMark : kPrE);
    pos += nslot;
  }
}

// Grid barrier with its wait accounted in the phase probe.
__device__ __forceinline__ bool grid_sync_probed(const FimDev &d, uint32_t nblocks, uint64_t timeout_ns, int where)
{
  PROBE(kPrLight);  // whatever ran since the last mark
  const bool ok = grid_sync(d.ctl, nblocks, timeout_ns, where);
  PROBE(kPrBarrier);
  (void)d;
  return ok;
}

// TWO: two grid-synchronised phases per iteration (one endless window),
// else four (windows); one instantiation each, so that each holds only the
// update phases it runs.
template <bool TWO>
__global__ void __launch_bounds__(kThreads, 1) fim_solve_kernel(FimDev d, FimParams p)
{
  FimCtl *ctl = d.ctl;
  const uint32_t nblocks = gridDim.x;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  int64_t my_evals = 0, my_updates = 0, my_exact = 0;
  int where = 0;
  extern __shared__ __align__(16) unsigned char fim_smem[];
  BatchSh &sh = *reinterpret_cast<BatchSh *>(fim_smem);
  PROBE(-1);

  // reset_states_gpu + update_events_gpu: phi = INF, far; seeds narrow.
  // (warm start: every vertex narrow at its given time instead)
  for (int64_t v = gtid; v < d.nV; v += nthreads) {
    const double x = d.phi_init ? d.phi_init[v] : FIM_INF;
    set_phi_both(d, v, x); d.sw[v] = x < FIM_INF ? ST_NARROW : ST_FAR; d.tst[v] = ST_FAR;
  }
  // failure-detection test hook: this block never arrives at the barrier (a
  // flag that nothing sets), so the others' bounded waits must expire
  if (p.withhold_block > 0 && (int64_t)blockIdx.x == (int64_t)p.withhold_block - 1) return;
  if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;
  for (int64_t i = gtid; i < d.nseed; i += nthreads) {
    const int32_t v = d.seed_v[i];
    set_phi_both(d, v, d.seed_t[i]); d.sw[v] = ST_NARROW;
  }
  if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;

  int64_t it = 0;  // global iteration counter (identical in every block)
  double cur_time = 0.0, phi_start = 0.0;
  for (int32_t step = 0; step < p.n_steps; ++step) {
    phi_start = cur_time;
    cur_time += p.dt;
    const double lower = phi_start - p.front_width;
    const float lower_lo = __double2float_rd(lower), lower_hi = __double2float_ru(lower);
    int s = (int)(it % 3);
    if (gtid == 0) {
      for (int k = 0; k < 3; ++k) { ctl->n_narrow[k] = 0; ctl->n_frozen[k] = 0; ctl->n_marked[k] = 0; }
    }
    // sync_step2 (cuda_fim.cu:1752-1787): every copy of a mesh vertex takes
    // the minimum over its copies; copies that were larger become narrow.
    // (The reference indexes its interface table with the thread id instead
    // of the loop index; that equals this whenever #vertices <= 256 *
    // #submeshes, i.e. one vertex per thread.)
    if (d.gptr) {
      for (int64_t g = gtid; g < d.nG; g += nthreads) {
        const int64_t k0 = d.gptr[g], k1 = d.gptr[g + 1];
        double mn = FIM_INF;
        for (int64_t k = k0; k < k1; ++k) {
          const double v = __ldcg(d.phi + d.gcopy[k]);
          if (v < mn) mn = v;
        }
        for (int64_t k = k0; k < k1; ++k) {
          const int32_t c = d.gcopy[k];
          if (mn < __ldcg(d.phi + c)) { set_phi_both(d, c, mn); d.sw[c] = ST_NARROW; }
        }
      }
    }
    if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;
    // update_states (cuda_fim.cu:1790-1845) -> narrow list of this window
    for (int64_t v = gtid; v < d.nV; v += nthreads) {
      uint8_t stv = (uint8_t)sw_state(d.sw[v]);
      if (stv == ST_NEXT) { stv = ST_NARROW; d.sw[v] = stv; }
      else if (p.apd >= 0.0 && stv == ST_FROZEN) {
        if (!(d.phi[v] + p.apd > cur_time)) d.sw[v] = ST_TAIL;
      } else if (p.apd >= 0.0 && stv == ST_TAIL) {
        if (!(d.phi[v] + p.apd / 0.91 > cur_time)) {
          set_phi_both(d, v, FIM_INF); d.sw[v] = ST_FAR;
        }
      }
      if (stv == ST_NARROW) d.list[s][atomicAdd(&ctl->n_narrow[s], 1)] = (int32_t)v;
    }
    if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;

    int64_t it_window = 0;
    for (;;) {
      s = (int)(it % 3);
      const int s1 = (int)((it + 1) % 3), s2 = (int)((it + 2) % 3);
      const int32_t nn = ld_volatile_i32(&ctl->n_narrow[s]);
      if (nn == 0) break;
      if ((p.max_iter > 0 && it_window >= p.max_iter) || it >= kMaxStampIterations) {
        if (gtid == 0 && atomicCAS(&ctl->error, KERR_NONE, KERR_MAX_ITER) == KERR_NONE) ctl->error_where = where;
        return;
      }
      const uint32_t stamp = (uint32_t)(it + 1);
      const int32_t *lst = d.list[s];
      int32_t *lnext = d.list[s1];
      if (gtid == 0) { ctl->n_narrow[s2] = 0; ctl->n_frozen[s2] = 0; ctl->n_marked[s2] = 0; }
      ListOut lo;
      lo.next = lnext; lo.n_next = &ctl->n_narrow[s1]; lo.n_frozen = &ctl->n_frozen[s];
      lo.n_marked = &ctl->n_marked[s];
      PROBE_COUNT(kPrPhases);

      if (TWO) {
        // X -- update the narrow list, mark the downwind neighbours of the
        // vertices frozen now (cuda_fim.cu:2102-2205)
        update_phase<kNarrow2>(d, sh, lst, nn, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, stamp,
                               lo, my_evals, my_exact);
        my_updates += (gtid == 0) ? nn : 0;
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;

        // Y -- apply the narrow list's times and states (the block's share
        // of the list, cuda_fim.cu:2291-2317), then re-solve the marked
        // neighbours (cuda_fim.cu:2215-2289), which read the new times from
        // phi2 and see every marked vertex as "neig"
        {
          const int64_t per_block = ((int64_t)nn + gridDim.x - 1) / gridDim.x;
          const int64_t lbeg = min((int64_t)nn, (int64_t)blockIdx.x * per_block);
          const int64_t lend = min((int64_t)nn, lbeg + per_block);
          for (int64_t i0 = lbeg; i0 < lend; i0 += kThreads) {
            const int64_t i = i0 + threadIdx.x;
            bool push = false;
            int32_t v = 0;
            if (i < lend) {
              v = lst[i];
              const uint32_t w = __ldcg(d.sw + v);
              const uint8_t tv = __ldcg(d.tst + v);
              const double x = __ldcg(d.phi2 + v);
              const float xf = __ldcg(d.phi2_f + v);
              if (sw_stamp(w) != stamp) {  // (a narrow vertex is never marked here)
                d.phi[v] = x;
                d.phi_f[v] = xf;
                if (sw_state(w) == ST_NARROW) {
                  if (tv == ST_FROZEN) d.sw[v] = ST_FROZEN;
                  else push = true;
                }
              }
            }
            const int pp = warp_append(lo.n_next, push, lane);
            if (pp >= 0) lnext[pp] = v;
          }
        }
        PROBE(kPrLight);
        const int32_t nm = ld_volatile_i32(&ctl->n_marked[s]);
        update_phase<kMarked2>(d, sh, d.lmarked, nm, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0,
                               stamp, lo, my_evals, my_exact);
        my_updates += (gtid == 0) ? nm : 0;
        ++it;
        ++it_window;
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;
      } else {
        // P1 -- solve on elements + reduce per vertex (cuda_fim.cu:2102-2163)
        update_phase<kNarrow4>(d, sh, lst, nn, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, stamp,
                               lo, my_evals, my_exact);
        my_updates += (gtid == 0) ? nn : 0;
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;

        // P2 -- apply the narrow times; mark downwind neighbours of the
        // vertices frozen now (cuda_fim.cu:2172-2205).  The two are
        // independent: the marking runs on groups of kMarkLanes threads from
        // the bottom of the grid, the apply on threads from the top, so that
        // their dependent load chains overlap.
        for (int64_t i = nthreads - 1 - gtid; i < nn; i += nthreads) {
          const int32_t v = lst[i];
          set_phi(d, v, __ldcg(d.phi2 + v));
        }
        const int32_t nf = ld_volatile_i32(&ctl->n_frozen[s]);
        for (int64_t i = gtid / kMarkLanes; i < nf; i += nthreads / kMarkLanes) {
          const int32_t n = d.lfrozen[i];
          const double pn = __ldcg(d.phi2 + n);
          for (int64_t k = d.nptr[n] + gtid % kMarkLanes; k < d.nptr[n + 1]; k += kMarkLanes) {
            // both loads at once; the word changes only by the exchange below,
            // so w is still v's word there unless another frozen vertex won
            const int32_t v = __ldg(d.nbr + k);
            const uint32_t w = __ldcg(d.sw + v);
            const double pv = __ldcg(d.phi2 + v);
            if (sw_state(w) != ST_NARROW && sw_stamp(w) != stamp && pn < pv) {
              if (atomicCAS(d.sw + v, w, sw_make(ST_NEIG, stamp)) == w) {
                d.tst[v] = (uint8_t)sw_state(w);
                d.lmarked[atomicAdd(&ctl->n_marked[s], 1)] = v;
              }
            }
          }
        }
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;

        // P3 -- solve elements for neighbours + reduce (cuda_fim.cu:2215-2289)
        const int32_t nm = ld_volatile_i32(&ctl->n_marked[s]);
        update_phase<kMarked4>(d, sh, d.lmarked, nm, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0,
                               stamp, lo, my_evals, my_exact);
        my_updates += (gtid == 0) ? nm : 0;
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;

        // P4 -- apply, update neighbour states, next narrow list (cuda_fim.cu:2291-2317):
        // the re-solved neighbours, then (one index space, so that both run
        // at once: they touch disjoint vertices) the narrow vertices that
        // were not re-solved
        for (int64_t i = gtid; i < (int64_t)nm + nn; i += nthreads) {
          if (i < nm) {
            const int32_t v = d.lmarked[i];
            uint8_t sv = __ldcg(d.dec + i);
            const uint8_t tv = __ldcg(d.tst + v);
            set_phi(d, v, __ldcg(d.phi2 + v));
            if (sv == ST_NARROW) {
              if (tv == ST_FROZEN) sv = ST_FROZEN;
              else lnext[atomicAdd(&ctl->n_narrow[s1], 1)] = v;
            }
            d.sw[v] = sw_make(sv, stamp);  // keeps the stamp: the narrow loop below skips it
          } else {
            // the three loads at once (a re-solved vertex's are not used)
            const int32_t v = lst[i - nm];
            const uint32_t w = __ldcg(d.sw + v);
            const uint8_t tv = __ldcg(d.tst + v);
            if (sw_stamp(w) == stamp) continue;  // re-solved above
            if (sw_state(w) == ST_NARROW) {
              if (tv == ST_FROZEN) d.sw[v] = ST_FROZEN;
              else lnext[atomicAdd(&ctl->n_narrow[s1], 1)] = v;
            }
          }
        }
        ++it;
        ++it_window;
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;
      }
    }
  }

  // local -> global gather (cuda_fim.cu:2466-2485): min time, max state;
  // with one submesh the states as bytes
  if (d.gptr) {
    for (int64_t g = gtid; g < d.nG; g += nthreads) {
      double mn = FIM_INF;
      uint8_t mx = ST_FAR;
      for (int64_t k = d.gptr[g]; k < d.gptr[g + 1]; ++k) {
        const int32_t c = d.gcopy[k];
        const double pc = __ldcg(d.phi + c);
        const uint8_t sc = (uint8_t)sw_state(__ldcg(d.sw + c));
        if (pc < mn) mn = pc;
        if (sc > mx) mx = sc;
      }
      d.phi_out[g] = mn;
      d.st_out[g] = mx;
    }
  } else {
    for (int64_t v = gtid; v < d.nV; v += nthreads) d.st[v] = (uint8_t)sw_state(__ldcg(d.sw + v));
  }

  // statistics
  __shared__ unsigned long long s_evals, s_exact;
  if (threadIdx.x == 0) { s_evals = 0; s_exact = 0; }
  __syncthreads();
  atomicAdd(&s_evals, (unsigned long long)my_evals);
  atomicAdd(&s_exact, (unsigned long long)my_exact);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd((unsigned long long *)&ctl->corner_evals, s_evals);
    atomicAdd((unsigned long long *)&ctl->exact_evals, s_exact);
  }
  if (gtid == 0) {
    ctl->iterations = it;
    atomicAdd((unsigned long long *)&ctl->vertex_updates, (unsigned long long)my_updates);
  }
}
// ---------------------------------------------------------------------------
// launch wrappers

cudaError_t launch_metric(const int32_t *tslots, const int64_t *cidx, const double *xyz,
                          const double *fib, const double *cf, const double *ct, int64_t e0, int64_t e1,
                          double *cgeo, float *cgf, uint4 *crec, unsigned long long *bad, cudaStream_t stream)
{
  if (e1 <= e0) return cudaSuccess;
  const int block = 256;
  int64_t grid = (e1 - e0 + block - 1) / block;
  if (grid > 152 * 64) grid = 152 * 64;
  fim_metric_kernel<<<(unsigned)grid, block, 0, stream>>>(tslots, cidx, xyz, fib, cf, ct, e0, e1, cgeo, cgf, crec,
                                                          bad);
  return cudaGetLastError();
}

cudaError_t solve_grid_size(int device, int block, int *grid)
{
  int sms = 0, per_sm = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fim_solve_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BatchSh));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fim_solve_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BatchSh));
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fim_solve_kernel<false>, block, sizeof(BatchSh));
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  *grid = sms * per_sm;
  return cudaSuccess;
}

cudaError_t launch_solve(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream)
{
  FimDev dd = d;
  FimParams pp = p;
  void *args[] = {&dd, &pp};
  const void *fn = p.two_phase ? (const void *)fim_solve_kernel<true> : (const void *)fim_solve_kernel<false>;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), args, sizeof(BatchSh), stream);
}

__global__ void fim_copy_kernel(const double *__restrict__ src, double *__restrict__ dst, int64_t n)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __ldcg(src + i);
}

cudaError_t launch_copy(const double *src, double *dst, int64_t n, cudaStream_t stream)
{
  if (n <= 0) return cudaSuccess;
  int64_t grid = (n + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  fim_copy_kernel<<<(unsigned)grid, 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError();
}

}  // namespace fimgb
