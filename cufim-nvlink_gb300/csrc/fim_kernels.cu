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
//    neighbours to re-solve), separated by a bounded grid barrier.
#include "fim_internal.h"
#include "fim_filter.cuh"

#include <cfloat>
#include <cstdint>

namespace fimgb {

#define FIM_INF DBL_MAX
#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------------------
// local solver, FP64 with the reference's float-typed triangle intermediates

// solve_tri_cu, cuda_fim.h:1256-1300
__device__ __forceinline__ double tri_ref(double e12, double e13, double e23, double p1, double p2)
{
  const double a = e23;
  const double b = -0.5 * (e12 + e23 - e13);
  const double c = e12;
  const double p12 = p2 - p1;
  float dv = (float)(p12 * p12 - c);
  const float sv = (float)((double)dv * (b * b - a * c));
  if ((double)dv != 0.0 && (double)sv >= 0.0) {
    dv = (float)(c * (double)dv);
    const float st = sqrtf(sv);
    const float l1 = (float)(-(b * p12 * p12 - b * c - (double)st * p12) / (double)dv);
    const float l2 = (float)(-(b * p12 * p12 - b * c + (double)st * p12) / (double)dv);
    float r1 = (float)(p2 - (double)l1 * p12 + sqrt(a + 2.0 * (double)l1 * b + (double)(l1 * l1) * c));
    if (!(((double)l1 >= 0.0) && ((double)l1 <= 1.0))) r1 = (float)FIM_INF;
    float r2 = (float)(p2 - (double)l2 * p12 + sqrt(a + 2.0 * (double)l2 * b + (double)(l2 * l2) * c));
    if (!(((double)l2 >= 0.0) && ((double)l2 <= 1.0))) r2 = (float)FIM_INF;
    return (double)fminf(r1, r2);
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

__global__ void fim_metric_kernel(const int32_t *__restrict__ tslots, const int64_t *__restrict__ cidx,
                                  const double *__restrict__ xyz, const double *__restrict__ fib,
                                  const double *__restrict__ cf, const double *__restrict__ ct,
                                  int64_t nT, double *__restrict__ cgeo, float *__restrict__ cgf)
{
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nT;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double f0 = fib[3 * e + 0], f1 = fib[3 * e + 1], f2 = fib[3 * e + 2];
    const double fa = f0*f0, fb = f0*f1, fc = f0*f2, fd = f1*f1, fe = f1*f2, ff = f2*f2;
    const double vf = 1. / cf[e] / cf[e], vs = 1. / ct[e] / ct[e];
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
    double g[6], s[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      // load_edge(a, b) = x_a - x_b (types.h:210-216); aMb_sym (types.h:165-171)
      const double ex = xyz[3 * (int64_t)va[k] + 0] - xyz[3 * (int64_t)vb[k] + 0];
      const double ey = xyz[3 * (int64_t)va[k] + 1] - xyz[3 * (int64_t)vb[k] + 1];
      const double ez = xyz[3 * (int64_t)va[k] + 2] - xyz[3 * (int64_t)vb[k] + 2];
      g[k] = (M0*ex + M1*ey + M2*ez)*ex + (M1*ex + M3*ey + M4*ez)*ey + (M2*ex + M4*ey + M5*ez)*ez;
      s[k] = sqrt(g[k]);
    }
    // scale 2^-k (k even) of the float screen record: edge norms O(1)
    double gmax = g[0];
#pragma unroll
    for (int kk = 1; kk < 6; ++kk) gmax = fmax(gmax, g[kk]);
    int ex = 0;
    frexp(gmax, &ex);
    int ks = ex & ~1;
    const bool ok = isfinite(gmax) && gmax > 0.0 && ks <= 50 && ks >= -50;
    if (!ok) ks = 0;
    const double sg = ldexp(1.0, -ks);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int64_t c = cidx[4 * e + t];
      double *o = cgeo + 10 * c;
      o[0] = g[sel_of(t, 0)]; o[1] = g[sel_of(t, 1)]; o[2] = g[sel_of(t, 2)];
      o[3] = g[sel_of(t, 3)]; o[4] = g[sel_of(t, 4)]; o[5] = g[sel_of(t, 5)];
      o[6] = s[sel_of(t, 4)]; o[7] = s[sel_of(t, 5)]; o[8] = s[sel_of(t, 2)];
      o[9] = 0.0;
      float4 *of = reinterpret_cast<float4 *>(cgf + 12 * c);
      of[0] = make_float4((float)(o[0] * sg), (float)(o[1] * sg), (float)(o[2] * sg), (float)(o[3] * sg));
      of[1] = make_float4((float)(o[4] * sg), (float)(o[5] * sg), (float)o[6], (float)o[7]);
      of[2] = make_float4((float)o[8], (float)ks, ok ? 0.f : 1.f, 0.f);
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

__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v)
{
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile_i32(const int32_t *p)
{
  return *(const volatile int32_t *)p;
}

// All blocks of the (co-resident) grid meet here.  Every wait is bounded by
// timeout_ns of %globaltimer and by a spin cap; on expiry the block records
// KERR_TIMEOUT and the phase, and every block leaves the kernel at its next
// barrier.  Returns false when the caller must return.
__device__ bool grid_sync(FimCtl *ctl, uint32_t nblocks, uint64_t timeout_ns, int where)
{
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const uint32_t gen = ld_acquire_u32(&ctl->bar_gen);
    __threadfence();
    const uint32_t arrived = atomicAdd(&ctl->bar_count, 1u) + 1u;
    if (arrived == nblocks) {
      atomicExch(&ctl->bar_count, 0u);
      __threadfence();
      st_release_u32(&ctl->bar_gen, gen + 1u);
    } else {
      const uint64_t t0 = global_timer();
      uint32_t spins = 0;
      while (ld_acquire_u32(&ctl->bar_gen) == gen) {
        ++spins;
        if ((spins & 63u) == 0u) {
          if (ld_volatile_i32(&ctl->error) != KERR_NONE) { ok = 0; break; }
          if (global_timer() - t0 > timeout_ns || spins > (1u << 30)) {
            if (atomicCAS(&ctl->error, KERR_NONE, KERR_TIMEOUT) == KERR_NONE) ctl->error_where = where;
            ok = 0;
            break;
          }
        }
        __nanosleep(64);
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

struct WarpCtx {
  int lane;
  int64_t gwarp;
  int64_t nwarps;
};

// One FP64 local solve of the reference for corner c: kind 0..2 are the
// triangle solves (1,2), (2,3), (1,3) and kind 3 the tet solve.  The caller
// guarantees the neighbours the solve uses are valid.
__device__ double exact_candidate(const FimDev &d, int64_t c, int kind)
{
  const int4 id = __ldg(d.cids + c);
  const double p1 = __ldcg(d.phi + id.x), p2 = __ldcg(d.phi + id.y), p3 = __ldcg(d.phi + id.z);
  const double2 *gp = reinterpret_cast<const double2 *>(d.cgeo + 10 * c);
  double g[6];
  {
    const double2 t0 = __ldg(gp), t1 = __ldg(gp + 1), t2 = __ldg(gp + 2);
    g[0] = t0.x; g[1] = t0.y; g[2] = t1.x; g[3] = t1.y; g[4] = t2.x; g[5] = t2.y;
  }
  if (kind == 3) return tet_ref(g[0], g[1], g[2], g[3], g[4], g[5], p1, p2, p3);
  if (kind == 0) return tri_ref(g[3], g[4], g[5], p1, p2);
  if (kind == 1) return tri_ref(g[1], g[5], g[2], p2, p3);
  return tri_ref(g[0], g[4], g[2], p1, p3);
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

constexpr int kThreads = 256;       // threads per block of the solve kernel
constexpr int kSlots = 32;          // vertices per batch (at most)
constexpr int kCornerCap = 768;     // corners per batch
constexpr int kTriCap = 1024;       // triangle screens per batch (more are screened on the spot)
constexpr int kTetCap = 768;        // tet screens per batch
constexpr int kQcap = 512;          // exact solves queued per kind and batch

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

// Shared memory of one batch of vertex updates.
struct BatchSh {
  int32_t vtx[kSlots];
  int64_t c0[kSlots];
  int32_t cp[kSlots + 1];           // corner prefix over the batch's vertices
  double old[kSlots];
  unsigned long long res[kSlots];   // dkey of the running minimum (exact values)
  unsigned int bhi[kSlots];         // fkey of a float upper bound of the new time
  // per corner of the batch: float times of the other three vertices,
  // float edge lengths, validity bits
  float pf[kCornerCap][3];
  float sf[kCornerCap][3];
  uint8_t vm[kCornerCap];
  // compacted screen lists: item (corner j | pair k << 16) and lower bound
  uint32_t tri[kTriCap];
  float tri_lb[kTriCap];
  uint32_t tet[kTetCap];
  float tet_lb[kTetCap];
  uint32_t q[2][kQcap];             // queued exact solves: [0] tets, [1] triangles
  int ntri, ntet, nq[2];
  int nslot;                        // vertices of the current batch
};

// Queue item: slot (5 bits) | kind (2 bits) | corner offset in the vertex (25 bits).
__device__ __forceinline__ uint32_t make_item(int slot, int kind, int64_t off)
{
  return (uint32_t)slot | ((uint32_t)kind << 5) | ((uint32_t)off << 7);
}

__device__ __forceinline__ int slot_of(const BatchSh &sh, int nslot, int j)
{
  int lo = 0, hi = nslot - 1;  // last slot with cp[slot] <= j
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sh.cp[mid] <= j) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Appends one item per lane with `need` to a list in shared memory
// (warp-ballot compaction).  Returns the item's position, or -1.
__device__ __forceinline__ int warp_append(int *counter, bool need, int lane)
{
  const unsigned mask = __ballot_sync(FULL_MASK, need);
  if (mask == 0) return -1;
  int base = 0;
  if (lane == 0) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(FULL_MASK, base, 0);
  return need ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

// Queues an exact solve (or runs it on the spot when the queue is full).
// qi (0: tets, 1: triangles) must be the same on every lane of the warp; the
// item's kind may differ per lane.
__device__ __forceinline__ void queue_exact(const FimDev &d, BatchSh &sh, bool need, int qi, int kind, int slot,
                                            int64_t c, int lane)
{
  const int pos = warp_append(&sh.nq[qi], need, lane);
  if (pos < 0) return;
  if (pos < kQcap) {
    sh.q[qi][pos] = make_item(slot, kind, c - sh.c0[slot]);
  } else {
    const double val = exact_candidate(d, c, kind);
    if (val < FIM_INF) atomicMin(&sh.res[slot], dkey(val));
  }
}

// Triangle screen of pair k (0: (1,2), 1: (2,3), 2: (1,3)) of corner c.
__device__ __forceinline__ CandBound tri_screen_of(const FimDev &d, int64_t c, int k, const float *pf)
{
  const float4 *rp = reinterpret_cast<const float4 *>(d.cgf + 12 * c);
  const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2);
  const float tk = re_pow2f((int)r2.y);
  // scaled e13, e23, e34, e12, e14, e24 -> true units
  const float g[6] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y};
  const int i12 = k == 0 ? 3 : (k == 1 ? 1 : 0);   // e12 role
  const int i13 = k == 0 ? 4 : (k == 1 ? 5 : 4);   // e13 role
  const int i23 = k == 0 ? 5 : 2;                  // e23 role
  const int a = k == 0 ? 0 : (k == 1 ? 1 : 0), b = k == 0 ? 1 : 2;
  return tri_screen(re_scale(re_in(g[i12]), tk), re_scale(re_in(g[i13]), tk), re_scale(re_in(g[i23]), tk),
                    re_in(pf[a]), re_in(pf[b]));
}

// Tet screen of corner c.
__device__ __forceinline__ CandBound tet_screen_of(const FimDev &d, int64_t c, const float *pf)
{
  const float4 *rp = reinterpret_cast<const float4 *>(d.cgf + 12 * c);
  const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2);
  const Re gs[6] = {re_in(r0.x), re_in(r0.y), re_in(r0.z), re_in(r0.w), re_in(r1.x), re_in(r1.y)};
  return tet_screen(gs, re_in(pf[0]), re_in(pf[1]), re_in(pf[2]), (int)r2.y);
}

// Writes a time and its float copy.
__device__ __forceinline__ void set_phi(const FimDev &d, int64_t v, double x)
{
  d.phi[v] = x;
  d.phi_f[v] = (float)x;
}

// One update phase over a vertex list.  Every block takes a contiguous part
// of the list and processes it in batches of up to kSlots vertices / up to
// kCornerCap corners, the corners of a batch spread over all threads:
//  A -- load every corner: validity of the neighbours (state >= narrow and
//       phi > phi_start - front_width, on the float copies when conclusive,
//       else on the FP64 times), float edge bounds -> per-vertex upper bound
//       bhi of the new time;
//  B -- exact FP64 edge candidates that can still be the minimum; triangle
//       and tet solves whose trivial bound min(neighbour times) <= bhi are
//       appended to compacted screen lists (warp-ballot compaction);
//  S -- the screens run over the lists with full warps (triangles and tets
//       on separate warps); certain upper bounds tighten bhi;
//  C -- solves whose lower bound does not exceed bhi are queued;
//  D -- the queued solves run in FP64 (tets and triangles on separate warps);
//  E -- the reference's per-vertex decision on the exact minimum:
//   mode 0 -- narrow vertices: window test (next), freeze test
//             (cuda_fim.cu:2125-2163);
//   mode 1 -- re-solved neighbours: keep or restore the state
//             (cuda_fim.cu:2255-2289).
// The minimum over everything equals the reference's update_per_element
// minimum over all corners (cuda_fim.h:1362-1411).
__device__ void update_phase(const FimDev &d, BatchSh &sh, const int32_t *list, int32_t n, int mode, double lower,
                             float lower_lo, float lower_hi, double phi_start, double dt, bool exact_all, int s,
                             int64_t &n_filtered, int64_t &n_exact)
{
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t per_block = ((int64_t)n + gridDim.x - 1) / gridDim.x;
  const int64_t lbeg = min((int64_t)n, (int64_t)blockIdx.x * per_block);
  const int64_t lend = min((int64_t)n, lbeg + per_block);
  int64_t pos = lbeg;
  while (pos < lend) {
    // batch: the longest run of vertices with <= kCornerCap corners (>= 1 vertex)
    const int cand = (int)min((int64_t)kSlots, lend - pos);
    if (tid < cand) {
      const int32_t v = __ldcg(list + pos + tid);
      const double old = __ldcg(d.phi + v);
      sh.vtx[tid] = v;
      sh.c0[tid] = d.cptr[v];
      sh.cp[tid + 1] = (int32_t)(d.cptr[v + 1] - d.cptr[v]);
      sh.old[tid] = old;
      sh.res[tid] = dkey(old);
      sh.bhi[tid] = fkey(exact_all ? INFINITY : re_hi(re_in(__ldcg(d.phi_f + v))));
    }
    if (tid == 0) {
      sh.cp[0] = 0;
      sh.ntri = 0; sh.ntet = 0; sh.nq[0] = 0; sh.nq[1] = 0;
    }
    __syncthreads();
    if (tid == 0) {
      int k = 1;
      for (; k <= cand; ++k) {
        const int t = sh.cp[k - 1] + sh.cp[k];
        if (t > kCornerCap && k > 1) break;
        sh.cp[k] = t;
      }
      sh.nslot = k - 1;
    }
    __syncthreads();
    const int nslot = sh.nslot;
    const int total = sh.cp[nslot];     // may exceed kCornerCap for a single huge vertex
    const int kept = min(total, kCornerCap);

    // A: load, validity, float edge bounds
    for (int j = tid; j < total; j += kThreads) {
      const int slot = slot_of(sh, nslot, j);
      const int64_t c = sh.c0[slot] + (j - sh.cp[slot]);
      const int4 id = __ldg(d.cids + c);
      const int32_t nb[3] = {id.x, id.y, id.z};
      const float4 *rp = reinterpret_cast<const float4 *>(d.cgf + 12 * c);
      const float4 r1 = __ldg(rp + 1), r2 = __ldg(rp + 2);
      const float sv[3] = {r1.z, r1.w, r2.x};
      uint32_t m = 0;
      float pf[3];
      float ub = INFINITY;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        pf[i] = __ldcg(d.phi_f + nb[i]);
        const Re P = re_in(pf[i]);
        bool ok = __ldcg(d.st + nb[i]) >= ST_NARROW;
        if (ok) {
          if (re_lo(P) > lower_hi) ok = true;
          else if (re_hi(P) <= lower_lo) ok = false;
          else ok = __ldcg(d.phi + nb[i]) > lower;
        }
        if (ok) {
          m |= 1u << i;
          ub = fminf(ub, re_hi(P + re_in(sv[i])));
        }
      }
      if (m) ++n_filtered;
      if (!exact_all && ub < INFINITY) atomicMin(&sh.bhi[slot], fkey(ub));
      if (j < kCornerCap) {
        sh.vm[j] = (uint8_t)m;
#pragma unroll
        for (int i = 0; i < 3; ++i) { sh.pf[j][i] = pf[i]; sh.sf[j][i] = sv[i]; }
      }
    }
    __syncthreads();

    // B: exact edges; screen lists
    for (int jb = 0; jb < kept; jb += kThreads) {
      const int j = jb + tid;
      const bool in = j < kept;
      int slot = 0;
      int64_t c = 0;
      uint32_t m = 0;
      float bhi = 0.f, lo[3] = {0.f, 0.f, 0.f};
      if (in) {
        slot = slot_of(sh, nslot, j);
        c = sh.c0[slot] + (j - sh.cp[slot]);
        m = sh.vm[j];
        bhi = funkey(sh.bhi[slot]);
        const int4 id = __ldg(d.cids + c);
        const int32_t nb[3] = {id.x, id.y, id.z};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const Re P = re_in(sh.pf[j][i]);
          lo[i] = re_lo(P);
          if ((m >> i) & 1u) {
            if (!(re_lo(P + re_in(sh.sf[j][i])) > bhi)) {
              const double val = __ldcg(d.phi + nb[i]) + __ldg(d.cgeo + 10 * c + 6 + i);
              atomicMin(&sh.res[slot], dkey(val));
            }
          }
        }
      }
      // triangle pairs (1,2), (2,3), (1,3) and the tet
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int a = k == 1 ? 1 : 0, b = k == 0 ? 1 : 2;
        const bool need = in && ((m >> a) & 1u) && ((m >> b) & 1u) && !(fminf(lo[a], lo[b]) > bhi);
        const int p = warp_append(&sh.ntri, need, lane);
        if (p >= 0) {
          if (p < kTriCap) {
            sh.tri[p] = (uint32_t)j | ((uint32_t)k << 16);
          } else {  // list full: screen here
            CandBound cb;
            if (exact_all) { cb.some = CAND_SOME; cb.lb = NAN; cb.ub = INFINITY; }
            else cb = tri_screen_of(d, c, k, sh.pf[j]);
            if (cb.some && !(cb.lb > bhi)) {
              const double val = exact_candidate(d, c, k);
              if (val < FIM_INF) atomicMin(&sh.res[slot], dkey(val));
            }
          }
        }
      }
      {
        const bool need = in && m == 7u && !(fminf(lo[0], fminf(lo[1], lo[2])) > bhi);
        const int p = warp_append(&sh.ntet, need, lane);
        if (p >= 0) sh.tet[p] = (uint32_t)j;  // kTetCap == kCornerCap: never full
      }
    }
    // corners beyond kCornerCap (a single vertex with very many corners):
    // every solve of them goes to FP64
    for (int jb = kept; jb < total; jb += kThreads) {
      const int j = jb + tid;
      if (j >= total) continue;
      const int slot = slot_of(sh, nslot, j);
      const int64_t c = sh.c0[slot] + (j - sh.cp[slot]);
      const int4 id = __ldg(d.cids + c);
      const int32_t nb[3] = {id.x, id.y, id.z};
      uint32_t m = 0;
      for (int i = 0; i < 3; ++i) {
        const double p = __ldcg(d.phi + nb[i]);
        if (__ldcg(d.st + nb[i]) >= ST_NARROW && p > lower) {
          m |= 1u << i;
          atomicMin(&sh.res[slot], dkey(p + __ldg(d.cgeo + 10 * c + 6 + i)));
        }
      }
      for (int k = 0; k < 4; ++k) {
        const bool use = k == 3 ? m == 7u : (((m >> (k == 1 ? 1 : 0)) & 1u) && ((m >> (k == 0 ? 1 : 2)) & 1u));
        if (!use) continue;
        const double val = exact_candidate(d, c, k);
        if (val < FIM_INF) atomicMin(&sh.res[slot], dkey(val));
      }
    }
    __syncthreads();

    // S: screens over the compacted lists; tets from thread 0, triangles from
    // the next warp boundary
    {
      const int ntet = min(sh.ntet, kTetCap), ntri = min(sh.ntri, kTriCap);
      const int tri0 = (ntet + 31) & ~31;
      for (int i = tid; i < tri0 + ntri; i += kThreads) {
        if (i < ntet) {
          const int j = (int)sh.tet[i];
          const int slot = slot_of(sh, nslot, j);
          const int64_t c = sh.c0[slot] + (j - sh.cp[slot]);
          CandBound cb;
          if (exact_all) { cb.some = CAND_SOME; cb.lb = NAN; cb.ub = INFINITY; }
          else cb = tet_screen_of(d, c, sh.pf[j]);
          sh.tet_lb[i] = !cb.some ? NAN : (isnan(cb.lb) ? -INFINITY : cb.lb);
          if (!exact_all && cb.some && cb.ub < INFINITY) atomicMin(&sh.bhi[slot], fkey(cb.ub));
        } else if (i >= tri0) {
          const int t = i - tri0;
          const int j = (int)(sh.tri[t] & 0xffffu), k = (int)(sh.tri[t] >> 16);
          const int slot = slot_of(sh, nslot, j);
          const int64_t c = sh.c0[slot] + (j - sh.cp[slot]);
          CandBound cb;
          if (exact_all) { cb.some = CAND_SOME; cb.lb = NAN; cb.ub = INFINITY; }
          else cb = tri_screen_of(d, c, k, sh.pf[j]);
          sh.tri_lb[t] = !cb.some ? NAN : (isnan(cb.lb) ? -INFINITY : cb.lb);
          if (!exact_all && cb.some && cb.ub < INFINITY) atomicMin(&sh.bhi[slot], fkey(cb.ub));
        }
      }
    }
    __syncthreads();

    // C: queue the solves that can still be the minimum
    {
      const int ntet = min(sh.ntet, kTetCap), ntri = min(sh.ntri, kTriCap);
      for (int ib = 0; ib < ntet + ntri; ib += kThreads) {
        const int i = ib + tid;
        bool need = false;
        int kind = 0, slot = 0;
        int64_t c = 0;
        if (i < ntet + ntri) {
          int j;
          float l;
          if (i < ntet) { j = (int)sh.tet[i]; kind = 3; l = sh.tet_lb[i]; }
          else { const uint32_t it = sh.tri[i - ntet]; j = (int)(it & 0xffffu); kind = (int)(it >> 16); l = sh.tri_lb[i - ntet]; }
          slot = slot_of(sh, nslot, j);
          c = sh.c0[slot] + (j - sh.cp[slot]);
          need = l <= funkey(sh.bhi[slot]);  // NaN (no value) never
        }
        // separate ballots per queue keep each queue warp-compacted
        queue_exact(d, sh, need && kind == 3, 0, kind, slot, c, lane);
        queue_exact(d, sh, need && kind != 3, 1, kind, slot, c, lane);
      }
    }
    __syncthreads();

    // D: exact solves; tets from thread 0, triangles from the next warp boundary
    {
      const int ntet = min(sh.nq[0], kQcap), ntri = min(sh.nq[1], kQcap);
      const int tri0 = (ntet + 31) & ~31;
      for (int j = tid; j < tri0 + ntri; j += kThreads) {
        uint32_t it;
        if (j < ntet) it = sh.q[0][j];
        else if (j >= tri0) it = sh.q[1][j - tri0];
        else continue;
        const int slot = it & 31, kind = (it >> 5) & 3;
        const int64_t c = sh.c0[slot] + (int64_t)(it >> 7);
        const double val = exact_candidate(d, c, kind);
        ++n_exact;
        if (val < FIM_INF) atomicMin(&sh.res[slot], dkey(val));
      }
    }
    __syncthreads();

    // E: decisions
    if (tid < nslot) {
      const int slot = tid;
      const int32_t v = sh.vtx[slot];
      const double old = sh.old[slot];
      const double nw = dunkey(sh.res[slot]);
      d.phi2[v] = nw;
      if (mode == 0) {
        d.tst[v] = ST_FAR;
        if (nw - phi_start > dt) {
          d.st[v] = ST_NEXT;
        } else if (fabs(old - nw) < (1e-6 * (1 + (old + nw) * .5))) {
          d.tst[v] = ST_FROZEN;
          d.lfrozen[atomicAdd(&d.ctl->n_frozen[s], 1)] = v;
        }
      } else {
        d.dec[pos + slot] = (nw < old) ? (uint8_t)ST_NARROW : __ldcg(d.tst + v);
      }
    }
    __syncthreads();
    pos += nslot;
  }
}

__global__ void __launch_bounds__(256) fim_solve_kernel(FimDev d, FimParams p)
{
  FimCtl *ctl = d.ctl;
  const uint32_t nblocks = gridDim.x;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  WarpCtx w;
  w.lane = threadIdx.x & 31;
  w.gwarp = gtid >> 5;
  w.nwarps = nthreads >> 5;
  int64_t my_evals = 0, my_updates = 0, my_exact = 0;
  int where = 0;
  __shared__ BatchSh sh;

  // reset_states_gpu + update_events_gpu: phi = INF, far; seeds narrow.
  for (int64_t v = gtid; v < d.nV; v += nthreads) {
    set_phi(d, v, FIM_INF); d.phi2[v] = FIM_INF; d.st[v] = ST_FAR; d.tst[v] = ST_FAR; d.flag[v] = 0;
  }
  // failure-detection test hook: this block never arrives at the barrier (a
  // flag that nothing sets), so the others' bounded waits must expire
  if (p.withhold_block > 0 && (int64_t)blockIdx.x == (int64_t)p.withhold_block - 1) return;
  if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;
  for (int64_t i = gtid; i < d.nseed; i += nthreads) {
    const int32_t v = d.seed_v[i];
    set_phi(d, v, d.seed_t[i]); d.phi2[v] = d.seed_t[i]; d.st[v] = ST_NARROW;
  }
  if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;

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
          if (mn < __ldcg(d.phi + c)) { set_phi(d, c, mn); d.phi2[c] = mn; d.st[c] = ST_NARROW; }
        }
      }
    }
    if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;
    // update_states (cuda_fim.cu:1790-1845) -> narrow list of this window
    for (int64_t v = gtid; v < d.nV; v += nthreads) {
      uint8_t stv = d.st[v];
      if (stv == ST_NEXT) { stv = ST_NARROW; d.st[v] = stv; }
      else if (p.apd >= 0.0 && stv == ST_FROZEN) {
        if (!(d.phi[v] + p.apd > cur_time)) d.st[v] = ST_TAIL;
      } else if (p.apd >= 0.0 && stv == ST_TAIL) {
        if (!(d.phi[v] + p.apd / 0.91 > cur_time)) {
          set_phi(d, v, FIM_INF); d.phi2[v] = FIM_INF; d.st[v] = ST_FAR;
        }
      }
      if (stv == ST_NARROW) d.list[s][atomicAdd(&ctl->n_narrow[s], 1)] = (int32_t)v;
    }
    if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;

    int64_t it_window = 0;
    for (;;) {
      s = (int)(it % 3);
      const int s1 = (int)((it + 1) % 3), s2 = (int)((it + 2) % 3);
      const int32_t nn = ld_volatile_i32(&ctl->n_narrow[s]);
      if (nn == 0) break;
      if (p.max_iter > 0 && it_window >= p.max_iter) {
        if (gtid == 0 && atomicCAS(&ctl->error, KERR_NONE, KERR_MAX_ITER) == KERR_NONE) ctl->error_where = where;
        return;
      }
      const int32_t stamp = (int32_t)(it + 1);
      const int32_t *lst = d.list[s];
      int32_t *lnext = d.list[s1];
      if (gtid == 0) { ctl->n_narrow[s2] = 0; ctl->n_frozen[s2] = 0; ctl->n_marked[s2] = 0; }

      // P1 -- solve on elements + reduce per vertex (cuda_fim.cu:2102-2163)
      update_phase(d, sh, lst, nn, 0, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, s, my_evals, my_exact);
      my_updates += (gtid == 0) ? nn : 0;
      if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;

      // P2 -- apply the narrow times; mark downwind neighbours of the
      // vertices frozen now (cuda_fim.cu:2172-2205)
      for (int64_t i = gtid; i < nn; i += nthreads) {
        const int32_t v = lst[i];
        set_phi(d, v, __ldcg(d.phi2 + v));
      }
      const int32_t nf = ld_volatile_i32(&ctl->n_frozen[s]);
      for (int64_t i = w.gwarp; i < nf; i += w.nwarps) {
        const int32_t n = d.lfrozen[i];
        const double pn = __ldcg(d.phi2 + n);
        for (int64_t k = d.nptr[n] + w.lane; k < d.nptr[n + 1]; k += 32) {
          const int32_t v = __ldg(d.nbr + k);
          if (__ldcg(d.st + v) != ST_NARROW && pn < __ldcg(d.phi2 + v)) {
            if (atomicExch(d.flag + v, stamp) != stamp) {
              d.tst[v] = __ldcg(d.st + v);
              d.st[v] = ST_NEIG;
              d.lmarked[atomicAdd(&ctl->n_marked[s], 1)] = v;
            }
          }
        }
      }
      if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;

      // P3 -- solve elements for neighbours + reduce (cuda_fim.cu:2215-2289)
      const int32_t nm = ld_volatile_i32(&ctl->n_marked[s]);
      update_phase(d, sh, d.lmarked, nm, 1, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, s, my_evals, my_exact);
      my_updates += (gtid == 0) ? nm : 0;
      if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;

      // P4 -- apply, update neighbour states, next narrow list (cuda_fim.cu:2291-2317)
      for (int64_t i = gtid; i < nm; i += nthreads) {
        const int32_t v = d.lmarked[i];
        set_phi(d, v, __ldcg(d.phi2 + v));
        uint8_t sv = __ldcg(d.dec + i);
        if (sv == ST_NARROW) {
          if (__ldcg(d.tst + v) == ST_FROZEN) sv = ST_FROZEN;
          else lnext[atomicAdd(&ctl->n_narrow[s1], 1)] = v;
        }
        d.st[v] = sv;
      }
      for (int64_t i = gtid; i < nn; i += nthreads) {
        const int32_t v = lst[i];
        if (__ldcg(d.flag + v) == stamp) continue;  // re-solved above
        if (__ldcg(d.st + v) == ST_NARROW) {
          if (__ldcg(d.tst + v) == ST_FROZEN) d.st[v] = ST_FROZEN;
          else lnext[atomicAdd(&ctl->n_narrow[s1], 1)] = v;
        }
      }
      ++it;
      ++it_window;
      if (!grid_sync(ctl, nblocks, p.timeout_ns, ++where)) return;
    }
  }

  // local -> global gather (cuda_fim.cu:2466-2485): min time, max state
  if (d.gptr) {
    for (int64_t g = gtid; g < d.nG; g += nthreads) {
      double mn = FIM_INF;
      uint8_t mx = ST_FAR;
      for (int64_t k = d.gptr[g]; k < d.gptr[g + 1]; ++k) {
        const int32_t c = d.gcopy[k];
        const double pc = __ldcg(d.phi + c);
        const uint8_t sc = __ldcg(d.st + c);
        if (pc < mn) mn = pc;
        if (sc > mx) mx = sc;
      }
      d.phi_out[g] = mn;
      d.st_out[g] = mx;
    }
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
                          const double *fib, const double *cf, const double *ct, int64_t nT,
                          double *cgeo, float *cgf, cudaStream_t stream)
{
  if (nT <= 0) return cudaSuccess;
  const int block = 256;
  int64_t grid = (nT + block - 1) / block;
  if (grid > 152 * 64) grid = 152 * 64;
  fim_metric_kernel<<<(unsigned)grid, block, 0, stream>>>(tslots, cidx, xyz, fib, cf, ct, nT, cgeo, cgf);
  return cudaGetLastError();
}

cudaError_t solve_grid_size(int device, int block, int *grid)
{
  int sms = 0, per_sm = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fim_solve_kernel, block, 0);
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
  return cudaLaunchCooperativeKernel((const void *)fim_solve_kernel, dim3(grid), dim3(block), args, 0, stream);
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
