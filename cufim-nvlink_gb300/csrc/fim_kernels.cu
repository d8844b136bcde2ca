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
//  * edge_vector_kernel -- the six edge vectors of every tet, staged once
//    per mesh for the metric kernel;
//  * the support check and warm-start reset of a warm-started solve.
// The solve itself, fim_solve_kernel (fim_solve.cuh, compiled once per
// batch shape by fim_solve_s*.cu), is one persistent cooperative launch for
// the whole solve: reset + seeding (reset_states_gpu / update_events_gpu,
// cuda_fim.cu:479-542, 632-683), per window update_states
// (cuda_fim.cu:1790-1845), then FIM iterations with the phases of
// compute_step (cuda_fim.cu:1992-2334) as global Jacobi steps over
// compacted lists (narrow list, vertices frozen this iteration, neighbours
// to re-solve), separated by a bounded grid barrier: three phases per
// iteration with windows, two with one endless window.
#include "fim_device.cuh"

#include <cmath>

namespace fimgb {

// ---------------------------------------------------------------------------
// metric kernel

__global__ void fim_metric_kernel(const int32_t *__restrict__ tslots, const int64_t *__restrict__ cidx,
                                  const double *__restrict__ xyz, const double *__restrict__ evec, int64_t nT,
                                  const double *__restrict__ fib,
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
    double g[6];
    if (evec) {
      // the edge vectors of the mesh, staged once (edge_vector_kernel)
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const double ex = evec[(3 * k + 0) * nT + e], ey = evec[(3 * k + 1) * nT + e], ez = evec[(3 * k + 2) * nT + e];
        g[k] = (M0*ex + M1*ey + M2*ez)*ex + (M1*ex + M3*ey + M4*ez)*ey + (M2*ex + M4*ey + M5*ez)*ez;
      }
    } else {
      const int32_t v0 = tslots[4 * e + 0], v1 = tslots[4 * e + 1];
      const int32_t v2 = tslots[4 * e + 2], v3 = tslots[4 * e + 3];
      const int32_t va[6] = {v0, v0, v1, v0, v1, v2};
      const int32_t vb[6] = {v1, v2, v2, v3, v3, v3};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        // load_edge(a, b) = x_a - x_b (types.h:210-216); aMb_sym (types.h:165-171)
        const double ex = xyz[3 * (int64_t)va[k] + 0] - xyz[3 * (int64_t)vb[k] + 0];
        const double ey = xyz[3 * (int64_t)va[k] + 1] - xyz[3 * (int64_t)vb[k] + 1];
        const double ez = xyz[3 * (int64_t)va[k] + 2] - xyz[3 * (int64_t)vb[k] + 2];
        g[k] = (M0*ex + M1*ey + M2*ez)*ex + (M1*ex + M3*ey + M4*ez)*ey + (M2*ex + M4*ey + M5*ez)*ez;
      }
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

// Edge vectors of every tet in the metric kernel's edge order, x_a - x_b
// for (a, b) = (0,1) (0,2) (1,2) (0,3) (1,3) (2,3) of its slots
// (load_edge, types.h:210-216): they depend on the mesh only, so
// fim_set_mesh stages them once and every conduction upload saves their 18
// FP64 subtractions per tet.  Layout: evec[(3 k + axis) nT + e].
__global__ void edge_vector_kernel(const int32_t *__restrict__ tslots, const double *__restrict__ xyz, int64_t nT,
                                   double *__restrict__ evec)
{
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nT; e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v0 = tslots[4 * e + 0], v1 = tslots[4 * e + 1];
    const int32_t v2 = tslots[4 * e + 2], v3 = tslots[4 * e + 3];
    const int32_t va[6] = {v0, v0, v1, v0, v1, v2};
    const int32_t vb[6] = {v1, v2, v2, v3, v3, v3};
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int a = 0; a < 3; ++a) evec[(3 * k + a) * nT + e] = xyz[3 * (int64_t)va[k] + a] - xyz[3 * (int64_t)vb[k] + a];
  }
}

// ---------------------------------------------------------------------------
// launch wrappers

cudaError_t launch_edge_vectors(const int32_t *tslots, const double *xyz, int64_t nT, double *evec,
                                cudaStream_t stream)
{
  if (nT <= 0) return cudaSuccess;
  edge_vector_kernel<<<152 * 8, 256, 0, stream>>>(tslots, xyz, nT, evec);
  return cudaGetLastError();
}

cudaError_t launch_metric(const int32_t *tslots, const int64_t *cidx, const double *xyz, const double *evec,
                          int64_t nT, const double *fib, const double *cf, const double *ct, int64_t e0, int64_t e1,
                          double *cgeo, float *cgf, uint4 *crec, unsigned long long *bad, cudaStream_t stream)
{
  if (e1 <= e0) return cudaSuccess;
  const int block = 256;
  int64_t grid = (e1 - e0 + block - 1) / block;
  if (grid > 152 * 64) grid = 152 * 64;
  fim_metric_kernel<<<(unsigned)grid, block, 0, stream>>>(tslots, cidx, xyz, evec, nT, fib, cf, ct, e0, e1, cgeo, cgf,
                                                          crec, bad);
  return cudaGetLastError();
}

// batch shapes (fim_solve_s*.cu); shape 0 is the default
cudaError_t solve_prepare_s192(int device, int block, int *max_grid);
cudaError_t solve_prepare_s160(int device, int block, int *max_grid);
cudaError_t solve_prepare_s96(int device, int block, int *max_grid);
cudaError_t solve_launch_s192(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream);
cudaError_t solve_launch_s160(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream);
cudaError_t solve_launch_s96(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream);

const ShapeDesc kShapes[kNumShapes] = {{"192x4096", 192, 4096}, {"160x3072", 160, 3072}, {"96x2048", 96, 2048}};

cudaError_t solve_prepare(int shape, int device, int block, int *max_grid)
{
  switch (shape) {
    case 0: return solve_prepare_s192(device, block, max_grid);
    case 1: return solve_prepare_s160(device, block, max_grid);
    case 2: return solve_prepare_s96(device, block, max_grid);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_solve(const FimDev &d, const FimParams &p, int shape, int grid, int block, cudaStream_t stream)
{
  switch (shape) {
    case 0: return solve_launch_s192(d, p, grid, block, stream);
    case 1: return solve_launch_s160(d, p, grid, block, stream);
    case 2: return solve_launch_s96(d, p, grid, block, stream);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// support check of a warm-started solve
//
// FIM only lowers times, so a start below the true time of a vertex would
// stay there.  Such a time is not attained by any candidate its neighbours
// can give: the reference's edge, triangle and tet updates
// (update_per_element, cuda_fim.h:1362-1411) all return at least the
// smallest time involved plus a distance.  The check bounds every candidate
// of every corner from below with the same rigorous FP32 bounds the screens
// use (edge: time + length; triangle pairs and tet: smallest time +
// root-term bound, solve_lo) and flags a reached, non-seed vertex whose
// time is strictly below all of them.  A cold solve never trips it: each of
// its times was a candidate when it was set, and neighbour times only fall
// afterwards, which only lowers the bounds.

__global__ void fim_support_kernel(FimDev d, double lower, float lower_lo, float lower_hi,
                                   const uint8_t *__restrict__ is_seed)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < d.nV; v += stride) {
    const double pv = __ldcg(d.phi + v);
    if (!(pv < FIM_INF) || is_seed[v]) continue;
    float L = INFINITY;
    for (int64_t c = d.cptr[v]; c < d.cptr[v + 1]; ++c) {
      const uint4 h0 = __ldg(d.crec + kCrecWords * c), h1 = __ldg(d.crec + kCrecWords * c + 1);
      const int32_t nb[3] = {(int32_t)h0.x, (int32_t)h0.y, (int32_t)h0.z};
      const float len[3] = {__uint_as_float(h1.x), __uint_as_float(h1.y), __uint_as_float(h1.z)};
      float lo[3], hi[3];
      bool ok[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const Re P = re_in(__ldcg(d.phi_f + nb[i]));
        bool valid = (__ldcg(d.sw + nb[i]) & 0xffu) >= ST_NARROW;
        if (valid) {
          if (re_lo(P) > lower_hi) valid = true;
          else if (re_hi(P) <= lower_lo) valid = false;
          else valid = __ldcg(d.phi + nb[i]) > lower;
        }
        ok[i] = valid;
        lo[i] = re_lo(P);
        hi[i] = re_hi(P);
        if (valid) L = fminf(L, re_lo(P + re_len(len[i])));
      }
      if (ok[0] && ok[1]) L = fminf(L, solve_lo(fminf(lo[0], lo[1]), fmaxf(hi[0], hi[1]), half_lo(h0.w)));
      if (ok[1] && ok[2]) L = fminf(L, solve_lo(fminf(lo[1], lo[2]), fmaxf(hi[1], hi[2]), half_hi(h0.w)));
      if (ok[0] && ok[2]) L = fminf(L, solve_lo(fminf(lo[0], lo[2]), fmaxf(hi[0], hi[2]), half_lo(h1.w)));
      if (ok[0] && ok[1] && ok[2])
        L = fminf(L, solve_lo(fminf(lo[0], fminf(lo[1], lo[2])), fmaxf(hi[0], fmaxf(hi[1], hi[2])), half_hi(h1.w)));
    }
    if ((double)L > pv) {
      atomicAdd(&d.ctl->n_bad, 1);
      atomicMin(&d.ctl->tmin_key, dkey(pv));
    }
  }
}

__global__ void fim_mark_seeds_kernel(const int32_t *__restrict__ seed_v, int32_t n, uint8_t *is_seed)
{
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) is_seed[seed_v[i]] = 1;
}

__global__ void fim_warm_reset_kernel(FimDev d, double tmin)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < d.nV; v += stride) {
    const double x = d.phi[v];
    d.tst[v] = ST_FAR;
    if (x >= tmin) {
      d.phi[v] = FIM_INF; d.phi2[v] = FIM_INF;
      d.phi_f[v] = (float)FIM_INF; d.phi2_f[v] = (float)FIM_INF;
      d.sw[v] = ST_FAR;
    } else if (x < FIM_INF) {
      d.sw[v] = ST_NARROW;
    }
  }
}

__global__ void fim_reseed_kernel(FimDev d)
{
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nseed; i += gridDim.x * blockDim.x) {
    const int32_t v = d.seed_v[i];
    const double x = d.seed_t[i];
    d.phi[v] = x; d.phi2[v] = x;
    d.phi_f[v] = (float)x; d.phi2_f[v] = (float)x;
    d.sw[v] = ST_NARROW;
  }
}

// float bounds of a double (round down / up), on the host
static float f_rd(double x)
{
  float f = (float)x;
  if ((double)f > x) f = std::nextafter(f, -INFINITY);
  return f;
}
static float f_ru(double x)
{
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, INFINITY);
  return f;
}

static unsigned grid_for(int64_t n, int block, unsigned cap)
{
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  return (unsigned)(g > cap ? cap : g);
}

cudaError_t launch_support_check(const FimDev &d, double lower, const uint8_t *is_seed, cudaStream_t stream)
{
  fim_support_kernel<<<grid_for(d.nV, 256, 152 * 16), 256, 0, stream>>>(d, lower, f_rd(lower), f_ru(lower),
                                                                        is_seed);
  return cudaGetLastError();
}

cudaError_t launch_mark_seeds(const FimDev &d, uint8_t *is_seed, cudaStream_t stream)
{
  if (d.nseed <= 0) return cudaSuccess;
  fim_mark_seeds_kernel<<<grid_for(d.nseed, 256, 152), 256, 0, stream>>>(d.seed_v, d.nseed, is_seed);
  return cudaGetLastError();
}

cudaError_t launch_warm_reset(const FimDev &d, double tmin, cudaStream_t stream)
{
  fim_warm_reset_kernel<<<grid_for(d.nV, 256, 152 * 16), 256, 0, stream>>>(d, tmin);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || d.nseed <= 0) return e;
  fim_reseed_kernel<<<grid_for(d.nseed, 256, 152), 256, 0, stream>>>(d);
  return cudaGetLastError();
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
