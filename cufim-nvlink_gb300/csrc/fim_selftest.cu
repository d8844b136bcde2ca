// fim_selftest.cu -- checks the FP32 screens (fim_filter.cuh) against the
// FP64 local solves they bound (tri_ref / tet_ref, the reference's
// solve_tri_cu / solve_tet_cu, cuda_fim.h:1256-1360) on random corners: the
// screens are what let the solve skip most FP64 work, and the solve is
// bit-exact only while every bound they report holds.
//
// A corner: target x4 at the origin and x1, x2, x3 at random offsets of
// random size (log-uniform over three decades, degenerate shapes included),
// a random anisotropic metric M = cf^-2 f f^T + ct^-2 (I - f f^T), and times
// from one of three regimes (a plane wave through the corner with noise, a
// random spread, nearly equal times), offset by up to 100.  The screens get
// what the solve gives them: the squared edge norms scaled by 2^-k (k even,
// the largest in [0.5, 4)) as floats and the float copies of the times.
// Both tet screens are checked (with branches, and the branch-free one the
// solve uses).  Violations: a solve with a value that a screen calls impossible or puts
// outside [lb, ub], or a certain upper bound where the solve has no value.
//
// No counterpart in the reference.
#include "fim_device.cuh"
#include "fim_filter.cuh"

#include "../../include/fim.h"

#include <string>

namespace fimgb {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t s;
  __device__ double uni() { s = mix64(s); return (double)(s >> 11) * 0x1p-53; }  // [0, 1)
  __device__ double sym() { return 2.0 * uni() - 1.0; }                          // [-1, 1)
};

__device__ double norm_m(const double *M, const double *e)
{
  return (M[0] * e[0] + M[1] * e[1] + M[2] * e[2]) * e[0] + (M[1] * e[0] + M[3] * e[1] + M[4] * e[2]) * e[1] +
         (M[2] * e[0] + M[4] * e[1] + M[5] * e[2]) * e[2];
}

// out: [0] tets checked, [1] tet violations, [2] tets with a value,
//      [3] triangles checked, [4] triangle violations, [5] triangles with a value
__global__ void screen_selftest_kernel(int64_t n, uint64_t seed, unsigned long long *out)
{
  unsigned long long cnt[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    Rng r{mix64(seed ^ (uint64_t)i * 0x2545f4914f6cdd1dull)};
    const double h = exp10(-3.0 + 3.0 * r.uni());  // corner size, log-uniform in [1e-3, 1]
    double x[4][3];
    for (int v = 0; v < 3; ++v)
      for (int c = 0; c < 3; ++c) x[v][c] = h * r.sym();
    x[3][0] = x[3][1] = x[3][2] = 0.0;
    double f[3] = {r.sym(), r.sym(), r.sym()};
    const double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]) + 1e-300;
    for (int c = 0; c < 3; ++c) f[c] /= fl;
    const double cf = 0.05 + 0.95 * r.uni(), ct = cf * (0.2 + 0.8 * r.uni());
    const double a = 1.0 / (cf * cf), b = 1.0 / (ct * ct);
    const double M[6] = {b + (a - b) * f[0] * f[0], (a - b) * f[0] * f[1], (a - b) * f[0] * f[2],
                         b + (a - b) * f[1] * f[1], (a - b) * f[1] * f[2], b + (a - b) * f[2] * f[2]};
    // edges in the solve's order: e13 e23 e34 e12 e14 e24 (the target is "4")
    const int ea[6] = {0, 1, 2, 0, 0, 1}, eb[6] = {2, 2, 3, 1, 3, 3};
    double g[6];
    for (int k = 0; k < 6; ++k) {
      const double e[3] = {x[ea[k]][0] - x[eb[k]][0], x[ea[k]][1] - x[eb[k]][1], x[ea[k]][2] - x[eb[k]][2]};
      g[k] = norm_m(M, e);
    }
    // times
    const int mode = (int)(i % 3);
    const double t0 = 100.0 * r.uni();
    double p[3];
    if (mode == 0) {  // a plane wave (direction d, speed between ct and cf) with a little noise
      double d[3] = {r.sym(), r.sym(), r.sym()};
      const double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + 1e-300;
      const double sp = ct + (cf - ct) * r.uni();
      for (int v = 0; v < 3; ++v)
        p[v] = t0 + (d[0] * x[v][0] + d[1] * x[v][1] + d[2] * x[v][2]) / (dl * sp) + 0.05 * h / sp * r.sym();
    } else if (mode == 1) {  // a random spread of a few travel times over the corner
      for (int v = 0; v < 3; ++v) p[v] = t0 + 3.0 * h / ct * r.uni();
    } else {  // nearly equal
      for (int v = 0; v < 3; ++v) p[v] = t0 + 1e-6 * h * r.sym();
    }
    // the screens' inputs, as the metric kernel and the solve make them
    double gmax = g[0];
    for (int k = 1; k < 6; ++k) gmax = fmax(gmax, g[k]);
    int ex = 0;
    frexp(gmax, &ex);
    int ks = ex & ~1;
    if (ks > 50 || ks < -50) ks = 0;
    float gs[6];
    for (int k = 0; k < 6; ++k) gs[k] = (float)ldexp(g[k], -ks);
    const float pf[3] = {(float)p[0], (float)p[1], (float)p[2]};

    // tet
    {
      const double v = tet_ref(g[0], g[1], g[2], g[3], g[4], g[5], p[0], p[1], p[2]);
      const bool has = v < FIM_INF;  // a value (not INF, not NaN)
      bool bad = false;
#pragma unroll
      for (int bf = 0; bf < 2; ++bf) {  // both variants: with branches, and the solve's branch-free one
        const CandBound cb = bf ? tet_screen_bf(gs, pf[0], pf[1], pf[2], ks) : tet_screen(gs, pf[0], pf[1], pf[2], ks);
        if (has) bad = bad || cb.some == CAND_NONE || (!isnan(cb.lb) && cb.lb > v) || cb.ub < v;
        else bad = bad || cb.ub < INFINITY;
      }
      if (has) ++cnt[2];
      ++cnt[0];
      if (bad) ++cnt[1];
    }
    // triangle pairs (1,2), (2,3), (1,3) of the same corner
    const float tk = ldexpf(1.f, ks);
    for (int k = 0; k < 3; ++k) {
      const int ia = k == 1 ? 1 : 0, ib = k == 0 ? 1 : 2;
      // tri_ref(e12, e13, e23, p1, p2) with the pair's norms: (1,2): e12 e14 e24, (2,3): e23 e24 e34, (1,3): e13 e14 e34
      const int s12 = k == 0 ? 3 : (k == 1 ? 1 : 0), s13 = k == 1 ? 5 : 4, s23 = k == 0 ? 5 : 2;
      const double v = tri_ref(g[s12], g[s13], g[s23], p[ia], p[ib]);
      const CandBound cb = tri_screen_bf(re_scale(re_in(gs[s12]), tk), re_scale(re_in(gs[s13]), tk),
                                         re_scale(re_in(gs[s23]), tk), re_in(pf[ia]), re_in(pf[ib]));
      const bool has = v < FIM_INF;
      bool bad = false;
      if (has) {
        bad = cb.some == CAND_NONE || (!isnan(cb.lb) && cb.lb > v) || cb.ub < v;
        ++cnt[5];
      } else {
        bad = cb.ub < INFINITY;
      }
      ++cnt[3];
      if (bad) ++cnt[4];
    }
  }
  for (int k = 0; k < 6; ++k)
    if (cnt[k]) atomicAdd(&out[k], cnt[k]);
}

}  // namespace
}  // namespace fimgb

extern "C" int fim_selftest_screens(int device, int64_t n, uint64_t seed, int64_t *out)
{
  using namespace fimgb;
  if (!out || n < 0) { set_last_error("fim_selftest_screens: bad arguments"); return FIM_ERR_INVALID_ARGUMENT; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    set_last_error("fim_selftest_screens: no such CUDA device");
    return FIM_ERR_NO_DEVICE;
  }
  cudaError_t e = cudaSetDevice(device);
  unsigned long long *d = nullptr;
  unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMalloc(&d, sizeof h);
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof h);
  if (e == cudaSuccess) {
    screen_selftest_kernel<<<1024, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    set_last_error((std::string("fim_selftest_screens: ") + cudaGetErrorString(e)).c_str());
    return FIM_ERR_CUDA;
  }
  for (int k = 0; k < 6; ++k) out[k] = (int64_t)h[k];
  return FIM_OK;
}
