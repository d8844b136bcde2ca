// fim_mlp.cu -- the learned warm start: per-vertex features and a small
// MLP (7 -> 128 -> 128 -> 128 -> 1, ReLU) trained and evaluated on the GPU.
//
// The three hidden-layer products are BF16 x BF16 -> FP32 tensor-core GEMMs
// (mma.sync m16n8k16), one tile kernel for every shape the forward and
// backward passes need, with the epilogue fused: bias + ReLU + BF16 store
// (forward), ReLU mask + BF16 store (backward), FP32 store (weight
// gradients).
// The output layer (128 -> 1), the loss, the bias gradients and Adam are
// element-wise FP32 kernels.  Master weights are FP32; the GEMMs read BF16
// copies refreshed after every update.  The input width is padded from 7
// features to kMlpIn = 64 columns (zeros), so that every GEMM dimension is a
// multiple of the 64 x 64 tile.
//
// No counterpart in the reference.
#include "fim_internal.h"

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace fimgb {

namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16;

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, const uint32_t *b)
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M x N] = A'[M x K] B'[K x N] with A' = A (row-major, lda) or A^T (A is
// K x M), B' = B (K x N) or B^T (B is N x K); M, N multiples of 64, K of 16.
// Epilogues:
//   kEpiBiasRelu: out_bf16 = relu(C + bias[n])
//   kEpiMask:     out_bf16 = C * (mask_bf16 > 0)
//   kEpiF32:      out_f32  = C
enum { kEpiBiasRelu = 0, kEpiMask = 1, kEpiF32 = 2 };

template <int EPI>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, int lda,
                                                        int transA, const __nv_bfloat16 *__restrict__ B, int ldb,
                                                        int transB, const float *__restrict__ bias,
                                                        const __nv_bfloat16 *__restrict__ mask, __nv_bfloat16 *out16,
                                                        float *out32, int ldc)
{
  __shared__ __nv_bfloat16 As[kBM][kBK + 2];
  __shared__ __nv_bfloat16 Bs[kBK][kBN + 2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;          // warp tile 32 x 32
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int g = lane >> 2, t = lane & 3;
  float acc[2][4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kBK) {
    // tiles to shared memory (64 x 16 of A', 16 x 64 of B'), 8 elements per thread each
    for (int e = tid; e < kBM * kBK; e += 128) {
      const int r = e / kBK, c = e % kBK;
      const int m = m0 + r, k = k0 + c;
      As[r][c] = transA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
    }
    for (int e = tid; e < kBK * kBN; e += 128) {
      const int r = e / kBN, c = e % kBN;
      const int k = k0 + r, n = n0 + c;
      Bs[r][c] = transB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
    }
    __syncthreads();
#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
      const int rb = wm * 32 + mi * 16;
      uint32_t a[4];
      a[0] = pack_bf16(As[rb + g][2 * t], As[rb + g][2 * t + 1]);
      a[1] = pack_bf16(As[rb + g + 8][2 * t], As[rb + g + 8][2 * t + 1]);
      a[2] = pack_bf16(As[rb + g][2 * t + 8], As[rb + g][2 * t + 9]);
      a[3] = pack_bf16(As[rb + g + 8][2 * t + 8], As[rb + g + 8][2 * t + 9]);
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        const int cb = wn * 32 + ni * 8;
        uint32_t b[2];
        b[0] = pack_bf16(Bs[2 * t][cb + g], Bs[2 * t + 1][cb + g]);
        b[1] = pack_bf16(Bs[2 * t + 8][cb + g], Bs[2 * t + 9][cb + g]);
        mma_bf16(acc[mi][ni], a, b);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int m = m0 + wm * 32 + mi * 16 + g + (q >> 1) * 8;
        const int n = n0 + wn * 32 + ni * 8 + 2 * t + (q & 1);
        const float v = acc[mi][ni][q];
        const size_t o = (size_t)m * ldc + n;
        if (EPI == kEpiBiasRelu) out16[o] = __float2bfloat16(fmaxf(v + bias[n], 0.f));
        else if (EPI == kEpiMask) out16[o] = __float2bfloat16(__bfloat162float(mask[o]) > 0.f ? v : 0.f);
        else out32[o] = v;
      }
}

}  // namespace

cudaError_t mlp_gemm(int epi, int M, int N, int K, const void *A, int lda, int transA, const void *B, int ldb,
                     int transB, const float *bias, const void *mask, void *out16, float *out32, int ldc,
                     cudaStream_t st)
{
  if (M % kBM || N % kBN || K % kBK) return cudaErrorInvalidValue;
  const dim3 grid(N / kBN, M / kBM);
  const auto *a = static_cast<const __nv_bfloat16 *>(A);
  const auto *b = static_cast<const __nv_bfloat16 *>(B);
  const auto *mk = static_cast<const __nv_bfloat16 *>(mask);
  auto *o16 = static_cast<__nv_bfloat16 *>(out16);
  if (epi == kEpiBiasRelu)
    gemm_bf16_kernel<kEpiBiasRelu><<<grid, 128, 0, st>>>(M, N, K, a, lda, transA, b, ldb, transB, bias, mk, o16, out32, ldc);
  else if (epi == kEpiMask)
    gemm_bf16_kernel<kEpiMask><<<grid, 128, 0, st>>>(M, N, K, a, lda, transA, b, ldb, transB, bias, mk, o16, out32, ldc);
  else
    gemm_bf16_kernel<kEpiF32><<<grid, 128, 0, st>>>(M, N, K, a, lda, transA, b, ldb, transB, bias, mk, o16, out32, ldc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// element-wise parts of the network

namespace {

// y[r] = H3[r] . w4 + b4 (FP32 over the BF16 activations); with targets, the
// squared error is summed into loss and dy[r] = 2 (y - t) / n.
__global__ void out_forward_kernel(int n, const __nv_bfloat16 *__restrict__ H3, const float *__restrict__ w4,
                                   const float *__restrict__ b4, float *y, const float *__restrict__ tgt, float *dy,
                                   float *loss)
{
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= n) return;
  float s = 0.f;
  for (int c = lane; c < kMlpH; c += 32) s += __bfloat162float(H3[(size_t)r * kMlpH + c]) * w4[c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  s += b4[0];
  if (lane == 0) {
    y[r] = s;
    if (tgt) {
      const float e = s - tgt[r];
      dy[r] = 2.f * e / (float)n;
      atomicAdd(loss, e * e);
    }
  }
}

// dZ3[r][c] = bf16(dy[r] w4[c]) where H3 > 0; gw4[c] += sum_r H3[r][c] dy[r];
// gb4 += sum_r dy[r].  One block per 64 rows, one thread per column.
__global__ void out_backward_kernel(int n, const __nv_bfloat16 *__restrict__ H3, const float *__restrict__ w4,
                                    const float *__restrict__ dy, __nv_bfloat16 *dZ3, float *gw4, float *gb4)
{
  const int c = threadIdx.x;  // kMlpH threads
  const int r0 = blockIdx.x * 64;
  float sw = 0.f, sb = 0.f;
  for (int r = r0; r < min(n, r0 + 64); ++r) {
    const float h = __bfloat162float(H3[(size_t)r * kMlpH + c]);
    sw += h * dy[r];
    sb += dy[r];
    dZ3[(size_t)r * kMlpH + c] = __float2bfloat16(h > 0.f ? dy[r] * w4[c] : 0.f);
  }
  atomicAdd(&gw4[c], sw);
  if (c == 0) atomicAdd(gb4, sb);
}

// gb[c] += sum_r dZ[r][c] (bias gradients), one block per 64 rows.
__global__ void colsum_kernel(int n, const __nv_bfloat16 *__restrict__ dZ, float *gb)
{
  const int c = threadIdx.x;
  const int r0 = blockIdx.x * 64;
  float s = 0.f;
  for (int r = r0; r < min(n, r0 + 64); ++r) s += __bfloat162float(dZ[(size_t)r * kMlpH + c]);
  atomicAdd(&gb[c], s);
}

// Adam (bias-corrected) on every parameter, then the BF16 copies of the
// three GEMM weight matrices.
__global__ void adam_kernel(int np, float *P, const float *__restrict__ G, float *m, float *v, float lr, float b1,
                            float b2, float eps, float c1, float c2, __nv_bfloat16 *W16)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float g = G[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float p = P[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    P[i] = p;
    if (i < kMlpW16) W16[i] = __float2bfloat16(p);
  }
}

__global__ void to_bf16_kernel(int n, const float *__restrict__ src, __nv_bfloat16 *dst)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16(src[i]);
}

}  // namespace

// ---------------------------------------------------------------------------
// per-vertex features: [x, y, z] scaled to the bounding box, the metric
// distance to the nearest stimulus (its start time plus the straight-line
// distance in the vertex's metric), cf, ct, the fibre angle in the xy-plane

namespace {

__device__ __forceinline__ unsigned int ord_key(float x)
{
  const unsigned int b = __float_as_uint(x);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord_val(unsigned int k)
{
  return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k);
}

__global__ void feat_accum_kernel(int64_t nT, const int32_t *__restrict__ tslots, const double *__restrict__ fib,
                                  const double *__restrict__ cf, const double *__restrict__ ct, float *acc)
{
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nT; e += (int64_t)gridDim.x * blockDim.x) {
    const float f0 = (float)fib[3 * e], f1 = (float)fib[3 * e + 1], f2 = (float)fib[3 * e + 2];
    const float a = (float)cf[e], b = (float)ct[e];
    for (int t = 0; t < 4; ++t) {
      float *q = acc + 6 * (int64_t)tslots[4 * e + t];
      atomicAdd(q + 0, f0); atomicAdd(q + 1, f1); atomicAdd(q + 2, f2);
      atomicAdd(q + 3, a); atomicAdd(q + 4, b); atomicAdd(q + 5, 1.f);
    }
  }
}

// acc -> per-vertex fibre (unit), cf, ct in place; distance; reductions:
// red[0..2] bounding-box minimum, red[3..5] maximum, red[6] largest distance
__global__ void feat_dist_kernel(int nV, const double *__restrict__ xyz, float *acc, int nseed,
                                 const int32_t *__restrict__ seed_v, const double *__restrict__ seed_t, float *dist,
                                 unsigned int *red)
{
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    float *q = acc + 6 * (int64_t)v;
    const float x = (float)xyz[3 * (int64_t)v], y = (float)xyz[3 * (int64_t)v + 1], z = (float)xyz[3 * (int64_t)v + 2];
    atomicMin(red + 0, ord_key(x)); atomicMin(red + 1, ord_key(y)); atomicMin(red + 2, ord_key(z));
    atomicMax(red + 3, ord_key(x)); atomicMax(red + 4, ord_key(y)); atomicMax(red + 5, ord_key(z));
    const float cnt = q[5];
    if (!(cnt > 0.f)) { dist[v] = 0.f; continue; }
    float f0 = q[0], f1 = q[1], f2 = q[2];
    const float fn = sqrtf(f0 * f0 + f1 * f1 + f2 * f2);
    if (fn > 0.f) { f0 /= fn; f1 /= fn; f2 /= fn; } else { f0 = 1.f; f1 = f2 = 0.f; }
    const float a = q[3] / cnt, b = q[4] / cnt;
    q[0] = f0; q[1] = f1; q[2] = f2; q[3] = a; q[4] = b;
    const float ia = 1.f / (a * a), ib = 1.f / (b * b);
    float best = INFINITY;
    for (int i = 0; i < nseed; ++i) {
      const int64_t s = seed_v[i];
      const float dx = x - (float)xyz[3 * s], dy = y - (float)xyz[3 * s + 1], dz = z - (float)xyz[3 * s + 2];
      const float along = dx * f0 + dy * f1 + dz * f2;
      const float d2 = ia * along * along + ib * (dx * dx + dy * dy + dz * dz - along * along);
      best = fminf(best, (float)seed_t[i] + sqrtf(fmaxf(d2, 0.f)));
    }
    dist[v] = best;
    if (best < INFINITY) atomicMax(red + 6, ord_key(best));
  }
}

__global__ void feat_write_kernel(int nV, const double *__restrict__ xyz, const float *__restrict__ acc,
                                  const float *__restrict__ dist, const unsigned int *__restrict__ red,
                                  __nv_bfloat16 *X)
{
  float lo[3], hi[3];
  for (int k = 0; k < 3; ++k) { lo[k] = ord_val(red[k]); hi[k] = ord_val(red[3 + k]); }
  const float T = fmaxf(ord_val(red[6]), 1e-30f);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const float *q = acc + 6 * (int64_t)v;
    float f[kMlpFeatures];
    for (int k = 0; k < 3; ++k) {
      const float c = 0.5f * (lo[k] + hi[k]), h = fmaxf(0.5f * (hi[k] - lo[k]), 1e-30f);
      f[k] = ((float)xyz[3 * (int64_t)v + k] - c) / h;
    }
    const bool in = q[5] > 0.f;
    f[3] = in ? dist[v] / T : 0.f;
    f[4] = in ? q[3] : 0.f;
    f[5] = in ? q[4] : 0.f;
    f[6] = in ? atan2f(q[1], q[0]) * 0.31830988618379067f : 0.f;
    __nv_bfloat16 *row = X + (int64_t)v * kMlpIn;
    for (int k = 0; k < kMlpIn; ++k) row[k] = __float2bfloat16(k < kMlpFeatures ? f[k] : 0.f);
  }
}

}  // namespace

cudaError_t launch_features(int nV, int64_t nT, const double *xyz, const int32_t *tslots, const double *fib,
                            const double *cf, const double *ct, int nseed, const int32_t *seed_v,
                            const double *seed_t, float *acc, float *dist, unsigned int *red, void *X,
                            cudaStream_t st)
{
  cudaError_t e;
  if ((e = cudaMemsetAsync(acc, 0, sizeof(float) * 6 * (size_t)nV, st)) != cudaSuccess) return e;
  const unsigned int init[7] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u};
  if ((e = cudaMemcpyAsync(red, init, sizeof(init), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
  const int grid = 152 * 8;
  feat_accum_kernel<<<grid, 256, 0, st>>>(nT, tslots, fib, cf, ct, acc);
  feat_dist_kernel<<<grid, 256, 0, st>>>(nV, xyz, acc, nseed, seed_v, seed_t, dist, red);
  feat_write_kernel<<<grid, 256, 0, st>>>(nV, xyz, acc, dist, red, static_cast<__nv_bfloat16 *>(X));
  return cudaGetLastError();
}

float features_scale(const unsigned int *host_red)
{
  const unsigned int k = host_red[6];
  const unsigned int b = (k >> 31) ? (k & 0x7fffffffu) : ~k;
  float f;
  memcpy(&f, &b, sizeof(f));
  return f;
}

}  // namespace fimgb

// ---------------------------------------------------------------------------
// C ABI of the network (include/fim.h)

#include "../../include/fim.h"

using namespace fimgb;

static_assert(FIM_MLP_PARAMS == kMlpParams, "parameter count of the C ABI");
static_assert(FIM_MLP_INPUTS == kMlpIn, "feature width of the C ABI");

struct fim_mlp {
  int device = 0;
  cudaStream_t st = nullptr;
  float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr, *loss = nullptr;
  __nv_bfloat16 *W16 = nullptr;
  int64_t cap = 0;
  __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *dA = nullptr, *dB = nullptr;
  float *y = nullptr, *dy = nullptr;
  int64_t steps = 0;
};

namespace {

int mlp_fail(const char *what, cudaError_t e)
{
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  set_last_error(m.c_str());
  return e == cudaErrorMemoryAllocation ? FIM_ERR_OUT_OF_MEMORY : FIM_ERR_CUDA;
}

#define MLP_TRY(what, call)                                   \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return mlp_fail((what), _e);       \
  } while (0)

void mlp_free_acts(fim_mlp *m)
{
  cudaFree(m->H1); cudaFree(m->H2); cudaFree(m->H3); cudaFree(m->dA); cudaFree(m->dB);
  cudaFree(m->y); cudaFree(m->dy);
  m->H1 = m->H2 = m->H3 = m->dA = m->dB = nullptr;
  m->y = m->dy = nullptr;
  m->cap = 0;
}

int mlp_reserve(fim_mlp *m, int64_t n)
{
  if (n <= m->cap) return FIM_OK;
  mlp_free_acts(m);
  const size_t a = sizeof(__nv_bfloat16) * kMlpH * (size_t)n;
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->H1, a));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->H2, a));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->H3, a));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->dA, a));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->dB, a));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->y, sizeof(float) * n));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->dy, sizeof(float) * n));
  m->cap = n;
  return FIM_OK;
}

int mlp_check_n(int64_t n, const char *who)
{
  if (n <= 0 || n % 64 != 0 || n > (int64_t)1 << 30) {
    std::string msg = std::string(who) + ": row count must be a positive multiple of 64";
    set_last_error(msg.c_str());
    return FIM_ERR_INVALID_ARGUMENT;
  }
  return FIM_OK;
}

// forward pass of n rows of X; with targets also the loss and dy
cudaError_t mlp_forward(fim_mlp *m, int n, const void *X, const float *tgt)
{
  cudaError_t e;
  const float *P = m->P;
  if ((e = mlp_gemm(0, n, kMlpH, kMlpIn, X, kMlpIn, 0, m->W16 + kMlpOW1, kMlpH, 0, P + kMlpOB1, nullptr, m->H1,
                    nullptr, kMlpH, m->st)) != cudaSuccess) return e;
  if ((e = mlp_gemm(0, n, kMlpH, kMlpH, m->H1, kMlpH, 0, m->W16 + kMlpOW2, kMlpH, 0, P + kMlpOB2, nullptr, m->H2,
                    nullptr, kMlpH, m->st)) != cudaSuccess) return e;
  if ((e = mlp_gemm(0, n, kMlpH, kMlpH, m->H2, kMlpH, 0, m->W16 + kMlpOW3, kMlpH, 0, P + kMlpOB3, nullptr, m->H3,
                    nullptr, kMlpH, m->st)) != cudaSuccess) return e;
  out_forward_kernel<<<(n + 7) / 8, 256, 0, m->st>>>(n, m->H3, P + kMlpOW4, P + kMlpOB4, m->y, tgt, m->dy, m->loss);
  return cudaGetLastError();
}

// backward pass after mlp_forward with targets: gradients into G (zeroed by the caller)
cudaError_t mlp_backward(fim_mlp *m, int n, const void *X)
{
  cudaError_t e;
  float *G = m->G;
  const int blocks = (n + 63) / 64;
  out_backward_kernel<<<blocks, kMlpH, 0, m->st>>>(n, m->H3, m->P + kMlpOW4, m->dy, m->dA, G + kMlpOW4, G + kMlpOB4);
  // layer 3: dW3 = H2^T dZ3, db3, dZ2 = (dZ3 W3^T) o [H2 > 0]
  if ((e = mlp_gemm(2, kMlpH, kMlpH, n, m->H2, kMlpH, 1, m->dA, kMlpH, 0, nullptr, nullptr, nullptr, G + kMlpOW3,
                    kMlpH, m->st)) != cudaSuccess) return e;
  colsum_kernel<<<blocks, kMlpH, 0, m->st>>>(n, m->dA, G + kMlpOB3);
  if ((e = mlp_gemm(1, n, kMlpH, kMlpH, m->dA, kMlpH, 0, m->W16 + kMlpOW3, kMlpH, 1, nullptr, m->H2, m->dB, nullptr,
                    kMlpH, m->st)) != cudaSuccess) return e;
  // layer 2
  if ((e = mlp_gemm(2, kMlpH, kMlpH, n, m->H1, kMlpH, 1, m->dB, kMlpH, 0, nullptr, nullptr, nullptr, G + kMlpOW2,
                    kMlpH, m->st)) != cudaSuccess) return e;
  colsum_kernel<<<blocks, kMlpH, 0, m->st>>>(n, m->dB, G + kMlpOB2);
  if ((e = mlp_gemm(1, n, kMlpH, kMlpH, m->dB, kMlpH, 0, m->W16 + kMlpOW2, kMlpH, 1, nullptr, m->H1, m->dA, nullptr,
                    kMlpH, m->st)) != cudaSuccess) return e;
  // layer 1
  if ((e = mlp_gemm(2, kMlpIn, kMlpH, n, X, kMlpIn, 1, m->dA, kMlpH, 0, nullptr, nullptr, nullptr, G + kMlpOW1,
                    kMlpH, m->st)) != cudaSuccess) return e;
  colsum_kernel<<<blocks, kMlpH, 0, m->st>>>(n, m->dA, G + kMlpOB1);
  return cudaGetLastError();
}

int mlp_loss_grads(fim_mlp *m, int64_t n, const void *X, const float *tgt, float *loss_out)
{
  int rc;
  if ((rc = mlp_reserve(m, n)) != FIM_OK) return rc;
  MLP_TRY("fim_mlp: clear", cudaMemsetAsync(m->G, 0, sizeof(float) * kMlpParams, m->st));
  MLP_TRY("fim_mlp: clear", cudaMemsetAsync(m->loss, 0, sizeof(float), m->st));
  MLP_TRY("fim_mlp: forward", mlp_forward(m, (int)n, X, tgt));
  MLP_TRY("fim_mlp: backward", mlp_backward(m, (int)n, X));
  if (loss_out) {
    float l = 0.f;
    MLP_TRY("fim_mlp: loss", cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY("fim_mlp: sync", cudaStreamSynchronize(m->st));
    *loss_out = l / (float)n;
  }
  return FIM_OK;
}

}  // namespace

extern "C" int fim_mlp_create(int device, uint64_t seed, fim_mlp **out)
{
  if (!out) { set_last_error("fim_mlp_create: out is NULL"); return FIM_ERR_INVALID_ARGUMENT; }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_last_error("fim_mlp_create: no CUDA device");
    return FIM_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) { set_last_error("fim_mlp_create: bad device"); return FIM_ERR_INVALID_ARGUMENT; }
  MLP_TRY("fim_mlp_create: set device", cudaSetDevice(device));
  fim_mlp *m = new fim_mlp();
  m->device = device;
  int rc = FIM_OK;
  auto fail = [&](int code) { fim_mlp_destroy(m); return code; };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&m->st, cudaStreamDefault)) != cudaSuccess ||
      (e = cudaMalloc(&m->P, sizeof(float) * kMlpParams)) != cudaSuccess ||
      (e = cudaMalloc(&m->G, sizeof(float) * kMlpParams)) != cudaSuccess ||
      (e = cudaMalloc(&m->M, sizeof(float) * kMlpParams)) != cudaSuccess ||
      (e = cudaMalloc(&m->V, sizeof(float) * kMlpParams)) != cudaSuccess ||
      (e = cudaMalloc(&m->loss, sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&m->W16, sizeof(__nv_bfloat16) * kMlpW16)) != cudaSuccess)
    return fail(mlp_fail("fim_mlp_create", e));
  // He initialisation (fixed seed); padded input rows and biases zero
  std::vector<float> h(kMlpParams, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int i = 0; i < kMlpFeatures; ++i)
    for (int j = 0; j < kMlpH; ++j) h[kMlpOW1 + i * kMlpH + j] = nd(rng) * std::sqrt(2.f / kMlpFeatures);
  for (int i = 0; i < kMlpH * kMlpH; ++i) h[kMlpOW2 + i] = nd(rng) * std::sqrt(2.f / kMlpH);
  for (int i = 0; i < kMlpH * kMlpH; ++i) h[kMlpOW3 + i] = nd(rng) * std::sqrt(2.f / kMlpH);
  for (int i = 0; i < kMlpH; ++i) h[kMlpOW4 + i] = nd(rng) * std::sqrt(1.f / kMlpH);
  rc = fim_mlp_set_params(m, h.data());
  if (rc != FIM_OK) return fail(rc);
  *out = m;
  return FIM_OK;
}

extern "C" int fim_mlp_destroy(fim_mlp *m)
{
  if (!m) return FIM_OK;
  cudaSetDevice(m->device);
  if (m->st) cudaStreamSynchronize(m->st);
  mlp_free_acts(m);
  cudaFree(m->P); cudaFree(m->G); cudaFree(m->M); cudaFree(m->V); cudaFree(m->loss); cudaFree(m->W16);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  return FIM_OK;
}

extern "C" int fim_mlp_set_params(fim_mlp *m, const float *params)
{
  if (!m || !params) { set_last_error("fim_mlp_set_params: NULL argument"); return FIM_ERR_INVALID_ARGUMENT; }
  MLP_TRY("fim_mlp_set_params: set device", cudaSetDevice(m->device));
  MLP_TRY("fim_mlp_set_params", cudaMemcpyAsync(m->P, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, m->st));
  MLP_TRY("fim_mlp_set_params", cudaMemsetAsync(m->M, 0, sizeof(float) * kMlpParams, m->st));
  MLP_TRY("fim_mlp_set_params", cudaMemsetAsync(m->V, 0, sizeof(float) * kMlpParams, m->st));
  to_bf16_kernel<<<64, 256, 0, m->st>>>(kMlpW16, m->P, m->W16);
  MLP_TRY("fim_mlp_set_params", cudaGetLastError());
  MLP_TRY("fim_mlp_set_params", cudaStreamSynchronize(m->st));
  m->steps = 0;
  return FIM_OK;
}

extern "C" int fim_mlp_get_params(const fim_mlp *m, float *params)
{
  if (!m || !params) { set_last_error("fim_mlp_get_params: NULL argument"); return FIM_ERR_INVALID_ARGUMENT; }
  MLP_TRY("fim_mlp_get_params: set device", cudaSetDevice(m->device));
  MLP_TRY("fim_mlp_get_params", cudaMemcpy(params, m->P, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  return FIM_OK;
}

extern "C" int fim_mlp_gradients(fim_mlp *m, int64_t n, const void *d_features, const float *d_targets,
                                 float *grads, float *loss)
{
  if (!m || !d_features || !d_targets || !grads) {
    set_last_error("fim_mlp_gradients: NULL argument");
    return FIM_ERR_INVALID_ARGUMENT;
  }
  int rc;
  if ((rc = mlp_check_n(n, "fim_mlp_gradients")) != FIM_OK) return rc;
  MLP_TRY("fim_mlp_gradients: set device", cudaSetDevice(m->device));
  if ((rc = mlp_loss_grads(m, n, d_features, d_targets, loss)) != FIM_OK) return rc;
  MLP_TRY("fim_mlp_gradients", cudaMemcpyAsync(grads, m->G, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->st));
  MLP_TRY("fim_mlp_gradients", cudaStreamSynchronize(m->st));
  return FIM_OK;
}

extern "C" int fim_mlp_train_step(fim_mlp *m, int64_t n, const void *d_features, const float *d_targets, float lr,
                                  float *loss)
{
  if (!m || !d_features || !d_targets) {
    set_last_error("fim_mlp_train_step: NULL argument");
    return FIM_ERR_INVALID_ARGUMENT;
  }
  if (!(lr > 0.f) || !std::isfinite(lr)) { set_last_error("fim_mlp_train_step: bad learning rate"); return FIM_ERR_INVALID_ARGUMENT; }
  int rc;
  if ((rc = mlp_check_n(n, "fim_mlp_train_step")) != FIM_OK) return rc;
  MLP_TRY("fim_mlp_train_step: set device", cudaSetDevice(m->device));
  if ((rc = mlp_loss_grads(m, n, d_features, d_targets, loss)) != FIM_OK) return rc;
  const float b1 = 0.9f, b2 = 0.999f;
  ++m->steps;
  const float c1 = 1.f - std::pow(b1, (float)m->steps), c2 = 1.f - std::pow(b2, (float)m->steps);
  adam_kernel<<<64, 256, 0, m->st>>>(kMlpParams, m->P, m->G, m->M, m->V, lr, b1, b2, 1e-8f, c1, c2, m->W16);
  MLP_TRY("fim_mlp_train_step: adam", cudaGetLastError());
  MLP_TRY("fim_mlp_train_step", cudaStreamSynchronize(m->st));
  return FIM_OK;
}

extern "C" int fim_mlp_predict(fim_mlp *m, int64_t n, const void *d_features, float *d_out)
{
  if (!m || !d_features || !d_out) { set_last_error("fim_mlp_predict: NULL argument"); return FIM_ERR_INVALID_ARGUMENT; }
  int rc;
  if ((rc = mlp_check_n(n, "fim_mlp_predict")) != FIM_OK) return rc;
  MLP_TRY("fim_mlp_predict: set device", cudaSetDevice(m->device));
  if ((rc = mlp_reserve(m, n)) != FIM_OK) return rc;
  MLP_TRY("fim_mlp_predict: forward", mlp_forward(m, (int)n, d_features, nullptr));
  MLP_TRY("fim_mlp_predict", cudaMemcpyAsync(d_out, m->y, sizeof(float) * n, cudaMemcpyDeviceToDevice, m->st));
  MLP_TRY("fim_mlp_predict", cudaStreamSynchronize(m->st));
  return FIM_OK;
}
