// fim_mlp.cu -- the learned warm start: per-vertex features and a small
// MLP (7 -> 128 -> 128 -> 128 -> 1, ReLU) trained and evaluated on the GPU.
//
// Every product of the three hidden layers, forward and backward, is one
// tcgen05 GEMM (C[M x 128] = A[M x K] B[128 x K]^T, BF16 operands staged by
// TMA with the 128-byte swizzle, FP32 accumulator in tensor memory) with the
// epilogue fused: bias + ReLU + BF16 store (forward), ReLU mask + BF16 store
// (backward data), FP32 store (weight gradients).  The forward GEMMs read
// transposed BF16 copies of the weights, the backward-data GEMMs the copies
// as stored, and the weight gradients transposed activations, so that every
// operand has K contiguous.
// The output layer (128 -> 1), the loss, the bias gradients and Adam are
// element-wise FP32 kernels.  Master weights are FP32; the GEMMs read BF16
// copies refreshed after every update.  The input width is padded from 7
// features to kMlpIn = 64 columns (zeros), one 128-byte K slice.
//
// No counterpart in the reference.
#include "fim_internal.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace fimgb {

namespace {

// ---------------------------------------------------------------------------
// tcgen05 GEMMs: C[M x 128] = A[M x K] B[128 x K]^T, A and B BF16 and
// K-major (rows of K contiguous), the FP32 accumulator in tensor memory.
// Operands are staged by TMA as 64-wide K slices (128 bytes, the swizzle
// span) with the 128-byte swizzle, and every mbarrier wait is bounded
// (%globaltimer): a wait that runs out sets the error word, the CTA skips
// its stores, waits (bounded) for the copies and MMAs it issued and frees
// its tensor memory.
//
// umma_gemm_kernel (the weight gradients: M <= 128, long K): one CTA of four
// warps per 128-row tile and split of K (a long K is split over up to 32
// CTAs, whose partial sums split_sum_kernel adds in a fixed order).  Warp 0
// (one lane) streams the K slices of A and B through a ring of kGemmStages
// stages (full/empty mbarriers); warp 1 (one
// lane) issues four tcgen05.mma (M = N = 128, K = 16) per slice and commits
// each slice's MMAs to the stage's empty barrier, the last one to the done
// barrier; warp 2 owns the 128 tensor-memory columns of the accumulator; all
// four warps then read it back (warp w: lanes 32w..32w+31, the tile rows)
// with tcgen05.ld and store FP32.
enum { kEpiBiasRelu = 0, kEpiMask = 1 };
constexpr int kGemmM = 128, kGemmN = 128, kGemmK = 64;  // tile rows, columns, K per stage (128 B of BF16)
constexpr int kGemmStages = 3;
constexpr uint32_t kGemmTileBytes = kGemmM * kGemmK * 2;  // one operand's slice: 16 KB (N == M)
constexpr int kGemmSmem = kGemmStages * 2 * kGemmTileBytes + 1024;  // + slack to align the ring to 1024 B
constexpr uint64_t kGemmWaitNs = 2000000000ull;  // bound of every mbarrier wait
constexpr int kGemmSplitSlices = 4;   // K slices per CTA of a split weight-gradient GEMM (at least)
constexpr int kGemmMaxSplits = 32;    // CTAs per 128-row tile at most
static_assert(kGemmN == kGemmM, "the ring holds equal A and B slices");

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t gtimer()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits until the phase with the given parity has completed; false after limit_ns
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns = kGemmWaitNs)
{
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  for (uint32_t n = 0;; ++n) {
    if (mbar_try(bar, parity)) return true;
    if ((n & 255u) == 255u && gtimer() - t0 > limit_ns) return false;
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, uint32_t src, int x, int y)
{
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
               ::"l"(reinterpret_cast<uint64_t>(map)), "r"(src), "r"(x), "r"(y)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Shared-memory matrix descriptor of a K-major operand slice with the
// 128-byte swizzle: rows of 128 B, 8-row groups 1024 B apart (stride byte
// offset), descriptor version 1, layout type 2 (128-byte swizzle).  The
// leading byte offset is unused for this layout (set to 16 B).
__device__ __forceinline__ uint64_t sdesc_k128(uint32_t addr)
{
  return (uint64_t)((addr & 0x3ffffu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits
// 4-5 = 1), BF16 A and B (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 =
// 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kGemmIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kGemmN >> 3) << 17) |
                                ((uint32_t)(kGemmM >> 4) << 24);
__device__ __forceinline__ void umma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
      ::"r"(tmem), "l"(a), "l"(b), "r"(kGemmIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 32 consecutive FP32 columns of this thread's tensor-memory lane (issued;
// tmem_wait_ld makes them readable)
__device__ __forceinline__ void tmem_ld32_issue(uint32_t taddr, uint32_t *v)
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t *v)
{
  tmem_ld32_issue(taddr, v);
  tmem_wait_ld();
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16(lo)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(hi)) << 16);
}

__global__ void __launch_bounds__(128, 1) umma_gemm_kernel(const __grid_constant__ CUtensorMap ta,
                                                           const __grid_constant__ CUtensorMap tb, int M, int K,
                                                           int kps, float *out32, int ldc, size_t split_stride,
                                                           unsigned int *err)
{
  extern __shared__ __align__(1024) unsigned char gemm_smem[];
  __shared__ __align__(8) uint64_t full_bar[kGemmStages], empty_bar[kGemmStages], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_fail, s_consumed;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ring = (smem_u32(gemm_smem) + 1023u) & ~1023u;
  const int m0 = blockIdx.x * kGemmM;
  // split blockIdx.y of K: slices [k0, k0 + nk), its partial sums at out32 + blockIdx.y * split_stride
  const int k0 = blockIdx.y * kps;
  const int nk = min(kps, K / kGemmK - k0);
  out32 += blockIdx.y * split_stride;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kGemmStages; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&done_bar), 1);
    s_fail = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&ta)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tb)) : "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kGemmN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  int issued = 0;
  if (warp == 0 && lane == 0) {
    // producer: K slice i into stage i % kGemmStages once the MMAs of slice
    // i - kGemmStages have released it
    for (int i = 0; i < nk; ++i) {
      const int s = i % kGemmStages;
      const uint32_t ph = (uint32_t)(i / kGemmStages) & 1u;
      if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u)) { s_fail = 1; break; }
      const uint32_t fb = smem_u32(&full_bar[s]);
      mbar_expect_tx(fb, 2 * kGemmTileBytes);
      tma_load_2d(ring + s * kGemmTileBytes, &ta, (k0 + i) * kGemmK, m0, fb);
      tma_load_2d(ring + (kGemmStages + s) * kGemmTileBytes, &tb, (k0 + i) * kGemmK, 0, fb);
      issued = i + 1;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: four K = 16 steps per slice (32 bytes apart within the
    // swizzled 128-byte rows)
    int i = 0;
    for (; i < nk; ++i) {
      const int s = i % kGemmStages;
      const uint32_t ph = (uint32_t)(i / kGemmStages) & 1u;
      if (!mbar_wait(smem_u32(&full_bar[s]), ph)) { s_fail = 1; break; }
      tc_fence_after();
      const uint32_t a = ring + s * kGemmTileBytes, b = ring + (kGemmStages + s) * kGemmTileBytes;
#pragma unroll
      for (int k = 0; k < kGemmK / 16; ++k)
        umma_bf16(tmem, sdesc_k128(a + 32 * k), sdesc_k128(b + 32 * k), (uint32_t)(i | k));
      umma_commit(smem_u32(&empty_bar[s]));
    }
    s_consumed = i;
    umma_commit(smem_u32(&done_bar));  // arrives once every MMA issued above has completed
  }
  __syncwarp();
  // the whole K loop runs before this completes: the bound grows with it
  if (!mbar_wait(smem_u32(&done_bar), 0, kGemmWaitNs + 20000ull * (uint64_t)nk)) s_fail = 1;
  tc_fence_after();
  const bool ok = s_fail == 0;

  // epilogue: this thread's row, 32 columns per tensor-memory load
  const int row = m0 + warp * 32 + lane;
  const bool store = ok && row < M;
#pragma unroll 1
  for (int c0 = 0; c0 < kGemmN; c0 += 32) {
    uint32_t v[32];
    tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
    if (!store) continue;
    float4 *o = reinterpret_cast<float4 *>(out32 + (size_t)row * ldc + c0);
#pragma unroll
    for (int q = 0; q < 8; ++q)
      o[q] = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]), __uint_as_float(v[4 * q + 2]),
                         __uint_as_float(v[4 * q + 3]));
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicOr(err, 1u);
    // copies issued but not consumed by an MMA still land in the ring: wait for them
    if (warp == 0 && lane == 0)
      for (int i = s_consumed; i < issued; ++i)
        (void)mbar_wait(smem_u32(&full_bar[i % kGemmStages]), (uint32_t)(i / kGemmStages) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 2)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kGemmN) : "memory");
}

// ---------------------------------------------------------------------------
// Persistent row-tile GEMM for the tall products (M = rows, K = 64 or 128):
// C[M x 128] = A[M x K] W[128 x K]^T, one CTA per SM looping over 128-row
// tiles.  The weights (B) are loaded once per CTA; warp 0 streams A tiles
// through a ring of kRowStages stages; warp 1 issues the MMAs of tile j into
// tensor-memory accumulator j % 2; warps 2-9 drain accumulator j % 2 (warp w
// reads lanes 32 (w % 4) .. +31, the tile rows, and columns 64 h .. 64 h + 63
// with h = (w - 2) / 4) while the MMAs of tile j + 1 run, release it (tempty)
// and then apply the epilogue:
//   kEpiBiasRelu:    out_bf16 = relu(C + bias)
//   kEpiMask:        out_bf16 = C * (mask_bf16 > 0)
//   kEpiBiasReluOut: h = bf16(relu(C + bias)) (stored when out_bf16 is set),
//                    y = h . w4 + b4 (the output layer), and with targets
//                    dy = 2 (y - t) / M and the summed squared error; the
//                    warps of columns 64..127 hand their partial dot
//                    products to those of columns 0..63 through shared
//                    memory (mbarrier ypart), which add them in a fixed
//                    order and release the accumulator after reading them.
enum { kEpiBiasReluOut = 3 };
constexpr int kRowStages = 3;
constexpr int kRowKMax = 128, kRowSlices = kRowKMax / kGemmK;
constexpr uint32_t kRowStageBytes = kRowSlices * kGemmTileBytes;     // one A tile (32 KB)
constexpr uint32_t kRowStgBytes = 32 * kGemmK * 2;  // one epilogue warp's 32 x 64 output box (4 KB)
constexpr int kRowEpiWarps = 8;
// B + the A ring + two output boxes per epilogue warp + alignment slack
constexpr int kRowSmem = (1 + kRowStages) * kRowStageBytes + 2 * kRowEpiWarps * kRowStgBytes + 1024;
constexpr int kRowThreads = 320;  // producer, MMA issuer, 8 epilogue warps

template <int EPI>
__global__ void __launch_bounds__(kRowThreads, 1) umma_rows_kernel(
    const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
    const __grid_constant__ CUtensorMap to, int M, int K, const float *__restrict__ bias,
    const __nv_bfloat16 *__restrict__ mask, int store, int ldc,
    const float *__restrict__ w4, const float *__restrict__ b4, float *y, const float *__restrict__ tgt, float *dy,
    float *loss, unsigned int *err)
{
  extern __shared__ __align__(1024) unsigned char gemm_smem[];
  __shared__ __align__(8) uint64_t bfull, afull[kRowStages], aempty[kRowStages], tfull[2], tempty[2], ypart[2];
  __shared__ float s_part[2][kGemmM];
  __shared__ uint32_t tmem_base;
  __shared__ float s_bias[kGemmN], s_w4[kGemmN];
  __shared__ volatile int s_fail;
  __shared__ int s_issued, s_consumed, s_mma_issued, s_drained;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t bsm = (smem_u32(gemm_smem) + 1023u) & ~1023u, aring = bsm + kRowStageBytes;
  const uint32_t stg0 = aring + kRowStages * kRowStageBytes;  // output boxes: [warp - 2][tile parity]
  const int nks = K / kGemmK;
  const uint32_t tile_bytes = (uint32_t)nks * kGemmTileBytes;
  const int ntiles = (M + kGemmM - 1) / kGemmM;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bfull), 1);
    for (int s = 0; s < kRowStages; ++s) {
      mbar_init(smem_u32(&afull[s]), 1);
      mbar_init(smem_u32(&aempty[s]), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(smem_u32(&tfull[a]), 1);
      mbar_init(smem_u32(&tempty[a]), 8);  // one arrival per epilogue warp
      mbar_init(smem_u32(&ypart[a]), 4);   // the warps of columns 64..127
    }
    s_fail = 0;
    s_issued = s_consumed = s_mma_issued = s_drained = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&ta)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tb)) : "memory");
    if (store) asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&to)) : "memory");
  }
  if (threadIdx.x < kGemmN) {
    s_bias[threadIdx.x] = (EPI == kEpiMask) ? 0.f : bias[threadIdx.x];
    s_w4[threadIdx.x] = (EPI == kEpiBiasReluOut) ? w4[threadIdx.x] : 0.f;
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(2 * kGemmN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      // producer: the weights once, then A tile j into stage j % kRowStages
      mbar_expect_tx(smem_u32(&bfull), tile_bytes);
      for (int ks = 0; ks < nks; ++ks)
        tma_load_2d(bsm + ks * kGemmTileBytes, &tb, ks * kGemmK, 0, smem_u32(&bfull));
      int j = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++j) {
        const int s = j % kRowStages;
        if (s_fail || !mbar_wait(smem_u32(&aempty[s]), ((uint32_t)(j / kRowStages) & 1u) ^ 1u)) { s_fail = 1; break; }
        const uint32_t fb = smem_u32(&afull[s]);
        mbar_expect_tx(fb, tile_bytes);
        for (int ks = 0; ks < nks; ++ks)
          tma_load_2d(aring + s * kRowStageBytes + ks * kGemmTileBytes, &ta, ks * kGemmK, tile * kGemmM, fb);
        s_issued = j + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: tile j into accumulator j % 2 once the epilogue has drained it
      if (!mbar_wait(smem_u32(&bfull), 0)) s_fail = 1;
      int j = 0;
      for (int tile = blockIdx.x; tile < ntiles && !s_fail; tile += gridDim.x, ++j) {
        const int s = j % kRowStages, acc = j & 1;
        if (!mbar_wait(smem_u32(&tempty[acc]), ((uint32_t)(j >> 1) & 1u) ^ 1u) ||
            !mbar_wait(smem_u32(&afull[s]), (uint32_t)(j / kRowStages) & 1u)) { s_fail = 1; break; }
        tc_fence_after();
        const uint32_t a = aring + s * kRowStageBytes, d = tmem + (uint32_t)(acc * kGemmN);
        for (int ks = 0; ks < nks; ++ks)
#pragma unroll
          for (int k = 0; k < kGemmK / 16; ++k)
            umma_bf16(d, sdesc_k128(a + ks * kGemmTileBytes + 32 * k), sdesc_k128(bsm + ks * kGemmTileBytes + 32 * k),
                      (uint32_t)(ks | k));
        umma_commit(smem_u32(&aempty[s]));
        umma_commit(smem_u32(&tfull[acc]));
        s_consumed = j + 1;
        s_mma_issued = j + 1;
      }
    }
  } else {
    // epilogue warps 2..9: tensor-memory lanes 32 q .. 32 q + 31 (tile rows),
    // columns cb .. cb + 63
    const int q = warp & 3, h = (warp - 2) >> 2, cb = 64 * h;
    auto release = [&](int acc, int j) {
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[acc])) : "memory");
      if (warp == 2 && lane == 0) s_drained = j + 1;
    };
    int j = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++j) {
      const int acc = j & 1;
      const uint32_t par = (uint32_t)(j >> 1) & 1u;
      if (s_fail || !mbar_wait(smem_u32(&tfull[acc]), par)) { s_fail = 1; break; }
      tc_fence_after();
      const int row = tile * kGemmM + q * 32 + lane;
      const bool in = row < M;
      uint32_t v[64];
      const uint32_t tv = tmem + (uint32_t)(acc * kGemmN) + ((uint32_t)(q * 32) << 16) + (uint32_t)cb;
      tmem_ld32_issue(tv, v);
      tmem_ld32_issue(tv + 32, v + 32);
      tmem_wait_ld();
      const bool combine = EPI == kEpiBiasReluOut && h == 0;  // releases after reading the partials
      if (!combine) release(acc, j);
      // this warp's 32 x 64 output box goes through shared memory (128-byte
      // swizzle: 16-byte chunk c of row r at chunk c ^ (r % 8)) and one TMA
      // store, which clips the rows past M; first the store issued from the
      // same buffer two tiles ago must have read it
      const uint32_t stg = stg0 + (uint32_t)(((warp - 2) * 2 + (j & 1)) * kRowStgBytes);
      if (store) {
        if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        __syncwarp();
      }
      float ysum = 0.f;
#pragma unroll
      for (int c = 0; c < 64; c += 32) {
        const int col = cb + c;
        uint32_t w[16];
        if (EPI == kEpiMask) {
          const uint4 *mk = reinterpret_cast<const uint4 *>(mask + (size_t)row * ldc + col);
#pragma unroll
          for (int q4 = 0; q4 < 4; ++q4) {
            const uint4 mm = in ? mk[q4] : make_uint4(0u, 0u, 0u, 0u);
            const uint32_t mw[4] = {mm.x, mm.y, mm.z, mm.w};
#pragma unroll
            for (int hh = 0; hh < 4; ++hh) {
              const int e = 4 * q4 + hh;
              const float lo = __bfloat162float(__ushort_as_bfloat16((unsigned short)(mw[hh] & 0xffffu)));
              const float hi = __bfloat162float(__ushort_as_bfloat16((unsigned short)(mw[hh] >> 16)));
              w[e] = pack_bf16(lo > 0.f ? __uint_as_float(v[c + 2 * e]) : 0.f,
                               hi > 0.f ? __uint_as_float(v[c + 2 * e + 1]) : 0.f);
            }
          }
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            w[e] = pack_bf16(fmaxf(__uint_as_float(v[c + 2 * e]) + s_bias[col + 2 * e], 0.f),
                             fmaxf(__uint_as_float(v[c + 2 * e + 1]) + s_bias[col + 2 * e + 1], 0.f));
            if (EPI == kEpiBiasReluOut) {  // the output layer on the stored (BF16) activations
              ysum += __bfloat162float(__ushort_as_bfloat16((unsigned short)(w[e] & 0xffffu))) * s_w4[col + 2 * e];
              ysum += __bfloat162float(__ushort_as_bfloat16((unsigned short)(w[e] >> 16))) * s_w4[col + 2 * e + 1];
            }
          }
        }
        if (store) {
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4) {
            const uint32_t chunk = (uint32_t)((c >> 3) + k4) ^ (uint32_t)(lane & 7);
            const uint32_t a = stg + (uint32_t)lane * 128u + chunk * 16u;
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(w[4 * k4]), "r"(w[4 * k4 + 1]),
                         "r"(w[4 * k4 + 2]), "r"(w[4 * k4 + 3])
                         : "memory");
          }
        }
      }
      if (store) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) tma_store_2d(&to, stg, cb, tile * kGemmM + q * 32);
      }
      if (EPI == kEpiBiasReluOut) {
        if (h == 1) {  // hand the partial dot product over
          s_part[acc][q * 32 + lane] = ysum;
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&ypart[acc])) : "memory");
        } else {
          const bool okp = mbar_wait(smem_u32(&ypart[acc]), par);
          if (!okp) s_fail = 1;
          const float p1 = s_part[acc][q * 32 + lane];
          release(acc, j);
          float se = 0.f;
          if (okp && in) {
            const float yv = (ysum + p1) + b4[0];
            y[row] = yv;
            if (tgt) {
              const float e = yv - tgt[row];
              dy[row] = 2.f * e / (float)M;
              se = e * e;
            }
          }
          if (tgt) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
            if (lane == 0) atomicAdd(loss, se);
          }
        }
      }
    }
    if (store && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // the output is written
  }
  __syncthreads();
  if (s_fail) {
    if (threadIdx.x == 0) {
      atomicOr(err, 1u);
      // the weights, copies issued but not consumed, MMAs issued but not
      // drained: let them land (bounded)
      (void)mbar_wait(smem_u32(&bfull), 0);
      for (int j = s_consumed; j < s_issued; ++j)
        (void)mbar_wait(smem_u32(&afull[j % kRowStages]), (uint32_t)(j / kRowStages) & 1u);
      for (int j = s_drained; j < s_mma_issued; ++j)
        (void)mbar_wait(smem_u32(&tfull[j & 1]), (uint32_t)(j >> 1) & 1u);
    }
    __syncthreads();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 2)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kGemmN) : "memory");
}

// out[c][r] = in[r][c] for an R x C BF16 matrix (R, C multiples of 32)
__global__ void transpose_bf16_kernel(int R, int C, const __nv_bfloat16 *__restrict__ in, __nv_bfloat16 *out)
{
  __shared__ __nv_bfloat16 t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) t[k][threadIdx.x] = in[(size_t)(r0 + k) * C + c0 + threadIdx.x];
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) out[(size_t)(c0 + k) * R + r0 + threadIdx.x] = t[threadIdx.x][k];
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// Tensor map of a rows x k BF16 matrix (row-major, k contiguous): boxes of
// 64 columns (128 B, the swizzle span) by 128 rows; rows beyond the matrix
// read as zeros.
bool make_map(CUtensorMap *map, const void *base, uint64_t k, uint64_t rows, uint32_t box_rows = kGemmM)
{
  const auto enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(base) & 15u) || k % kGemmK) return false;
  const cuuint64_t dims[2] = {k, rows};
  const cuuint64_t strides[1] = {k * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kGemmK, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

namespace {
// out[r][c] = sum over the splits, in split order (deterministic), of the
// partial sums ws[s][r][c] (row stride ldc, split stride M * ldc)
__global__ void split_sum_kernel(int M, int ldc, int splits, const float *__restrict__ ws, float *out)
{
  const int n = M * kGemmN;
  const size_t st = (size_t)M * ldc;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int r = i / kGemmN, c = i % kGemmN;
    const float *p = ws + (size_t)r * ldc + c;
    float acc = 0.f;
#pragma unroll 8
    for (int s = 0; s < splits; ++s) acc += p[s * st];
    out[(size_t)r * ldc + c] = acc;
  }
}
}  // namespace

// Weight gradients: C[M x 128] = A[M x K] B[128 x K]^T (FP32 out) for BF16
// A (rows_a >= M rows) and B (128 rows), both with K contiguous, K a
// multiple of 64 (the K loop of umma_gemm_kernel).  A long K is split over
// up to kGemmMaxSplits CTAs per 128-row tile (kGemmSplitSlices K slices
// each, partial sums in ws, which holds kGemmMaxSplits * M * ldc floats) and
// summed in split order; without ws one CTA per tile runs the whole K.
cudaError_t mlp_gemm_wgrad(int M, int K, const void *A, int rows_a, const void *B, float *out32, int ldc, float *ws,
                           unsigned int *err, cudaStream_t st)
{
  if (M <= 0 || K <= 0 || K % kGemmK || rows_a < M) return cudaErrorInvalidValue;
  CUtensorMap ta, tb;
  if (!make_map(&ta, A, (uint64_t)K, (uint64_t)rows_a) || !make_map(&tb, B, (uint64_t)K, kGemmN))
    return cudaErrorInvalidValue;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(umma_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem)) !=
      cudaSuccess) return e;
  const int nk = K / kGemmK;
  int kps = nk, splits = 1;
  if (ws && nk > kGemmSplitSlices) {
    kps = std::max(kGemmSplitSlices, (nk + kGemmMaxSplits - 1) / kGemmMaxSplits);
    splits = (nk + kps - 1) / kps;
  }
  const dim3 grid((M + kGemmM - 1) / kGemmM, splits);
  if (splits == 1) {
    umma_gemm_kernel<<<grid, 128, kGemmSmem, st>>>(ta, tb, M, K, kps, out32, ldc, 0, err);
    return cudaGetLastError();
  }
  umma_gemm_kernel<<<grid, 128, kGemmSmem, st>>>(ta, tb, M, K, kps, ws, ldc, (size_t)M * ldc, err);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  split_sum_kernel<<<(M * kGemmN + 255) / 256, 256, 0, st>>>(M, ldc, splits, ws, out32);
  return cudaGetLastError();
}

// The tall products: C[M x 128] = A[M x K] W[128 x K]^T with K = 64 or 128
// (umma_rows_kernel, one CTA per SM); epilogue arguments as the kernel's.
struct RowEpi {
  const float *bias = nullptr;
  const void *mask = nullptr;
  void *out16 = nullptr;
  const float *w4 = nullptr, *b4 = nullptr;
  float *y = nullptr;
  const float *tgt = nullptr;
  float *dy = nullptr, *loss = nullptr;
};

cudaError_t mlp_gemm_rows(int epi, int M, int K, const void *A, const void *W, const RowEpi &x, unsigned int *err,
                          cudaStream_t st)
{
  if (M <= 0 || (K != 64 && K != 128)) return cudaErrorInvalidValue;
  CUtensorMap ta, tb;
  CUtensorMap to;  // the output in 32 x 64 boxes (unused without a BF16 output)
  const int store = x.out16 != nullptr;
  if (!make_map(&ta, A, (uint64_t)K, (uint64_t)M) || !make_map(&tb, W, (uint64_t)K, kGemmN))
    return cudaErrorInvalidValue;
  if (!store) to = ta;
  else if (!make_map(&to, x.out16, kGemmN, (uint64_t)M, 32)) return cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  const int ntiles = (M + kGemmM - 1) / kGemmM;
  const dim3 grid(std::min(ntiles, nsm));
  const auto *mk = static_cast<const __nv_bfloat16 *>(x.mask);
#define FIM_ROWS_LAUNCH(E)                                                                                           \
  do {                                                                                                              \
    if ((e = cudaFuncSetAttribute(umma_rows_kernel<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRowSmem)) !=   \
        cudaSuccess)                                                                                                \
      return e;                                                                                                     \
    umma_rows_kernel<E><<<grid, kRowThreads, kRowSmem, st>>>(ta, tb, to, M, K, x.bias, mk, store, kGemmN, x.w4, x.b4, \
                                                             x.y, x.tgt, x.dy, x.loss, err);                       \
  } while (0)
  if (epi == kEpiBiasRelu) FIM_ROWS_LAUNCH(kEpiBiasRelu);
  else if (epi == kEpiMask) FIM_ROWS_LAUNCH(kEpiMask);
  else if (epi == kEpiBiasReluOut) FIM_ROWS_LAUNCH(kEpiBiasReluOut);
  else return cudaErrorInvalidValue;
#undef FIM_ROWS_LAUNCH
  return cudaGetLastError();
}

cudaError_t mlp_transpose(int R, int C, const void *in, void *out, cudaStream_t st)
{
  if (R % 32 || C % 32) return cudaErrorInvalidValue;
  transpose_bf16_kernel<<<dim3(C / 32, R / 32), dim3(32, 8), 0, st>>>(R, C, static_cast<const __nv_bfloat16 *>(in),
                                                                       static_cast<__nv_bfloat16 *>(out));
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// element-wise parts of the network

namespace {

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

// Index of weight i (W1 [kMlpIn x kMlpH], W2, W3 [kMlpH x kMlpH], each
// [in x out] row-major) in the transposed copies [out x in] that the forward
// GEMMs read as their K-major B operand.
__device__ __forceinline__ int transposed_index(int i)
{
  if (i < kMlpOW2) return kMlpOW1 + (i % kMlpH) * kMlpIn + i / kMlpH;
  const int off = i < kMlpOW3 ? kMlpOW2 : kMlpOW3, k = i - off;
  return off + (k % kMlpH) * kMlpH + k / kMlpH;
}

// Adam (bias-corrected) on every parameter, then the BF16 copies of the
// three GEMM weight matrices (as stored and transposed).
__global__ void adam_kernel(int np, float *P, const float *__restrict__ G, float *m, float *v, float lr, float b1,
                            float b2, float eps, float c1, float c2, __nv_bfloat16 *W16, __nv_bfloat16 *W16T)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float g = G[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float p = P[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    P[i] = p;
    if (i < kMlpW16) {
      W16[i] = __float2bfloat16(p);
      W16T[transposed_index(i)] = __float2bfloat16(p);
    }
  }
}

__global__ void to_bf16_kernel(const float *__restrict__ src, __nv_bfloat16 *W16, __nv_bfloat16 *W16T)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpW16; i += gridDim.x * blockDim.x) {
    W16[i] = __float2bfloat16(src[i]);
    W16T[transposed_index(i)] = __float2bfloat16(src[i]);
  }
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
  __nv_bfloat16 *W16 = nullptr, *W16T = nullptr;  // GEMM weights as stored ([in x out]) and transposed
  unsigned int *err = nullptr;                     // set by a GEMM whose bounded wait ran out
  unsigned int h_err = 0;
  int64_t cap = 0;
  __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *dA = nullptr, *dB = nullptr;
  __nv_bfloat16 *HT = nullptr, *DT = nullptr;     // [kMlpH x cap] transposes for the weight gradients
  float *y = nullptr, *dy = nullptr;
  float *ws = nullptr;                             // split-K partial sums of the weight gradients
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
  cudaFree(m->HT); cudaFree(m->DT);
  cudaFree(m->y); cudaFree(m->dy);
  m->H1 = m->H2 = m->H3 = m->dA = m->dB = m->HT = m->DT = nullptr;
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
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->HT, a));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->DT, a));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->y, sizeof(float) * n));
  MLP_TRY("fim_mlp: activations", cudaMalloc(&m->dy, sizeof(float) * n));
  m->cap = n;
  return FIM_OK;
}

// Queues the read of the GEMMs' error word (before the caller's stream
// synchronisation); mlp_gemm_status then reports it after the sync.
cudaError_t mlp_read_err(fim_mlp *m)
{
  return cudaMemcpyAsync(&m->h_err, m->err, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->st);
}
int mlp_gemm_status(fim_mlp *m, const char *who)
{
  if (m->h_err == 0) return FIM_OK;
  m->h_err = 0;
  cudaMemset(m->err, 0, sizeof(unsigned int));
  std::string msg = std::string(who) + ": a tensor-core GEMM wait ran out (results discarded)";
  set_last_error(msg.c_str());
  return FIM_ERR_TIMEOUT;
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
  // H_l = relu(H_{l-1} W_l + b_l): B operand = W_l^T [out x in]; the last
  // layer's epilogue also evaluates the output layer (and, with targets,
  // dy and the loss); H3 is stored only for the backward pass
  RowEpi x1, x2, x3;
  x1.bias = P + kMlpOB1; x1.out16 = m->H1;
  x2.bias = P + kMlpOB2; x2.out16 = m->H2;
  x3.bias = P + kMlpOB3; x3.out16 = tgt ? m->H3 : nullptr;
  x3.w4 = P + kMlpOW4; x3.b4 = P + kMlpOB4; x3.y = m->y; x3.tgt = tgt; x3.dy = m->dy; x3.loss = m->loss;
  if ((e = mlp_gemm_rows(kEpiBiasRelu, n, kMlpIn, X, m->W16T + kMlpOW1, x1, m->err, m->st)) != cudaSuccess) return e;
  if ((e = mlp_gemm_rows(kEpiBiasRelu, n, kMlpH, m->H1, m->W16T + kMlpOW2, x2, m->err, m->st)) != cudaSuccess) return e;
  if ((e = mlp_gemm_rows(kEpiBiasReluOut, n, kMlpH, m->H2, m->W16T + kMlpOW3, x3, m->err, m->st)) != cudaSuccess)
    return e;
  return cudaGetLastError();
}

// backward pass after mlp_forward with targets: gradients into G (zeroed by the caller)
cudaError_t mlp_backward(fim_mlp *m, int n, const void *X)
{
  cudaError_t e;
  float *G = m->G;
  const int blocks = (n + 63) / 64;
  out_backward_kernel<<<blocks, kMlpH, 0, m->st>>>(n, m->H3, m->P + kMlpOW4, m->dy, m->dA, G + kMlpOW4, G + kMlpOB4);
  // layer l: dW_l = H_{l-1}^T dZ_l (both transposed so that K = rows is
  // contiguous), db_l, dZ_{l-1} = (dZ_l W_l^T) o [H_{l-1} > 0] (B operand =
  // W_l as stored, [in x out])
  // layer 3
  if ((e = mlp_transpose(n, kMlpH, m->H2, m->HT, m->st)) != cudaSuccess) return e;
  if ((e = mlp_transpose(n, kMlpH, m->dA, m->DT, m->st)) != cudaSuccess) return e;
  if ((e = mlp_gemm_wgrad(kMlpH, n, m->HT, kMlpH, m->DT, G + kMlpOW3, kMlpH, m->ws, m->err, m->st)) != cudaSuccess) return e;
  colsum_kernel<<<blocks, kMlpH, 0, m->st>>>(n, m->dA, G + kMlpOB3);
  RowEpi xm;
  xm.mask = m->H2; xm.out16 = m->dB;
  if ((e = mlp_gemm_rows(kEpiMask, n, kMlpH, m->dA, m->W16 + kMlpOW3, xm, m->err, m->st)) != cudaSuccess) return e;
  // layer 2
  if ((e = mlp_transpose(n, kMlpH, m->H1, m->HT, m->st)) != cudaSuccess) return e;
  if ((e = mlp_transpose(n, kMlpH, m->dB, m->DT, m->st)) != cudaSuccess) return e;
  if ((e = mlp_gemm_wgrad(kMlpH, n, m->HT, kMlpH, m->DT, G + kMlpOW2, kMlpH, m->ws, m->err, m->st)) != cudaSuccess) return e;
  colsum_kernel<<<blocks, kMlpH, 0, m->st>>>(n, m->dB, G + kMlpOB2);
  xm.mask = m->H1; xm.out16 = m->dA;
  if ((e = mlp_gemm_rows(kEpiMask, n, kMlpH, m->dB, m->W16 + kMlpOW2, xm, m->err, m->st)) != cudaSuccess) return e;
  // layer 1: X^T is kMlpIn rows; the tile's other rows (left over in HT)
  // only reach output rows that are not stored
  if ((e = mlp_transpose(n, kMlpIn, X, m->HT, m->st)) != cudaSuccess) return e;
  if ((e = mlp_transpose(n, kMlpH, m->dA, m->DT, m->st)) != cudaSuccess) return e;
  if ((e = mlp_gemm_wgrad(kMlpIn, n, m->HT, kMlpH, m->DT, G + kMlpOW1, kMlpH, m->ws, m->err, m->st)) != cudaSuccess) return e;
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
      (e = cudaMalloc(&m->W16, sizeof(__nv_bfloat16) * kMlpW16)) != cudaSuccess ||
      (e = cudaMalloc(&m->W16T, sizeof(__nv_bfloat16) * kMlpW16)) != cudaSuccess ||
      (e = cudaMalloc(&m->err, sizeof(unsigned int))) != cudaSuccess ||
      (e = cudaMalloc(&m->ws, sizeof(float) * kGemmMaxSplits * kMlpH * kMlpH)) != cudaSuccess ||
      (e = cudaMemset(m->err, 0, sizeof(unsigned int))) != cudaSuccess)
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
  cudaFree(m->W16T); cudaFree(m->err); cudaFree(m->ws);
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
  to_bf16_kernel<<<64, 256, 0, m->st>>>(m->P, m->W16, m->W16T);
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
  MLP_TRY("fim_mlp_gradients", mlp_read_err(m));
  MLP_TRY("fim_mlp_gradients", cudaStreamSynchronize(m->st));
  return mlp_gemm_status(m, "fim_mlp_gradients");
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
  adam_kernel<<<64, 256, 0, m->st>>>(kMlpParams, m->P, m->G, m->M, m->V, lr, b1, b2, 1e-8f, c1, c2, m->W16, m->W16T);
  MLP_TRY("fim_mlp_train_step: adam", cudaGetLastError());
  MLP_TRY("fim_mlp_train_step", mlp_read_err(m));
  MLP_TRY("fim_mlp_train_step", cudaStreamSynchronize(m->st));
  return mlp_gemm_status(m, "fim_mlp_train_step");
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
  MLP_TRY("fim_mlp_predict", mlp_read_err(m));
  MLP_TRY("fim_mlp_predict", cudaStreamSynchronize(m->st));
  return mlp_gemm_status(m, "fim_mlp_predict");
}
