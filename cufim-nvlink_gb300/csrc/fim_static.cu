// fim_static.cu -- the fixed device scratch of fim_solve_noalloc.
//
// fim_solve_noalloc re-solves a solver's staged mesh for a new set of
// stimuli without allocating anything: the persistent solve kernel's
// per-solve working set (times, states, iteration stamps, the rotating
// lists, the control block) and the stimulus staging live in one
// file-scope device array of fixed size, instead of in the solver's
// cudaMalloc'd buffers.  The array belongs to this translation unit's
// module, so it is only loaded on devices where this path is used.
//
// Layout (every part starts on a 256-byte boundary): per vertex copy
// phi, phi2 (f64), sw (u32), list[3], lfrozen, lmarked (i32), phi_f,
// phi2_f (f32), st, tst, dec (u8); per mesh vertex the gathered states st_out (u8) and
// the stimulus keys (u64); the raw stimuli as given (i64 vertex, f64
// time), the stimulus entries expanded to vertex copies (i32, f64); the
// control block FimCtl.
//
// What must start at zero: only the FimCtl block (barrier counter and
// generation, list counters, error word).  fim_solve_noalloc clears it with
// cudaMemsetAsync before every launch.  Everything else is written before it
// is read within one call: the solve kernel resets phi/phi2/sw/tst of every
// copy, the lists are filled behind their counters, and the stimulus
// kernel sets the key of every stimulated vertex before it takes minima.
#include "fim_internal.h"

#include <mutex>

namespace fimgb {

namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

constexpr size_t kC = (size_t)kStaticMaxCopies;
constexpr size_t kG = (size_t)kStaticMaxVertices;
constexpr size_t kOffPhi = 0;
constexpr size_t kOffPhi2 = kOffPhi + align256(8 * kC);
constexpr size_t kOffSw = kOffPhi2 + align256(8 * kC);
constexpr size_t kOffList0 = kOffSw + align256(4 * kC);
constexpr size_t kOffList1 = kOffList0 + align256(4 * kC);
constexpr size_t kOffList2 = kOffList1 + align256(4 * kC);
constexpr size_t kOffFrozen = kOffList2 + align256(4 * kC);
constexpr size_t kOffMarked = kOffFrozen + align256(4 * kC);
constexpr size_t kOffPhiF = kOffMarked + align256(4 * kC);
constexpr size_t kOffPhi2F = kOffPhiF + align256(4 * kC);
constexpr size_t kOffSt = kOffPhi2F + align256(4 * kC);
constexpr size_t kOffTst = kOffSt + align256(kC);
constexpr size_t kOffDec = kOffTst + align256(kC);
constexpr size_t kOffStOut = kOffDec + align256(kC);
constexpr size_t kOffKey = kOffStOut + align256(kG);
constexpr size_t kOffRawV = kOffKey + align256(8 * kG);
constexpr size_t kOffRawT = kOffRawV + align256(8 * (size_t)kStaticMaxSeeds);
constexpr size_t kOffSeedV = kOffRawT + align256(8 * (size_t)kStaticMaxSeeds);
constexpr size_t kOffSeedT = kOffSeedV + align256(4 * (size_t)kStaticMaxSeedEntries);
constexpr size_t kOffCtl = kOffSeedT + align256(8 * (size_t)kStaticMaxSeedEntries);
constexpr size_t kScratchBytes = kOffCtl + align256(sizeof(FimCtl));

// The scratch itself: about 8.5 MB, zero at module load.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_base[kMaxDevices] = {};

// Order-preserving key of a finite double (smaller time -> smaller key).
// -0.0 is keyed as +0.0, as fim_set_stimuli takes it, so that a vertex given
// both gets the same seed on both paths.
__device__ __forceinline__ unsigned long long time_key(double t)
{
  unsigned long long b = (unsigned long long)__double_as_longlong(t);
  if ((b << 1) == 0ull) b = 0ull;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_time(unsigned long long k)
{
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

constexpr int kSeedThreads = 1024;

// Stimuli -> seed entries, in one block: every stimulated mesh vertex takes
// the earliest of its start times, and every vertex copy of it (one copy per
// submesh holding it; none for a vertex outside every tet) becomes one entry
// (the same rule as fim_set_stimuli).  A vertex given k times produces its
// entries k times over, all with the same copy and time, which the solve
// kernel's seeding writes idempotently.
__global__ void __launch_bounds__(kSeedThreads)
noalloc_seed_kernel(const int64_t *raw_v, const double *raw_t, int32_t n, unsigned long long *key,
                    const int64_t *gptr, const int32_t *gcopy, const int64_t *cptr, int32_t *seed_v,
                    double *seed_t)
{
  __shared__ int32_t scan[kSeedThreads];
  for (int32_t i = threadIdx.x; i < n; i += kSeedThreads) key[raw_v[i]] = ~0ull;
  __syncthreads();
  for (int32_t i = threadIdx.x; i < n; i += kSeedThreads) atomicMin(&key[raw_v[i]], time_key(raw_t[i]));
  __syncthreads();
  int32_t base = 0;
  for (int32_t chunk = 0; chunk < n; chunk += kSeedThreads) {
    const int32_t i = chunk + (int32_t)threadIdx.x;
    int64_t g = 0;
    int32_t c = 0;
    if (i < n) {
      g = raw_v[i];
      c = gptr ? (int32_t)(gptr[g + 1] - gptr[g]) : (cptr[g + 1] > cptr[g] ? 1 : 0);
    }
    // inclusive block scan of the entry counts (Hillis-Steele)
    scan[threadIdx.x] = c;
    __syncthreads();
    for (int off = 1; off < kSeedThreads; off <<= 1) {
      const int32_t add = threadIdx.x >= (unsigned)off ? scan[threadIdx.x - off] : 0;
      __syncthreads();
      scan[threadIdx.x] += add;
      __syncthreads();
    }
    const int32_t pos = base + scan[threadIdx.x] - c;
    if (c > 0) {
      const double t = key_time(key[g]);
      for (int32_t j = 0; j < c; ++j) {
        seed_v[pos + j] = gptr ? gcopy[gptr[g] + j] : (int32_t)g;
        seed_t[pos + j] = t;
      }
    }
    base += scan[kSeedThreads - 1];
    __syncthreads();
  }
}

}  // namespace

cudaError_t noalloc_scratch(int device, NoallocScratch *out)
{
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    base = g_base[device];
    if (!base) {
      // once per device, with that device current (the caller has set it):
      // loads this module there and yields the array's address
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return e;
      base = static_cast<unsigned char *>(p);
      g_base[device] = base;
    }
  }
  out->phi = reinterpret_cast<double *>(base + kOffPhi);
  out->phi2 = reinterpret_cast<double *>(base + kOffPhi2);
  out->sw = reinterpret_cast<uint32_t *>(base + kOffSw);
  out->list[0] = reinterpret_cast<int32_t *>(base + kOffList0);
  out->list[1] = reinterpret_cast<int32_t *>(base + kOffList1);
  out->list[2] = reinterpret_cast<int32_t *>(base + kOffList2);
  out->lfrozen = reinterpret_cast<int32_t *>(base + kOffFrozen);
  out->lmarked = reinterpret_cast<int32_t *>(base + kOffMarked);
  out->phi_f = reinterpret_cast<float *>(base + kOffPhiF);
  out->phi2_f = reinterpret_cast<float *>(base + kOffPhi2F);
  out->st = base + kOffSt;
  out->tst = base + kOffTst;
  out->dec = base + kOffDec;
  out->st_out = base + kOffStOut;
  out->key = reinterpret_cast<unsigned long long *>(base + kOffKey);
  out->raw_v = reinterpret_cast<int64_t *>(base + kOffRawV);
  out->raw_t = reinterpret_cast<double *>(base + kOffRawT);
  out->seed_v = reinterpret_cast<int32_t *>(base + kOffSeedV);
  out->seed_t = reinterpret_cast<double *>(base + kOffSeedT);
  out->ctl = reinterpret_cast<FimCtl *>(base + kOffCtl);
  return cudaSuccess;
}

cudaError_t launch_noalloc_seeds(const NoallocScratch &sc, int32_t n, const int64_t *gptr,
                                 const int32_t *gcopy, const int64_t *cptr, cudaStream_t stream)
{
  if (n <= 0) return cudaSuccess;
  noalloc_seed_kernel<<<1, kSeedThreads, 0, stream>>>(sc.raw_v, sc.raw_t, n, sc.key, gptr, gcopy, cptr,
                                                      sc.seed_v, sc.seed_t);
  return cudaGetLastError();
}

}  // namespace fimgb
