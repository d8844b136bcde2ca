// fim_internal.h -- shared declarations of the GB300 FIM solver (host side
// and kernels).  Not part of the C ABI.
#pragma once

#include <cstdint>
#include <cstddef>

#include <cuda_runtime.h>

namespace fimgb {

// Reference node states (types.h:85).
enum : uint8_t { ST_FAR = 0, ST_NEIG = 1, ST_NARROW = 2, ST_NEXT = 3, ST_FROZEN = 4, ST_TAIL = 5 };

// Doubles per corner of the FP64 record.
constexpr int kCgeoStride = 6;
// Floats per corner of the FP32 screen record (e13, e23, e34, e12, e14, e24
// times 2^-k, k, unused).
constexpr int kCgfStride = 8;
// The 32-byte record that every corner update reads first, as two uint4:
//   [0] ids of the other three vertices ("1","2","3"), root-term bounds of
//       the pairs (1,2) and (2,3) as two fp16 rounded down;
//   [1] float edge lengths towards the corner's vertex from "1","2","3",
//       root-term bounds of the pair (1,3) and of the tet as two fp16.
// The ids come from the mesh staging, the rest from the metric kernel.
constexpr int kCrecWords = 2;

// Threads per block of the persistent solve kernel (one block per SM).
#ifndef FIM_SOLVE_THREADS
#define FIM_SOLVE_THREADS 512
#endif
constexpr int kSolveThreads = FIM_SOLVE_THREADS;

// Kernel error codes written into FimCtl::error.
enum : int { KERR_NONE = 0, KERR_TIMEOUT = 1, KERR_MAX_ITER = 2 };

// Device control block: counters of the three rotating list slots, the grid
// barrier, the error word and statistics.  Lives in device memory; the host
// clears it before every launch.
struct FimCtl {
  int32_t n_narrow[3];      // narrow list length of the iteration using this slot
  int32_t n_frozen[3];      // vertices frozen in that iteration
  int32_t n_marked[3];      // neighbours re-solved in that iteration
  uint32_t bar_count;       // grid barrier arrival word (its top bit flips at every barrier)
  uint32_t bar_pad;
  int32_t error;            // KERR_*
  int32_t error_where;      // phase that failed
  int64_t iterations;
  int64_t vertex_updates;
  int64_t corner_evals;
  int64_t exact_evals;
  int32_t n_bad;                 // support check: reached times below every candidate bound
  int32_t pad2;
  unsigned long long tmin_key;   // dkey of the smallest such time
  unsigned long long win_iter_max;  // submesh sweeps: most iterations of a block in this window
  unsigned long long iters_total;   // submesh sweeps: iterations of all windows
};

// Everything the persistent kernel touches, as device pointers.
//
// Vertices of the kernel are vertex *copies*: with submesh tags every
// submesh holds its own copy of each of its vertices (the reference's
// per-submesh local numbering, extract_submeshes2, types.cpp:306-570), and a
// tet's corners only see the copies of its own submesh.  Without tags there
// is one submesh and copy == vertex.
struct FimDev {
  int32_t nV;                 // vertex copies
  int32_t nG;                 // mesh vertices
  const int64_t *gptr;        // [nG+1] copies of each mesh vertex (nullptr: copy == vertex)
  const int32_t *gcopy;
  double *phi_out;            // [nG] gathered results (min over copies)
  uint8_t *st_out;            // [nG] (max over copies)
  int64_t nT;
  int64_t nC;                 // corners = 4 * nT
  // topology
  const int64_t *cptr;        // [nV+1] corner range per vertex
  const uint4 *crec;          // [kCrecWords*nC] first-read record of each corner (kCrecWords)
  const double *cgeo;         // [nC*kCgeoStride] FP64 e13, e23, e34, e12, e14, e24
  const float *cgf;           // [nC*kCgfStride] float screen record: e13..e24 * 2^-k, k, unused
  float *phi_f;               // float copy (round to nearest) of phi, kept in step with it
  float *phi2_f;              // float copy of phi2
  const int64_t *nptr;        // [nV+1] vertex neighbourhood (self included)
  const int32_t *nbr;
  // state
  double *phi;                // current times
  double *phi2;               // next times (equal to phi outside the updated lists)
  uint32_t *sw;               // state word: state (low 8 bits) | iteration stamp of "marked" << 8
  uint8_t *st;                // states as bytes, written at the end of a solve (the result)
  uint8_t *tst;               // reference tmp_state
  int32_t *list[3];           // rotating narrow lists
  int32_t *lfrozen;           // frozen this iteration
  int32_t *lmarked;           // marked this iteration
  uint8_t *dec;               // decided state of marked vertices
  // stimuli
  const int32_t *seed_v;
  const double *seed_t;
  int32_t nseed;
  const double *phi_init;     // warm start per vertex (nullptr: cold start)
  FimCtl *ctl;
  unsigned long long *probe;  // per-block phase times (builds with FIM_PROBE only), else nullptr
  const int32_t *blk_ptr;     // [grid+1] submesh sweeps: the vertex copies each block owns (whole submeshes)
};

// Iteration stamps live in the upper 24 bits of the state word.
constexpr int64_t kMaxStampIterations = (int64_t(1) << 24) - 1;
constexpr int kProbeSlots = 28;  // phase-time accumulators per block (FIM_PROBE builds)

struct FimParams {
  double dt;            // window length (inf = endless)
  int32_t n_steps;
  double front_width;   // reference wavefront width
  double apd;           // < 0 disables the frozen->tail->far reset
  int64_t max_iter;     // per window
  uint64_t timeout_ns;  // per wait
  int32_t withhold_block;  // test hook: block k-1 skips its first barrier arrival (0 = off)
  int32_t exact_all;       // 1: every local solve in FP64, no interval filter
  int32_t two_phase;       // 1: two grid-synchronised phases per iteration (endless window only)
  int32_t dag_warps;       // warps running the FP64 tet prefix groups of a batch (1..kDagWarpsMax)
  int32_t resume;          // 1: keep the times and states as they are (no reset, no seeding)
  int32_t fp32;            // 1: FP32 local solves where their screens are conclusive (not bit-exact)
  int32_t local;           // 1: submesh sweeps (blocks own whole submeshes within a window; four phases)
};

// Most warps of a batch that run FP64 tet prefix groups (the scratch is
// sized for it).
constexpr int kDagWarpsMax = 12;

// Records the message returned by fim_last_error(NULL) on this thread.
void set_last_error(const char *msg);

// ---- kernels (fim_kernels.cu) ----
// FP64 metric + edge norms of tets [e0, e1) scattered into the corner
// records; the first tet with a non-positive or non-finite speed or a
// non-finite fibre lowers *bad to its index.
// evec: the mesh's edge vectors (launch_edge_vectors), or null to form them
// from xyz.
cudaError_t launch_metric(const int32_t *tslots, const int64_t *cidx, const double *xyz, const double *evec,
                          int64_t nT, const double *fib, const double *cf, const double *ct, int64_t e0, int64_t e1,
                          double *cgeo, float *cgf, uint4 *crec, unsigned long long *bad, cudaStream_t stream);
// Stages the six edge vectors of every tet (18 doubles, SoA) for the
// metric kernel.
cudaError_t launch_edge_vectors(const int32_t *tslots, const double *xyz, int64_t nT, double *evec,
                                cudaStream_t stream);
// The persistent cooperative solve is compiled once per batch shape
// (fim_solve_s*.cu: vertices x corners a block stages per batch); the
// autotuner picks the shape, the grid and the tet-prefix warps per problem.
constexpr int kNumShapes = 3;
struct ShapeDesc {
  const char *name;
  int slots;    // vertices per batch
  int corners;  // corners per batch
};
extern const ShapeDesc kShapes[kNumShapes];
// Sets the shape's shared-memory size and returns its largest co-resident grid.
cudaError_t solve_prepare(int shape, int device, int block, int *max_grid);
// Persistent cooperative solve with batch shape `shape`.
cudaError_t launch_solve(const FimDev &d, const FimParams &p, int shape, int grid, int block, cudaStream_t stream);
// Writes phi (any order) into out.
cudaError_t launch_copy(const double *src, double *dst, int64_t n, cudaStream_t stream);
// Support check of a finished solve (fim_kernels.cu): every reached vertex
// that is not a seed (is_seed[v] == 0) and whose time lies below a rigorous
// lower bound of every candidate of its neighbours counts into ctl->n_bad
// and lowers ctl->tmin_key to its time.
cudaError_t launch_support_check(const FimDev &d, double lower, const uint8_t *is_seed, cudaStream_t stream);
// Marks the seeds of d in is_seed (after the caller cleared it).
cudaError_t launch_mark_seeds(const FimDev &d, uint8_t *is_seed, cudaStream_t stream);
// Resets every vertex with a time >= tmin to INF / far, lists every other
// reached vertex as narrow, then re-seeds the stimuli (two launches).
cudaError_t launch_warm_reset(const FimDev &d, double tmin, cudaStream_t stream);

// ---- learned warm start (fim_mlp.cu) ----
// Network 7 (padded to kMlpIn) -> kMlpH -> kMlpH -> kMlpH -> 1.  Parameter
// vector: the three GEMM weight matrices first ([in][out], row-major; their
// BF16 copies cover exactly this prefix), then b1, b2, b3, w4, b4.
constexpr int kMlpIn = 64, kMlpH = 128, kMlpFeatures = 7;
constexpr int kMlpOW1 = 0, kMlpOW2 = kMlpIn * kMlpH, kMlpOW3 = kMlpOW2 + kMlpH * kMlpH;
constexpr int kMlpW16 = kMlpOW3 + kMlpH * kMlpH;
constexpr int kMlpOB1 = kMlpW16, kMlpOB2 = kMlpOB1 + kMlpH, kMlpOB3 = kMlpOB2 + kMlpH;
constexpr int kMlpOW4 = kMlpOB3 + kMlpH, kMlpOB4 = kMlpOW4 + kMlpH;
constexpr int kMlpParams = kMlpOB4 + 1;

// Feature rows of the learned warm start (fim_mlp.cu); red receives the
// bounding box and the largest stimulus distance (features_scale reads it).
cudaError_t launch_features(int nV, int64_t nT, const double *xyz, const int32_t *tslots, const double *fib,
                            const double *cf, const double *ct, int nseed, const int32_t *seed_v,
                            const double *seed_t, float *acc, float *dist, unsigned int *red, void *X,
                            cudaStream_t st);
float features_scale(const unsigned int *host_red);

// ---- fixed scratch of fim_solve_noalloc (fim_static.cu) ----
constexpr int64_t kStaticMaxCopies = 131072;       // vertex copies of the mesh
constexpr int64_t kStaticMaxVertices = 131072;     // mesh vertices
constexpr int64_t kStaticMaxSeeds = 8192;          // stimulus entries as given
constexpr int64_t kStaticMaxSeedEntries = 32768;   // stimulus entries expanded to vertex copies

// Pointers into the fixed scratch of one device.
struct NoallocScratch {
  double *phi, *phi2;
  uint32_t *sw;
  int32_t *list[3], *lfrozen, *lmarked;
  float *phi_f, *phi2_f;
  uint8_t *st, *tst, *dec, *st_out;
  unsigned long long *key;   // per mesh vertex: earliest stimulus time (order-preserving key)
  int64_t *raw_v;            // stimuli as given
  double *raw_t;
  int32_t *seed_v;           // stimuli expanded to vertex copies
  double *seed_t;
  FimCtl *ctl;
};
// Resolves the scratch address on `device` (must be the current device); the
// first call per device does the lookup, later calls reuse it.
cudaError_t noalloc_scratch(int device, NoallocScratch *out);
// Expands sc.raw_v/raw_t[n] into sc.seed_v/seed_t (one block).
cudaError_t launch_noalloc_seeds(const NoallocScratch &sc, int32_t n, const int64_t *gptr,
                                 const int32_t *gcopy, const int64_t *cptr, cudaStream_t stream);

}  // namespace fimgb
