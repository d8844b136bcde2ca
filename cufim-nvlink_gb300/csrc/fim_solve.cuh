// fim_solve.cuh -- the persistent FIM solve kernel, compiled once per batch
// shape.  A translation unit defines FIM_SLOTS (vertices per batch),
// FIM_CORNER_CAP (corners per batch) and FIM_SHAPE_NS (a namespace of its
// own, since the batch layout differs per shape) and includes this file;
// fim_solve_s*.cu are those units, and the autotuner (fim_solver.cpp)
// chooses among them per problem.
#pragma once

#include "fim_device.cuh"

#if !defined(FIM_SLOTS) || !defined(FIM_CORNER_CAP) || !defined(FIM_SHAPE_NS)
#error "define FIM_SLOTS, FIM_CORNER_CAP and FIM_SHAPE_NS before including fim_solve.cuh"
#endif

namespace fimgb {
namespace FIM_SHAPE_NS {

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


// One block of 16 warps per SM: the FP64 solves of a batch are packed into
// as few warps as possible, and those warps sit on different SM
// sub-partitions (an FP64 warp instruction occupies its sub-partition's
// FP64 pipe for 64 cycles whatever its active lanes, so two blocks per SM
// would stack their FP64 warps on the same sub-partitions).
constexpr int kThreads = kSolveThreads;  // threads per block of the solve kernel
#ifndef FIM_MARK_LANES
#define FIM_MARK_LANES 16
#endif
constexpr int kMarkLanes = FIM_MARK_LANES;  // threads per frozen vertex in the neighbour marking
static_assert(kThreads % kMarkLanes == 0, "marking groups must tile the grid");
// the two-phase path's marking (phase X): groups of kMarkLanesX threads,
// two neighbours per thread and round
constexpr int kMarkLanesX = 8;
static_assert(kThreads % kMarkLanesX == 0, "marking groups must tile the block");
constexpr int kSlots = FIM_SLOTS;             // vertices per batch (at most)
constexpr int kCornerCap = FIM_CORNER_CAP;    // corners per batch
constexpr int kTriCap = kCornerCap * 6 / 5;  // triangle screens per batch (more are screened on the spot)
constexpr int kTetCap = kCornerCap; // tet screens per batch: never full
constexpr int kQcap = 768;          // exact solves queued per kind and batch (more run on the spot)
// Phase D runs the queued tets on at most FimParams::dag_warps (<=
// kDagWarpsMax) warps, one group of kDagLanes lanes per tet (scratch:
// kDagGroups * kDagSlots doubles).
constexpr int kDagWarps = kDagWarpsMax * 32 <= kThreads ? kDagWarpsMax : kThreads / 32;
constexpr int kDagGroups = kDagWarps * 32 / kDagLanes;

// Update phases.  With windows (finite dt) an iteration runs the reference's
// four steps as four grid-synchronised phases: kNarrow4 (update the narrow
// list), the apply + neighbour marking, kMarked4 (re-solve the marked
// neighbours), the apply + next list.  With one endless window no vertex
// can leave the narrow list for "next" inside the window, so an iteration
// needs only two: kNarrow2 updates the narrow list and marks the downwind
// neighbours of the vertices it freezes, kMarked2 re-solves them, applies
// everything and builds the next list.
// With windows the re-solve applies its own results too (kMarked3: the
// times into both buffers, the decided state, the next list), so that
// iteration needs three phases: a re-solved vertex is seen as "neig" by every
// other re-solve of the phase, so nothing reads what it writes.
enum : int { kNarrow4 = 0, kMarked4 = 1, kNarrow2 = 2, kMarked2 = 3, kMarked3 = 4 };
__host__ __device__ constexpr bool is_marked_mode(int m) { return m == kMarked4 || m == kMarked2 || m == kMarked3; }

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
  uint8_t tsv[kSlots];              // kMarked2, kMarked3: tmp_state of each vertex
  int32_t fz[kSlots];               // kNarrow2: slots frozen in this batch
  // per corner of the batch
  union {
    struct {
      float pf[kCornerCap][3];      // their float times
      float lbv[kCornerCap][4];     // lower bounds of the triangle pairs (1,2), (2,3), (1,3) and the tet (+inf: not valid)
      float elo[kCornerCap];        // smallest lower bound of the corner's valid edges (+inf: none)
    };
    double dag[kDagGroups][kDagSlots];  // phase D (where pf and sf are dead): scratch of the tet prefix groups
  };
  uint8_t vm[kCornerCap];           // validity bits of the three neighbours
  uint8_t cs[kCornerCap];           // slot of the corner's vertex
  // compacted screen lists: items corner j | pair k << 14 (triangles), corner j (tets)
  uint16_t tri[kTriCap];
  uint16_t tet[kTetCap];
  uint16_t edg[kCornerCap];         // corners whose best edge can still be the minimum (phase B): never full
  uint32_t q[3][kQcap];             // queued exact solves: [0] tets, [1] triangles, [2] edges
  float qlb[3][kQcap];              // their lower bounds (rechecked against the final bhi)
  int ntri, ntet, nedge, nq[3];
  int next_item;                    // next unclaimed screen item (phase S)
  int wsum[kSlots / 32];            // corner counts of each warp's 32 slots (setup)
  int nfit;                         // slots whose corners end within kCornerCap (setup)
  int nfz;                          // kNarrow2: frozen slots of the batch
};

// (for small shapes the tet prefix scratch is the larger member of the union)

// Queue item: slot (8 bits) | kind (2 bits) | corner index in the batch (22 bits).
// kind: triangle pair 0..2 or 3 (tet) in queues 0 and 1, edge 0..2 in queue 2.
static_assert(kSlots <= 256 && kCornerCap <= (1 << 14), "queue item and screen list fields");
// the slot prefix scan and the warp-aggregated appends of phase E run on
// whole warps over the slots
static_assert(kSlots % 32 == 0 && kSlots <= kThreads, "slots must fill whole warps of the block");
static_assert(kCornerCap % 32 == 0, "corner capacity in whole warps");
static_assert(kDagWarps >= 1 && 32 * kDagWarps <= kThreads, "tet prefix warps within the block");
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

// Appends v to a global list from inside a divergent branch: one atomic per
// group of lanes that reach it together (instead of one per lane on the
// list's single counter).
__device__ __forceinline__ void append_active(int32_t *list, int32_t *counter, int32_t v)
{
  const unsigned act = __activemask();
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(act) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(act));
  base = __shfl_sync(act, base, leader);
  list[base + __popc(act & ((1u << lane) - 1u))] = v;
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
// 2^-k and k (an array of its own, read only by the corners phase B lists;
// an L1 prefetch of it issued in phase B measured slower).
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

__device__ __forceinline__ CandBound tet_screen_sm(const FimDev &d, const BatchSh &sh, int j, int *why = nullptr)
{
  float g[7];
  screen_record(d, sh, j, g);
  return tet_screen_bf(g, sh.pf[j][0], sh.pf[j][1], sh.pf[j][2], (int)g[6], why);
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
  int32_t *frozen;    // kNarrow4: vertices frozen now
  int32_t *n_frozen;
  int32_t *marked;    // kNarrow2: neighbours marked now
  int32_t *n_marked;
  uint8_t *dec;       // kMarked4: decided state per position of the marked list
  bool local;         // the list is this block's own (submesh sweeps): no split over the grid
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
                             float lower_lo, float lower_hi, double phi_start, double dt, bool exact_all, bool fp32,
                             uint32_t stamp, int dag_warps, const ListOut &lo_, int64_t &n_filtered,
                             int64_t &n_exact)
{
  constexpr bool kMarkedMode = is_marked_mode(MODE);
  const double *ph = MODE == kMarked2 ? d.phi2 : d.phi;      // times this phase reads
  const float *phf = MODE == kMarked2 ? d.phi2_f : d.phi_f;
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t per_block = lo_.local ? (int64_t)n : ((int64_t)n + gridDim.x - 1) / gridDim.x;
  const int64_t lbeg = lo_.local ? 0 : min((int64_t)n, (int64_t)blockIdx.x * per_block);
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
      if (MODE == kMarked2 || MODE == kMarked3) sh.tsv[tid] = __ldcg(d.tst + v);
    }
    if (tid == 0) {
      sh.cp[0] = 0;
      sh.nfit = 0;
      sh.ntri = 0; sh.ntet = 0; sh.nedge = 0; sh.nq[0] = 0; sh.nq[1] = 0; sh.nq[2] = 0; sh.next_item = 0; sh.nfz = 0;
    }
    __syncthreads();
    // corner prefix over the slots: each warp scans its 32 slots, the warp
    // totals are added after one barrier; then every slot marks its corners
    // with its index (phase A reads the slot of a corner instead of
    // searching the prefix) and the slots whose corners end within
    // kCornerCap are counted (the batch: that run, at least one slot)
    int cnt_own = 0, incl = 0;
    if (tid < kSlots) {  // whole warps
      cnt_own = tid < cand ? sh.cnt[tid] : 0;
      incl = cnt_own;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += u;
      }
      if (lane == 31) sh.wsum[tid >> 5] = incl;
    }
    __syncthreads();
    if (tid < kSlots) {
      for (int w = 0; w < (tid >> 5); ++w) incl += sh.wsum[w];
      sh.cp[tid + 1] = incl;
      const int fit = __popc(__ballot_sync(FULL_MASK, tid < cand && incl <= kCornerCap));
      if (lane == 0 && fit) atomicAdd(&sh.nfit, fit);
      const int j1 = min(incl, kCornerCap);
      for (int j = incl - cnt_own; j < j1; ++j) sh.cs[j] = (uint8_t)tid;
    }
    __syncthreads();
    const int nslot = max(1, sh.nfit);
    const int total = sh.cp[nslot];     // may exceed kCornerCap for a single huge vertex
    const int kept = min(total, kCornerCap);
    __syncthreads();
    PROBE(kPrSetup);

    // A: load, validity, float edge bounds.  Every thread walks its corners
    // j = tid, tid + kThreads, ...: the first-read record (ids, float
    // lengths, fp16 bounds) of the next corner is loaded while the
    // neighbours' states and float times of the current one are (they need
    // its ids), so that a thread's corners are not a chain of round trips.
    {
      uint4 n0 = make_uint4(0u, 0u, 0u, 0u), n1 = n0;
      if (tid < kept) {
        const int sl = sh.cs[tid];
        const int64_t c = sh.c0[sl] + (tid - sh.cp[sl]);
        n0 = __ldg(d.crec + kCrecWords * c);
        n1 = __ldg(d.crec + kCrecWords * c + 1);
      }
      for (int j = tid; j < kept; j += kThreads) {
        const uint4 h0 = n0, h1 = n1;
        const int slot = sh.cs[j];
        const int jn = j + kThreads;
        if (jn < kept) {  // prefetch the next corner's record
          const int sl = sh.cs[jn];
          const int64_t c = sh.c0[sl] + (jn - sh.cp[sl]);
          n0 = __ldg(d.crec + kCrecWords * c);
          n1 = __ldg(d.crec + kCrecWords * c + 1);
        }
        float pf[3];
        uint8_t stn[3];
        const int32_t nbs[3] = {(int32_t)h0.x, (int32_t)h0.y, (int32_t)h0.z};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          pf[i] = __ldcg(phf + nbs[i]);
          stn[i] = (uint8_t)sw_seen(__ldcg(d.sw + nbs[i]), kMarkedMode, stamp);
        }
        const float len[3] = {__uint_as_float(h1.x), __uint_as_float(h1.y), __uint_as_float(h1.z)};
        uint32_t m = 0;
        float ub = INFINITY, elo = INFINITY, lo[3], hi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const Re P = re_in(pf[i]);
          lo[i] = re_lo(P);
          hi[i] = re_hi(P);
          bool ok = stn[i] >= ST_NARROW;
          if (ok) {
            if (lo[i] > lower_hi) ok = true;
            else if (hi[i] <= lower_lo) ok = false;
            else ok = __ldcg(ph + nbs[i]) > lower;  // rare: the FP64 time decides
          }
          if (ok) {
            m |= 1u << i;
            const Re E = P + re_len(len[i]);
            ub = fminf(ub, re_hi(E));
            elo = fminf(elo, re_lo(E));
          }
          sh.pf[j][i] = pf[i];
        }
        // lower bounds of the triangle pairs and the tet: min(times) +
        // root-term bound (fp16, rounded down), for phase B's screen lists
        const float hv[4] = {half_lo(h0.w), half_hi(h0.w), half_lo(h1.w), half_hi(h1.w)};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int a = k == 1 ? 1 : 0, b = k == 0 ? 1 : 2;
          sh.lbv[j][k] = ((m >> a) & (m >> b) & 1u) ? solve_lo(fminf(lo[a], lo[b]), fmaxf(hi[a], hi[b]), hv[k])
                                                     : INFINITY;
        }
        sh.lbv[j][3] = m == 7u ? solve_lo(fminf(lo[0], fminf(lo[1], lo[2])), fmaxf(hi[0], fmaxf(hi[1], hi[2])), hv[3])
                               : INFINITY;
        sh.elo[j] = elo;
        if (m) ++n_filtered;
        if (!exact_all && ub < INFINITY) atomicMin(&sh.bhi[slot], fkey(ub));
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
      float bhi = 0.f, lb[4] = {0.f, 0.f, 0.f, 0.f}, elo = 0.f;
      if (in) {
        slot = sh.cs[j];
        m = sh.vm[j];
        bhi = funkey(sh.bhi[slot]);
        lb[0] = sh.lbv[j][0]; lb[1] = sh.lbv[j][1]; lb[2] = sh.lbv[j][2]; lb[3] = sh.lbv[j][3];
        elo = sh.elo[j];
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
            sh.tri[p] = (uint16_t)(j | (k << 14));
          } else {  // list full: screen here
            tri_list_full(d, ph, sh, j, k, slot, bhi, exact_all);
          }
        }
      }
      {
        const bool need = in && m == 7u && !(lb[3] > bhi);
        const int p = warp_append(&sh.ntet, need, lane);
        if (p >= 0) sh.tet[p] = (uint16_t)j;  // kTetCap == kCornerCap: never full
      }
      {
        // the corners with an edge that can still be the minimum: the
        // smallest edge lower bound (phase A) against bhi; the FP32 mode
        // lists every corner with a valid edge
        bool need = false;
        if (in) need = fp32 ? m != 0u : !(elo > bhi);
        const int p = warp_append(&sh.nedge, need, lane);
        if (p >= 0) sh.edg[p] = (uint16_t)j;  // one entry per corner at most: never full
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
      const int nedge = sh.nedge;
      const int nclaim = edge_c0 + ((nedge + 31) & ~31);
      for (;;) {
        // claims of 32: tet chunks, then triangle chunks of 64 (two per
        // lane), then edge chunks of 32 corners
        int cl = 0;
        if (lane == 0) cl = atomicAdd(&sh.next_item, 32);
        cl = __shfl_sync(FULL_MASK, cl, 0);
        if (cl >= nclaim) break;
#ifdef FIM_PROBE
        const unsigned long long pt0 = global_timer();
#define PROBE_CHUNK(k) do { if (lane == 0) atomicAdd(&d.probe[blockIdx.x * kProbeSlots + (k)], global_timer() - pt0); } while (0)
#else
#define PROBE_CHUNK(k) ((void)0)
#endif
        if (cl >= edge_c0) {
          // the edges that can still be the minimum, over the corners phase
          // B listed (their float lengths from the first-read record again)
          const int e = cl - edge_c0 + lane;
          const bool in = e < nedge;
          const int j = in ? (int)sh.edg[e] : 0;
          int slot = 0;
          uint32_t m = 0;
          float bhi = 0.f;
          uint4 r1 = make_uint4(0u, 0u, 0u, 0u);
          if (in) {
            slot = sh.cs[j]; m = sh.vm[j]; bhi = funkey(sh.bhi[slot]);
            r1 = __ldg(d.crec + kCrecWords * (sh.c0[slot] + (j - sh.cp[slot])) + 1);
          }
          const float len[3] = {__uint_as_float(r1.x), __uint_as_float(r1.y), __uint_as_float(r1.z)};
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const float le = in ? re_lo(re_in(sh.pf[j][i]) + re_len(len[i])) : 0.f;
            bool need = in && ((m >> i) & 1u) && !(le > bhi);
            if (fp32 && need) {  // FP32 mode: the float edge sum is the value
              atomicMin(&sh.res[slot], dkey((double)(sh.pf[j][i] + len[i])));
              need = false;
            }
            queue_exact(d, ph, sh, need, 2, i, slot, j, le, lane);
          }
          PROBE_CHUNK(13);
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
#ifdef FIM_PROBE
            else {
              int why = 3;
              cb = tet_screen_sm(d, sh, j, &why);
              // outcomes: sqt < 0, sqt undecided, no accepted root, a value (pruned / queued below)
              atomicAdd(&d.probe[blockIdx.x * kProbeSlots + 16 + (why < 3 ? why : 3)], 1ull);
              if (why == 3 && cb.lb > funkey(sh.bhi[slot])) atomicAdd(&d.probe[blockIdx.x * kProbeSlots + 20], 1ull);
            }
#else
            else cb = tet_screen_sm(d, sh, j);
#endif
            if (!exact_all && cb.some && cb.ub < INFINITY) atomicMin(&sh.bhi[slot], fkey(cb.ub));
            lb = isnan(cb.lb) ? -INFINITY : cb.lb;
            need = cb.some && !(lb > funkey(sh.bhi[slot]));
            if (fp32 && need && cb.ub < INFINITY && !isnan(cb.lb)) {  // FP32 mode: conclusive screen
              atomicMin(&sh.res[slot], dkey((double)(0.5f * (cb.lb + cb.ub))));
              need = false;
            }
          }
          queue_exact(d, ph, sh, need, 0, 3, slot, j, lb, lane);
          PROBE_CHUNK(11);
        } else {
          int jj[2], kk[2], sl[2];
          bool in[2];
          CandBound cb[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int i = ib + 32 * h + lane;
            in[h] = i < tri0 + ntri;
            const uint32_t it = in[h] ? (uint32_t)sh.tri[i - tri0] : 0u;
            jj[h] = (int)(it & 0x3fffu);
            kk[h] = (int)(it >> 14);
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
#ifdef FIM_PROBE
              // triangle outcomes: no value, a value above bhi, a value below
              atomicAdd(&d.probe[blockIdx.x * kProbeSlots + (!cb[h].some ? 21 : (need ? 23 : 22))], 1ull);
#endif
              if (fp32 && need && cb[h].ub < INFINITY && !isnan(cb[h].lb)) {  // FP32 mode: conclusive screen
                atomicMin(&sh.res[sl[h]], dkey((double)(0.5f * (cb[h].lb + cb[h].ub))));
                need = false;
              }
            }
            queue_exact(d, ph, sh, need, 1, kk[h], sl[h], jj[h], lb, lane);
          }
          PROBE_CHUNK(12);
        }
#undef PROBE_CHUNK
      }
    }
    __syncthreads();
    PROBE(kPrS);
#ifdef FIM_PROBE
    __shared__ unsigned long long s_d_start, s_d_tri_end;
    if (tid == 0) { s_d_start = global_timer(); s_d_tri_end = 0; }
    __syncthreads();
#endif

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
      const int tet_warps = min(dag_warps, (ntet * kDagLanes + 31) / 32);
      const int tri0 = 32 * tet_warps;
#ifdef FIM_PROBE
      if (tid == 0) {  // queued FP64 solves of the batch: tets (and batches with > 48), triangles
        d.probe[blockIdx.x * kProbeSlots + 14] += (unsigned long long)ntet + ((unsigned long long)(ntet > 48) << 32);
        d.probe[blockIdx.x * kProbeSlots + 15] += (unsigned long long)ntri + ((unsigned long long)nedge << 32);
      }
#endif
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
#ifdef FIM_PROBE
        if (tid == 0) {  // the tet part of D, in batches that have one
          d.probe[blockIdx.x * kProbeSlots + 24] += global_timer() - s_d_start;
          d.probe[blockIdx.x * kProbeSlots + 26] += 1;
        }
#endif
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
#ifdef FIM_PROBE
        atomicMax(&s_d_tri_end, global_timer());
#endif
      }
    }
    __syncthreads();
#ifdef FIM_PROBE
    if (tid == 0 && s_d_tri_end > s_d_start) {  // the triangle/edge part of D
      d.probe[blockIdx.x * kProbeSlots + 25] += s_d_tri_end - s_d_start;
      d.probe[blockIdx.x * kProbeSlots + 27] += 1;
    }
#endif
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
            append_active(lo_.frozen, lo_.n_frozen, v);
          }
        } else {
          lo_.dec[pos + slot] = (nw < old) ? (uint8_t)ST_NARROW : __ldcg(d.tst + v);
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
      // kMarkLanesX threads per frozen vertex, two neighbours per thread and
      // round with their loads issued together
      const int nfz = sh.nfz;
      for (int g = tid / kMarkLanesX; g < nfz; g += kThreads / kMarkLanesX) {
        const int slot = sh.fz[g];
        const double pn = dunkey(sh.res[slot]);
        const int64_t k0 = sh.n0[slot], k1 = k0 + sh.ncnt[slot];
        for (int64_t k = k0 + tid % kMarkLanesX; k < k1; k += 2 * kMarkLanesX) {
          const int64_t kk[2] = {k, k + kMarkLanesX};
          int32_t v[2];
          uint32_t w[2];
          double pv[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) v[h] = kk[h] < k1 ? __ldg(d.nbr + kk[h]) : -1;
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            w[h] = v[h] >= 0 ? __ldcg(d.sw + v[h]) : 0u;
            pv[h] = v[h] >= 0 ? __ldcg(d.phi2 + v[h]) : 0.0;
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if (v[h] >= 0 && sw_state(w[h]) != ST_NARROW && sw_stamp(w[h]) != stamp && pn < pv[h]) {
              if (atomicCAS(d.sw + v[h], w[h], sw_make(sw_state(w[h]), stamp)) == w[h]) {
                d.tst[v[h]] = (uint8_t)sw_state(w[h]);
                append_active(lo_.marked, lo_.n_marked, v[h]);
              }
            }
          }
        }
      }
    } else {  // kMarked2, kMarked3
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

// One window of submesh sweeps: the block owns the vertex copies [c0, c1)
// -- whole submeshes -- and runs the reference's compute_step
// (cuda_fim.cu:1992-2334) on them until they converge, with block barriers
// only: within a window the submeshes do not exchange times (sync_step2
// runs only between windows), so each block iterates at its own pace.  The
// four phases per iteration are those of the grid path (P1 update narrow,
// P2 apply + mark, P3 re-solve, P4 apply + next list) on the block's own
// lists (its segment of each list array) with counters in shared memory.
// Returns false after recording an error.
__device__ bool local_window(const FimDev &d, BatchSh &sh, const FimParams &p, double lower, float lower_lo,
                             float lower_hi, double phi_start, double cur_time, int64_t &it, int dag,
                             int64_t &my_evals, int64_t &my_exact, int64_t &my_updates, int where)
{
  __shared__ int32_t b_narrow[3], b_frozen, b_marked;
  const int tid = threadIdx.x;
  const int32_t c0 = d.blk_ptr[blockIdx.x], c1 = d.blk_ptr[blockIdx.x + 1];
  int s = (int)(it % 3);
  if (tid == 0) { b_narrow[0] = 0; b_narrow[1] = 0; b_narrow[2] = 0; b_frozen = 0; b_marked = 0; }
  __syncthreads();
  // update_states (cuda_fim.cu:1790-1845) on the block's copies
  for (int32_t v = c0 + tid; v < c1; v += kThreads) {
    uint8_t stv = (uint8_t)sw_state(d.sw[v]);
    if (stv == ST_NEXT) { stv = ST_NARROW; d.sw[v] = stv; }
    else if (p.apd >= 0.0 && stv == ST_FROZEN) {
      if (!(d.phi[v] + p.apd > cur_time)) d.sw[v] = ST_TAIL;
    } else if (p.apd >= 0.0 && stv == ST_TAIL) {
      if (!(d.phi[v] + p.apd / 0.91 > cur_time)) {
        set_phi_both(d, v, FIM_INF); d.sw[v] = ST_FAR;
      }
    }
    if (stv == ST_NARROW) d.list[s][c0 + atomicAdd(&b_narrow[s], 1)] = v;
  }
  __syncthreads();
  int64_t it_window = 0;
  for (;;) {
    s = (int)(it % 3);
    const int s1 = (int)((it + 1) % 3), s2 = (int)((it + 2) % 3);
    const int32_t nn = b_narrow[s];
    if (nn == 0) break;
    if ((p.max_iter > 0 && it_window >= p.max_iter) || it >= kMaxStampIterations) {
      if (tid == 0 && atomicCAS(&d.ctl->error, KERR_NONE, KERR_MAX_ITER) == KERR_NONE) d.ctl->error_where = where;
      return false;
    }
    const uint32_t stamp = (uint32_t)(it + 1);
    const int32_t *lst = d.list[s] + c0;
    int32_t *lnext = d.list[s1] + c0;
    __syncthreads();  // every thread has read the counters of the last iteration
    if (tid == 0) { b_narrow[s2] = 0; b_frozen = 0; b_marked = 0; }
    __syncthreads();
    ListOut lo;
    lo.next = lnext; lo.n_next = &b_narrow[s1];
    lo.frozen = d.lfrozen + c0; lo.n_frozen = &b_frozen;
    lo.marked = d.lmarked + c0; lo.n_marked = &b_marked;
    lo.dec = d.dec + c0; lo.local = true;

    // P1 -- update the narrow list
    update_phase<kNarrow4>(d, sh, lst, nn, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0,
                           p.fp32 != 0, stamp, dag, lo, my_evals, my_exact);
    if (tid == 0) my_updates += nn;
    // P2 -- apply; mark the downwind neighbours of the vertices frozen now
    for (int32_t i = tid; i < nn; i += kThreads) {
      const int32_t v = lst[i];
      set_phi(d, v, __ldcg(d.phi2 + v));
    }
    const int32_t nf = b_frozen;
    for (int32_t i = tid / kMarkLanes; i < nf; i += kThreads / kMarkLanes) {
      const int32_t n = lo.frozen[i];
      const double pn = __ldcg(d.phi2 + n);
      for (int64_t k = d.nptr[n] + tid % kMarkLanes; k < d.nptr[n + 1]; k += kMarkLanes) {
        const int32_t v = __ldg(d.nbr + k);
        const uint32_t w = __ldcg(d.sw + v);
        const double pv = __ldcg(d.phi2 + v);
        if (sw_state(w) != ST_NARROW && sw_stamp(w) != stamp && pn < pv) {
          if (atomicCAS(d.sw + v, w, sw_make(ST_NEIG, stamp)) == w) {
            d.tst[v] = (uint8_t)sw_state(w);
            lo.marked[atomicAdd(&b_marked, 1)] = v;
          }
        }
      }
    }
    __syncthreads();
    // P3 -- re-solve the marked neighbours
    const int32_t nm = b_marked;
    update_phase<kMarked4>(d, sh, lo.marked, nm, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0,
                           p.fp32 != 0, stamp, dag, lo, my_evals, my_exact);
    if (tid == 0) my_updates += nm;
    // P4 -- apply, decided states, next narrow list
    for (int32_t i = tid; i < nm + nn; i += kThreads) {
      if (i < nm) {
        const int32_t v = lo.marked[i];
        uint8_t sv = __ldcg(lo.dec + i);
        const uint8_t tv = __ldcg(d.tst + v);
        set_phi(d, v, __ldcg(d.phi2 + v));
        if (sv == ST_NARROW) {
          if (tv == ST_FROZEN) sv = ST_FROZEN;
          else lnext[atomicAdd(&b_narrow[s1], 1)] = v;
        }
        d.sw[v] = sw_make(sv, stamp);
      } else {
        const int32_t v = lst[i - nm];
        const uint32_t w = __ldcg(d.sw + v);
        const uint8_t tv = __ldcg(d.tst + v);
        if (sw_stamp(w) == stamp) continue;
        if (sw_state(w) == ST_NARROW) {
          if (tv == ST_FROZEN) d.sw[v] = ST_FROZEN;
          else lnext[atomicAdd(&b_narrow[s1], 1)] = v;
        }
      }
    }
    ++it;
    ++it_window;
    __syncthreads();
  }
  if (tid == 0) atomicMax(&d.ctl->win_iter_max, (unsigned long long)it_window);
  return true;
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

// PATH: kPathFour -- four grid-synchronised phases per iteration (windows);
// kPathTwo -- two (one endless window); kPathLocal -- submesh sweeps (blocks
// own whole submeshes within a window).  One instantiation each, so that each
// holds only the update phases it runs (no spills at 128 registers).
enum : int { kPathFour = 0, kPathTwo = 1, kPathLocal = 2 };
#pragma nv_diag_suppress 128  // the grid-wide window code is unreachable in the submesh-sweep instantiation
template <int PATH>
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
  const int dag = min(max(p.dag_warps, 1), kDagWarps);
  PROBE(-1);

  // reset_states_gpu + update_events_gpu: phi = INF, far; seeds narrow.
  // (warm start: every vertex narrow at its given time instead; resume: the
  // times and states as they are, the narrow ones listed below)
  if (!p.resume) {
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
  }

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
    if (PATH == kPathLocal) {
      // submesh sweeps: each block runs its own submeshes through the window
      if (!local_window(d, sh, p, lower, lower_lo, lower_hi, phi_start, cur_time, it, dag, my_evals, my_exact,
                        my_updates, where))
        return;
      if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;
      if (gtid == 0) {  // the window took as many iterations as its slowest block
        ctl->iters_total += ctl->win_iter_max;
        ctl->win_iter_max = 0;
      }
      continue;
    }
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
      if (stv == ST_NARROW) append_active(d.list[s], &ctl->n_narrow[s], (int32_t)v);
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
      lo.next = lnext; lo.n_next = &ctl->n_narrow[s1];
      lo.frozen = d.lfrozen; lo.n_frozen = &ctl->n_frozen[s];
      lo.marked = d.lmarked; lo.n_marked = &ctl->n_marked[s];
      lo.dec = d.dec; lo.local = false;
      PROBE_COUNT(kPrPhases);

      if (PATH == kPathTwo) {
        // X -- update the narrow list, mark the downwind neighbours of the
        // vertices frozen now (cuda_fim.cu:2102-2205)
        update_phase<kNarrow2>(d, sh, lst, nn, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, p.fp32 != 0, stamp, dag,
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
        update_phase<kMarked2>(d, sh, d.lmarked, nm, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, p.fp32 != 0,
                               stamp, dag, lo, my_evals, my_exact);
        my_updates += (gtid == 0) ? nm : 0;
        ++it;
        ++it_window;
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;
      } else {
        // P1 -- solve on elements + reduce per vertex (cuda_fim.cu:2102-2163)
        update_phase<kNarrow4>(d, sh, lst, nn, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, p.fp32 != 0, stamp, dag,
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
                append_active(d.lmarked, &ctl->n_marked[s], v);
              }
            }
          }
        }
        if (!grid_sync_probed(d, nblocks, p.timeout_ns, ++where)) return;

        // P3 -- the narrow vertices that are not re-solved now go to the next
        // list (or freeze), then the marked neighbours are re-solved
        // (cuda_fim.cu:2215-2289), each applying its own result, decided
        // state and next-list entry (cuda_fim.cu:2291-2317): the two touch
        // disjoint vertices, and a narrow vertex's state change leaves it a
        // valid neighbour
        for (int64_t i = gtid; i < nn; i += nthreads) {
          const int32_t v = lst[i];
          const uint32_t w = __ldcg(d.sw + v);
          const uint8_t tv = __ldcg(d.tst + v);
          if (sw_stamp(w) == stamp) continue;  // re-solved below
          if (sw_state(w) == ST_NARROW) {
            if (tv == ST_FROZEN) d.sw[v] = ST_FROZEN;
            else append_active(lnext, &ctl->n_narrow[s1], v);
          }
        }
        const int32_t nm = ld_volatile_i32(&ctl->n_marked[s]);
        update_phase<kMarked3>(d, sh, d.lmarked, nm, lower, lower_lo, lower_hi, phi_start, p.dt, p.exact_all != 0, p.fp32 != 0,
                               stamp, dag, lo, my_evals, my_exact);
        my_updates += (gtid == 0) ? nm : 0;
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
    ctl->iterations = p.local ? (int64_t)ctl->iters_total : it;
  }
  if (my_updates) atomicAdd((unsigned long long *)&ctl->vertex_updates, (unsigned long long)my_updates);
}

#pragma nv_diag_default 128

// Sets the kernels' shared-memory size and returns the largest co-resident
// grid on `device` (the cooperative launch's limit).
inline cudaError_t prepare(int device, int block, int *max_grid)
{
  int sms = 0, per_sm = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fim_solve_kernel<kPathFour>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(BatchSh));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fim_solve_kernel<kPathTwo>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(BatchSh));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fim_solve_kernel<kPathLocal>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(BatchSh));
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fim_solve_kernel<kPathFour>, block, sizeof(BatchSh));
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  *max_grid = sms * per_sm;
  return cudaSuccess;
}

// A cooperative launch (every block co-resident: the grid barrier relies on
// it), through cudaLaunchKernelEx so that stream capture records it as a
// cooperative kernel node.
inline cudaError_t launch(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream)
{
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = sizeof(BatchSh);
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (p.local) return cudaLaunchKernelEx(&cfg, fim_solve_kernel<kPathLocal>, d, p);
  if (p.two_phase) return cudaLaunchKernelEx(&cfg, fim_solve_kernel<kPathTwo>, d, p);
  return cudaLaunchKernelEx(&cfg, fim_solve_kernel<kPathFour>, d, p);
}

}  // namespace FIM_SHAPE_NS
}  // namespace fimgb
