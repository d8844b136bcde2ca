// fim_solver.cpp -- C ABI of the GB300 FIM solver (include/fim.h): solver
// objects, mesh staging on the host, device buffers and launches.
//
// Host staging replaces the reference's CudaSolverFIM constructor
// (src/eikonal/cuda_fim.cu:1218-1501): instead of per-submesh blobs with
// in-blob pointers it builds flat device arrays --
//   * the reference's vertex order inside every tet (extract_submeshes2,
//     src/core/types.cpp:306-570: first appearance inside the tet's submesh,
//     then ascending local id), which the local solver's result depends on;
//   * one "corner" record per (vertex, tet): the other three vertices in the
//     relabelled order of the reference's gray-code tables and the tet's six
//     squared edge norms in that order (filled by the FP64 metric kernel);
//   * the vertex neighbourhood (n2n incl. self, types.cpp:141-220).
#include "fim_internal.h"
#include "../../include/fim.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace fimgb;

namespace {

thread_local std::string g_last_error;

constexpr int kDefaultDagWarps = 10;

template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count)
  {
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
  // keeps the buffer when it already holds count elements
  cudaError_t reserve(size_t count)
  {
    if (p && n >= (count ? count : 1)) return cudaSuccess;
    return alloc(count);
  }
  void release()
  {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DevBuf() { release(); }
};

}  // namespace

void fimgb::set_last_error(const char *msg) { g_last_error = msg; }

// fim_set_conduction uploads the field in up to kCondChunks pieces of at
// least kCondChunkMin tets.
constexpr int kCondChunks = 8;
constexpr int64_t kCondChunkMin = int64_t(1) << 18;

struct fim_solver {
  fim_opts opts{};
  int device = 0;
  cudaStream_t own_stream = nullptr;  // created by fim_create (blocking: ordered after legacy-stream work)
  cudaStream_t stream = nullptr;      // working stream (own_stream unless fim_set_stream)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // the persistent launch as a CUDA graph: captured on cap_stream, replayed
  // while the launch's arguments (gd, gp) and configuration stay the same
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t gexec = nullptr;
  FimDev gd{};
  FimParams gp{};
  int gshape = -1, ggrid = 0, gblock = 0;
  bool graph_ok = true;  // false once capture turned out to be unavailable
  // conduction upload: copy stream, one event per chunk (chunk copies
  // overlap the metric kernel of the chunk before), first invalid tet
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_dep = nullptr, ev_chunk[kCondChunks] = {};
  std::string err;
  int block = kSolveThreads;
  // launch configuration of the solve kernel: batch shape, grid, tet-prefix
  // warps (defaults, or the autotuner's choice for the staged problem)
  int max_grid[kNumShapes] = {};
  int shape = 0, grid = 0, dag_warps = kDefaultDagWarps;
  int local = 0;                    // submesh sweeps for meshes with several submeshes (tuned)
  bool tuned = false;
  fim_tune_info tune{};

  // mesh (nL vertex copies: nL == nV with one submesh)
  int64_t nV = 0, nT = 0, nC = 0, nL = 0;
  int32_t n_submeshes = 1;
  std::vector<int64_t> h_sub_ptr;   // first vertex copy of every submesh (+ end)
  std::vector<int64_t> h_cptr;      // corner offsets of the vertex copies (host copy)
  DevBuf<int32_t> blk_ptr;          // submesh sweeps: copies owned by each block
  int blk_grid = -1;                // grid blk_ptr was computed for
  std::vector<uint8_t> in_tet;
  std::vector<int64_t> h_gptr;
  std::vector<int32_t> h_gcopy;
  DevBuf<int64_t> gptr;
  DevBuf<int32_t> gcopy;
  DevBuf<double> phi_out;
  DevBuf<uint8_t> st_out;
  bool have_mesh = false, have_cond = false, have_stim = false, solved = false;
  double front_width = 0.0;
  DevBuf<double> xyz;
  DevBuf<int32_t> tslots;
  DevBuf<double> evec;  // edge vectors of every tet (metric kernel); empty when they did not fit
  DevBuf<int64_t> cidx, cptr, nptr;
  DevBuf<uint4> crec;
  DevBuf<double> cgeo;
  DevBuf<float> cgf, phi_f, phi2_f;
  DevBuf<int32_t> nbr;
  DevBuf<double> fib, cf, ct;
  DevBuf<unsigned long long> bad;  // first invalid tet of the last conduction upload
  // state
  DevBuf<double> phi, phi2;
  DevBuf<uint8_t> st, tst, dec;
  DevBuf<uint32_t> sw;
  DevBuf<int32_t> list0, list1, list2, lfrozen, lmarked;
  DevBuf<unsigned long long> probe;  // phase times (FIM_PROBE builds)
  DevBuf<int32_t> seed_v;
  DevBuf<double> seed_t;
  int32_t nseed = 0;
  DevBuf<FimCtl> ctl;
  FimCtl last_ctl{};
  fim_stats stats{};
  const double *warm = nullptr;  // caller's warm-start times (device) or nullptr
};

static int set_err(fim_solver *s, int code, const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  g_last_error = buf;
  return code;
}

#define CUDA_TRY(s, call)                                                                     \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess) {                                                                  \
      return set_err((s), _e == cudaErrorMemoryAllocation ? FIM_ERR_OUT_OF_MEMORY : FIM_ERR_CUDA, \
                     "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
    }                                                                                         \
  } while (0)

extern "C" void fim_default_opts(fim_opts *o)
{
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->device = 0;
  o->dt = std::numeric_limits<double>::infinity();
  o->n_steps = 1;
  o->front_width = -1.0;
  o->apd = -1.0;
  o->max_iterations = 0;
  o->timeout_s = 10.0;
  o->verbose = 0;
}

extern "C" const char *fim_last_error(const fim_solver *s)
{
  if (s) return s->err.c_str();
  return g_last_error.c_str();
}

// Loads every batch shape of the solve kernel and records its largest
// co-resident grid; the default configuration is shape 0 on its full grid.
static cudaError_t prepare_shapes(fim_solver *s)
{
  for (int k = 0; k < kNumShapes; ++k) {
    const cudaError_t e = solve_prepare(k, s->device, s->block, &s->max_grid[k]);
    if (e != cudaSuccess) return e;
  }
  s->shape = 0;
  s->grid = s->max_grid[0];
  s->dag_warps = kDefaultDagWarps;
  return cudaSuccess;
}

static cudaError_t create_chunk_events(fim_solver *s)
{
  for (cudaEvent_t &ev : s->ev_chunk) {
    const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

extern "C" int fim_create(const fim_opts *opts, fim_solver **out)
{
  if (!out) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_create: out is NULL");
  *out = nullptr;
  fim_opts o;
  if (opts) o = *opts;
  else fim_default_opts(&o);
  if (o.n_steps < 1) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_create: n_steps must be >= 1");
  if (!(o.dt > 0.0)) o.dt = std::numeric_limits<double>::infinity();
  if (!(o.timeout_s > 0.0)) o.timeout_s = 10.0;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return set_err(nullptr, FIM_ERR_NO_DEVICE, "fim_create: no CUDA device (%s)", cudaGetErrorString(e));
  if (o.device < 0 || o.device >= ndev)
    return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_create: device %d out of range [0,%d)", o.device, ndev);
  fim_solver *s = new (std::nothrow) fim_solver();
  if (!s) return set_err(nullptr, FIM_ERR_OUT_OF_MEMORY, "fim_create: out of host memory");
  s->opts = o;
  s->device = o.device;
  if ((e = cudaSetDevice(s->device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamDefault)) != cudaSuccess ||
      (e = cudaEventCreate(&s->ev0)) != cudaSuccess || (e = cudaEventCreate(&s->ev1)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamDefault)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&s->ev_dep, cudaEventDisableTiming)) != cudaSuccess ||
      (e = create_chunk_events(s)) != cudaSuccess || (e = s->bad.alloc(1)) != cudaSuccess ||
      (e = prepare_shapes(s)) != cudaSuccess || (e = s->ctl.alloc(1)) != cudaSuccess) {
    int rc = set_err(nullptr, FIM_ERR_CUDA, "fim_create: %s", cudaGetErrorString(e));
    fim_destroy(s);
    return rc;
  }
  s->stream = s->own_stream;
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, s->device);
  if (!coop) {
    fim_destroy(s);
    return set_err(nullptr, FIM_ERR_NO_DEVICE, "fim_create: device does not support cooperative launch");
  }
  *out = s;
  return FIM_OK;
}

extern "C" int fim_destroy(fim_solver *s)
{
  if (!s) return FIM_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->own_stream) cudaStreamSynchronize(s->own_stream);
  if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->ev_dep) cudaEventDestroy(s->ev_dep);
  for (cudaEvent_t ev : s->ev_chunk)
    if (ev) cudaEventDestroy(ev);
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  s->own_stream = nullptr;
  s->stream = nullptr;
  delete s;  // DevBuf destructors free device memory
  return FIM_OK;
}

extern "C" int fim_set_stream(fim_solver *s, void *stream)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_set_stream: solver is NULL");
  CUDA_TRY(s, cudaSetDevice(s->device));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  s->stream = stream ? (cudaStream_t)stream : s->own_stream;
  return FIM_OK;
}

// ---------------------------------------------------------------------------
// mesh staging

namespace {

// The reference's slot order of every tet: aggregates numbered by first
// appearance of their tag, local vertex ids by first appearance while
// walking the aggregate's tets in increasing tet index with each tet's
// global ids ascending, then each tet's local ids ascending
// (types.cpp:63-67, 331-345, 383-398, 473).
//   slots  -- 4*nT mesh vertex ids in slot order (for the metric)
//   cslots -- 4*nT vertex-copy ids in slot order (for the corners)
//   gptr/gcopy -- copies of every mesh vertex (left empty with one submesh,
//                 where copy == vertex)
struct Staging {
  std::vector<int32_t> slots, cslots;
  int64_t n_copies = 0;
  int32_t n_submeshes = 1;
  std::vector<int64_t> sub_ptr;   // first vertex copy of every submesh (n_submeshes + 1)
  std::vector<int64_t> gptr;
  std::vector<int32_t> gcopy;
};

void reference_slots(int64_t nV, int64_t nT, const int64_t *tets, const int32_t *atags, Staging &S)
{
  S.slots.resize(4 * nT);
  S.cslots.resize(4 * nT);
  std::vector<int32_t> agg(nT, 0);
  int32_t nagg = 1;
  if (atags) {
    std::unordered_map<int32_t, int32_t> t2a;
    nagg = 0;
    for (int64_t e = 0; e < nT; ++e) {
      auto it = t2a.find(atags[e]);
      if (it == t2a.end()) it = t2a.emplace(atags[e], nagg++).first;
      agg[e] = it->second;
    }
  }
  S.n_submeshes = nagg;
  // tets grouped by aggregate, increasing index inside each group
  std::vector<int64_t> aptr(nagg + 1, 0), order(nT);
  for (int64_t e = 0; e < nT; ++e) aptr[agg[e] + 1]++;
  for (int32_t a = 0; a < nagg; ++a) aptr[a + 1] += aptr[a];
  {
    std::vector<int64_t> fill(aptr.begin(), aptr.end() - 1);
    for (int64_t e = 0; e < nT; ++e) order[fill[agg[e]]++] = e;
  }
  std::vector<int64_t> rank(nV, -1);  // first-appearance rank inside the current aggregate
  std::vector<int32_t> touched;
  std::vector<int32_t> copy_owner;    // copy -> mesh vertex (several submeshes)
  int64_t base = 0;
  for (int32_t a = 0; a < nagg; ++a) {
    int64_t next = 0;
    for (int64_t k = aptr[a]; k < aptr[a + 1]; ++k) {
      const int64_t e = order[k];
      int64_t g[4] = {tets[4 * e], tets[4 * e + 1], tets[4 * e + 2], tets[4 * e + 3]};
      std::sort(g, g + 4);
      for (int j = 0; j < 4; ++j)
        if (rank[g[j]] < 0) {
          rank[g[j]] = next++;
          touched.push_back((int32_t)g[j]);
          if (nagg > 1) copy_owner.push_back((int32_t)g[j]);
        }
      std::sort(g, g + 4, [&](int64_t x, int64_t y) { return rank[x] < rank[y]; });
      for (int j = 0; j < 4; ++j) {
        S.slots[4 * e + j] = (int32_t)g[j];
        S.cslots[4 * e + j] = nagg > 1 ? (int32_t)(base + rank[g[j]]) : (int32_t)g[j];
      }
    }
    S.sub_ptr.push_back(base);
    base += next;
    for (int32_t v : touched) rank[v] = -1;
    touched.clear();
  }
  if (nagg > 1) {
    S.n_copies = base;
    S.gptr.assign(nV + 1, 0);
    for (int32_t g : copy_owner) S.gptr[g + 1]++;
    for (int64_t v = 0; v < nV; ++v) S.gptr[v + 1] += S.gptr[v];
    S.gcopy.resize(base);
    std::vector<int64_t> fill(S.gptr.begin(), S.gptr.end() - 1);
    for (int64_t c = 0; c < base; ++c) S.gcopy[fill[copy_owner[c]]++] = (int32_t)c;
  } else {
    S.n_copies = nV;
  }
}

}  // namespace

extern "C" int fim_set_mesh(fim_solver *s, int64_t nV, const double *xyz, int64_t nT, const int64_t *tets,
                            const int32_t *atags)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_set_mesh: solver is NULL");
  if (nV <= 0 || nT <= 0 || !xyz || !tets)
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_mesh: empty mesh or NULL array");
  if (nV >= (int64_t)INT32_MAX || 4 * nT >= (int64_t)INT32_MAX)
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_mesh: mesh too large (%lld vertices, %lld tets)",
                   (long long)nV, (long long)nT);
  for (int64_t i = 0; i < 4 * nT; ++i)
    if (tets[i] < 0 || tets[i] >= nV)
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_mesh: tet %lld has vertex %lld outside [0,%lld)",
                     (long long)(i / 4), (long long)tets[i], (long long)nV);
  for (int64_t e = 0; e < nT; ++e) {
    const int64_t *t = tets + 4 * e;
    if (t[0] == t[1] || t[0] == t[2] || t[0] == t[3] || t[1] == t[2] || t[1] == t[3] || t[2] == t[3])
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_mesh: tet %lld repeats a vertex", (long long)e);
  }
  for (int64_t i = 0; i < 3 * nV; ++i)
    if (!std::isfinite(xyz[i]))
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_mesh: coordinate %lld is not finite", (long long)i);

  Staging S;
  reference_slots(nV, nT, tets, atags, S);
  const std::vector<int32_t> &slots = S.slots;
  const int64_t nL = S.n_copies;

  // corners of every vertex copy, in increasing tet index
  const int64_t nC = 4 * nT;
  std::vector<int64_t> cptr(nL + 1, 0), cidx(nC);
  for (int64_t i = 0; i < nC; ++i) cptr[S.cslots[i] + 1]++;
  for (int64_t v = 0; v < nL; ++v) cptr[v + 1] += cptr[v];
  std::vector<int4> cids(nC);
  {
    std::vector<int64_t> fill(cptr.begin(), cptr.end() - 1);
    for (int64_t e = 0; e < nT; ++e)
      for (int t = 0; t < 4; ++t) {
        const int32_t v = S.cslots[4 * e + t];
        const int64_t c = fill[v]++;
        cidx[4 * e + t] = c;
        cids[c] = make_int4(S.cslots[4 * e + ((t + 1) & 3)], S.cslots[4 * e + ((t + 2) & 3)],
                            S.cslots[4 * e + ((t + 3) & 3)], (int)e);
      }
  }
  // neighbourhood of every copy incl. itself (sorted), two passes
  std::vector<int64_t> nptr(nL + 1, 0);
  std::vector<int32_t> nbr;
  {
    std::vector<int32_t> cnt(nL);
#pragma omp parallel
    {
      std::vector<int32_t> buf;
#pragma omp for schedule(static)
      for (int64_t v = 0; v < nL; ++v) {
        buf.clear();
        buf.push_back((int32_t)v);
        for (int64_t c = cptr[v]; c < cptr[v + 1]; ++c) {
          buf.push_back(cids[c].x); buf.push_back(cids[c].y); buf.push_back(cids[c].z);
        }
        std::sort(buf.begin(), buf.end());
        cnt[v] = (int32_t)(std::unique(buf.begin(), buf.end()) - buf.begin());
      }
    }
    for (int64_t v = 0; v < nL; ++v) nptr[v + 1] = nptr[v] + cnt[v];
    nbr.resize(nptr[nL]);
#pragma omp parallel
    {
      std::vector<int32_t> buf;
#pragma omp for schedule(static)
      for (int64_t v = 0; v < nL; ++v) {
        buf.clear();
        buf.push_back((int32_t)v);
        for (int64_t c = cptr[v]; c < cptr[v + 1]; ++c) {
          buf.push_back(cids[c].x); buf.push_back(cids[c].y); buf.push_back(cids[c].z);
        }
        std::sort(buf.begin(), buf.end());
        const int64_t m = std::unique(buf.begin(), buf.end()) - buf.begin();
        std::copy(buf.begin(), buf.begin() + m, nbr.begin() + nptr[v]);
      }
    }
  }
  // vertices in at least one tet (seeds elsewhere are dropped, as the
  // reference seeds through submeshes only)
  std::vector<uint8_t> in_tet(nV, 0);
  for (int64_t i = 0; i < nC; ++i) in_tet[slots[i]] = 1;
  // reference front width: 1.01 * longest edge / 0.6 (compute_dwf, cuda_fim.h:1536-1576)
  double maxe2 = 0.0;
  for (int64_t e = 0; e < nT; ++e)
    for (int i = 0; i < 4; ++i)
      for (int j = i + 1; j < 4; ++j) {
        const int64_t a = tets[4 * e + i], b = tets[4 * e + j];
        const double dx = xyz[3 * b] - xyz[3 * a], dy = xyz[3 * b + 1] - xyz[3 * a + 1], dz = xyz[3 * b + 2] - xyz[3 * a + 2];
        const double l = dx * dx + dy * dy + dz * dz;
        if (l > maxe2) maxe2 = l;
      }
  s->front_width = 1.01 * std::sqrt(maxe2) / 0.6;

  CUDA_TRY(s, cudaSetDevice(s->device));
  s->warm = nullptr;  // a warm start belongs to the previous mesh
  if (s->tuned) {      // so does a tuned launch configuration
    s->tuned = false;
    s->shape = 0; s->grid = s->max_grid[0]; s->dag_warps = kDefaultDagWarps; s->local = 0;
  }
  s->have_mesh = s->have_cond = s->have_stim = s->solved = false;
  s->nV = nV; s->nT = nT; s->nC = nC; s->nL = nL;
  s->n_submeshes = S.n_submeshes;
  S.sub_ptr.push_back(nL);
  s->h_sub_ptr.swap(S.sub_ptr);
  s->blk_grid = -1;
  s->in_tet.swap(in_tet);
  s->h_gptr.swap(S.gptr);
  s->h_gcopy.swap(S.gcopy);
  const bool multi = S.n_submeshes > 1;
  CUDA_TRY(s, s->xyz.alloc(3 * nV));
  CUDA_TRY(s, s->tslots.alloc(4 * nT));
  CUDA_TRY(s, s->cidx.alloc(nC));
  CUDA_TRY(s, s->cptr.alloc(nL + 1));
  CUDA_TRY(s, s->crec.alloc((size_t)kCrecWords * nC));
  CUDA_TRY(s, s->cgeo.alloc((size_t)kCgeoStride * nC));
  CUDA_TRY(s, s->cgf.alloc((size_t)kCgfStride * nC));
  CUDA_TRY(s, s->nptr.alloc(nL + 1));
  CUDA_TRY(s, s->nbr.alloc(nbr.size()));
  CUDA_TRY(s, s->fib.alloc(3 * nT));
  CUDA_TRY(s, s->cf.alloc(nT));
  CUDA_TRY(s, s->ct.alloc(nT));
  CUDA_TRY(s, s->phi.alloc(nL));
  CUDA_TRY(s, s->phi_f.alloc(nL));
  CUDA_TRY(s, s->phi2.alloc(nL));
  CUDA_TRY(s, s->phi2_f.alloc(nL));
  CUDA_TRY(s, s->st.alloc(nL));
  CUDA_TRY(s, s->tst.alloc(nL));
  CUDA_TRY(s, s->dec.alloc(nL));
  CUDA_TRY(s, s->sw.alloc(nL));
  CUDA_TRY(s, s->list0.alloc(nL));
  CUDA_TRY(s, s->list1.alloc(nL));
  CUDA_TRY(s, s->list2.alloc(nL));
  CUDA_TRY(s, s->lfrozen.alloc(nL));
  CUDA_TRY(s, s->lmarked.alloc(nL));
  if (multi) {
    CUDA_TRY(s, s->gptr.alloc(nV + 1));
    CUDA_TRY(s, s->gcopy.alloc(nL));
    CUDA_TRY(s, s->phi_out.alloc(nV));
    CUDA_TRY(s, s->st_out.alloc(nV));
  } else {
    s->gptr.release(); s->gcopy.release(); s->phi_out.release(); s->st_out.release();
  }
  cudaStream_t st = s->stream;
  CUDA_TRY(s, cudaMemcpyAsync(s->xyz.p, xyz, sizeof(double) * 3 * nV, cudaMemcpyHostToDevice, st));
  CUDA_TRY(s, cudaMemcpyAsync(s->tslots.p, slots.data(), sizeof(int32_t) * 4 * nT, cudaMemcpyHostToDevice, st));
  // the edge vectors for the metric kernel (144 B per tet); without room
  // for them the kernel forms them from xyz
  if (s->evec.alloc((size_t)18 * nT) == cudaSuccess) {
    CUDA_TRY(s, launch_edge_vectors(s->tslots.p, s->xyz.p, nT, s->evec.p, st));
  } else {
    cudaGetLastError();
    s->evec.release();
  }
  CUDA_TRY(s, cudaMemcpyAsync(s->cidx.p, cidx.data(), sizeof(int64_t) * nC, cudaMemcpyHostToDevice, st));
  CUDA_TRY(s, cudaMemcpyAsync(s->cptr.p, cptr.data(), sizeof(int64_t) * (nL + 1), cudaMemcpyHostToDevice, st));
  CUDA_TRY(s, cudaStreamSynchronize(st));
  s->h_cptr.swap(cptr);
  {
    // the ids part of the first-read records (the metric kernel fills the rest)
    std::vector<uint4> crec((size_t)kCrecWords * nC);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nC; ++c) {
      crec[kCrecWords * c] = make_uint4((unsigned)cids[c].x, (unsigned)cids[c].y, (unsigned)cids[c].z, 0u);
      crec[kCrecWords * c + 1] = make_uint4(0u, 0u, 0u, 0u);
    }
    CUDA_TRY(s, cudaMemcpyAsync(s->crec.p, crec.data(), sizeof(uint4) * crec.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(s, cudaStreamSynchronize(st));
  }
  CUDA_TRY(s, cudaMemcpyAsync(s->nptr.p, nptr.data(), sizeof(int64_t) * (nL + 1), cudaMemcpyHostToDevice, st));
  CUDA_TRY(s, cudaMemcpyAsync(s->nbr.p, nbr.data(), sizeof(int32_t) * nbr.size(), cudaMemcpyHostToDevice, st));
  if (multi) {
    CUDA_TRY(s, cudaMemcpyAsync(s->gptr.p, s->h_gptr.data(), sizeof(int64_t) * (nV + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(s, cudaMemcpyAsync(s->gcopy.p, s->h_gcopy.data(), sizeof(int32_t) * nL, cudaMemcpyHostToDevice, st));
  }
  CUDA_TRY(s, cudaStreamSynchronize(st));
  s->stats.n_corners = nC;
  s->have_mesh = true;
  return FIM_OK;
}

// Uploads a conduction field and runs the metric kernel.  The arrays (host
// or device, by `host`) are copied over the copy stream in chunks, and each
// chunk's metric launch waits only for its own copy, so the transfers
// overlap the FP64 metric work.  The
// kernel also checks the field (positive finite speeds, finite fibres): on a
// bad tet the call fails and the solver has no conduction until a later call
// succeeds.
static int run_metric(fim_solver *s, const double *fib, const double *cf, const double *ct, bool host,
                      const char *who)
{
  const int64_t nT = s->nT;
  const int nch = (int)std::max<int64_t>(1, std::min<int64_t>(kCondChunks, nT / kCondChunkMin));
  const cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  cudaStream_t cs = s->copy_stream;
  s->have_cond = false;
  s->solved = false;
  CUDA_TRY(s, cudaMemsetAsync(s->bad.p, 0xff, sizeof(unsigned long long), s->stream));
  // the copies overwrite arrays that earlier work on the working stream may read
  CUDA_TRY(s, cudaEventRecord(s->ev_dep, s->stream));
  CUDA_TRY(s, cudaStreamWaitEvent(cs, s->ev_dep, 0));
  for (int i = 0; i < nch; ++i) {
    const int64_t e0 = nT * i / nch, e1 = nT * (i + 1) / nch;
    CUDA_TRY(s, cudaMemcpyAsync(s->fib.p + 3 * e0, fib + 3 * e0, sizeof(double) * 3 * (e1 - e0), kind, cs));
    CUDA_TRY(s, cudaMemcpyAsync(s->cf.p + e0, cf + e0, sizeof(double) * (e1 - e0), kind, cs));
    CUDA_TRY(s, cudaMemcpyAsync(s->ct.p + e0, ct + e0, sizeof(double) * (e1 - e0), kind, cs));
    CUDA_TRY(s, cudaEventRecord(s->ev_chunk[i], cs));
    CUDA_TRY(s, cudaStreamWaitEvent(s->stream, s->ev_chunk[i], 0));
    if (i == 0) CUDA_TRY(s, cudaEventRecord(s->ev0, s->stream));
    CUDA_TRY(s, launch_metric(s->tslots.p, s->cidx.p, s->xyz.p, s->evec.p, s->nT, s->fib.p, s->cf.p, s->ct.p, e0,
                              e1, s->cgeo.p, s->cgf.p, s->crec.p, s->bad.p, s->stream));
  }
  CUDA_TRY(s, cudaEventRecord(s->ev1, s->stream));
  CUDA_TRY(s, cudaEventSynchronize(s->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  s->stats.metric_ms = ms;
  unsigned long long bad = 0;
  CUDA_TRY(s, cudaMemcpy(&bad, s->bad.p, sizeof bad, cudaMemcpyDeviceToHost));
  if (bad < (unsigned long long)nT) {
    const int64_t e = (int64_t)bad;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // cf, ct, fibre
    CUDA_TRY(s, cudaMemcpy(v, s->cf.p + e, sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(s, cudaMemcpy(v + 1, s->ct.p + e, sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(s, cudaMemcpy(v + 2, s->fib.p + 3 * e, 3 * sizeof(double), cudaMemcpyDeviceToHost));
    if (!(v[0] > 0.0) || !(v[1] > 0.0) || !std::isfinite(v[0]) || !std::isfinite(v[1]))
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "%s: tet %lld has speed cf=%g ct=%g", who, (long long)e, v[0], v[1]);
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "%s: tet %lld has a non-finite fibre", who, (long long)e);
  }
  s->have_cond = true;
  return FIM_OK;
}

extern "C" int fim_set_conduction(fim_solver *s, const double *fib, const double *cf, const double *ct)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_set_conduction: solver is NULL");
  if (!s->have_mesh) return set_err(s, FIM_ERR_NOT_READY, "fim_set_conduction: no mesh");
  if (!fib || !cf || !ct) return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_conduction: NULL array");
  CUDA_TRY(s, cudaSetDevice(s->device));
  return run_metric(s, fib, cf, ct, true, "fim_set_conduction");
}

extern "C" int fim_set_conduction_device(fim_solver *s, const double *d_fib, const double *d_cf, const double *d_ct)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_set_conduction_device: solver is NULL");
  if (!s->have_mesh) return set_err(s, FIM_ERR_NOT_READY, "fim_set_conduction_device: no mesh");
  if (!d_fib || !d_cf || !d_ct) return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_conduction_device: NULL array");
  CUDA_TRY(s, cudaSetDevice(s->device));
  return run_metric(s, d_fib, d_cf, d_ct, false, "fim_set_conduction_device");
}

extern "C" int fim_set_stimuli(fim_solver *s, int64_t n, const int64_t *vertices, const double *t0)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_set_stimuli: solver is NULL");
  if (!s->have_mesh) return set_err(s, FIM_ERR_NOT_READY, "fim_set_stimuli: no mesh");
  if (n < 0 || (n > 0 && (!vertices || !t0)))
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_stimuli: bad count or NULL array");
  // one entry per vertex: the earliest start time
  std::unordered_map<int64_t, double> first;
  for (int64_t i = 0; i < n; ++i) {
    if (vertices[i] < 0 || vertices[i] >= s->nV)
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_stimuli: vertex %lld outside [0,%lld)",
                     (long long)vertices[i], (long long)s->nV);
    if (!std::isfinite(t0[i]))
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_stimuli: start time %lld is not finite", (long long)i);
    const double ti = t0[i] == 0.0 ? 0.0 : t0[i];  // -0.0 counts as +0.0
    auto it = first.find(vertices[i]);
    if (it == first.end()) first.emplace(vertices[i], ti);
    else if (ti < it->second) it->second = ti;
  }
  // every copy of a stimulated vertex is seeded (update_events_gpu seeds
  // through the submeshes holding the vertex, cuda_fim.cu:1422-1487)
  std::vector<int32_t> v;
  std::vector<double> t;
  v.reserve(first.size());
  t.reserve(first.size());
  for (int64_t i = 0; i < n; ++i) {
    auto it = first.find(vertices[i]);
    if (it == first.end()) continue;
    const int64_t g = it->first;
    if (s->in_tet[g]) {
      if (s->h_gptr.empty()) { v.push_back((int32_t)g); t.push_back(it->second); }
      else
        for (int64_t k = s->h_gptr[g]; k < s->h_gptr[g + 1]; ++k) { v.push_back(s->h_gcopy[k]); t.push_back(it->second); }
    }
    first.erase(it);
  }
  CUDA_TRY(s, cudaSetDevice(s->device));
  CUDA_TRY(s, s->seed_v.reserve(v.size()));
  CUDA_TRY(s, s->seed_t.reserve(t.size()));
  if (!v.empty()) {
    CUDA_TRY(s, cudaMemcpyAsync(s->seed_v.p, v.data(), sizeof(int32_t) * v.size(), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(s->seed_t.p, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  }
  s->nseed = (int32_t)v.size();
  s->have_stim = true;
  s->solved = false;
  return FIM_OK;
}

// Two grid-synchronised phases per FIM iteration need one endless window:
// only then can no vertex leave the narrow list for "next" in mid-window,
// which lets the neighbour marking run inside the narrow update.
static bool two_phase_ok(const FimParams &p)
{
  return std::isinf(p.dt) && p.dt > 0.0;
}

#ifdef FIM_PROBE
// Per-phase device time of the last solve, averaged over the blocks
// (instrumented builds only).
static void print_probe(fim_solver *s, int grid)
{
  std::vector<unsigned long long> h((size_t)grid * kProbeSlots);
  if (cudaMemcpy(h.data(), s->probe.p, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return;
  static const char *names[14] = {"setup", "A", "B", "S", "D", "E", "mark", "barrier", "light", "batches",
                                  "phases", "S-tet warp-ms", "S-tri warp-ms", "S-edge warp-ms"};
  std::fprintf(stderr, "probe (mean per block):");
  for (int k = 0; k < 14; ++k) {
    double sum = 0.0;
    for (int b = 0; b < grid; ++b) sum += (double)h[(size_t)b * kProbeSlots + k];
    sum /= grid;
    if (k < 9 || k >= 11) std::fprintf(stderr, " %s %.3f ms", names[k], sum * 1e-6);
    else std::fprintf(stderr, " %s %.1f", names[k], sum);
  }
  // queued FP64 solves per block: tets (low word; batches with more than 48
  // in the high word), triangles (low) and edges (high)
  double q[4] = {0, 0, 0, 0};
  for (int b = 0; b < grid; ++b) {
    const unsigned long long a = h[(size_t)b * kProbeSlots + 14], c = h[(size_t)b * kProbeSlots + 15];
    q[0] += (double)(a & 0xffffffffull); q[1] += (double)(a >> 32);
    q[2] += (double)(c & 0xffffffffull); q[3] += (double)(c >> 32);
  }
  std::fprintf(stderr, " queued tets %.1f (batches > 48: %.1f) tris %.1f edges %.1f", q[0] / grid, q[1] / grid,
               q[2] / grid, q[3] / grid);
  static const char *outc[8] = {"tet sqt<0", "tet sqt undecided", "tet no root", "tet value", "tet value>bhi",
                                "tri none", "tri >bhi", "tri <=bhi"};
  for (int k = 16; k < 24; ++k) {
    double sum = 0.0;
    for (int b = 0; b < grid; ++b) sum += (double)h[(size_t)b * kProbeSlots + k];
    std::fprintf(stderr, " %s %.0f", outc[k - 16], sum / grid);
  }
  double dt[4] = {0, 0, 0, 0};
  for (int b = 0; b < grid; ++b)
    for (int k = 0; k < 4; ++k) dt[k] += (double)h[(size_t)b * kProbeSlots + 24 + k];
  std::fprintf(stderr, " D tet part %.2f us in %.1f batches, D tri part %.2f us in %.1f batches",
               dt[2] > 0 ? dt[0] / dt[2] * 1e-3 : 0.0, dt[2] / grid, dt[3] > 0 ? dt[1] / dt[3] * 1e-3 : 0.0,
               dt[3] / grid);
  std::fprintf(stderr, "\n");
}
#endif

static int tune_solver(fim_solver *s, cudaStream_t st);
static int warm_check(fim_solver *s, cudaStream_t st);

// Submesh sweeps: whole submeshes to blocks, contiguous in copy order, with
// about the same number of corners each (the corners are the work).
static void block_ranges(const fim_solver *s, int grid, std::vector<int32_t> &out)
{
  const std::vector<int64_t> &sp = s->h_sub_ptr;
  const int nsub = (int)sp.size() - 1;
  const int64_t total = s->h_cptr[s->nL];
  out.assign(grid + 1, (int32_t)s->nL);
  out[0] = 0;
  int b = 1;
  for (int a = 0; a < nsub && b < grid; ++a) {
    // close block b-1 after submesh a once it holds its share
    const int64_t done = s->h_cptr[sp[a + 1]];
    while (b < grid && done * grid >= total * b) out[b++] = (int32_t)sp[a + 1];
  }
}

// Launch parameters and device view of the solver's staged problem.
static void solve_args(const fim_solver *s, FimDev &d, FimParams &p)
{
  // zeroed bytewise (padding included): the graph cache compares them bytewise
  std::memset(static_cast<void *>(&d), 0, sizeof d);
  d.nV = (int32_t)s->nL; d.nG = (int32_t)s->nV; d.nT = s->nT; d.nC = s->nC;
  d.gptr = s->gptr.p; d.gcopy = s->gcopy.p; d.phi_out = s->phi_out.p; d.st_out = s->st_out.p;
  d.cptr = s->cptr.p; d.crec = s->crec.p; d.cgeo = s->cgeo.p; d.cgf = s->cgf.p; d.nptr = s->nptr.p; d.nbr = s->nbr.p;
  d.phi_f = s->phi_f.p; d.phi2_f = s->phi2_f.p;
  d.phi = s->phi.p; d.phi2 = s->phi2.p; d.sw = s->sw.p; d.st = s->st.p; d.tst = s->tst.p;
  d.list[0] = s->list0.p; d.list[1] = s->list1.p; d.list[2] = s->list2.p;
  d.lfrozen = s->lfrozen.p; d.lmarked = s->lmarked.p; d.dec = s->dec.p;
  d.seed_v = s->seed_v.p; d.seed_t = s->seed_t.p; d.nseed = s->nseed;
  d.phi_init = s->warm;
  d.ctl = s->ctl.p;
  std::memset(static_cast<void *>(&p), 0, sizeof p);
  p.dt = s->opts.dt;
  p.n_steps = s->opts.n_steps;
  p.front_width = s->opts.front_width >= 0.0 ? s->opts.front_width : s->front_width;
  p.apd = s->opts.apd;
  p.max_iter = s->opts.max_iterations > 0 ? s->opts.max_iterations : 10000000;
  p.timeout_ns = (uint64_t)(s->opts.timeout_s * 1e9);
  p.exact_all = s->opts.exact_all ? 1 : 0;
  p.fp32 = (s->opts.fp32_update && !s->opts.exact_all) ? 1 : 0;
  p.two_phase = two_phase_ok(p) ? 1 : 0;
}

// The persistent launch as a CUDA graph: graph_prepare keeps the cached
// graph when the kernel's arguments and configuration equal those it was
// captured with, else captures the launch on cap_stream (thread-local mode,
// so other threads' CUDA calls are not affected) and instantiates it; it
// returns whether the graph can be launched.  Where capture or instantiation
// fails the solver launches directly from then on.  It runs before the
// solve's timing events, so capturing costs no measured device time.
static bool graph_prepare(fim_solver *s, const FimDev &d, const FimParams &p, int shape, int grid, bool *captured)
{
  *captured = false;
  if (!s->graph_ok) return false;
  if (s->gexec && s->gshape == shape && s->ggrid == grid && s->gblock == s->block &&
      std::memcmp(&s->gd, &d, sizeof d) == 0 && std::memcmp(&s->gp, &p, sizeof p) == 0)
    return true;
  if (s->gexec) { cudaGraphExecDestroy(s->gexec); s->gexec = nullptr; }
  cudaError_t e = cudaSuccess;
  if (!s->cap_stream) e = cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking);
  cudaGraph_t g = nullptr;
  if (e == cudaSuccess) e = cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const cudaError_t el = launch_solve(d, p, shape, grid, s->block, s->cap_stream);
    const cudaError_t ec = cudaStreamEndCapture(s->cap_stream, &g);
    e = el != cudaSuccess ? el : ec;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&s->gexec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();  // not sticky: clear it and launch directly from now on
    s->gexec = nullptr;
    s->graph_ok = false;
    return false;
  }
  std::memcpy(static_cast<void *>(&s->gd), &d, sizeof d);
  std::memcpy(static_cast<void *>(&s->gp), &p, sizeof p);
  s->gshape = shape; s->ggrid = grid; s->gblock = s->block;
  *captured = true;
  return true;
}

// One solve with launch configuration (shape, grid, dag_warps); resume keeps
// the times and states in place instead of resetting and seeding them.
static int run_solve(fim_solver *s, cudaStream_t st, int shape, int grid, int dag_warps, bool resume = false,
                     int local = -1)
{
  if (local < 0) local = s->local;
  FimDev d{};
  FimParams p{};
  solve_args(s, d, p);
  p.withhold_block = (s->opts.test_withhold_block > 0 && s->opts.test_withhold_block <= grid)
                         ? s->opts.test_withhold_block : 0;
  p.dag_warps = dag_warps;
  p.resume = resume ? 1 : 0;
  if (local && s->n_submeshes > 1) {
    p.local = 1;
    p.two_phase = 0;
    if (s->blk_grid != grid) {
      std::vector<int32_t> ranges;
      block_ranges(s, grid, ranges);
      CUDA_TRY(s, s->blk_ptr.reserve(ranges.size()));
      CUDA_TRY(s, cudaMemcpyAsync(s->blk_ptr.p, ranges.data(), sizeof(int32_t) * ranges.size(),
                                  cudaMemcpyHostToDevice, st));
      s->blk_grid = grid;
    }
    d.blk_ptr = s->blk_ptr.p;
  }
#ifdef FIM_PROBE
  CUDA_TRY(s, s->probe.reserve((size_t)grid * kProbeSlots));
  CUDA_TRY(s, cudaMemsetAsync(s->probe.p, 0, sizeof(unsigned long long) * grid * kProbeSlots, st));
  d.probe = s->probe.p;
#endif
  CUDA_TRY(s, cudaMemsetAsync(s->ctl.p, 0, sizeof(FimCtl), st));
  bool captured = false;
  const bool replayed = graph_prepare(s, d, p, shape, grid, &captured);
  CUDA_TRY(s, cudaEventRecord(s->ev0, st));
  if (replayed) CUDA_TRY(s, cudaGraphLaunch(s->gexec, st));
  else CUDA_TRY(s, launch_solve(d, p, shape, grid, s->block, st));
  CUDA_TRY(s, cudaEventRecord(s->ev1, st));
  CUDA_TRY(s, cudaMemcpyAsync(&s->last_ctl, s->ctl.p, sizeof(FimCtl), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(s, cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  s->stats.solve_ms = ms;
  s->stats.iterations = s->last_ctl.iterations;
  s->stats.vertex_updates = s->last_ctl.vertex_updates;
  s->stats.corner_evals = s->last_ctl.corner_evals;
  s->stats.exact_evals = s->last_ctl.exact_evals;
  s->stats.grid_blocks = grid;
  s->stats.block_threads = s->block;
  s->stats.batch_slots = kShapes[shape].slots;
  s->stats.batch_corners = kShapes[shape].corners;
  s->stats.dag_warps = dag_warps;
  s->stats.submesh_sweeps = p.local;
  s->stats.graph_launch = replayed ? 1 : 0;
  s->stats.graph_captured = captured ? 1 : 0;
#ifdef FIM_PROBE
  print_probe(s, grid);
#endif
  if (s->last_ctl.error == KERR_TIMEOUT)
    return set_err(s, FIM_ERR_TIMEOUT, "fim_solve: a grid barrier wait exceeded %.3f s (phase %d)",
                   s->opts.timeout_s, s->last_ctl.error_where);
  if (s->last_ctl.error == KERR_MAX_ITER)
    return set_err(s, FIM_ERR_MAX_ITERATIONS, "fim_solve: iteration cap %lld reached in a window",
                   (long long)p.max_iter);
  s->solved = true;
  return FIM_OK;
}

extern "C" int fim_solve(fim_solver *s, void *stream)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_solve: solver is NULL");
  if (!s->have_mesh || !s->have_cond || !s->have_stim)
    return set_err(s, FIM_ERR_NOT_READY, "fim_solve: mesh, conduction and stimuli must be set first");
  CUDA_TRY(s, cudaSetDevice(s->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
  if (s->opts.autotune && !s->tuned) {
    const int rc = tune_solver(s, st);
    if (rc != FIM_OK) return rc;
  }
  int rc = run_solve(s, st, s->shape, s->grid, s->dag_warps);
  s->stats.warm_reset = 0;
  s->stats.warm_rounds = 0;
  if (rc != FIM_OK || !s->warm || !(std::isinf(s->opts.dt) && s->opts.n_steps == 1)) return rc;
  return warm_check(s, st);
}

// ---------------------------------------------------------------------------
// support check of warm-started solves
//
// FIM only lowers times, so a start below the true time of a vertex would
// stay wrong.  After a warm-started solve, fim_support_kernel flags every
// reached non-seed vertex whose time lies below a rigorous lower bound of
// every candidate of its neighbours (a cold solve never has one).  Such a
// vertex, and every vertex downwind of it, has a time at least as large as
// the smallest flagged time tmin, so all times >= tmin are reset to INF and
// FIM resumes from the times below tmin (and the stimuli); the check then
// runs again.  After kWarmRounds rounds that still find flagged vertices,
// the solve is redone cold.
constexpr int kWarmRounds = 3;

static int warm_check(fim_solver *s, cudaStream_t st)
{
  FimDev d{};
  FimParams p{};
  solve_args(s, d, p);
  const double lower = -p.front_width;
  double total_ms = s->stats.solve_ms;
  int64_t iters = s->stats.iterations, upd = s->stats.vertex_updates;
  int64_t reset = 0;
  int rounds = 0;
  for (;;) {
    float ms = 0.f;
    CUDA_TRY(s, cudaEventRecord(s->ev0, st));
    CUDA_TRY(s, cudaMemsetAsync(s->dec.p, 0, s->nL, st));
    CUDA_TRY(s, launch_mark_seeds(d, s->dec.p, st));
    CUDA_TRY(s, cudaMemsetAsync(&s->ctl.p->n_bad, 0, sizeof(int32_t), st));
    CUDA_TRY(s, cudaMemsetAsync(&s->ctl.p->tmin_key, 0xff, sizeof(unsigned long long), st));
    CUDA_TRY(s, launch_support_check(d, lower, s->dec.p, st));
    CUDA_TRY(s, cudaEventRecord(s->ev1, st));
    FimCtl h{};
    CUDA_TRY(s, cudaMemcpyAsync(&h, s->ctl.p, sizeof(FimCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(s, cudaStreamSynchronize(st));
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    total_ms += ms;
    if (h.n_bad == 0) break;
    reset += h.n_bad;
    int rc;
    if (rounds == kWarmRounds) {  // give up on the start: a cold solve
      const double *w = s->warm;
      s->warm = nullptr;
      rc = run_solve(s, st, s->shape, s->grid, s->dag_warps);
      s->warm = w;
      if (rc != FIM_OK) return rc;
      total_ms += s->stats.solve_ms;
      iters += s->stats.iterations;
      upd += s->stats.vertex_updates;
      ++rounds;
      break;
    }
    const unsigned long long k = h.tmin_key;
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double tmin;
    std::memcpy(&tmin, &b, sizeof tmin);
    CUDA_TRY(s, cudaEventRecord(s->ev0, st));
    CUDA_TRY(s, launch_warm_reset(d, tmin, st));
    CUDA_TRY(s, cudaEventRecord(s->ev1, st));
    if ((rc = run_solve(s, st, s->shape, s->grid, s->dag_warps, true)) != FIM_OK) return rc;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    total_ms += ms + s->stats.solve_ms;
    iters += s->stats.iterations;
    upd += s->stats.vertex_updates;
    ++rounds;
  }
  s->stats.solve_ms = total_ms;
  s->stats.iterations = iters;
  s->stats.vertex_updates = upd;
  s->stats.warm_reset = reset;
  s->stats.warm_rounds = rounds;
  return FIM_OK;
}

// ---------------------------------------------------------------------------
// autotuner (replaces the reference's external partition and its fixed
// block size, types.cpp:306-570, cuda_fim.cu:2435)
//
// The solve's speed depends on the problem: how many vertices a FIM
// iteration updates (the front), how many corners they have, how many of
// their local solves survive the FP32 screens.  The tuner times full solves
// of the staged problem under candidate launch configurations and keeps the
// fastest: first the batch shape (vertices x corners a block stages at once)
// on its full grid, then the grid (fewer persistent blocks cost less per
// grid barrier and give each block more vertices), then the number of warps
// running the FP64 tet prefixes.  Every configuration computes the same
// times bit for bit; only the speed differs.

// Device time of one solve under a configuration (the better of two runs
// for short solves).
static int time_config(fim_solver *s, cudaStream_t st, int shape, int grid, int dag, double *ms)
{
  int rc = run_solve(s, st, shape, grid, dag);
  if (rc != FIM_OK) return rc;
  double best = s->stats.solve_ms;
  if (best < 200.0) {
    rc = run_solve(s, st, shape, grid, dag);
    if (rc != FIM_OK) return rc;
    best = std::min(best, s->stats.solve_ms);
  }
  *ms = best;
  return FIM_OK;
}

static int tune_solver(fim_solver *s, cudaStream_t st)
{
  int n = 0;
  double def_ms = 0.0;
  s->local = 0;
  int rc = time_config(s, st, 0, s->max_grid[0], kDefaultDagWarps, &def_ms);
  if (rc != FIM_OK) return rc;
  ++n;
  int b_shape = 0, b_grid = s->max_grid[0], b_dag = kDefaultDagWarps;
  double b_ms = def_ms;
  auto consider = [&](int shape, int grid, int dag) -> int {
    double ms = 0.0;
    const int r = time_config(s, st, shape, grid, dag, &ms);
    if (r != FIM_OK) return r;
    ++n;
    if (ms < b_ms) { b_ms = ms; b_shape = shape; b_grid = grid; b_dag = dag; }
    return FIM_OK;
  };
  for (int k = 1; k < kNumShapes; ++k)
    if ((rc = consider(k, s->max_grid[k], kDefaultDagWarps)) != FIM_OK) return rc;
  const int full = s->max_grid[b_shape];
  for (int div : {2, 4})
    if (full / div >= 1 && (rc = consider(b_shape, full / div, kDefaultDagWarps)) != FIM_OK) return rc;
  const int g = b_grid;
  for (int dag : {6, 8, 12})
    if ((rc = consider(b_shape, g, dag)) != FIM_OK) return rc;
  int b_local = 0;
  if (s->n_submeshes > 1) {  // submesh sweeps against grid-wide iterations
    s->local = 1;
    double ms = 0.0;
    if ((rc = time_config(s, st, b_shape, b_grid, b_dag, &ms)) != FIM_OK) return rc;
    ++n;
    if (ms < b_ms) { b_ms = ms; b_local = 1; }
  }
  s->local = b_local;
  s->shape = b_shape; s->grid = b_grid; s->dag_warps = b_dag;
  s->tuned = true;
  s->tune.batch_slots = kShapes[b_shape].slots;
  s->tune.batch_corners = kShapes[b_shape].corners;
  s->tune.grid_blocks = b_grid;
  s->tune.dag_warps = b_dag;
  s->tune.submesh_sweeps = b_local;
  s->tune.default_ms = def_ms;
  s->tune.tuned_ms = b_ms;
  s->tune.candidates = n;
  return FIM_OK;
}

extern "C" int fim_autotune(fim_solver *s, void *stream, fim_tune_info *info)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_autotune: solver is NULL");
  if (!s->have_mesh || !s->have_cond || !s->have_stim)
    return set_err(s, FIM_ERR_NOT_READY, "fim_autotune: mesh, conduction and stimuli must be set first");
  CUDA_TRY(s, cudaSetDevice(s->device));
  const int rc = tune_solver(s, stream ? (cudaStream_t)stream : s->stream);
  if (rc != FIM_OK) return rc;
  if (info) *info = s->tune;
  return FIM_OK;
}

extern "C" int fim_set_tune(fim_solver *s, const fim_tune_info *cfg)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_set_tune: solver is NULL");
  if (!cfg) {  // back to the default configuration
    s->tuned = false;
    s->shape = 0; s->grid = s->max_grid[0]; s->dag_warps = kDefaultDagWarps; s->local = 0;
    return FIM_OK;
  }
  int shape = -1;
  for (int k = 0; k < kNumShapes; ++k)
    if (kShapes[k].slots == cfg->batch_slots && kShapes[k].corners == cfg->batch_corners) shape = k;
  if (shape < 0) {
    std::string have;
    for (int k = 0; k < kNumShapes; ++k) have += std::string(k ? ", " : "") + kShapes[k].name;
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_tune: no batch shape %dx%d (compiled: %s)", cfg->batch_slots,
                   cfg->batch_corners, have.c_str());
  }
  if (cfg->grid_blocks < 1 || cfg->grid_blocks > s->max_grid[shape])
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_tune: grid %d outside [1,%d]", cfg->grid_blocks,
                   s->max_grid[shape]);
  if (cfg->dag_warps < 1 || cfg->dag_warps > kDagWarpsMax)
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_tune: dag_warps %d outside [1,%d]", cfg->dag_warps,
                   kDagWarpsMax);
  s->shape = shape; s->grid = cfg->grid_blocks; s->dag_warps = cfg->dag_warps;
  s->local = cfg->submesh_sweeps ? 1 : 0;
  s->tuned = true;
  s->tune = *cfg;
  return FIM_OK;
}

extern "C" int fim_get_tune(const fim_solver *s, fim_tune_info *info)
{
  if (!s || !info) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_get_tune: NULL argument");
  if (s->tuned) {
    *info = s->tune;
  } else {
    std::memset(info, 0, sizeof(*info));
    info->batch_slots = kShapes[s->shape].slots;
    info->batch_corners = kShapes[s->shape].corners;
    info->grid_blocks = s->grid;
    info->dag_warps = s->dag_warps;
    info->submesh_sweeps = s->local;
  }
  return FIM_OK;
}

extern "C" int fim_get_times(fim_solver *s, double *phi, int32_t *state)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_get_times: solver is NULL");
  if (!s->solved) return set_err(s, FIM_ERR_NOT_READY, "fim_get_times: no finished solve");
  CUDA_TRY(s, cudaSetDevice(s->device));
  const double *dphi = s->phi_out.p ? s->phi_out.p : s->phi.p;
  const uint8_t *dst = s->st_out.p ? s->st_out.p : s->st.p;
  if (phi) CUDA_TRY(s, cudaMemcpyAsync(phi, dphi, sizeof(double) * s->nV, cudaMemcpyDeviceToHost, s->stream));
  std::vector<uint8_t> st8;
  if (state) {
    st8.resize(s->nV);
    CUDA_TRY(s, cudaMemcpyAsync(st8.data(), dst, s->nV, cudaMemcpyDeviceToHost, s->stream));
  }
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  if (state)
    for (int64_t v = 0; v < s->nV; ++v) state[v] = st8[v];
  return FIM_OK;
}

extern "C" int fim_get_times_device(fim_solver *s, double *d_phi)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_get_times_device: solver is NULL");
  if (!s->solved) return set_err(s, FIM_ERR_NOT_READY, "fim_get_times_device: no finished solve");
  if (!d_phi) return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_get_times_device: NULL pointer");
  CUDA_TRY(s, cudaSetDevice(s->device));
  CUDA_TRY(s, launch_copy(s->phi_out.p ? s->phi_out.p : s->phi.p, d_phi, s->nV, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  return FIM_OK;
}

extern "C" int fim_get_stats(const fim_solver *s, fim_stats *out)
{
  if (!s || !out) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_get_stats: NULL argument");
  *out = s->stats;
  return FIM_OK;
}

// ---------------------------------------------------------------------------
// allocation-free re-solve (no counterpart in the reference)
//
// Meant for callers that re-solve one staged mesh for many stimulus sets from
// a loop sharing the device with other work: fim_set_stimuli grows its seed
// buffers whenever a stimulus set is larger than all before it (cudaFree,
// which waits for the whole device, then cudaMalloc, which can fail once the
// caller's own pool holds the free memory).  Here the
// stimuli and the solve's working set go to the fixed scratch of
// fim_static.cu, the result to the caller's device buffer; the solver's own
// buffers and last results are left as they were.
extern "C" int fim_solve_noalloc(fim_solver *s, int64_t n, const int64_t *vertices, const double *t0,
                                 double *d_phi, void *stream)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_solve_noalloc: solver is NULL");
  if (!s->have_mesh || !s->have_cond)
    return set_err(s, FIM_ERR_NOT_READY, "fim_solve_noalloc: mesh and conduction must be set first");
  if (!d_phi) return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_solve_noalloc: d_phi is NULL");
  if (n < 0 || (n > 0 && (!vertices || !t0)))
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_solve_noalloc: bad count or NULL array");
  if (s->nL > kStaticMaxCopies || s->nV > kStaticMaxVertices)
    return set_err(s, FIM_ERR_INVALID_ARGUMENT,
                   "fim_solve_noalloc: the mesh has %lld vertices (%lld vertex copies); the fixed scratch "
                   "holds at most %lld of each -- use fim_set_stimuli + fim_solve",
                   (long long)s->nV, (long long)s->nL, (long long)kStaticMaxCopies);
  if (n > kStaticMaxSeeds)
    return set_err(s, FIM_ERR_INVALID_ARGUMENT,
                   "fim_solve_noalloc: %lld stimulus entries; the fixed scratch holds at most %lld",
                   (long long)n, (long long)kStaticMaxSeeds);
  int64_t entries = 0;  // stimulus entries once expanded to vertex copies
  for (int64_t i = 0; i < n; ++i) {
    const int64_t g = vertices[i];
    if (g < 0 || g >= s->nV)
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_solve_noalloc: vertex %lld outside [0,%lld)",
                     (long long)g, (long long)s->nV);
    if (!std::isfinite(t0[i]))
      return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_solve_noalloc: start time %lld is not finite",
                     (long long)i);
    entries += s->h_gptr.empty() ? (s->in_tet[g] ? 1 : 0) : s->h_gptr[g + 1] - s->h_gptr[g];
  }
  if (entries > kStaticMaxSeedEntries)
    return set_err(s, FIM_ERR_INVALID_ARGUMENT,
                   "fim_solve_noalloc: the stimuli expand to %lld vertex copies; the fixed scratch holds at "
                   "most %lld", (long long)entries, (long long)kStaticMaxSeedEntries);
  CUDA_TRY(s, cudaSetDevice(s->device));
  NoallocScratch sc{};
  CUDA_TRY(s, noalloc_scratch(s->device, &sc));
  cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
  if (n > 0) {
    CUDA_TRY(s, cudaMemcpyAsync(sc.raw_v, vertices, sizeof(int64_t) * n, cudaMemcpyHostToDevice, st));
    CUDA_TRY(s, cudaMemcpyAsync(sc.raw_t, t0, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CUDA_TRY(s, launch_noalloc_seeds(sc, (int32_t)n, s->gptr.p, s->gcopy.p, s->cptr.p, st));
  }
  const bool multi = s->gptr.p != nullptr;
  FimDev d{};
  d.nV = (int32_t)s->nL; d.nG = (int32_t)s->nV; d.nT = s->nT; d.nC = s->nC;
  d.gptr = s->gptr.p; d.gcopy = s->gcopy.p;
  d.phi_out = multi ? d_phi : nullptr; d.st_out = multi ? sc.st_out : nullptr;
  d.cptr = s->cptr.p; d.crec = s->crec.p; d.cgeo = s->cgeo.p; d.cgf = s->cgf.p; d.nptr = s->nptr.p; d.nbr = s->nbr.p;
  d.phi_f = sc.phi_f; d.phi2_f = sc.phi2_f;
  d.phi = sc.phi; d.phi2 = sc.phi2; d.sw = sc.sw; d.st = sc.st; d.tst = sc.tst;
  d.list[0] = sc.list[0]; d.list[1] = sc.list[1]; d.list[2] = sc.list[2];
  d.lfrozen = sc.lfrozen; d.lmarked = sc.lmarked; d.dec = sc.dec;
  d.seed_v = sc.seed_v; d.seed_t = sc.seed_t; d.nseed = (int32_t)entries;
  d.phi_init = s->warm;  // the caller's own device array (fim_set_warm_start): nothing to allocate
  d.ctl = sc.ctl;
  FimParams p{};
  p.dt = s->opts.dt;
  p.n_steps = s->opts.n_steps;
  p.front_width = s->opts.front_width >= 0.0 ? s->opts.front_width : s->front_width;
  p.apd = s->opts.apd;
  p.max_iter = s->opts.max_iterations > 0 ? s->opts.max_iterations : 10000000;
  p.timeout_ns = (uint64_t)(s->opts.timeout_s * 1e9);
  p.withhold_block = 0;
  p.exact_all = s->opts.exact_all ? 1 : 0;
  p.fp32 = (s->opts.fp32_update && !s->opts.exact_all) ? 1 : 0;
  p.two_phase = two_phase_ok(p) ? 1 : 0;
  p.dag_warps = s->dag_warps;
  CUDA_TRY(s, cudaMemsetAsync(sc.ctl, 0, sizeof(FimCtl), st));
  CUDA_TRY(s, launch_solve(d, p, s->shape, s->grid, s->block, st));
  if (!multi) CUDA_TRY(s, launch_copy(sc.phi, d_phi, s->nV, st));
  FimCtl ctl{};
  CUDA_TRY(s, cudaMemcpyAsync(&ctl, sc.ctl, sizeof(FimCtl), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(s, cudaStreamSynchronize(st));
  if (ctl.error == KERR_TIMEOUT)
    return set_err(s, FIM_ERR_TIMEOUT, "fim_solve_noalloc: a grid barrier wait exceeded %.3f s (phase %d)",
                   s->opts.timeout_s, ctl.error_where);
  if (ctl.error == KERR_MAX_ITER)
    return set_err(s, FIM_ERR_MAX_ITERATIONS, "fim_solve_noalloc: iteration cap %lld reached in a window",
                   (long long)p.max_iter);
  return FIM_OK;
}

// ---------------------------------------------------------------------------
// batched solves (no counterpart in the reference)
//
// Independent problems are staged as ONE disjoint mesh in an internal
// solver: every FIM iteration of the persistent kernel advances all of them,
// so the per-iteration latencies (grid barriers, batch phase chains) are
// paid once for the whole batch.  A problem's vertices only ever meet its
// own tets, and with one endless window and start times >= 0 the reference's
// front-width test never rejects a reached time, so each problem evolves
// exactly as it would alone (a problem that has converged simply has an
// empty narrow list).

struct fim_batch {
  fim_opts opts{};
  fim_solver *s = nullptr;
  std::string err;
  struct Problem {
    int64_t nV = 0, nT = 0;
    int64_t v0 = 0;  // first vertex in the union
  };
  std::vector<Problem> probs;
  std::vector<double> xyz, fib, cf, ct, stim_t;
  std::vector<int64_t> tets, stim_v;
  bool staged = false, solved = false;
  std::vector<double> phi;
  std::vector<int32_t> st;
};

static int batch_err(fim_batch *b, int code, const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  g_last_error = buf;
  return code;
}

extern "C" int fim_batch_create(const fim_opts *opts, fim_batch **out)
{
  if (!out) return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_batch_create: out is NULL");
  *out = nullptr;
  fim_opts o;
  if (opts) o = *opts;
  else fim_default_opts(&o);
  if ((o.dt > 0.0 && std::isfinite(o.dt)) || o.n_steps != 1)
    return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT,
                     "fim_batch_create: batched solves run one endless window (dt <= 0, n_steps = 1)");
  fim_batch *b = new (std::nothrow) fim_batch();
  if (!b) return batch_err(nullptr, FIM_ERR_OUT_OF_MEMORY, "fim_batch_create: out of host memory");
  b->opts = o;
  const int rc = fim_create(&o, &b->s);
  if (rc != FIM_OK) {
    const std::string m = fim_last_error(nullptr);
    delete b;
    return batch_err(nullptr, rc, "fim_batch_create: %s", m.c_str());
  }
  *out = b;
  return FIM_OK;
}

extern "C" int fim_batch_destroy(fim_batch *b)
{
  if (!b) return FIM_OK;
  fim_destroy(b->s);
  delete b;
  return FIM_OK;
}

extern "C" const char *fim_batch_last_error(const fim_batch *b)
{
  return b ? b->err.c_str() : g_last_error.c_str();
}

extern "C" int fim_batch_add(fim_batch *b, int64_t nV, const double *xyz, int64_t nT, const int64_t *tets,
                             const double *fib, const double *cf, const double *ct, int64_t n_stim,
                             const int64_t *stim_v, const double *stim_t, int64_t *problem)
{
  if (!b) return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_batch_add: batch is NULL");
  if (nV <= 0 || nT <= 0 || !xyz || !tets || !fib || !cf || !ct || n_stim < 0 || (n_stim > 0 && (!stim_v || !stim_t)))
    return batch_err(b, FIM_ERR_INVALID_ARGUMENT, "fim_batch_add: bad size or NULL array");
  const int64_t v0 = b->probs.empty() ? 0 : b->probs.back().v0 + b->probs.back().nV;
  if (v0 + nV > INT32_MAX || (int64_t)(b->tets.size() / 4) + nT > INT32_MAX / 4)
    return batch_err(b, FIM_ERR_INVALID_ARGUMENT, "fim_batch_add: the batch exceeds 2^31 vertices or 2^29 tets");
  for (int64_t i = 0; i < 4 * nT; ++i)
    if (tets[i] < 0 || tets[i] >= nV)
      return batch_err(b, FIM_ERR_INVALID_ARGUMENT, "fim_batch_add: tet %lld refers to vertex %lld outside [0,%lld)",
                       (long long)(i / 4), (long long)tets[i], (long long)nV);
  for (int64_t i = 0; i < n_stim; ++i) {
    if (stim_v[i] < 0 || stim_v[i] >= nV)
      return batch_err(b, FIM_ERR_INVALID_ARGUMENT, "fim_batch_add: stimulus vertex %lld outside [0,%lld)",
                       (long long)stim_v[i], (long long)nV);
    if (!(stim_t[i] >= 0.0) || !std::isfinite(stim_t[i]))
      return batch_err(b, FIM_ERR_INVALID_ARGUMENT,
                       "fim_batch_add: start time %lld is %g; batched solves need finite times >= 0", (long long)i,
                       stim_t[i]);
  }
  try {
    b->xyz.insert(b->xyz.end(), xyz, xyz + 3 * nV);
    for (int64_t i = 0; i < 4 * nT; ++i) b->tets.push_back(tets[i] + v0);
    b->fib.insert(b->fib.end(), fib, fib + 3 * nT);
    b->cf.insert(b->cf.end(), cf, cf + nT);
    b->ct.insert(b->ct.end(), ct, ct + nT);
    for (int64_t i = 0; i < n_stim; ++i) { b->stim_v.push_back(stim_v[i] + v0); b->stim_t.push_back(stim_t[i]); }
    fim_batch::Problem p;
    p.nV = nV; p.nT = nT; p.v0 = v0;
    b->probs.push_back(p);
  } catch (const std::bad_alloc &) {
    return batch_err(b, FIM_ERR_OUT_OF_MEMORY, "fim_batch_add: out of host memory");
  }
  if (problem) *problem = (int64_t)b->probs.size() - 1;
  b->staged = b->solved = false;
  return FIM_OK;
}

// Stages every problem of the batch as one disjoint mesh (once after adds).
static int batch_stage(fim_batch *b, const char *who)
{
  if (b->staged) return FIM_OK;
  fim_solver *s = b->s;
  int rc;
  const int64_t nV = (int64_t)b->xyz.size() / 3, nT = (int64_t)b->tets.size() / 4;
  if ((rc = fim_set_mesh(s, nV, b->xyz.data(), nT, b->tets.data(), nullptr)) != FIM_OK ||
      (rc = fim_set_conduction(s, b->fib.data(), b->cf.data(), b->ct.data())) != FIM_OK ||
      (rc = fim_set_stimuli(s, (int64_t)b->stim_v.size(), b->stim_v.data(), b->stim_t.data())) != FIM_OK)
    return batch_err(b, rc, "%s: %s", who, fim_last_error(s));
  b->staged = true;
  return FIM_OK;
}

extern "C" int fim_batch_autotune(fim_batch *b, void *stream, fim_tune_info *info)
{
  if (!b) return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_batch_autotune: batch is NULL");
  if (b->probs.empty()) return batch_err(b, FIM_ERR_NOT_READY, "fim_batch_autotune: no problems added");
  int rc = batch_stage(b, "fim_batch_autotune");
  if (rc != FIM_OK) return rc;
  if ((rc = fim_autotune(b->s, stream, info)) != FIM_OK)
    return batch_err(b, rc, "fim_batch_autotune: %s", fim_last_error(b->s));
  b->solved = false;
  return FIM_OK;
}

extern "C" int fim_batch_set_warm_start(fim_batch *b, const double *d_phi_init)
{
  if (!b) return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_batch_set_warm_start: batch is NULL");
  if (d_phi_init && b->probs.empty())
    return batch_err(b, FIM_ERR_NOT_READY, "fim_batch_set_warm_start: no problems added");
  if (d_phi_init) {
    const int rc = batch_stage(b, "fim_batch_set_warm_start");
    if (rc != FIM_OK) return rc;
  }
  const int rc = fim_set_warm_start(b->s, d_phi_init);
  if (rc != FIM_OK) return batch_err(b, rc, "fim_batch_set_warm_start: %s", fim_last_error(b->s));
  b->solved = false;
  return FIM_OK;
}

extern "C" int fim_batch_solve(fim_batch *b, void *stream)
{
  if (!b) return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_batch_solve: batch is NULL");
  if (b->probs.empty()) return batch_err(b, FIM_ERR_NOT_READY, "fim_batch_solve: no problems added");
  fim_solver *s = b->s;
  int rc = batch_stage(b, "fim_batch_solve");
  if (rc != FIM_OK) return rc;
  if ((rc = fim_solve(s, stream)) != FIM_OK) return batch_err(b, rc, "fim_batch_solve: %s", fim_last_error(s));
  try {
    b->phi.resize(b->xyz.size() / 3);
    b->st.resize(b->xyz.size() / 3);
  } catch (const std::bad_alloc &) {
    return batch_err(b, FIM_ERR_OUT_OF_MEMORY, "fim_batch_solve: out of host memory");
  }
  if ((rc = fim_get_times(s, b->phi.data(), b->st.data())) != FIM_OK)
    return batch_err(b, rc, "fim_batch_solve: %s", fim_last_error(s));
  b->solved = true;
  return FIM_OK;
}

extern "C" int fim_batch_get_times(fim_batch *b, int64_t problem, double *phi, int32_t *state)
{
  if (!b) return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_batch_get_times: batch is NULL");
  if (!b->solved) return batch_err(b, FIM_ERR_NOT_READY, "fim_batch_get_times: no finished solve");
  if (problem < 0 || problem >= (int64_t)b->probs.size())
    return batch_err(b, FIM_ERR_INVALID_ARGUMENT, "fim_batch_get_times: problem %lld outside [0,%lld)",
                     (long long)problem, (long long)b->probs.size());
  const fim_batch::Problem &p = b->probs[problem];
  if (phi) std::copy(b->phi.begin() + p.v0, b->phi.begin() + p.v0 + p.nV, phi);
  if (state) std::copy(b->st.begin() + p.v0, b->st.begin() + p.v0 + p.nV, state);
  return FIM_OK;
}

extern "C" int fim_batch_get_stats(const fim_batch *b, fim_stats *out)
{
  if (!b || !out) return batch_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_batch_get_stats: NULL argument");
  return fim_get_stats(b->s, out);
}

// ---------------------------------------------------------------------------
// learned warm start: features of the staged problem, warm-start times

extern "C" int fim_features(fim_solver *s, void *d_features, float *time_scale)
{
  if (!s || !d_features) return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_features: NULL argument");
  if (!s->have_mesh || !s->have_cond || !s->have_stim)
    return set_err(s, FIM_ERR_NOT_READY, "fim_features: mesh, conduction and stimuli must be set first");
  if (s->gptr.p) return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_features: meshes with submesh tags are not supported");
  CUDA_TRY(s, cudaSetDevice(s->device));
  DevBuf<float> acc, dist;
  DevBuf<unsigned int> red;
  CUDA_TRY(s, acc.alloc(6 * (size_t)s->nV));
  CUDA_TRY(s, dist.alloc((size_t)s->nV));
  CUDA_TRY(s, red.alloc(8));
  CUDA_TRY(s, launch_features((int)s->nV, s->nT, s->xyz.p, s->tslots.p, s->fib.p, s->cf.p, s->ct.p, s->nseed,
                              s->seed_v.p, s->seed_t.p, acc.p, dist.p, red.p, d_features, s->stream));
  unsigned int h[8] = {};
  CUDA_TRY(s, cudaMemcpyAsync(h, red.p, sizeof(unsigned int) * 7, cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  if (time_scale) *time_scale = features_scale(h);
  return FIM_OK;
}

extern "C" int fim_set_warm_start(fim_solver *s, const double *d_phi_init)
{
  if (!s) return set_err(nullptr, FIM_ERR_INVALID_ARGUMENT, "fim_set_warm_start: solver is NULL");
  if (d_phi_init && (!s->have_mesh || s->gptr.p))
    return set_err(s, FIM_ERR_INVALID_ARGUMENT, "fim_set_warm_start: needs a mesh without submesh tags");
  s->warm = d_phi_init;
  s->solved = false;
  return FIM_OK;
}
