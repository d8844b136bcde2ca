/*
 * fim.h -- C ABI of the GB300 Fast Iterative Method eikonal solver.
 *
 * Drop-in for the solve of the reference's tw::CudaSolverFIM
 * (src/eikonal/cuda_fim.h:1443-1577 of tomstrident/cufim-nvlink): the
 * constructor's staging (src/eikonal/cuda_fim.cu:1218-1501) maps to
 * fim_set_mesh / fim_set_conduction / fim_set_stimuli, CudaSolverFIM::solve
 * (src/eikonal/cuda_fim.cu:2386-2503) maps to fim_solve + fim_get_times.
 *
 * Conventions
 *  - Plain C types only; every function returns a fim_status (0 = FIM_OK).
 *    Nothing here exits the process or throws; the message of the last error
 *    of a solver is fim_last_error(solver) (fim_last_error(NULL) for errors
 *    before a solver exists).
 *  - Vertex and tet ids are int64_t as in the reference (idx_t, types.h:45).
 *  - Times, lengths and speeds are in any consistent unit system (the
 *    reference's files use um, um/us and us).
 *  - A solver object is used from one host thread at a time.
 *  - Device arrays passed in must be complete when the call is made.  The
 *    library's own streams are blocking streams, so its work is ordered
 *    after earlier work on the legacy default stream (PyTorch's default
 *    stream); data written on any other stream must be synchronised by the
 *    caller, or that stream passed where a call takes one (fim_solve).
 *  - Solve semantics are those of the reference's CudaSolverFIM::solve with
 *    every tet in one submesh: windows of length dt, n_steps of them,
 *    narrow/next/frozen/tail states, the front-width rule and the APD reset
 *    (src/eikonal/cuda_fim.cu:1790-1845, 1992-2334).  With dt <= 0 (or
 *    infinite) and n_steps = 1 the solve runs to convergence in one window.
 *    Arithmetic is FP64 with the reference's float-typed triangle
 *    intermediates and no fused multiply-adds, so results are bit-identical
 *    to the reference's source semantics.
 */
#ifndef FIM_GB300_H_
#define FIM_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FIM_OK = 0,
  FIM_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size, index or option       */
  FIM_ERR_CUDA = 2,             /* a CUDA runtime call failed               */
  FIM_ERR_NOT_READY = 3,        /* mesh / conduction / stimuli missing      */
  FIM_ERR_TIMEOUT = 4,          /* a bounded in-kernel wait expired         */
  FIM_ERR_MAX_ITERATIONS = 5,   /* iteration cap reached before convergence */
  FIM_ERR_IO = 6,               /* file could not be read / written         */
  FIM_ERR_OUT_OF_MEMORY = 7,
  FIM_ERR_NO_DEVICE = 8
} fim_status;

/* Reference node states (types.h:85). */
enum { FIM_FAR = 0, FIM_NEIG = 1, FIM_NARROW = 2, FIM_NEXT = 3, FIM_FROZEN = 4, FIM_TAIL = 5 };

typedef struct fim_solver fim_solver;

typedef struct {
  int device;            /* CUDA device ordinal                                     */
  double dt;             /* window length; <= 0 or inf: one window without end      */
  int n_steps;           /* number of windows (>= 1)                                */
  double front_width;    /* < 0: reference rule 1.01 * longest edge / 0.6           */
  double apd;            /* frozen->tail after apd, tail->far after apd/0.91;
                            < 0: disabled (reference: 3e5 us, cuda_fim.cu:1815)     */
  int64_t max_iterations;/* cap on FIM iterations per window; 0: 1e7                */
  double timeout_s;      /* limit of every in-kernel wait; <= 0: 10 s               */
  int verbose;
  int test_withhold_block; /* failure-detection test hook: k > 0 makes block k-1
                              skip its first grid-barrier arrival, so the other
                              blocks' bounded waits expire and fim_solve returns
                              FIM_ERR_TIMEOUT; 0 = off                             */
  int exact_all;         /* 1: solve every triangle/tet candidate in FP64 instead of
                              screening them with FP32 interval bounds first; the
                              results are identical, only slower (cross-check)     */
  int autotune;          /* 1: the first fim_solve after fim_set_mesh (or
                              fim_batch_solve after an add) runs fim_autotune first */
  int fp32_update;       /* 1: take each triangle, tet and edge candidate's FP32
                              value wherever its running-error screen is
                              conclusive, FP64 only where it is not (the
                              degenerate branch).  NOT bit-exact: the
                              reference's freeze rule amplifies float rounding;
                              bench.py --precision fp32 reports the error   */
} fim_opts;

/* Defaults: device 0, one endless window, reference front width, APD off. */
void fim_default_opts(fim_opts *opts);

/* Creates a solver on opts->device (NULL opts = defaults). */
int fim_create(const fim_opts *opts, fim_solver **out);
int fim_destroy(fim_solver *s);
const char *fim_last_error(const fim_solver *s);

/* Mesh: xyz[3*n_vertices] (x,y,z per vertex), tets[4*n_tets] (any vertex
 * order), atags[n_tets] submesh tags or NULL.  The tags fix the reference's
 * vertex order inside every tet (extract_submeshes2, types.cpp:306-570);
 * NULL is one submesh.  Replaces the ctor's extract_submeshes2 and staging
 * (cuda_fim.cu:1218-1411). */
int fim_set_mesh(fim_solver *s, int64_t n_vertices, const double *xyz, int64_t n_tets,
                 const int64_t *tets, const int32_t *atags);

/* Conduction per tet (host pointers): unit fibre fib[3*n_tets], speed along
 * the fibre cf[n_tets] and across it ct[n_tets].  The FP64 per-tet metric
 * M = cf^-2 f f^T + ct^-2 (I - f f^T) and its six squared edge norms are
 * computed on the GPU (compute_velocity_tensor_f3 + compute_geo,
 * types.h:173-188, types.cpp:227-257; the reference hard-codes fibre (1,0,0)
 * and 0.6 there, vtk.cpp:99-101, types.cpp:231).  The arrays are uploaded
 * in chunks whose transfers overlap the metric kernel (pinned host memory
 * lets them run asynchronously) and are read until the call returns.  The
 * GPU checks the field: a tet with a non-positive or non-finite speed or a
 * non-finite fibre fails the call with FIM_ERR_INVALID_ARGUMENT, naming the
 * first such tet, and the solver then has no conduction until a later call
 * succeeds. */
int fim_set_conduction(fim_solver *s, const double *fib, const double *cf, const double *ct);
/* Same, with device pointers (already resident in HBM on the solver's
 * device), with the same check. */
int fim_set_conduction_device(fim_solver *s, const double *d_fib, const double *d_cf,
                              const double *d_ct);

/* Stimuli: n vertices with their start times (the reference seeds every
 * stimulus at time 0, update_events_gpu, cuda_fim.cu:632-683).  A vertex
 * given several times starts at the earliest; -0.0 counts as +0.0. */
int fim_set_stimuli(fim_solver *s, int64_t n, const int64_t *vertices, const double *t0);

/* Runs the solve on `stream` (a cudaStream_t, NULL = the solver's working
 * stream) and waits for it.  The persistent launch is captured once into a
 * CUDA graph (on a stream of the solver's own) and replayed by every later
 * solve whose device buffers, stimulus count, options and launch
 * configuration are unchanged; anything else captures a new graph.  Where
 * capture is not available the kernel is launched directly (fim_stats
 * graph_launch = 0). */
int fim_solve(fim_solver *s, void *stream);

/* Sets the working stream (a cudaStream_t on the solver's device) of all
 * later transfers and launches of this solver; NULL restores its own. */
int fim_set_stream(fim_solver *s, void *stream);

/* Results of the last solve: phi[n_vertices] (FP64; the reference's INF,
 * DBL_MAX, for unreached vertices) and state[n_vertices] (or NULL). */
int fim_get_times(fim_solver *s, double *phi, int32_t *state);
/* Same into device memory (phi on the solver's device). */
int fim_get_times_device(fim_solver *s, double *d_phi);

typedef struct {
  int64_t iterations;      /* FIM iterations (all windows)                  */
  int64_t vertex_updates;  /* vertex solves (narrow + re-solved neighbours) */
  int64_t corner_evals;    /* (vertex, tet) corners screened                */
  int64_t exact_evals;     /* triangle/tet solves done in FP64              */
  double solve_ms;         /* device time of the last fim_solve             */
  double metric_ms;        /* device time of the last metric precompute     */
  int64_t n_corners;       /* (vertex, tet) pairs of the mesh               */
  int grid_blocks;         /* persistent grid size of the FIM kernel        */
  int block_threads;
  int batch_slots;         /* batch shape of the last solve: vertices ...   */
  int batch_corners;       /* ... and corners a block stages at once        */
  int dag_warps;           /* warps running FP64 tet prefixes per batch     */
  int64_t warm_reset;      /* warm start: times the support check rejected  */
  int warm_rounds;         /* warm start: check-reset-resume rounds run     */
  int submesh_sweeps;      /* 1: blocks ran whole submeshes per window      */
  int graph_launch;        /* 1: the persistent launch ran as the replay of
                              a CUDA graph instantiated by the solver        */
  int graph_captured;      /* 1: this solve captured (and instantiated) that
                              graph; later solves with the same staged
                              buffers, stimuli count and launch configuration
                              replay it without capturing again              */
} fim_stats;
int fim_get_stats(const fim_solver *s, fim_stats *out);

/* Autotuner -- replaces the reference's external partition and fixed block
 * size (extract_submeshes2, src/core/types.cpp:306-570; compute_step<<<nA,
 * 256>>>, src/eikonal/cuda_fim.cu:2435).  Times full solves of the staged
 * problem (mesh, conduction, stimuli set) under candidate launch
 * configurations of the persistent kernel -- the batch shape (vertices x
 * corners a block stages at once), the number of persistent blocks and the
 * warps running the FP64 tet prefixes -- and keeps the fastest for every
 * later solve of this mesh (fim_set_mesh forgets it).  Every configuration
 * gives bit-identical times; the solver's last results are those of the
 * last timed run.  info (or NULL) receives the choice. */
typedef struct {
  int batch_slots;      /* chosen batch shape: vertices ...                       */
  int batch_corners;    /* ... and corners per batch                              */
  int grid_blocks;      /* persistent blocks                                      */
  int dag_warps;        /* warps running FP64 tet prefixes                        */
  int submesh_sweeps;   /* meshes with several submeshes: 1 = every block runs its
                           own whole submeshes through each window with block
                           barriers only (grid barriers only between windows),
                           0 = grid-wide iterations; results are identical     */
  double default_ms;    /* solve time with the default configuration (0: untuned) */
  double tuned_ms;      /* solve time with the chosen one                         */
  int candidates;       /* configurations timed                                   */
} fim_tune_info;
int fim_autotune(fim_solver *s, void *stream, fim_tune_info *info);
/* The configuration in use (the default one until tuned). */
int fim_get_tune(const fim_solver *s, fim_tune_info *info);
/* Pins a configuration (e.g. one fim_autotune chose in an earlier run):
 * batch_slots/batch_corners must name a compiled batch shape (192x4096,
 * 160x3072, 96x2048), grid_blocks lie in [1, the shape's co-resident grid],
 * dag_warps in [1, 12]; the timing fields are ignored.  NULL restores the
 * default configuration (grid-wide iterations). */
int fim_set_tune(fim_solver *s, const fim_tune_info *cfg);

/* Allocation-free re-solve -- no counterpart in the reference.
 * Solves s's mesh and conduction for the stimuli given here (host arrays,
 * the rules of fim_set_stimuli) and writes the times of all n_vertices into
 * d_phi (device memory on s's device), on `stream` (NULL = the solver's
 * working stream), and waits for it.  Results are bit-identical to
 * fim_set_stimuli + fim_solve + fim_get_times_device.
 *
 * It calls no allocator: the solve's working set lives in a fixed device
 * array of the library (about 8.5 MB per device), for callers that must not
 * allocate between solves -- e.g. a loop re-solving one mesh for many
 * stimulus sets while other streams run, where fim_set_stimuli grows its
 * seed buffers whenever a stimulus set is larger than all before it (a
 * cudaFree that waits for the whole device, then a cudaMalloc that can fail
 * once the caller's own pool holds the memory).  Limits: at most 131072 mesh
 * vertices and 131072 vertex copies (one per submesh holding a vertex),
 * 8192 stimulus entries, 32768 stimulus vertex copies; larger inputs are
 * rejected with FIM_ERR_INVALID_ARGUMENT.  The solver's own buffers, stats
 * and last results are not touched.  A warm start set by fim_set_warm_start
 * applies here as in fim_solve (it is the caller's own device array).
 *
 * The first call on a device resolves the array's address (and loads its
 * code there); make it before any stream capture.  The array is shared by
 * every call on that device in this process: calls that overlap in time
 * (from several host threads) race on it and return wrong times, so they
 * must be serialised by the caller. */
int fim_solve_noalloc(fim_solver *s, int64_t n, const int64_t *vertices, const double *t0,
                      double *d_phi, void *stream);

/* Self-test of the FP32 screens -- no counterpart in the reference.  The
 * solve screens every triangle and tet candidate with rigorous FP32 bounds
 * before it runs the FP64 solve, and stays bit-exact only while those
 * bounds hold.  This checks them on n random corners (random shapes and
 * anisotropic metrics, plane-wave, spread and nearly equal times) against
 * the FP64 solves on `device`: out[0] tets checked, out[1] tet violations,
 * out[2] tets with a value, out[3] triangle pairs checked, out[4] triangle
 * violations, out[5] triangle pairs with a value.  A violation is a value
 * the screen calls impossible or bounds wrongly. */
int fim_selftest_screens(int device, int64_t n, uint64_t seed, int64_t *out);

/* Batched solves -- no counterpart in the reference: many solves of uneven
 * size in one persistent launch.
 * Independent problems (mesh + conduction + stimuli, each with its own
 * vertex numbering) are staged as one disjoint mesh and solved by ONE launch
 * of the persistent kernel: every FIM iteration advances all of them.  Each
 * problem's times are bit-identical to solving it alone with fim_solve.
 * Batches run one endless window (opts->dt <= 0 or inf, n_steps = 1) and
 * take start times >= 0, where the front-width rule never fires.  Problems
 * are copied at fim_batch_add; staging happens at the first fim_batch_solve
 * after an add.  Errors: fim_batch_last_error(batch). */
typedef struct fim_batch fim_batch;
int fim_batch_create(const fim_opts *opts, fim_batch **out);
int fim_batch_destroy(fim_batch *b);
const char *fim_batch_last_error(const fim_batch *b);
/* Adds a problem (host arrays as for fim_set_mesh / fim_set_conduction /
 * fim_set_stimuli; tets index 0..n_vertices-1) and returns its index. */
int fim_batch_add(fim_batch *b, int64_t n_vertices, const double *xyz, int64_t n_tets, const int64_t *tets,
                  const double *fib, const double *cf, const double *ct, int64_t n_stim,
                  const int64_t *stim_vertices, const double *stim_t0, int64_t *problem);
/* Solves every problem of the batch (one persistent launch) and waits. */
int fim_batch_solve(fim_batch *b, void *stream);
/* Times (and states, or NULL) of one problem after fim_batch_solve. */
int fim_batch_get_times(fim_batch *b, int64_t problem, double *phi, int32_t *state);
/* Statistics of the last batch solve (all problems together). */
int fim_batch_get_stats(const fim_batch *b, fim_stats *out);
/* Stages the batch if needed and runs fim_autotune on it (all problems in
 * one launch, as fim_batch_solve runs them); results are then those of the
 * batch's last timed solve. */
int fim_batch_autotune(fim_batch *b, void *stream, fim_tune_info *info);
/* Warm start of every problem at once: d_phi_init (device, FP64) holds the
 * start times of all problems' vertices in the order they were added (as
 * fim_set_warm_start; the support check runs over the whole batch); NULL
 * restores the cold start.  Stages the batch if needed. */
int fim_batch_set_warm_start(fim_batch *b, const double *d_phi_init);

/* Learned warm start -- no counterpart in the reference.
 * A per-vertex MLP (features -> 128 -> 128 -> 128 -> 1, ReLU; BF16 weights
 * on the tensor cores, FP32 accumulation, FP32 master weights and Adam)
 * predicts activation times; fim_set_warm_start makes the next fim_solve
 * start from given times (every vertex narrow at its start value, stimuli at
 * their start times) and correct them downwards.  Such a solve is NOT
 * bit-identical to the cold solve: the reference's FIM stops above the
 * fixed point of its local solver, and that fixed point is not unique.
 * Feature rows: FIM_MLP_INPUTS BF16 values per vertex, the first 7 used
 * (x, y, z scaled to the bounding box; metric distance to the nearest
 * stimulus over the time scale; cf; ct; fibre angle in the xy-plane / pi).
 * Row counts passed to the network are multiples of 64 (pad with zeros). */
#define FIM_MLP_INPUTS 64
#define FIM_MLP_PARAMS 41473
typedef struct fim_mlp fim_mlp;
int fim_mlp_create(int device, uint64_t seed, fim_mlp **out);
int fim_mlp_destroy(fim_mlp *m);
/* Parameters (FIM_MLP_PARAMS floats: W1 [64x128], W2, W3 [128x128] row-major
 * [in][out], then b1, b2, b3, w4, b4); setting them resets Adam. */
int fim_mlp_set_params(fim_mlp *m, const float *params);
int fim_mlp_get_params(const fim_mlp *m, float *params);
/* Mean-squared-error gradients (host, FIM_MLP_PARAMS floats) and loss of n
 * rows of d_features (device, BF16 [n x FIM_MLP_INPUTS]) against
 * d_targets (device, FP32 [n]). */
int fim_mlp_gradients(fim_mlp *m, int64_t n, const void *d_features, const float *d_targets, float *grads,
                      float *loss);
/* One Adam step on those n rows (learning rate lr); loss before the step. */
int fim_mlp_train_step(fim_mlp *m, int64_t n, const void *d_features, const float *d_targets, float lr,
                       float *loss);
/* Predictions (device, FP32 [n]) for n feature rows. */
int fim_mlp_predict(fim_mlp *m, int64_t n, const void *d_features, float *d_out);
/* Feature rows (device, BF16 [n_vertices x FIM_MLP_INPUTS]) of the solver's
 * mesh, conduction and stimuli (one submesh); *time_scale receives the
 * largest stimulus distance, the unit of the distance feature and of the
 * normalised times the network predicts. */
int fim_features(fim_solver *s, void *d_features, float *time_scale);
/* Start times (device, FP64 [n_vertices], complete before and kept by the
 * caller until the solve) for the next solves; NULL restores the cold start.
 * FIM only lowers times, so a start below the true time of a vertex would
 * stay wrong.  With one endless window every warm-started fim_solve
 * therefore ends with a support check: a reached vertex (not a stimulus)
 * whose time lies below a rigorous lower bound of every candidate its
 * neighbours give -- the reference's edge, triangle and tet updates all
 * return at least their smallest input time plus a distance, and a cold
 * solve never violates this -- marks its time tmin; every time >= tmin
 * (the flagged vertices and everything downwind of them) is reset to INF and
 * FIM resumes from the rest and the stimuli; the check repeats, and after 3
 * rounds that still flag vertices the solve is redone cold.  fim_stats
 * reports the rejected times (warm_reset) and rounds; solve_ms and the
 * counts cover all rounds.  A start only slightly below the truth can pass
 * the check.  A start below the earliest stimulus time can keep the
 * iteration from settling (it then stops at max_iterations). */
int fim_set_warm_start(fim_solver *s, const double *d_phi_init);

/* Reference-compatible files.  fim_vtk_* read/write the legacy ASCII VTK
 * that the reference reads and writes (load_vtk / save_vtk,
 * src/io/vtk.cpp:11-211); fim_read_tags reads a partition file
 * (read_vector_txt, src/io/io_base.h:81-86).  Sizes-first protocol: call
 * with NULL arrays to get the sizes, then with arrays of those sizes. */
int fim_vtk_read(const char *path, int64_t *n_vertices, int64_t *n_tets, double *xyz,
                 int64_t *tets, int32_t *etags);
int fim_vtk_write(const char *path, int64_t n_vertices, int64_t n_tets, const double *xyz,
                  const int64_t *tets, const int32_t *etags, const double *phi,
                  const double *states);
int fim_read_tags(const char *path, int64_t *n, int32_t *tags);

/* Plan + config (load_options / load_plan, src/io/io_json.cpp:228-317):
 * dt and n_steps (the plan's deltatime*1000 and timesteps override the cfg),
 * stimulus vertices of the active events (sizes-first), the first region's
 * CVref speeds (vf, vs, vn) and the first event's start time. */
typedef struct {
  double dt;
  int64_t n_steps;
  int64_t n_events;
  int64_t n_stim_vertices;
  double cv[3];
  double tstart;
  int has_cv;
} fim_plan_info;
int fim_load_plan(const char *cfg_path, const char *plan_path, fim_plan_info *info,
                  int64_t *stim_vertices);

#ifdef __cplusplus
}
#endif
#endif /* FIM_GB300_H_ */
