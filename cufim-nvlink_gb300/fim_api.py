"""Python front end of the GB300 FIM solver: a ctypes binding of the C ABI in
include/fim.h (libfim_gb300.so, built in-tree by build.py).

This module is glue for tests, benchmarks and scripting; all arithmetic runs
in the library's CUDA kernels.  Loading fails loudly when the library is
missing -- there is no fallback path.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# FIM_GB300_LIB selects another build of the same library (e.g. one compiled
# with per-phase timing instrumentation)
LIB_PATH = os.environ.get("FIM_GB300_LIB") or os.path.join(HERE, "_build", "libfim_gb300.so")
INF = np.finfo(np.float64).max  # the reference's INF (DBL_MAX) for unreached vertices

FIM_OK = 0
STATUS = {0: "FIM_OK", 1: "FIM_ERR_INVALID_ARGUMENT", 2: "FIM_ERR_CUDA", 3: "FIM_ERR_NOT_READY",
          4: "FIM_ERR_TIMEOUT", 5: "FIM_ERR_MAX_ITERATIONS", 6: "FIM_ERR_IO", 7: "FIM_ERR_OUT_OF_MEMORY",
          8: "FIM_ERR_NO_DEVICE"}
FAR, NEIG, NARROW, NEXT, FROZEN, TAIL = range(6)

# every symbol declared in include/fim.h
EXPORTS = ["fim_default_opts", "fim_create", "fim_destroy", "fim_last_error", "fim_set_mesh",
           "fim_set_conduction", "fim_set_conduction_device", "fim_set_stimuli", "fim_solve",
           "fim_get_times", "fim_get_times_device", "fim_get_stats", "fim_vtk_read", "fim_vtk_write",
           "fim_read_tags", "fim_load_plan", "fim_set_stream", "fim_solve_noalloc", "fim_batch_create",
           "fim_batch_destroy", "fim_batch_last_error", "fim_batch_add", "fim_batch_solve", "fim_batch_get_times",
           "fim_batch_get_stats", "fim_mlp_create", "fim_mlp_destroy", "fim_mlp_set_params", "fim_mlp_get_params",
           "fim_mlp_gradients", "fim_mlp_train_step", "fim_mlp_predict", "fim_features", "fim_set_warm_start",
           "fim_autotune", "fim_get_tune", "fim_set_tune", "fim_batch_autotune", "fim_batch_set_warm_start",
           "fim_selftest_screens"]
MLP_INPUTS = 64
MLP_PARAMS = 41473


class FimOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("dt", C.c_double), ("n_steps", C.c_int), ("front_width", C.c_double),
                ("apd", C.c_double), ("max_iterations", C.c_int64), ("timeout_s", C.c_double),
                ("verbose", C.c_int), ("test_withhold_block", C.c_int), ("exact_all", C.c_int),
                ("autotune", C.c_int), ("fp32_update", C.c_int)]


class FimStats(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("vertex_updates", C.c_int64), ("corner_evals", C.c_int64),
                ("exact_evals", C.c_int64), ("solve_ms", C.c_double), ("metric_ms", C.c_double), ("n_corners", C.c_int64),
                ("grid_blocks", C.c_int), ("block_threads", C.c_int), ("batch_slots", C.c_int),
                ("batch_corners", C.c_int), ("dag_warps", C.c_int), ("warm_reset", C.c_int64),
                ("warm_rounds", C.c_int), ("submesh_sweeps", C.c_int), ("graph_launch", C.c_int),
                ("graph_captured", C.c_int)]


class FimTuneInfo(C.Structure):
    _fields_ = [("batch_slots", C.c_int), ("batch_corners", C.c_int), ("grid_blocks", C.c_int),
                ("dag_warps", C.c_int), ("submesh_sweeps", C.c_int), ("default_ms", C.c_double),
                ("tuned_ms", C.c_double), ("candidates", C.c_int)]


class FimPlanInfo(C.Structure):
    _fields_ = [("dt", C.c_double), ("n_steps", C.c_int64), ("n_events", C.c_int64),
                ("n_stim_vertices", C.c_int64), ("cv", C.c_double * 3), ("tstart", C.c_double),
                ("has_cv", C.c_int)]


class FimError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib():
    """Load libfim_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FimError(8, f"{LIB_PATH} not built; run cufim-nvlink_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        P, d, i32, i64, vp = C.POINTER, C.c_double, C.c_int32, C.c_int64, C.c_void_p
        L.fim_default_opts.argtypes = [P(FimOpts)]
        L.fim_default_opts.restype = None
        L.fim_create.argtypes = [P(FimOpts), P(vp)]
        L.fim_destroy.argtypes = [vp]
        L.fim_last_error.argtypes = [vp]
        L.fim_last_error.restype = C.c_char_p
        L.fim_set_mesh.argtypes = [vp, i64, P(d), i64, P(i64), P(i32)]
        L.fim_set_conduction.argtypes = [vp, P(d), P(d), P(d)]
        L.fim_set_conduction_device.argtypes = [vp, vp, vp, vp]
        L.fim_set_stimuli.argtypes = [vp, i64, P(i64), P(d)]
        L.fim_solve.argtypes = [vp, vp]
        L.fim_set_stream.argtypes = [vp, vp]
        L.fim_get_times.argtypes = [vp, P(d), P(i32)]
        L.fim_get_times_device.argtypes = [vp, vp]
        L.fim_get_stats.argtypes = [vp, P(FimStats)]
        L.fim_solve_noalloc.argtypes = [vp, i64, P(i64), P(d), vp, vp]
        L.fim_batch_create.argtypes = [P(FimOpts), P(vp)]
        L.fim_batch_destroy.argtypes = [vp]
        L.fim_batch_last_error.argtypes = [vp]
        L.fim_batch_last_error.restype = C.c_char_p
        L.fim_batch_add.argtypes = [vp, i64, P(d), i64, P(i64), P(d), P(d), P(d), i64, P(i64), P(d), P(i64)]
        L.fim_batch_solve.argtypes = [vp, vp]
        L.fim_batch_get_times.argtypes = [vp, i64, P(d), P(i32)]
        L.fim_batch_get_stats.argtypes = [vp, P(FimStats)]
        f32 = C.c_float
        L.fim_mlp_create.argtypes = [C.c_int, C.c_uint64, P(vp)]
        L.fim_mlp_destroy.argtypes = [vp]
        L.fim_mlp_set_params.argtypes = [vp, P(f32)]
        L.fim_mlp_get_params.argtypes = [vp, P(f32)]
        L.fim_mlp_gradients.argtypes = [vp, i64, vp, vp, P(f32), P(f32)]
        L.fim_mlp_train_step.argtypes = [vp, i64, vp, vp, f32, P(f32)]
        L.fim_mlp_predict.argtypes = [vp, i64, vp, vp]
        L.fim_features.argtypes = [vp, vp, P(f32)]
        L.fim_set_warm_start.argtypes = [vp, vp]
        L.fim_autotune.argtypes = [vp, vp, P(FimTuneInfo)]
        L.fim_get_tune.argtypes = [vp, P(FimTuneInfo)]
        L.fim_set_tune.argtypes = [vp, P(FimTuneInfo)]
        L.fim_batch_autotune.argtypes = [vp, vp, P(FimTuneInfo)]
        L.fim_batch_set_warm_start.argtypes = [vp, vp]
        L.fim_selftest_screens.argtypes = [C.c_int, i64, C.c_uint64, P(i64)]
        L.fim_vtk_read.argtypes = [C.c_char_p, P(i64), P(i64), P(d), P(i64), P(i32)]
        L.fim_vtk_write.argtypes = [C.c_char_p, i64, i64, P(d), P(i64), P(i32), P(d), P(d)]
        L.fim_read_tags.argtypes = [C.c_char_p, P(i64), P(i32)]
        L.fim_load_plan.argtypes = [C.c_char_p, C.c_char_p, P(FimPlanInfo), P(i64)]
        for name in EXPORTS:
            getattr(L, name)
        _lib = L
    return _lib


def selftest_screens(n, seed=1, device=0):
    """The FP32 screens against the FP64 solves on n random corners
    (fim_selftest_screens): a dict of counts, violations included."""
    out = np.zeros(6, dtype=np.int64)
    _check(lib().fim_selftest_screens(device, n, seed, out.ctypes.data_as(C.POINTER(C.c_int64))))
    keys = ["tets", "tet_violations", "tets_with_value", "tris", "tri_violations", "tris_with_value"]
    return {k: int(v) for k, v in zip(keys, out)}


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def _check(rc, handle=None):
    if rc != FIM_OK:
        msg = lib().fim_last_error(handle)
        raise FimError(rc, msg.decode() if msg else "")


def default_opts(**kw):
    o = FimOpts()
    lib().fim_default_opts(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Solver:
    """One GPU solver object (a fim_solver handle)."""

    def __init__(self, **opts):
        self.h = C.c_void_p()
        o = default_opts(**opts)
        _check(lib().fim_create(C.byref(o), C.byref(self.h)))
        self.nV = 0
        self.nT = 0

    def close(self):
        if self.h:
            lib().fim_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_mesh(self, xyz, tets, atags=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        tets = np.ascontiguousarray(tets, dtype=np.int64)
        at = None if atags is None else np.ascontiguousarray(atags, dtype=np.int32)
        self.nV = xyz.shape[0]
        self.nT = tets.shape[0]
        _check(lib().fim_set_mesh(self.h, self.nV, _ptr(xyz, C.c_double), self.nT, _ptr(tets, C.c_int64),
                                  _ptr(at, C.c_int32)), self.h)

    def set_conduction(self, fib, cf, ct):
        fib = np.ascontiguousarray(fib, dtype=np.float64)
        cf = np.ascontiguousarray(cf, dtype=np.float64)
        ct = np.ascontiguousarray(ct, dtype=np.float64)
        _check(lib().fim_set_conduction(self.h, _ptr(fib, C.c_double), _ptr(cf, C.c_double),
                                        _ptr(ct, C.c_double)), self.h)

    def set_conduction_device(self, fib_ptr, cf_ptr, ct_ptr):
        _check(lib().fim_set_conduction_device(self.h, C.c_void_p(fib_ptr), C.c_void_p(cf_ptr),
                                               C.c_void_p(ct_ptr)), self.h)

    def set_stimuli(self, vertices, t0):
        v = np.ascontiguousarray(vertices, dtype=np.int64)
        t = np.ascontiguousarray(t0, dtype=np.float64)
        _check(lib().fim_set_stimuli(self.h, v.shape[0], _ptr(v, C.c_int64), _ptr(t, C.c_double)), self.h)

    def solve(self, stream=None):
        _check(lib().fim_solve(self.h, C.c_void_p(stream) if stream else None), self.h)

    def set_stream(self, stream):
        """Working stream (an integer cudaStream_t, e.g. torch's stream.cuda_stream; 0/None = own)."""
        _check(lib().fim_set_stream(self.h, C.c_void_p(stream) if stream else None), self.h)

    def times(self, with_state=True):
        phi = np.empty(self.nV, dtype=np.float64)
        st = np.empty(self.nV, dtype=np.int32) if with_state else None
        _check(lib().fim_get_times(self.h, _ptr(phi, C.c_double), _ptr(st, C.c_int32)), self.h)
        return (phi, st) if with_state else phi

    def times_device(self, dptr):
        _check(lib().fim_get_times_device(self.h, C.c_void_p(dptr)), self.h)

    def solve_noalloc(self, vertices, t0, d_phi, stream=None):
        """Allocation-free solve for these stimuli into device buffer d_phi (an address of n_vertices f64)."""
        v = np.ascontiguousarray(vertices, dtype=np.int64)
        t = np.ascontiguousarray(t0, dtype=np.float64)
        _check(lib().fim_solve_noalloc(self.h, v.shape[0], _ptr(v, C.c_int64), _ptr(t, C.c_double),
                                       C.c_void_p(d_phi), C.c_void_p(stream) if stream else None), self.h)

    def stats(self):
        s = FimStats()
        _check(lib().fim_get_stats(self.h, C.byref(s)), self.h)
        return {k: getattr(s, k) for k, _ in FimStats._fields_}

    def autotune(self, stream=None):
        """Times candidate launch configurations on the staged problem and keeps the fastest (dict)."""
        t = FimTuneInfo()
        _check(lib().fim_autotune(self.h, C.c_void_p(stream) if stream else None, C.byref(t)), self.h)
        return {k: getattr(t, k) for k, _ in FimTuneInfo._fields_}

    def tune_info(self):
        t = FimTuneInfo()
        _check(lib().fim_get_tune(self.h, C.byref(t)), self.h)
        return {k: getattr(t, k) for k, _ in FimTuneInfo._fields_}

    def set_tune(self, slots=None, corners=None, grid=None, dag_warps=None, submesh_sweeps=None):
        """Pins a launch configuration (all None: back to the default)."""
        if slots is None and corners is None and grid is None and dag_warps is None and submesh_sweeps is None:
            _check(lib().fim_set_tune(self.h, None), self.h)
            return
        cur = self.tune_info()
        t = FimTuneInfo(batch_slots=slots or cur["batch_slots"], batch_corners=corners or cur["batch_corners"],
                        grid_blocks=grid or cur["grid_blocks"], dag_warps=dag_warps or cur["dag_warps"],
                        submesh_sweeps=cur["submesh_sweeps"] if submesh_sweeps is None else int(submesh_sweeps))
        _check(lib().fim_set_tune(self.h, C.byref(t)), self.h)

    def features(self, d_features):
        """Writes the BF16 feature rows [n_vertices x MLP_INPUTS] to device memory; returns the time scale."""
        ts = C.c_float()
        _check(lib().fim_features(self.h, C.c_void_p(d_features), C.byref(ts)), self.h)
        return ts.value

    def set_warm_start(self, d_phi):
        """Device address of FP64 start times [n_vertices] (kept alive by the caller), or None."""
        _check(lib().fim_set_warm_start(self.h, C.c_void_p(d_phi) if d_phi else None), self.h)


class Mlp:
    """The warm-start network (a fim_mlp handle); device buffers are passed as addresses."""

    def __init__(self, device=0, seed=1):
        self.h = C.c_void_p()
        _check(lib().fim_mlp_create(device, seed, C.byref(self.h)))

    def close(self):
        if self.h:
            lib().fim_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def get_params(self):
        p = np.empty(MLP_PARAMS, dtype=np.float32)
        _check(lib().fim_mlp_get_params(self.h, _ptr(p, C.c_float)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (MLP_PARAMS,)
        _check(lib().fim_mlp_set_params(self.h, _ptr(p, C.c_float)))

    def gradients(self, n, d_features, d_targets):
        g = np.empty(MLP_PARAMS, dtype=np.float32)
        loss = C.c_float()
        _check(lib().fim_mlp_gradients(self.h, n, C.c_void_p(d_features), C.c_void_p(d_targets), _ptr(g, C.c_float),
                                       C.byref(loss)))
        return g, loss.value

    def train_step(self, n, d_features, d_targets, lr):
        loss = C.c_float()
        _check(lib().fim_mlp_train_step(self.h, n, C.c_void_p(d_features), C.c_void_p(d_targets), lr, C.byref(loss)))
        return loss.value

    def predict(self, n, d_features, d_out):
        _check(lib().fim_mlp_predict(self.h, n, C.c_void_p(d_features), C.c_void_p(d_out)))


def _bcheck(rc, b):
    if rc != FIM_OK:
        msg = lib().fim_batch_last_error(b)
        raise FimError(rc, msg.decode() if msg else "")


class Batch:
    """Many independent problems solved by one persistent launch (a fim_batch handle)."""

    def __init__(self, **opts):
        self.h = C.c_void_p()
        o = default_opts(**opts)
        _check(lib().fim_batch_create(C.byref(o), C.byref(self.h)))
        self.sizes = []

    def close(self):
        if self.h:
            lib().fim_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add(self, xyz, tets, fib, cf, ct, seed_v, seed_t):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        tets = np.ascontiguousarray(tets, dtype=np.int64)
        fib = np.ascontiguousarray(fib, dtype=np.float64)
        cf = np.ascontiguousarray(cf, dtype=np.float64)
        ct = np.ascontiguousarray(ct, dtype=np.float64)
        sv = np.ascontiguousarray(seed_v, dtype=np.int64)
        st = np.ascontiguousarray(seed_t, dtype=np.float64)
        pid = C.c_int64()
        _bcheck(lib().fim_batch_add(self.h, xyz.shape[0], _ptr(xyz, C.c_double), tets.shape[0], _ptr(tets, C.c_int64),
                                    _ptr(fib, C.c_double), _ptr(cf, C.c_double), _ptr(ct, C.c_double), sv.shape[0],
                                    _ptr(sv, C.c_int64), _ptr(st, C.c_double), C.byref(pid)), self.h)
        self.sizes.append(xyz.shape[0])
        return pid.value

    def solve(self, stream=None):
        _bcheck(lib().fim_batch_solve(self.h, C.c_void_p(stream) if stream else None), self.h)

    def times(self, problem, with_state=True):
        n = self.sizes[problem]
        phi = np.empty(n, dtype=np.float64)
        st = np.empty(n, dtype=np.int32) if with_state else None
        _bcheck(lib().fim_batch_get_times(self.h, problem, _ptr(phi, C.c_double), _ptr(st, C.c_int32)), self.h)
        return (phi, st) if with_state else phi

    def stats(self):
        s = FimStats()
        _bcheck(lib().fim_batch_get_stats(self.h, C.byref(s)), self.h)
        return {k: getattr(s, k) for k, _ in FimStats._fields_}

    def autotune(self, stream=None):
        t = FimTuneInfo()
        _bcheck(lib().fim_batch_autotune(self.h, C.c_void_p(stream) if stream else None, C.byref(t)), self.h)
        return {k: getattr(t, k) for k, _ in FimTuneInfo._fields_}

    def set_warm_start(self, d_phi):
        """Start times of all problems' vertices (device FP64, in add order); None: cold."""
        _bcheck(lib().fim_batch_set_warm_start(self.h, C.c_void_p(d_phi) if d_phi else None), self.h)


def solve_case(case, atags=None, **opts):
    """Convenience: one solve of a case dict (xyz, tets, fib, cf, ct, seed_v, seed_t)."""
    with Solver(**opts) as s:
        s.set_mesh(case["xyz"], case["tets"], atags)
        s.set_conduction(case["fib"], case["cf"], case["ct"])
        s.set_stimuli(case["seed_v"], case["seed_t"])
        s.solve()
        phi, st = s.times()
        return phi, st, s.stats()


# ---------------------------------------------------------------------------
# reference-compatible files

def vtk_read(path):
    nV, nT = C.c_int64(), C.c_int64()
    _check(lib().fim_vtk_read(path.encode(), C.byref(nV), C.byref(nT), None, None, None))
    xyz = np.empty((nV.value, 3), dtype=np.float64)
    tets = np.empty((nT.value, 4), dtype=np.int64)
    et = np.empty(nT.value, dtype=np.int32)
    _check(lib().fim_vtk_read(path.encode(), C.byref(nV), C.byref(nT), _ptr(xyz, C.c_double),
                              _ptr(tets, C.c_int64), _ptr(et, C.c_int32)))
    return xyz, tets, et


def vtk_write(path, xyz, tets, etags=None, phi=None, states=None):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    tets = np.ascontiguousarray(tets, dtype=np.int64)
    et = None if etags is None else np.ascontiguousarray(etags, dtype=np.int32)
    ph = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
    sd = None if states is None else np.ascontiguousarray(states, dtype=np.float64)
    _check(lib().fim_vtk_write(path.encode(), xyz.shape[0], tets.shape[0], _ptr(xyz, C.c_double),
                               _ptr(tets, C.c_int64), _ptr(et, C.c_int32), _ptr(ph, C.c_double),
                               _ptr(sd, C.c_double)))


def read_tags(path):
    n = C.c_int64(0)
    _check(lib().fim_read_tags(path.encode(), C.byref(n), None))
    tags = np.empty(n.value, dtype=np.int32)
    _check(lib().fim_read_tags(path.encode(), C.byref(n), _ptr(tags, C.c_int32)))
    return tags


def load_plan(cfg_path, plan_path):
    info = FimPlanInfo()
    cfg = cfg_path.encode() if cfg_path else None
    _check(lib().fim_load_plan(cfg, plan_path.encode(), C.byref(info), None))
    stim = np.empty(info.n_stim_vertices, dtype=np.int64)
    _check(lib().fim_load_plan(cfg, plan_path.encode(), C.byref(info), _ptr(stim, C.c_int64)))
    return dict(dt=info.dt, n_steps=info.n_steps, n_events=info.n_events, stim=stim,
                cv=tuple(info.cv) if info.has_cv else None, tstart=info.tstart)
