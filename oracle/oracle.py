"""ctypes front end of the oracle (fim_oracle.c) and of the reference's own
host code (oracle/_ref).  TEST INFRASTRUCTURE ONLY: used by tests/, by
``__graft_entry__.smoke`` and by the CPU-baseline leg of bench.py as the
checker, never by the product path."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
INF = np.finfo(np.float64).max  # the reference's INF (DBL_MAX)

ST_FAR, ST_NEIG, ST_NARROW, ST_NEXT, ST_FROZEN, ST_TAIL = range(6)

_lib = None
_ref = None


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def lib():
    global _lib
    if _lib is None:
        from oracle import build as _b  # noqa: F401  (package import when run from repo root)
        path = _b.build_oracle()
        L = C.CDLL(path)
        d, i32, i64 = C.c_double, C.c_int32, C.c_int64
        P = C.POINTER
        L.orc_solve_tri.restype = d
        L.orc_solve_tri.argtypes = [d, d, d, d, d, C.c_int]
        L.orc_solve_tet.restype = d
        L.orc_solve_tet.argtypes = [d] * 9
        L.orc_corner_update.restype = d
        L.orc_corner_update.argtypes = [P(d), C.c_int, P(d), C.c_int]
        L.orc_corner_tables.argtypes = [C.c_int, P(C.c_int), P(C.c_int)]
        L.orc_metric_geo.argtypes = [i64, P(i32), P(d), P(d), P(d), P(d), P(d)]
        L.orc_reference_slots.restype = C.c_int
        L.orc_reference_slots.argtypes = [C.c_int, i64, P(i32), P(i32), P(i32), P(i32), P(i32)]
        L.orc_solve_reference.restype = C.c_long
        L.orc_solve_reference.argtypes = [C.c_int, i64, P(i32), P(i32), P(d), C.c_int, P(i32), P(d),
                                          d, C.c_int, d, d, C.c_int, C.c_int, P(d), P(i32)]
        L.orc_solve_pure.restype = C.c_long
        L.orc_solve_pure.argtypes = [C.c_int, i64, P(i32), P(d), C.c_int, P(i32), P(d), C.c_int,
                                     C.c_int, C.c_long, P(d), P(i32), P(C.c_long)]
        L.orc_fixed_point.restype = C.c_long
        L.orc_fixed_point.argtypes = [C.c_int, i64, P(i32), P(d), C.c_int, P(i32), P(d), C.c_int,
                                      C.c_int, C.c_long, P(d), P(d)]
        L.orc_front_width.restype = d
        L.orc_front_width.argtypes = [i64, P(i32), P(d), d]
        L.orc_support.argtypes = [C.c_int, i64, P(i32), P(d), P(d), P(i32), C.c_int, P(d)]
        L.orc_support.restype = None
        _lib = L
    return _lib


def corner_tables(t):
    sel = (C.c_int * 6)()
    oth = (C.c_int * 3)()
    lib().orc_corner_tables(t, sel, oth)
    return list(sel), list(oth)


def solve_tri(e12, e13, e23, p1, p2, tri_f32=True):
    return lib().orc_solve_tri(e12, e13, e23, p1, p2, int(tri_f32))


def solve_tet(*args):
    return lib().orc_solve_tet(*args)


def corner_update(geo6, t, ph4, tri_f32=True):
    g = np.ascontiguousarray(geo6, dtype=np.float64)
    p = np.ascontiguousarray(ph4, dtype=np.float64)
    return lib().orc_corner_update(_p(g, C.c_double), int(t), _p(p, C.c_double), int(tri_f32))


def reference_slots(nV, tets, atags=None):
    """Per-tet global vertex ids in the reference's slot order, aggregate of
    each tet and its local ids.  Returns (slots [nT,4] int32, agg [nT], local [nT,4], nagg)."""
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    nT = tets.shape[0]
    slots = np.empty((nT, 4), dtype=np.int32)
    agg = np.empty(nT, dtype=np.int32)
    loc = np.empty((nT, 4), dtype=np.int32)
    at = None if atags is None else np.ascontiguousarray(atags, dtype=np.int32)
    na = lib().orc_reference_slots(int(nV), nT, _p(tets, C.c_int32),
                                   None if at is None else _p(at, C.c_int32),
                                   _p(slots, C.c_int32), _p(agg, C.c_int32), _p(loc, C.c_int32))
    return slots, agg, loc, na


def metric_geo(tet_slots, xyz, fib, cf, ct):
    tet_slots = np.ascontiguousarray(tet_slots, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    fib = np.ascontiguousarray(fib, dtype=np.float64)
    cf = np.ascontiguousarray(cf, dtype=np.float64)
    ct = np.ascontiguousarray(ct, dtype=np.float64)
    nT = tet_slots.shape[0]
    geo = np.empty((nT, 6), dtype=np.float64)
    lib().orc_metric_geo(nT, _p(tet_slots, C.c_int32), _p(xyz, C.c_double), _p(fib, C.c_double),
                         _p(cf, C.c_double), _p(ct, C.c_double), _p(geo, C.c_double))
    return geo


def front_width(tets, xyz, speed=0.6):
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    return lib().orc_front_width(tets.shape[0], _p(tets, C.c_int32), _p(xyz, C.c_double), speed)


def solve_reference(nV, tets, atags, geo_slots, seed_v, seed_t, dt, n_steps, fw, apd_us=3e5,
                    tri_f32=True, max_iter=0):
    """Reference-semantics solve (aggregates, time windows, sync). Returns (phi, state, iters)."""
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    at = None if atags is None else np.ascontiguousarray(atags, dtype=np.int32)
    geo = np.ascontiguousarray(geo_slots, dtype=np.float64)
    sv = np.ascontiguousarray(seed_v, dtype=np.int32)
    st = np.ascontiguousarray(seed_t, dtype=np.float64)
    phi = np.empty(nV, dtype=np.float64)
    state = np.empty(nV, dtype=np.int32)
    it = lib().orc_solve_reference(int(nV), tets.shape[0], _p(tets, C.c_int32),
                                   None if at is None else _p(at, C.c_int32), _p(geo, C.c_double),
                                   len(sv), _p(sv, C.c_int32), _p(st, C.c_double), float(dt), int(n_steps),
                                   float(fw), float(apd_us), int(tri_f32), int(max_iter),
                                   _p(phi, C.c_double), _p(state, C.c_int32))
    return phi, state, it


def solve_pure(nV, tet_slots, geo_slots, seed_v, seed_t, tri_f32=True, threads=0, max_iter=0):
    """Single-aggregate, single-window reference FIM with active lists.
    Returns (phi, state, iterations, vertex_updates)."""
    ts = np.ascontiguousarray(tet_slots, dtype=np.int32)
    geo = np.ascontiguousarray(geo_slots, dtype=np.float64)
    sv = np.ascontiguousarray(seed_v, dtype=np.int32)
    st = np.ascontiguousarray(seed_t, dtype=np.float64)
    phi = np.empty(nV, dtype=np.float64)
    state = np.empty(nV, dtype=np.int32)
    upd = C.c_long(0)
    it = lib().orc_solve_pure(int(nV), ts.shape[0], _p(ts, C.c_int32), _p(geo, C.c_double), len(sv),
                              _p(sv, C.c_int32), _p(st, C.c_double), int(tri_f32), int(threads),
                              int(max_iter), _p(phi, C.c_double), _p(state, C.c_int32), C.byref(upd))
    return phi, state, it, upd.value


def fixed_point(nV, tet_slots, geo_slots, seed_v, seed_t, tri_f32=True, threads=0, max_sweeps=0,
                phi_init=None):
    ts = np.ascontiguousarray(tet_slots, dtype=np.int32)
    geo = np.ascontiguousarray(geo_slots, dtype=np.float64)
    sv = np.ascontiguousarray(seed_v, dtype=np.int32)
    st = np.ascontiguousarray(seed_t, dtype=np.float64)
    phi = np.empty(nV, dtype=np.float64)
    pi = None if phi_init is None else np.ascontiguousarray(phi_init, dtype=np.float64)
    sw = lib().orc_fixed_point(int(nV), ts.shape[0], _p(ts, C.c_int32), _p(geo, C.c_double), len(sv),
                               _p(sv, C.c_int32), _p(st, C.c_double), int(tri_f32), int(threads),
                               int(max_sweeps), None if pi is None else _p(pi, C.c_double),
                               _p(phi, C.c_double))
    return phi, sw


# ---------------------------------------------------------------------------
# the reference's own host code (present only where the reference tree was)
def ref_lib():
    """Load oracle/_ref/libfimref.so, or return None when it was not built."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libfimref.so")
        if not os.path.exists(path):
            return None
        L = C.CDLL(path)
        d, i32, i64 = C.c_double, C.c_int32, C.c_int64
        P = C.POINTER
        L.ref_solve_tri.restype = d
        L.ref_solve_tri.argtypes = [d] * 5
        L.ref_solve_tet.restype = d
        L.ref_solve_tet.argtypes = [d] * 9
        L.ref_gray_tables.argtypes = [P(i64), P(i64), P(i64)]
        L.ref_update_corner.restype = d
        L.ref_update_corner.argtypes = [P(d), C.c_int, P(i32), P(d), d, d]
        L.ref_extract.restype = C.c_int
        L.ref_extract.argtypes = [i64, i64, P(d), P(i64), P(i32), P(i64), P(d), P(i32)]
        L.ref_load_vtk.restype = C.c_int
        L.ref_load_vtk.argtypes = [C.c_char_p, P(i64), P(i64), P(d), P(i64), P(i32)]
        L.ref_save_vtk.restype = C.c_int
        L.ref_save_vtk.argtypes = [C.c_char_p, i64, i64, P(d), P(i64), P(i32), P(d), P(d)]
        L.ref_load_plan.restype = C.c_int
        L.ref_load_plan.argtypes = [C.c_char_p, C.c_char_p, P(d), P(i64), P(i64), P(i64), P(i64), P(d), P(d)]
        _ref = L
    return _ref


def support(nV, tet_slots, geo_slots, phi, state, tri_f32=True):
    """Per vertex, the minimum local update from its neighbours' final times
    (orc_support): a reached time below it is unsupported."""
    ts = np.ascontiguousarray(tet_slots, dtype=np.int32)
    g = np.ascontiguousarray(geo_slots, dtype=np.float64)
    ph = np.ascontiguousarray(phi, dtype=np.float64)
    st = np.ascontiguousarray(state, dtype=np.int32)
    U = np.empty(nV)
    lib().orc_support(nV, ts.shape[0], _p(ts, C.c_int32), _p(g, C.c_double), _p(ph, C.c_double),
                      _p(st, C.c_int32), 1 if tri_f32 else 0, _p(U, C.c_double))
    return U
