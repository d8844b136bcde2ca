"""Generates the golden fixtures of tests/golden from the reference itself.

Run in a checkout where the reference tree is present ($FIM_REFERENCE_ROOT,
else ``../reference`` beside the repository) after ``python oracle/build.py`` has compiled the
reference's own host code into oracle/_ref/libfimref.so:

    python tests/golden/make_golden.py [--ref-root DIR]

Outputs (committed, small):
  * ut_mesh.npz  -- the reference's unit mesh (points, tets, element tags),
    its two partition files, the plan's stimulus vertices, dt and steps as
    read by the reference's own load_options/load_plan, and the reference's
    golden solver output data/output/cuda_fim_res.vtk (phi, states).
  * corners.npz  -- local-solver vectors: random corners (geo, target slot,
    neighbour states/times) and update_per_element's result computed by the
    reference's own code.
  * extract.npz  -- per-tet slot order and edge norms from the reference's
    extract_submeshes2 + compute_geo on the unit mesh (both partitions) and
    on a jittered cube with random tags.
  * ut_mesh_written.vtk -- save_vtk's output for the unit mesh with the
    golden phi/states (byte-compatibility fixture for the writer).
"""
import argparse
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cufim-nvlink_gb300"))

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402


def P(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def read_point_data(path, n):
    lines = open(path).read().split("\n")
    i = lines.index("SCALARS phi double 1")
    phi = np.array([float(x) for x in lines[i + 2:i + 2 + n]])
    j = lines.index("SCALARS states double 1")
    st = np.array([float(x) for x in lines[j + 2:j + 2 + n]])
    return phi, st


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=obuild.reference_root())
    a = ap.parse_args()
    obuild.build_ref(a.ref_root)
    R = O.ref_lib()
    assert R is not None, "oracle/_ref/libfimref.so was not built"
    data = os.path.join(a.ref_root, "data")

    # --- unit mesh through the reference's own reader
    path = os.path.join(data, "ut_mesh", "ut_mesh.vtk").encode()
    nV, nT = C.c_int64(), C.c_int64()
    R.ref_load_vtk(path, C.byref(nV), C.byref(nT), None, None, None)
    xyz = np.empty((nV.value, 3))
    tets = np.empty((nT.value, 4), dtype=np.int64)
    et = np.empty(nT.value, dtype=np.int32)
    R.ref_load_vtk(path, C.byref(nV), C.byref(nT), P(xyz, C.c_double), P(tets, C.c_int64), P(et, C.c_int32))
    tags = np.loadtxt(os.path.join(data, "ut_mesh", "ut_mesh.tags"), dtype=np.int32)
    tags_p = np.loadtxt(os.path.join(data, "ut_mesh", "ut_mesh_p.tags"), dtype=np.int32)
    dt = C.c_double()
    ns, nev, nvx = C.c_int64(), C.c_int64(), C.c_int64()
    vtx = np.zeros(64, dtype=np.int64)
    t0 = C.c_double()
    cv = np.zeros(3)
    R.ref_load_plan(os.path.join(data, "default.cfg").encode(),
                    os.path.join(data, "ut_mesh", "ut_mesh.plan.json").encode(),
                    C.byref(dt), C.byref(ns), C.byref(nev), P(vtx, C.c_int64), C.byref(nvx), C.byref(t0),
                    P(cv, C.c_double))
    gphi, gst = read_point_data(os.path.join(data, "output", "cuda_fim_res.vtk"), nV.value)
    np.savez_compressed(os.path.join(HERE, "ut_mesh.npz"), xyz=xyz, tets=tets, etags=et, tags=tags, tags_p=tags_p,
                        stim=vtx[:nvx.value], plan_dt=dt.value, plan_steps=ns.value, plan_events=nev.value,
                        plan_tstart=t0.value, plan_cv=cv, golden_phi=gphi, golden_states=gst,
                        golden_dt=150000.0, golden_steps=3)

    # --- local solver vectors from update_per_element
    rng = np.random.default_rng(20221201)
    pairs = [(0, 1), (0, 2), (1, 2), (0, 3), (1, 3), (2, 3)]
    N = 6000
    geo = np.empty((N, 6))
    tgt = np.empty(N, dtype=np.int32)
    states = np.empty((N, 4), dtype=np.int32)
    phis = np.empty((N, 4))
    res = np.empty(N)
    kuhn = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [1, 1, 1]], float)
    for i in range(N):
        X = kuhn + rng.uniform(-.2, .2, size=(4, 3)) if i % 2 else rng.normal(size=(4, 3))
        A = rng.normal(size=(3, 3))
        M = A @ A.T + 0.1 * np.eye(3)
        g = np.array([(X[p] - X[q]) @ M @ (X[p] - X[q]) for p, q in pairs])
        t = int(rng.integers(4))
        ph = rng.uniform(0, 3, size=4) * 10 ** rng.uniform(-2, 5)
        st = np.where(rng.random(4) < 0.2, 0, 2).astype(np.int32)
        geo[i], tgt[i], states[i], phis[i] = g, t, st, ph
        res[i] = R.ref_update_corner(P(g, C.c_double), t, P(st, C.c_int32), P(ph, C.c_double), 0.0, 1e300)
    adf = (C.c_int64 * 12)()
    bce = (C.c_int64 * 12)()
    phm = (C.c_int64 * 12)()
    R.ref_gray_tables(adf, bce, phm)
    np.savez_compressed(os.path.join(HERE, "corners.npz"), geo=geo, target=tgt, states=states, phi=phis,
                        result=res, adf=np.array(adf[:]), bce=np.array(bce[:]), phimap=np.array(phm[:]))

    # --- extract_submeshes2 + compute_geo
    def extract(xyz_, tets_, tags_):
        n = tets_.shape[0]
        sl = np.empty((n, 4), dtype=np.int64)
        gg = np.empty((n, 6))
        ag = np.empty(n, dtype=np.int32)
        t64 = np.ascontiguousarray(tets_, dtype=np.int64)
        tg = np.ascontiguousarray(tags_, dtype=np.int32)
        R.ref_extract(xyz_.shape[0], n, P(xyz_, C.c_double), P(t64, C.c_int64), P(tg, C.c_int32),
                      P(sl, C.c_int64), P(gg, C.c_double), P(ag, C.c_int32))
        return sl, gg, ag

    import fim_mesh
    cx, ctt = fim_mesh.kuhn_box(5, 4, 3, 1.0, 0.8, 0.6, jitter=0.2, seed=7)
    ctags = rng.integers(0, 6, size=ctt.shape[0]).astype(np.int32)
    out = {}
    for name, (x_, t_, g_) in {"ut": (xyz, tets, tags), "utp": (xyz, tets, tags_p), "cube": (cx, ctt, ctags)}.items():
        sl, gg, ag = extract(x_, t_, g_)
        out[name + "_slots"], out[name + "_geo"], out[name + "_agg"] = sl, gg, ag
    np.savez_compressed(os.path.join(HERE, "extract.npz"), cube_xyz=cx, cube_tets=ctt, cube_tags=ctags, **out)

    # --- the reference's VTK writer
    wpath = os.path.join(HERE, "ut_mesh_written.vtk")
    st_d = gst.astype(np.float64)
    ph = np.where(gphi < 0, O.INF, gphi)
    ts = np.ascontiguousarray(np.sort(tets, axis=1))
    R.ref_save_vtk(wpath.encode(), nV.value, nT.value, P(xyz, C.c_double), P(ts, C.c_int64), P(et, C.c_int32),
                   P(ph, C.c_double), P(st_d, C.c_double))
    print("written to", HERE)


if __name__ == "__main__":
    main()
