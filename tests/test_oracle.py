"""The oracle (oracle/fim_oracle.c) against the reference's own outputs:
local-solver vectors, slot order + edge norms, the gray-code identity and
the golden solver output on the reference's unit mesh.  CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def test_corner_tables_match_reference(O):
    z = np.load(os.path.join(GOLDEN, "corners.npz"))
    for t in range(4):
        sel, oth = O.corner_tables(t)
        assert sel[:3] == list(z["adf"][3 * t:3 * t + 3])
        assert sel[3:] == list(z["bce"][3 * t:3 * t + 3])
        assert oth == list(z["phimap"][3 * t:3 * t + 3])


def test_corner_update_bit_exact(O):
    """update_per_element of the reference vs the restatement, incl. invalid neighbours."""
    z = np.load(os.path.join(GOLDEN, "corners.npz"))
    bad = 0
    for g, t, st, ph, r in zip(z["geo"], z["target"], z["states"], z["phi"], z["result"]):
        p = np.where(st >= O.ST_NARROW, ph, O.INF)
        o = O.corner_update(g, int(t), p, True)
        if not (o == r or (np.isnan(o) and np.isnan(r))):
            bad += 1
    assert bad == 0


def test_corner_update_live_reference(O):
    """Same on fresh random corners when the reference's code was compiled here."""
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference tree not present: oracle/_ref not built")
    import ctypes as C
    rng = np.random.default_rng(11)
    pairs = [(0, 1), (0, 2), (1, 2), (0, 3), (1, 3), (2, 3)]
    for _ in range(3000):
        X = rng.normal(size=(4, 3))
        A = rng.normal(size=(3, 3))
        M = A @ A.T + 0.05 * np.eye(3)
        g = np.array([(X[a] - X[b]) @ M @ (X[a] - X[b]) for a, b in pairs])
        t = int(rng.integers(4))
        ph = rng.uniform(0, 5, size=4)
        st = np.where(rng.random(4) < 0.25, 0, 4).astype(np.int32)
        r = R.ref_update_corner(g.ctypes.data_as(C.POINTER(C.c_double)), t,
                                st.ctypes.data_as(C.POINTER(C.c_int32)),
                                ph.ctypes.data_as(C.POINTER(C.c_double)), 0.0, 1e300)
        o = O.corner_update(g, t, np.where(st >= O.ST_NARROW, ph, O.INF), True)
        assert o == r or (np.isnan(o) and np.isnan(r))


@pytest.mark.parametrize("name", ["ut", "utp", "cube"])
def test_slots_and_metric_match_reference(O, name):
    ex = np.load(os.path.join(GOLDEN, "extract.npz"))
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    if name == "cube":
        xyz, tets, tags = ex["cube_xyz"], ex["cube_tets"], ex["cube_tags"]
    else:
        xyz, tets = ut["xyz"], ut["tets"]
        tags = ut["tags"] if name == "ut" else ut["tags_p"]
    slots, agg, _, _ = O.reference_slots(xyz.shape[0], tets, tags)
    assert np.array_equal(slots, ex[name + "_slots"])
    assert np.array_equal(agg, ex[name + "_agg"])
    nT = tets.shape[0]
    geo = O.metric_geo(slots, xyz, np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.6), np.full(nT, 0.6))
    assert np.array_equal(geo, ex[name + "_geo"])  # bit-exact


def test_gray_code_identity(O):
    """Known-answer test of the reference (test_gray_code, cuda_fim.cu:2595-2681),
    restated over every tet and target: the six tet coefficients from the
    gray-code mapping equal the direct e_i^T M e_j products."""
    import fim_mesh
    xyz, tets = fim_mesh.kuhn_box(4, 3, 3, jitter=0.2, seed=3)
    nT = tets.shape[0]
    rng = np.random.default_rng(4)
    f = rng.normal(size=(nT, 3))
    f /= np.linalg.norm(f, axis=1, keepdims=True)
    cf, ct = np.full(nT, 0.6), np.full(nT, 0.25)
    slots, _, _, _ = O.reference_slots(xyz.shape[0], tets, None)
    geo = O.metric_geo(slots, xyz, f, cf, ct)
    err = 0.0
    for e in range(nT):
        M = (1 / cf[e] ** 2) * np.outer(f[e], f[e]) + (1 / ct[e] ** 2) * (np.eye(3) - np.outer(f[e], f[e]))
        for t in range(4):
            sel, oth = O.corner_tables(t)
            x = xyz[slots[e]]
            x1, x2, x3, x4 = x[oth[0]], x[oth[1]], x[oth[2]], x[t]
            e13, e23, e34 = x3 - x1, x3 - x2, x4 - x3
            reg = [e13 @ M @ e13, e23 @ M @ e13, e34 @ M @ e13, e23 @ M @ e23, e34 @ M @ e23, e34 @ M @ e34]
            g = geo[e][sel]
            gray = [g[0], 0.5 * (g[1] + g[0] - g[3]), -0.5 * (g[2] + g[0] - g[4]), g[1],
                    -0.5 * (g[2] + g[1] - g[5]), g[2]]
            err = max(err, float(np.max(np.abs(np.array(gray) - np.array(reg)))))
    assert err < 1e-9


def _ut_setup(O, tag_key):
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    xyz, tets = ut["xyz"], np.sort(ut["tets"], axis=1)
    tags = ut[tag_key]
    nV, nT = xyz.shape[0], tets.shape[0]
    slots, _, _, _ = O.reference_slots(nV, tets, tags)
    geo = O.metric_geo(slots, xyz, np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.6), np.full(nT, 0.6))
    fw = O.front_width(tets.astype(np.int32), xyz)
    return ut, xyz, tets, tags, geo, fw


def test_golden_unit_mesh(O):
    """The reference's committed solver output (data/output/cuda_fim_res.vtk:
    4 submeshes, dt = 150000 us, 3 windows) is reproduced exactly."""
    ut, xyz, tets, tags, geo, fw = _ut_setup(O, "tags")
    stim = ut["stim"]
    phi, st, _ = O.solve_reference(xyz.shape[0], tets, tags, geo, stim, np.zeros(len(stim)),
                                   float(ut["golden_dt"]), int(ut["golden_steps"]), fw)
    written = np.round(np.where(phi < 1e50, phi, -1.0), 6)  # save_vtk prints %lf, INF as -1
    assert np.array_equal(written, ut["golden_phi"])
    assert np.array_equal(st, ut["golden_states"].astype(np.int32))
    # straight-edge exactness: 180000 um / 0.6 um/us
    assert abs(phi[0] - 300000.0) < 1e-6 and abs(phi[1] - 300000.0) < 1e-6


def test_plan_values(O):
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    assert float(ut["plan_dt"]) == 150000.0 and int(ut["plan_steps"]) == 4
    assert sorted(ut["stim"].tolist()) == [4, 5, 8, 9, 48, 49, 50, 51, 52, 53, 130]


@pytest.mark.parametrize("n", [4, 7, 10])
def test_active_list_fim_equals_reference_phases(O, n):
    """The active-list FIM (CPU baseline, large oracle runs) is the
    reference's compute_step with one submesh and one endless window."""
    import fim_mesh
    c = fim_mesh.cube_case(n)
    nV = c["xyz"].shape[0]
    slots, _, _, _ = O.reference_slots(nV, c["tets"], None)
    geo = O.metric_geo(slots, c["xyz"], c["fib"], c["cf"], c["ct"])
    p1, s1, _ = O.solve_reference(nV, c["tets"], None, geo, c["seed_v"], c["seed_t"], 1e300, 1, 1e300)
    p2, s2, _, _ = O.solve_pure(nV, slots, geo, c["seed_v"], c["seed_t"])
    assert np.array_equal(p1, p2) and np.array_equal(s1, s2)


def test_planar_front_known_answer(O):
    """Unjittered Kuhn box, isotropic speed, whole x = 0 face stimulated at
    t = 0: every vertex gets x / v (reached along x-edges)."""
    import fim_mesh
    xyz, tets = fim_mesh.kuhn_box(8, 3, 3, 8.0, 3.0, 3.0, jitter=0.0)
    nV, nT = xyz.shape[0], tets.shape[0]
    slots, _, _, _ = O.reference_slots(nV, tets, None)
    geo = O.metric_geo(slots, xyz, np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.5), np.full(nT, 0.5))
    seeds = np.nonzero(xyz[:, 0] == 0.0)[0]
    phi, _, _, _ = O.solve_pure(nV, slots, geo, seeds, np.zeros(len(seeds)))
    assert np.allclose(phi, xyz[:, 0] / 0.5, rtol=1e-6, atol=1e-9)


def test_mlp_oracle_gradients_finite_differences():
    """The network restatement's backward pass (FP64, no BF16 roundings)
    against central finite differences of its loss."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(4)
    n = 32
    p = np.zeros(M.NPARAMS)
    p[M.OW1:M.OW1 + 7 * M.H] = rng.normal(0, 0.5, 7 * M.H)
    p[M.OW2:M.OB1] = rng.normal(0, 0.12, 2 * M.H * M.H)
    p[M.OB1:M.OW4] = rng.normal(0, 0.05, 3 * M.H)
    p[M.OW4:M.OB4] = rng.normal(0, 0.1, M.H)
    X = np.zeros((n, M.IN))
    X[:, :7] = rng.normal(0, 1, (n, 7))
    t = rng.normal(0, 1, n)
    _, g = M.loss_and_gradients(p, X, t, exact=True)
    idx = np.concatenate([rng.choice(np.arange(a, b), size=min(6, b - a), replace=False)
                          for name, (a, b) in M.BLOCKS.items() if name != "W1"] +
                         [rng.choice(np.arange(M.OW1, M.OW1 + 7 * M.H), size=6, replace=False)])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.loss_and_gradients(pp, X, t, exact=True)[0] - M.loss_and_gradients(pm, X, t, exact=True)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


def test_high_valence_active_list_equals_reference_phases(O):
    """The active-list oracle and the phase-by-phase restatement agree on a
    vertex with thousands of incident tets (the neighbourhood lists of both
    grow with the valence; no fixed-size gather)."""
    pytest.importorskip("scipy")
    from scipy.spatial import ConvexHull
    rng = np.random.default_rng(3)
    p = rng.normal(size=(3000, 3))
    p /= np.linalg.norm(p, axis=1)[:, None]
    hull = ConvexHull(p)
    xyz = np.vstack([[[0.0, 0.0, 0.0]], p * rng.uniform(0.9, 1.1, (len(p), 1))])
    tets = np.hstack([np.zeros((len(hull.simplices), 1), dtype=np.int64), hull.simplices + 1])
    nT, nV = tets.shape[0], xyz.shape[0]
    ang = rng.uniform(0, np.pi, nT)
    fib = np.stack([np.cos(ang), np.sin(ang), np.zeros(nT)], axis=1)
    slots, _, _, _ = O.reference_slots(nV, tets, None)
    geo = O.metric_geo(slots, xyz, fib, np.full(nT, 0.6), np.full(nT, 0.25))
    sv, st0 = np.array([1, 2, 3]), np.array([0.0, 0.5, 1.0])
    phi, st, it, _ = O.solve_pure(nV, slots, geo, sv, st0)
    fw = O.front_width(tets, xyz)
    phi_r, st_r, it_r = O.solve_reference(nV, tets, None, geo, sv, st0, float("inf"), 1, fw, apd_us=-1.0)
    assert np.array_equal(phi, phi_r) and np.array_equal(st, st_r) and it == it_r
