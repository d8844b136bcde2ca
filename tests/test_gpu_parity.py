"""GPU solver vs the oracle, through the C ABI.  The solver reproduces the
reference's FP64 source semantics, so every comparison here is bit-exact
(times and states), at sizes the oracle finishes in seconds."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F(built_library):
    import fim_api
    return fim_api


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def oracle_single(O, case, tri_f32=True):
    nV = case["xyz"].shape[0]
    slots, _, _, _ = O.reference_slots(nV, case["tets"], None)
    geo = O.metric_geo(slots, case["xyz"], case["fib"], case["cf"], case["ct"])
    phi, st, it, upd = O.solve_pure(nV, slots, geo, case["seed_v"], case["seed_t"], tri_f32=tri_f32)
    return phi, st, it, upd


def assert_identical(phi_g, st_g, phi_o, st_o):
    diff = np.nonzero(phi_g != phi_o)[0]
    assert diff.size == 0, f"{diff.size} times differ, first {diff[:5]}: {phi_g[diff[:5]]} vs {phi_o[diff[:5]]}"
    assert np.array_equal(st_g, st_o)


@pytest.mark.parametrize("n", [3, 6, 12, 20])
def test_unit_cube_bit_exact(F, O, n):
    """The plain FIM configuration (unit cube, n^3 x 6 Kuhn tets, +-0.2h jitter,
    isotropic 0.6, stimulus at the origin); n = 20 is the 9,261-vertex case."""
    import fim_mesh
    c = fim_mesh.cube_case(n)
    phi, st, stats = F.solve_case(c)
    phi_o, st_o, it_o, upd_o = oracle_single(O, c)
    assert_identical(phi, st, phi_o, st_o)
    assert stats["iterations"] == it_o and stats["vertex_updates"] == upd_o


def test_anisotropic_slab_bit_exact(F, O):
    """Scaled-down anisotropic slab: rotating fibres, cf/ct, slow scar, 5
    surface stimuli with t0 in [0, 10]."""
    import fim_mesh
    c = fim_mesh.slab_case(cells=(40, 14, 6), size=(20.0, 7.0, 3.0), seed=5)
    phi, st, stats = F.solve_case(c)
    phi_o, st_o, it_o, _ = oracle_single(O, c)
    assert_identical(phi, st, phi_o, st_o)
    assert stats["iterations"] == it_o


def test_warm_start_bit_exact(F, O):
    """fim_set_warm_start: every vertex starts narrow at its given time (here
    1.05 x the cold result; unreached vertices stay far).  The oracle runs the
    same FIM seeded with every vertex at its start time, the stimuli after
    them so that their own times win, as they do on the GPU."""
    import fim_mesh
    torch = pytest.importorskip("torch")
    c = fim_mesh.slab_case(cells=(40, 14, 6), size=(20.0, 7.0, 3.0), seed=5)
    nV = c["xyz"].shape[0]
    cold, _, _ = F.solve_case(c)
    start = np.where(cold < F.INF, 1.05 * cold, F.INF)
    d_start = torch.from_numpy(start).cuda()
    torch.cuda.synchronize()
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        s.set_warm_start(d_start.data_ptr())
        s.solve()
        phi, st = s.times()
        it = s.stats()["iterations"]
        assert s.stats()["warm_reset"] == 0 and s.stats()["warm_rounds"] == 0  # an upper bound passes the check
    slots, _, _, _ = O.reference_slots(nV, c["tets"], None)
    geo = O.metric_geo(slots, c["xyz"], c["fib"], c["cf"], c["ct"])
    sv = np.concatenate([np.arange(nV), c["seed_v"]])
    st0 = np.concatenate([start, c["seed_t"]])
    keep = st0 < F.INF
    phi_o, st_o, it_o, _ = O.solve_pure(nV, slots, geo, sv[keep], st0[keep])
    assert_identical(phi, st, phi_o, st_o)
    assert it == it_o


@pytest.mark.parametrize("scale", [0.5, 0.9])
def test_warm_start_below_truth_is_reset(F, O, scale):
    """The truth a warm start approaches from above is the fixed point of the
    local solver (the oracle's fixed_point; the reference's cold FIM stops
    above it, here by up to 18 % of max(t)).  A start at scale x that fixed
    point in the middle third of the slab (1.05 x elsewhere) must trip the
    support check; a gross underestimate (0.5) must end within 1e-2 max(t) of
    the fixed point, and no start may end further below it than it began."""
    import fim_mesh
    torch = pytest.importorskip("torch")
    c = fim_mesh.slab_case(cells=(40, 14, 6), size=(20.0, 7.0, 3.0), seed=5)
    nV = c["xyz"].shape[0]
    cold, _, _ = F.solve_case(c)
    slots, _, _, _ = O.reference_slots(nV, c["tets"], None)
    geo = O.metric_geo(slots, c["xyz"], c["fib"], c["cf"], c["ct"])
    fp, _ = O.fixed_point(nV, slots, geo, c["seed_v"], c["seed_t"])
    x = c["xyz"][:, 0]
    mid = (x > 20.0 / 3) & (x < 40.0 / 3)
    reached = cold < F.INF
    start = np.where(reached, np.where(mid, scale, 1.05) * fp, F.INF)
    d_start = torch.from_numpy(start).cuda()
    torch.cuda.synchronize()
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        s.set_warm_start(d_start.data_ptr())
        s.solve()
        phi, _ = s.times()
        stt = s.stats()
        s.set_warm_start(None)
        s.solve()
        again, _ = s.times()
    assert np.array_equal(again, cold)  # the cold start is back
    assert stt["warm_reset"] > 0 and stt["warm_rounds"] >= 1
    assert np.array_equal(phi < F.INF, reached)
    tmax = cold[reached].max()
    below_start = max(0.0, np.max((fp - start)[reached]) / tmax)
    below_end = np.max((fp - phi)[reached]) / tmax
    assert below_end <= below_start + 1e-3, (below_start, below_end)
    if scale <= 0.5:
        assert below_end < 1e-2, f"a time ends {below_end:.3g} x max(t) below the fixed point"


def _ut(O, tag_key):
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    xyz, tets = ut["xyz"], np.sort(ut["tets"], axis=1)
    return ut, xyz, tets, ut[tag_key]


def test_unit_mesh_golden(F, O):
    """The reference's golden output (4 submeshes, 3 windows of 150000 us, APD reset)."""
    ut, xyz, tets, tags = _ut(O, "tags")
    nT = tets.shape[0]
    with F.Solver(dt=float(ut["golden_dt"]), n_steps=int(ut["golden_steps"]), apd=3e5) as s:
        s.set_mesh(xyz, tets, tags)
        s.set_conduction(np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.6), np.full(nT, 0.6))
        s.set_stimuli(ut["stim"], np.zeros(len(ut["stim"])))
        s.solve()
        phi, st = s.times()
    written = np.round(np.where(phi < 1e50, phi, -1.0), 6)
    assert np.array_equal(written, ut["golden_phi"])
    assert np.array_equal(st, ut["golden_states"].astype(np.int32))


@pytest.mark.parametrize("tag_key,steps", [("tags", 4), ("tags_p", 3), ("tags_p", 5)])
def test_unit_mesh_windows_bit_exact(F, O, tag_key, steps):
    ut, xyz, tets, tags = _ut(O, tag_key)
    nV, nT = xyz.shape[0], tets.shape[0]
    slots, _, _, _ = O.reference_slots(nV, tets, tags)
    geo = O.metric_geo(slots, xyz, np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.6), np.full(nT, 0.6))
    fw = O.front_width(tets.astype(np.int32), xyz)
    phi_o, st_o, _ = O.solve_reference(nV, tets, tags, geo, ut["stim"], np.zeros(len(ut["stim"])),
                                       150000.0, steps, fw)
    with F.Solver(dt=150000.0, n_steps=steps, apd=3e5) as s:
        s.set_mesh(xyz, tets, tags)
        s.set_conduction(np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.6), np.full(nT, 0.6))
        s.set_stimuli(ut["stim"], np.zeros(len(ut["stim"])))
        s.solve()
        phi, st = s.times()
    assert_identical(phi, st, phi_o, st_o)


def test_random_submeshes_windows_bit_exact(F, O):
    """Jittered box, 7 random submeshes, anisotropic, windows + APD reset."""
    import fim_mesh
    xyz, tets = fim_mesh.kuhn_box(9, 7, 5, 4.5, 3.5, 2.5, jitter=0.2, seed=9)
    nV, nT = xyz.shape[0], tets.shape[0]
    rng = np.random.default_rng(2)
    tags = rng.integers(0, 7, size=nT).astype(np.int32)
    fib = fim_mesh.fibre_rotation(fim_mesh.tet_centroids(xyz, tets)[:, 2], 0, 2.5, -60, 60)
    cf, ct = np.full(nT, 0.6), np.full(nT, 0.3)
    sv = np.array([0, 17, 200], dtype=np.int32)
    st0 = np.array([0.0, 1.0, 2.5])
    slots, _, _, _ = O.reference_slots(nV, tets, tags)
    geo = O.metric_geo(slots, xyz, fib, cf, ct)
    dt, steps, apd = 3.0, 6, 8.0
    fw = O.front_width(tets, xyz)
    phi_o, st_o, _ = O.solve_reference(nV, tets, tags, geo, sv, st0, dt, steps, fw, apd_us=apd)
    with F.Solver(dt=dt, n_steps=steps, apd=apd) as s:
        s.set_mesh(xyz, tets, tags)
        s.set_conduction(fib, cf, ct)
        s.set_stimuli(sv, st0)
        s.solve()
        phi, st = s.times()
    assert_identical(phi, st, phi_o, st_o)


def test_single_submesh_windows_bit_exact(F, O):
    import fim_mesh
    c = fim_mesh.cube_case(8)
    nV, nT = c["xyz"].shape[0], c["tets"].shape[0]
    slots, _, _, _ = O.reference_slots(nV, c["tets"], None)
    geo = O.metric_geo(slots, c["xyz"], c["fib"], c["cf"], c["ct"])
    fw = O.front_width(c["tets"], c["xyz"])
    phi_o, st_o, _ = O.solve_reference(nV, c["tets"], None, geo, c["seed_v"], c["seed_t"], 0.5, 5, fw, apd_us=1.0)
    with F.Solver(dt=0.5, n_steps=5, apd=1.0) as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        s.solve()
        phi, st = s.times()
    assert_identical(phi, st, phi_o, st_o)


def test_edge_cases(F, O):
    import fim_mesh
    c = fim_mesh.cube_case(3)
    nV = c["xyz"].shape[0]
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        # no stimuli: nothing is reached
        s.set_stimuli(np.zeros(0, dtype=np.int64), np.zeros(0))
        s.solve()
        phi, st = s.times()
        assert np.all(phi == F.INF) and np.all(st == F.FAR)
        # duplicate stimuli: the earliest start time wins
        s.set_stimuli([5, 5, 0], [2.0, 1.0, 0.0])
        s.solve()
        phi, _ = s.times()
        assert phi[5] <= 1.0 and phi[0] == 0.0
        # every vertex stimulated
        s.set_stimuli(np.arange(nV), np.zeros(nV))
        s.solve()
        phi, st = s.times()
        assert np.all(phi == 0.0) and np.all(st == F.FROZEN)
        for bad in ([nV], [-1]):
            with pytest.raises(F.FimError) as e:
                s.set_stimuli(bad, [0.0])
            assert e.value.code == 1
        with pytest.raises(F.FimError):
            s.set_conduction(c["fib"], np.zeros(len(c["cf"])), c["ct"])
    with F.Solver() as s:
        with pytest.raises(F.FimError) as e:
            s.solve()
        assert e.value.code == 3
        with pytest.raises(F.FimError):
            s.set_mesh(c["xyz"], np.array([[0, 1, 2, 2]]))
        with pytest.raises(F.FimError):
            s.set_mesh(c["xyz"], np.array([[0, 1, 2, nV]]))
    # one tet, one stimulus
    xyz = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    case = dict(xyz=xyz, tets=np.array([[0, 1, 2, 3]]), fib=np.array([[1.0, 0, 0]]), cf=np.array([0.5]),
                ct=np.array([0.5]), seed_v=np.array([0]), seed_t=np.array([0.0]))
    phi, st, _ = F.solve_case(case)
    assert np.allclose(phi, [0.0, 2.0, 2.0, 2.0])
    # an isolated vertex (no tet) is never seeded or reached, like the reference
    xyz2 = np.vstack([xyz, [[5.0, 5, 5]]])
    case2 = dict(case, xyz=xyz2, seed_v=np.array([0, 4]), seed_t=np.array([0.0, 0.0]))
    phi, st, _ = F.solve_case(case2)
    assert phi[4] == F.INF and st[4] == F.FAR


def test_bounded_wait_reports_timeout(F, O):
    """A block that never arrives at the grid barrier makes the others' waits
    expire: the solve returns FIM_ERR_TIMEOUT and the context stays usable."""
    import fim_mesh
    c = fim_mesh.cube_case(6)
    with F.Solver(timeout_s=0.5, test_withhold_block=1) as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        with pytest.raises(F.FimError) as e:
            s.solve()
        assert e.value.code == 4
    phi, st, _ = F.solve_case(c)
    phi_o, st_o, _, _ = oracle_single(O, c)
    assert_identical(phi, st, phi_o, st_o)


def test_iteration_cap(F):
    import fim_mesh
    c = fim_mesh.cube_case(6)
    with pytest.raises(F.FimError) as e:
        F.solve_case(c, max_iterations=2)
    assert e.value.code == 5


def test_device_resident_inputs_and_outputs(F, O):
    """fim_set_conduction_device / fim_get_times_device with torch tensors."""
    import torch
    import fim_mesh
    c = fim_mesh.cube_case(5)
    dev = torch.device("cuda:0")
    fib = torch.tensor(c["fib"], dtype=torch.float64, device=dev).contiguous()
    cf = torch.tensor(c["cf"], dtype=torch.float64, device=dev)
    ct = torch.tensor(c["ct"], dtype=torch.float64, device=dev)
    out = torch.empty(c["xyz"].shape[0], dtype=torch.float64, device=dev)
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction_device(fib.data_ptr(), cf.data_ptr(), ct.data_ptr())
        s.set_stimuli(c["seed_v"], c["seed_t"])
        s.solve()
        s.times_device(out.data_ptr())
    torch.cuda.synchronize()
    phi_o, _, _, _ = oracle_single(O, c)
    assert np.array_equal(out.cpu().numpy(), phi_o)


@pytest.mark.parametrize("exact_all", [0, 1])
def test_filtered_and_exact_paths_agree(F, O, exact_all):
    """The interval-screened path and the all-FP64 path both equal the oracle."""
    import fim_mesh
    c = fim_mesh.slab_case(cells=(30, 12, 6), size=(20.0, 7.0, 3.0), seed=8)
    phi, st, stats = F.solve_case(c, exact_all=exact_all)
    phi_o, st_o, _, _ = oracle_single(O, c)
    assert_identical(phi, st, phi_o, st_o)
    if exact_all:
        assert stats["exact_evals"] > 0


@pytest.mark.parametrize("scale", [1e-3, 1.0, 1e3, 1e5])
def test_unit_scales_bit_exact(F, O, scale):
    """The reference's tet solve is not scale invariant; the filters must
    stay exact in mm, um and larger units (the reference's files are um)."""
    import fim_mesh
    c = fim_mesh.slab_case(cells=(16, 8, 5), size=(4.0, 2.0, 1.25), scar_radius=0.5, seed=10)
    c = dict(c, xyz=c["xyz"] * scale, seed_t=c["seed_t"] * scale)
    phi, st, _ = F.solve_case(c)
    phi_o, st_o, _, _ = oracle_single(O, c)
    assert_identical(phi, st, phi_o, st_o)


def test_random_metrics_bit_exact(F, O):
    """Strongly anisotropic random fibres and speeds per tet."""
    import fim_mesh
    xyz, tets = fim_mesh.kuhn_box(14, 10, 8, 3.5, 2.5, 2.0, jitter=0.25, seed=21)
    nT = tets.shape[0]
    rng = np.random.default_rng(5)
    f = rng.normal(size=(nT, 3))
    f /= np.linalg.norm(f, axis=1, keepdims=True)
    cf = rng.uniform(0.2, 1.5, nT)
    ct = cf * rng.uniform(0.1, 1.0, nT)
    c = dict(xyz=xyz, tets=tets, fib=f, cf=cf, ct=ct, seed_v=np.array([0, 500, 1000]),
             seed_t=np.array([0.0, 0.3, 0.1]))
    phi, st, _ = F.solve_case(c)
    phi_o, st_o, _, _ = oracle_single(O, c)
    assert_identical(phi, st, phi_o, st_o)


def test_shell_bit_exact(F, O):
    """Scaled-down ventricle-like shell: curved wall, periodic seam, a hole
    at the apex, transmural fibre rotation, 8 endocardial stimuli."""
    import fim_mesh
    c = fim_mesh.shell_case(n_wall=4, n_circ=48, n_long=24)
    phi, st, stats = F.solve_case(c)
    phi_o, st_o, it_o, _ = oracle_single(O, c)
    assert_identical(phi, st, phi_o, st_o)
    assert stats["iterations"] == it_o


def _pincushion(n_sphere, seed):
    """A centre vertex joined to every face of a triangulated sphere around
    it: the centre has 2 n_sphere - 4 incident tets (more than one batch of
    the solve kernel holds), the sphere vertices a handful each."""
    from scipy.spatial import ConvexHull
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(n_sphere, 3))
    p /= np.linalg.norm(p, axis=1)[:, None]
    hull = ConvexHull(p)
    xyz = np.vstack([[[0.0, 0.0, 0.0]], p * rng.uniform(0.9, 1.1, (n_sphere, 1))])
    tets = np.hstack([np.zeros((len(hull.simplices), 1), dtype=np.int64), hull.simplices + 1])
    nT = tets.shape[0]
    ang = rng.uniform(0, np.pi, nT)
    fib = np.stack([np.cos(ang), np.sin(ang), np.zeros(nT)], axis=1)
    return dict(xyz=xyz, tets=tets, fib=fib, cf=np.full(nT, 0.6), ct=np.full(nT, 0.25),
                seed_v=np.array([1, 2, 3]), seed_t=np.array([0.0, 0.5, 1.0]))


@pytest.mark.parametrize("n_sphere", [1400, 1600, 3000])
def test_high_valence_vertex_bit_exact(F, O, n_sphere):
    """A vertex with 2,796 tets around it fills most of a batch (3,072
    corners) on its own; one with 3,196 or 5,996 has more corners than a
    batch holds and goes through the all-FP64 path for the excess; the
    result is still the oracle's, bit for bit, screened or not."""
    pytest.importorskip("scipy")
    c = _pincushion(n_sphere, 3)
    phi_o, st_o, it_o, _ = oracle_single(O, c)
    for exact_all in (0, 1):
        phi, st, stats = F.solve_case(c, exact_all=exact_all)
        assert_identical(phi, st, phi_o, st_o)
        assert stats["iterations"] == it_o
