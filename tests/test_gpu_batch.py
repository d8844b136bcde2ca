"""Batched solves (fim_batch_*): many independent problems of uneven size in
one persistent launch, each bit-identical to solving it alone and to the
FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F(built_library):
    import fim_api
    return fim_api


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _problems(n_meshes=6, n_solves=12, vmin=300, vmax=6000, seed=11):
    import fim_mesh
    meshes, solves = fim_mesh.batch_cases(n_meshes=n_meshes, n_solves=n_solves, vmin=vmin, vmax=vmax, seed=seed)
    out = []
    for sv in solves:
        m = meshes[sv["mesh"]]
        out.append(dict(xyz=m["xyz"], tets=m["tets"], fib=sv["fib"], cf=sv["cf"], ct=sv["ct"],
                        seed_v=sv["seed_v"], seed_t=sv["seed_t"]))
    return out


def test_batch_equals_single_solves(F, O):
    probs = _problems()
    with F.Batch() as b:
        ids = [b.add(p["xyz"], p["tets"], p["fib"], p["cf"], p["ct"], p["seed_v"], p["seed_t"]) for p in probs]
        b.solve()
        stats = b.stats()
        got = [b.times(i) for i in ids]
        # a second solve of the same batch (staging reused) gives the same times
        b.solve()
        again = [b.times(i) for i in ids]
    for (phi, st), (phi2, st2) in zip(got, again):
        assert np.array_equal(phi, phi2) and np.array_equal(st, st2)
    iters = []
    for p, (phi, st) in zip(probs, got):
        phi1, st1, s1 = F.solve_case(p)
        assert np.array_equal(phi, phi1) and np.array_equal(st, st1)
        iters.append(s1["iterations"])
    # the batch iterates as long as its slowest problem
    assert stats["iterations"] == max(iters)
    # two problems against the oracle as well
    for p, (phi, st) in list(zip(probs, got))[:2]:
        nV = p["xyz"].shape[0]
        slots, _, _, _ = O.reference_slots(nV, p["tets"], None)
        geo = O.metric_geo(slots, p["xyz"], p["fib"], p["cf"], p["ct"])
        phi_o, st_o, _, _ = O.solve_pure(nV, slots, geo, p["seed_v"], p["seed_t"])
        assert np.array_equal(phi, phi_o) and np.array_equal(st, st_o)


def test_batch_rejects_windows_and_negative_times(F):
    with pytest.raises(F.FimError) as e:
        F.Batch(dt=10.0)
    assert e.value.code == 1
    p = _problems(n_meshes=1, n_solves=1)[0]
    with F.Batch() as b:
        with pytest.raises(F.FimError) as e:
            b.add(p["xyz"], p["tets"], p["fib"], p["cf"], p["ct"], p["seed_v"], -np.ones(len(p["seed_v"])))
        assert e.value.code == 1 and "times >= 0" in str(e.value)
        with pytest.raises(F.FimError):
            b.solve()  # nothing added


def test_wide_batch_every_problem(F, O):
    """34 problems in one launch: 32 uneven boxes with 1-8 stimuli, a
    112,716-vertex anisotropic slab and a single-stimulus cube.  Every problem
    equals its own single solve bit for bit; four (the slab, the cube and
    the two smallest boxes) also equal the FP64 oracle."""
    import fim_mesh
    probs = _problems(n_meshes=12, n_solves=32, vmin=300, vmax=20000, seed=23)
    big = fim_mesh.slab_case(cells=(100, 35, 30), size=(20.0, 7.0, 3.0), seed=13)
    one = fim_mesh.cube_case(10, seed=4)
    assert len(one["seed_v"]) == 1 and big["xyz"].shape[0] > 100_000
    probs = probs + [{k: big[k] for k in ("xyz", "tets", "fib", "cf", "ct", "seed_v", "seed_t")},
                     {k: one[k] for k in ("xyz", "tets", "fib", "cf", "ct", "seed_v", "seed_t")}]
    with F.Batch() as b:
        ids = [b.add(p["xyz"], p["tets"], p["fib"], p["cf"], p["ct"], p["seed_v"], p["seed_t"]) for p in probs]
        b.solve()
        got = [b.times(i) for i in ids]
    for k, (p, (phi, st)) in enumerate(zip(probs, got)):
        phi1, st1, _ = F.solve_case(p)
        assert np.array_equal(phi, phi1) and np.array_equal(st, st1), f"problem {k} differs from its single solve"
    order = sorted(range(32), key=lambda i: probs[i]["xyz"].shape[0])
    for k in [32, 33] + order[:2]:
        p = probs[k]
        phi, st = got[k]
        nV = p["xyz"].shape[0]
        slots, _, _, _ = O.reference_slots(nV, p["tets"], None)
        geo = O.metric_geo(slots, p["xyz"], p["fib"], p["cf"], p["ct"])
        phi_o, st_o, _, _ = O.solve_pure(nV, slots, geo, p["seed_v"], p["seed_t"])
        assert np.array_equal(phi, phi_o) and np.array_equal(st, st_o), f"problem {k} differs from the oracle"


def test_batch_warm_start_equals_single_warm_solves(F):
    """fim_batch_set_warm_start: upper-bound starts (1.05 x the cold times)
    for three problems in one array, in add order; each problem's result
    equals its own warm-started single solve bit for bit."""
    import fim_mesh
    torch = pytest.importorskip("torch")
    cases = [fim_mesh.cube_case(n, seed=2 + n) for n in (6, 9, 7)]
    starts, singles = [], []
    for c in cases:
        cold, _, _ = F.solve_case(c)
        st = np.where(cold < F.INF, 1.05 * cold, F.INF)
        starts.append(st)
        d = torch.from_numpy(st).cuda()
        torch.cuda.synchronize()
        with F.Solver() as s:
            s.set_mesh(c["xyz"], c["tets"])
            s.set_conduction(c["fib"], c["cf"], c["ct"])
            s.set_stimuli(c["seed_v"], c["seed_t"])
            s.set_warm_start(d.data_ptr())
            s.solve()
            singles.append(s.times())
            assert s.stats()["warm_reset"] == 0
    d_all = torch.from_numpy(np.concatenate(starts)).cuda()
    torch.cuda.synchronize()
    with F.Batch() as b:
        for c in cases:
            b.add(c["xyz"], c["tets"], c["fib"], c["cf"], c["ct"], c["seed_v"], c["seed_t"])
        b.set_warm_start(d_all.data_ptr())
        b.solve()
        assert b.stats()["warm_reset"] == 0
        for i, (phi1, st1) in enumerate(singles):
            phi, st = b.times(i)
            assert np.array_equal(phi, phi1) and np.array_equal(st, st1)
