"""The persistent launch as a CUDA graph: the first solve captures it, later
solves with the same staged buffers and launch configuration replay it, and
anything that changes the kernel's arguments captures a new graph.  Every
result is bit-exact against the oracle."""
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


def oracle_times(O, case, seed_v, seed_t):
    nV = case["xyz"].shape[0]
    slots, _, _, _ = O.reference_slots(nV, case["tets"], None)
    geo = O.metric_geo(slots, case["xyz"], case["fib"], case["cf"], case["ct"])
    phi, st, _, _ = O.solve_pure(nV, slots, geo, seed_v, seed_t)
    return phi, st


def test_solves_replay_the_captured_graph(F, O):
    import fim_mesh
    c = fim_mesh.slab_case(cells=(30, 12, 6), size=(6.0, 2.4, 1.2), scar_radius=0.5, seed=9)
    nV = c["xyz"].shape[0]
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        s.solve()
        st1 = s.stats()
        phi1, sta1 = s.times()
        assert st1["graph_launch"] == 1 and st1["graph_captured"] == 1
        s.solve()
        st2 = s.stats()
        phi2, sta2 = s.times()
        assert st2["graph_launch"] == 1 and st2["graph_captured"] == 0  # replayed
        assert np.array_equal(phi1, phi2) and np.array_equal(sta1, sta2)
        phi_o, st_o = oracle_times(O, c, c["seed_v"], c["seed_t"])
        assert np.array_equal(phi1, phi_o) and np.array_equal(sta1, st_o)

        # other stimuli, same count: the same buffers, so the graph replays
        # and reads the new seeds
        rng = np.random.default_rng(4)
        v2 = rng.choice(nV, size=len(c["seed_v"]), replace=False).astype(np.int64)
        t2 = rng.uniform(0.0, 5.0, size=len(v2))
        s.set_stimuli(v2, t2)
        s.solve()
        st3 = s.stats()
        phi3, sta3 = s.times()
        assert st3["graph_launch"] == 1 and st3["graph_captured"] == 0
        phi_o, st_o = oracle_times(O, c, v2, t2)
        assert np.array_equal(phi3, phi_o) and np.array_equal(sta3, st_o)

        # a different stimulus count changes the kernel's arguments: new capture
        v4, t4 = v2[:2], t2[:2]
        s.set_stimuli(v4, t4)
        s.solve()
        st4 = s.stats()
        phi4, sta4 = s.times()
        assert st4["graph_launch"] == 1 and st4["graph_captured"] == 1
        phi_o, st_o = oracle_times(O, c, v4, t4)
        assert np.array_equal(phi4, phi_o) and np.array_equal(sta4, st_o)


def test_batched_launch_replays_its_graph(F):
    import fim_mesh
    cases = [fim_mesh.slab_case(cells=(12 + 3 * k, 6, 4), size=(3.0, 1.5, 1.0), scar_radius=0.3, seed=20 + k)
             for k in range(4)]
    b = F.Batch()
    try:
        for c in cases:
            b.add(c["xyz"], c["tets"], c["fib"], c["cf"], c["ct"], c["seed_v"], c["seed_t"])
        b.solve()
        st1 = b.stats()
        first = [b.times(i, with_state=False) for i in range(len(cases))]
        b.solve()
        st2 = b.stats()
        assert st1["graph_launch"] == 1 and st1["graph_captured"] == 1
        assert st2["graph_launch"] == 1 and st2["graph_captured"] == 0
        for i, c in enumerate(cases):
            assert np.array_equal(b.times(i, with_state=False), first[i])
            phi, _, _ = F.solve_case(c)
            assert np.array_equal(first[i], phi)
    finally:
        b.close()
