"""Launch configurations and the autotuner, through the C ABI.

Every compiled batch shape, grid size and tet-prefix warp count must give
the same times bit for bit (the configuration changes only the speed); the
autotuner must pick one of them, keep it for later solves of the mesh and
forget it with a new mesh."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

SHAPES = [(192, 4096), (160, 3072), (96, 2048)]


@pytest.fixture(scope="module")
def F(built_library):
    import fim_api
    return fim_api


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _oracle(O, case):
    nV = case["xyz"].shape[0]
    slots, _, _, _ = O.reference_slots(nV, case["tets"], None)
    geo = O.metric_geo(slots, case["xyz"], case["fib"], case["cf"], case["ct"])
    phi, st, it, _ = O.solve_pure(nV, slots, geo, case["seed_v"], case["seed_t"])
    return phi, st, it


def _same(phi, st, phi_o, st_o):
    diff = np.nonzero(phi != phi_o)[0]
    assert diff.size == 0, f"{diff.size} times differ, first {diff[:5]}"
    assert np.array_equal(st, st_o)


def test_every_configuration_bit_identical(F, O):
    """Shapes x grids x tet-prefix warps on an anisotropic slab whose narrow
    list outgrows one batch per block on the small grids."""
    import fim_mesh
    c = fim_mesh.slab_case(cells=(60, 21, 9), size=(20.0, 7.0, 3.0), seed=11)
    phi_o, st_o, it_o = _oracle(O, c)
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        full = s.tune_info()["grid_blocks"]
        for slots, corners in SHAPES:
            for grid in (full, 19, 1):
                for dag in (1, 12):
                    s.set_tune(slots=slots, corners=corners, grid=grid, dag_warps=dag)
                    s.solve()
                    st = s.stats()
                    assert (st["batch_slots"], st["batch_corners"], st["grid_blocks"], st["dag_warps"]) == \
                        (slots, corners, grid, dag)
                    assert st["iterations"] == it_o
                    phi, sts = s.times()
                    _same(phi, sts, phi_o, st_o)


def test_windowed_submeshes_on_small_shape(F):
    """The reference's golden unit-mesh output (4 submeshes, 3 windows, APD
    reset: the four-phase path) on the smallest shape and a small grid."""
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    xyz, tets, tags = ut["xyz"], np.sort(ut["tets"], axis=1), ut["tags"]
    nT = tets.shape[0]
    with F.Solver(dt=float(ut["golden_dt"]), n_steps=int(ut["golden_steps"]), apd=3e5) as s:
        s.set_mesh(xyz, tets, tags)
        s.set_conduction(np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.6), np.full(nT, 0.6))
        s.set_stimuli(ut["stim"], np.zeros(len(ut["stim"])))
        s.set_tune(slots=96, corners=2048, grid=7, dag_warps=3)
        s.solve()
        phi, st = s.times()
    written = np.round(np.where(phi < 1e50, phi, -1.0), 6)
    assert np.array_equal(written, ut["golden_phi"])
    assert np.array_equal(st, ut["golden_states"].astype(np.int32))


def test_autotune_chooses_keeps_and_forgets(F, O):
    import fim_mesh
    c = fim_mesh.cube_case(12)
    phi_o, st_o, _ = _oracle(O, c)
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        info = s.autotune()
        assert (info["batch_slots"], info["batch_corners"]) in SHAPES
        assert 1 <= info["grid_blocks"] and 1 <= info["dag_warps"] <= 12
        assert info["candidates"] >= 8 and 0 < info["tuned_ms"] <= info["default_ms"]
        phi, st = s.times()  # the last timed run
        _same(phi, st, phi_o, st_o)
        s.solve()
        stt = s.stats()
        assert (stt["batch_slots"], stt["grid_blocks"], stt["dag_warps"]) == \
            (info["batch_slots"], info["grid_blocks"], info["dag_warps"])
        phi, st = s.times()
        _same(phi, st, phi_o, st_o)
        assert s.tune_info() == info
        s.set_mesh(c["xyz"], c["tets"])  # a new mesh: back to the default
        assert s.tune_info()["default_ms"] == 0.0
    with F.Solver() as s:
        with pytest.raises(F.FimError):
            s.set_tune(slots=100, corners=1000, grid=1, dag_warps=1)


def test_autotune_option_and_batch(F, O):
    """opts.autotune tunes at the first solve; a batch tunes over all its
    problems in one launch and stays bit-exact per problem."""
    import fim_mesh
    c = fim_mesh.cube_case(8)
    phi_o, st_o, _ = _oracle(O, c)
    with F.Solver(autotune=1) as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        s.solve()
        assert s.tune_info()["candidates"] >= 8
        phi, st = s.times()
        _same(phi, st, phi_o, st_o)
    cases = [fim_mesh.cube_case(n) for n in (5, 9, 7)]
    with F.Batch() as b:
        for k in cases:
            b.add(k["xyz"], k["tets"], k["fib"], k["cf"], k["ct"], k["seed_v"], k["seed_t"])
        info = b.autotune()
        assert info["candidates"] >= 8
        b.solve()
        for i, k in enumerate(cases):
            phi_o, st_o, _ = _oracle(O, k)
            phi, st = b.times(i)
            _same(phi, st, phi_o, st_o)


@pytest.mark.parametrize("parts", [(3, 2, 2), (8, 3, 2)])
def test_submesh_sweeps_equal_grid_iterations(F, O, parts):
    """A partitioned slab with time windows: the submesh sweeps (each block
    runs whole submeshes through a window with block barriers only) and the
    grid-wide iterations give the oracle's reference-semantics result bit
    for bit, in the same number of iterations."""
    import fim_mesh
    c = fim_mesh.slab_case(cells=(40, 14, 6), size=(20.0, 7.0, 3.0), seed=5)
    xyz, tets = c["xyz"], c["tets"]
    tags = fim_mesh.block_tags(xyz, tets, parts)
    nV = xyz.shape[0]
    dt, steps = 3.0, 30
    slots, _, _, _ = O.reference_slots(nV, tets, tags)
    geo = O.metric_geo(slots, xyz, c["fib"], c["cf"], c["ct"])
    fw = O.front_width(tets.astype(np.int32), xyz)
    phi_o, st_o, _ = O.solve_reference(nV, tets, tags, geo, c["seed_v"], c["seed_t"], dt, steps, fw)
    iters = []
    for local in (1, 0):
        with F.Solver(dt=dt, n_steps=steps, apd=3e5) as s:
            s.set_mesh(xyz, tets, tags)
            s.set_conduction(c["fib"], c["cf"], c["ct"])
            s.set_stimuli(c["seed_v"], c["seed_t"])
            s.set_tune(submesh_sweeps=local)
            s.solve()
            st = s.stats()
            assert st["submesh_sweeps"] == local
            phi, sts = s.times()
        _same(phi, sts, phi_o, st_o)
        iters.append(st["iterations"])
    # a window takes as many iterations as its slowest submesh either way
    # (the oracle counts every submesh's own iterations instead)
    assert iters[0] == iters[1]
