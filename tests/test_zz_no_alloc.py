"""fim_solve_noalloc (the allocation-free re-solve backed by a fixed device
array) against the allocating entry points fim_set_stimuli + fim_solve +
fim_get_times_device, two calls in a row on the same solver.  Collected last
so that it also runs after every other GPU test in the same process; it
passes alone as well."""
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
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _existing(s, torch, v, t):
    """Times through the allocating entry points, into a device buffer."""
    s.set_stimuli(v, t)
    s.solve()
    out = torch.full((s.nV,), -1.0, dtype=torch.float64, device="cuda")
    s.times_device(out.data_ptr())
    return out.cpu().numpy()


def _noalloc(s, torch, v, t):
    out = torch.full((s.nV,), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    s.solve_noalloc(v, t, out.data_ptr())
    return out.cpu().numpy()


def _same(a, b):
    diff = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0]
    assert diff.size == 0, f"{diff.size} times differ, first {diff[:5]}: {a[diff[:5]]} vs {b[diff[:5]]}"


def test_noalloc_slab_two_calls(F, torch_cuda):
    """One submesh: two different stimulus sets back to back (the second with
    a vertex given twice, the earlier time winning); the solver's own last
    results stay as they were."""
    import fim_mesh
    torch = torch_cuda
    c = fim_mesh.slab_case(cells=(40, 14, 6), size=(20.0, 7.0, 3.0), seed=5)
    va, ta = c["seed_v"], c["seed_t"]
    vb = np.array([7, 300, 1200, 300, 2500], dtype=np.int64)
    tb = np.array([0.0, 4.0, 1.5, 2.25, 8.0])
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        ref_a = _existing(s, torch, va, ta)
        ref_b = _existing(s, torch, vb, tb)
        own_b = s.times(with_state=False)
        got_a = _noalloc(s, torch, va, ta)
        got_b = _noalloc(s, torch, vb, tb)
        _same(got_a, ref_a)
        _same(got_b, ref_b)
        assert not np.array_equal(ref_a, ref_b)
        _same(s.times(with_state=False), own_b)


def test_noalloc_warm_start_and_signed_zero(F, torch_cuda):
    """A warm start set on the solver applies to both paths alike, and a
    vertex given both -0.0 and +0.0 is seeded the same way on both."""
    import fim_mesh
    torch = torch_cuda
    c = fim_mesh.slab_case(cells=(30, 12, 5), size=(6.0, 2.4, 1.0), seed=9)
    v = np.concatenate([c["seed_v"], c["seed_v"][:1], c["seed_v"][:1]]).astype(np.int64)
    t = np.concatenate([c["seed_t"], [0.0], [-0.0]])
    t[0] = -0.0
    with F.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        cold = _existing(s, torch, v, t)
        _same(_noalloc(s, torch, v, t), cold)
        reached = cold < 1e300
        start = torch.tensor(np.where(reached, np.maximum(cold * 1.05, 0.0), np.finfo(np.float64).max),
                             dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        s.set_warm_start(start.data_ptr())
        warm_a = _existing(s, torch, v, t)
        got_a = _noalloc(s, torch, v, t)
        got_b = _noalloc(s, torch, v, t)
        s.set_warm_start(None)
        _same(got_a, warm_a)
        _same(got_b, warm_a)


def test_noalloc_submeshes_two_calls(F, torch_cuda):
    """The reference's unit mesh: 4 submeshes, 3 windows of 150000 us with the
    APD reset; the golden stimuli, then a single-vertex stimulus."""
    torch = torch_cuda
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    xyz, tets, tags = ut["xyz"], np.sort(ut["tets"], axis=1), ut["tags"]
    nT = tets.shape[0]
    va = ut["stim"].astype(np.int64)
    ta = np.zeros(len(va))
    vb = np.array([int(tets[nT // 2, 0])], dtype=np.int64)
    tb = np.array([12.5])
    with F.Solver(dt=float(ut["golden_dt"]), n_steps=int(ut["golden_steps"]), apd=3e5) as s:
        s.set_mesh(xyz, tets, tags)
        s.set_conduction(np.tile([1.0, 0, 0], (nT, 1)), np.full(nT, 0.6), np.full(nT, 0.6))
        ref_a = _existing(s, torch, va, ta)
        ref_b = _existing(s, torch, vb, tb)
        got_a = _noalloc(s, torch, va, ta)
        got_b = _noalloc(s, torch, vb, tb)
        _same(got_a, ref_a)
        _same(got_b, ref_b)
        written = np.round(np.where(got_a < 1e50, got_a, -1.0), 6)
        assert np.array_equal(written, ut["golden_phi"])


def test_noalloc_limits(F, torch_cuda):
    """Inputs beyond the fixed scratch are refused with a clear message, and
    the scratch still works afterwards."""
    import fim_mesh
    torch = torch_cuda
    big = fim_mesh.cube_case(51)  # 52^3 = 140,608 vertices > 131,072
    out = torch.empty(big["xyz"].shape[0], dtype=torch.float64, device="cuda")
    with F.Solver() as s:
        s.set_mesh(big["xyz"], big["tets"])
        s.set_conduction(big["fib"], big["cf"], big["ct"])
        with pytest.raises(F.FimError) as e:
            s.solve_noalloc(big["seed_v"], big["seed_t"], out.data_ptr())
        assert e.value.code == 1 and "fixed scratch" in str(e.value)
    small = fim_mesh.cube_case(6)
    with F.Solver() as s:
        s.set_mesh(small["xyz"], small["tets"])
        s.set_conduction(small["fib"], small["cf"], small["ct"])
        many = np.zeros(8193, dtype=np.int64)
        with pytest.raises(F.FimError) as e:
            s.solve_noalloc(many, np.zeros(8193), out.data_ptr())
        assert e.value.code == 1 and "fixed scratch" in str(e.value)
        _same(_noalloc(s, torch, small["seed_v"], small["seed_t"]),
              _existing(s, torch, small["seed_v"], small["seed_t"]))
