"""The learned warm start: the network's GPU kernels against the CPU
restatement (oracle/mlp_oracle.py), training on FIM maps, and warm-started
solves."""
import numpy as np
import pytest

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


def _random_problem(M, n, seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.NPARAMS, dtype=np.float32)
    p[M.OW1:M.OW1 + 7 * M.H] = rng.normal(0, 0.5, 7 * M.H)
    p[M.OW2:M.OB1] = rng.normal(0, 0.12, 2 * M.H * M.H)
    p[M.OB1:M.OW4] = rng.normal(0, 0.05, 3 * M.H)
    p[M.OW4:M.OB4] = rng.normal(0, 0.1, M.H)
    p[M.OB4] = 0.3
    X = np.zeros((n, M.IN), dtype=np.float32)
    X[:, :7] = rng.normal(0, 1, (n, 7))
    X = M.bf16(X)
    t = rng.normal(0.5, 0.3, n).astype(np.float32)
    return p, X, t


def _to_device_bf16(torch, X):
    bits = (np.ascontiguousarray(X, dtype=np.float32).view(np.uint32) >> 16).astype(np.uint16)
    return torch.from_numpy(bits.view(np.int16)).cuda()


def test_gradients_match_oracle(F, torch_cuda):
    from oracle import mlp_oracle as M
    torch = torch_cuda
    p, X, t = _random_problem(M, 256, 1)
    with F.Mlp(seed=3) as mlp:
        mlp.set_params(p)
        assert np.array_equal(mlp.get_params(), p)
        dX, dt = _to_device_bf16(torch, X), torch.from_numpy(t).cuda()
        g, loss = mlp.gradients(256, dX.data_ptr(), dt.data_ptr())
        y = torch.empty(256, dtype=torch.float32, device="cuda")
        mlp.predict(256, dX.data_ptr(), y.data_ptr())
    loss_o, g_o = M.loss_and_gradients(p, X, t)
    _, _, _, y_o = M.forward(p, X)
    assert np.allclose(y.cpu().numpy(), y_o, rtol=1e-3, atol=1e-3)
    assert abs(loss - loss_o) <= 1e-3 * abs(loss_o)
    for name, (a, b) in M.BLOCKS.items():
        ref = g_o[a:b]
        err = np.linalg.norm(g[a:b] - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 1e-2, (name, err)


@pytest.mark.parametrize("n", [192, 4096])
def test_tensor_core_gemms_ragged_tile_and_long_k(F, torch_cuda, n):
    """192 rows end in half a 128-row tile (rows past the matrix read as
    zeros and are not stored); 4096 rows make the weight gradients 64 K
    slices, many passes through the GEMM's stage ring."""
    from oracle import mlp_oracle as M
    torch = torch_cuda
    p, X, t = _random_problem(M, n, 11)
    with F.Mlp(seed=3) as mlp:
        mlp.set_params(p)
        dX, dt = _to_device_bf16(torch, X), torch.from_numpy(t).cuda()
        y = torch.empty(n, dtype=torch.float32, device="cuda")
        mlp.predict(n, dX.data_ptr(), y.data_ptr())
        g, loss = mlp.gradients(n, dX.data_ptr(), dt.data_ptr())
        y2 = torch.empty(n, dtype=torch.float32, device="cuda")
        mlp.predict(n, dX.data_ptr(), y2.data_ptr())
    _, _, _, y_o = M.forward(p, X)
    yg = y.cpu().numpy()
    # FP32 summation order differs from the oracle's: where that flips the
    # BF16 rounding of a stored activation, the row moves by a BF16 step
    bad = ~np.isclose(yg, y_o, rtol=1e-3, atol=1e-3)
    assert bad.mean() < 0.01, bad.sum()
    assert np.max(np.abs(yg - y_o)) < 0.05 * np.max(np.abs(y_o))
    assert np.array_equal(yg, y2.cpu().numpy())  # deterministic
    loss_o, g_o = M.loss_and_gradients(p, X, t)
    assert abs(loss - loss_o) <= 1e-3 * abs(loss_o)
    for name, (a, b) in M.BLOCKS.items():
        ref = g_o[a:b]
        err = np.linalg.norm(g[a:b] - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 1e-2, (name, err)


def test_row_count_must_be_multiple_of_64(F, torch_cuda):
    torch = torch_cuda
    with F.Mlp() as mlp:
        X = torch.zeros((100, F.MLP_INPUTS), dtype=torch.int16, device="cuda")
        y = torch.zeros(100, dtype=torch.float32, device="cuda")
        with pytest.raises(F.FimError) as e:
            mlp.predict(100, X.data_ptr(), y.data_ptr())
        assert e.value.code == 1


def test_training_beats_the_distance_feature_and_warm_solves(F, torch_cuda):
    """Trained on FIM maps of small slabs, the network predicts held-out maps
    better than the metric distance to the stimuli alone (what it gains over
    the method without it).  A warm-started solve only corrects downwards
    where its start passes the support check; an all-infinite warm start is
    the cold solve bit for bit."""
    import fim_warm
    torch = torch_cuda
    cells = (24, 9, 5)
    train_maps = fim_warm.make_maps(48, cells, 7, torch)
    test_maps = fim_warm.make_maps(6, cells, 8, torch)
    with F.Mlp(seed=5) as mlp:
        losses = fim_warm.train(mlp, train_maps, steps=600, batch=1024, lr=2e-3, torch=torch)
        assert np.mean(losses[-50:]) < 0.3 * np.mean(losses[:10])
        ev = fim_warm.evaluate(mlp, test_maps, torch)
        # measured on the GB300: network RMS error 0.19 of max(t) against 0.30
        # for the distance feature
        assert ev["net_rms"] < 0.8 * ev["dist_rms"], ev
        with F.Solver() as s:
            m = test_maps[0]
            phi, st, start = fim_warm.warm_solve(s, mlp, m, torch)
            other = np.ones(m.nV, dtype=bool)
            other[m.case["seed_v"]] = False
            if st["warm_reset"] == 0:
                assert np.all(phi[other] <= start[other])  # corrections only go down
            assert np.all(phi[m.case["seed_v"]] <= m.case["seed_t"])
            inf = torch.full((m.nV,), float(F.INF), dtype=torch.float64, device="cuda")
            c = m.case
            s.set_mesh(c["xyz"], c["tets"])
            s.set_conduction(c["fib"], c["cf"], c["ct"])
            s.set_stimuli(c["seed_v"], c["seed_t"])
            s.set_warm_start(inf.data_ptr())
            s.solve()
            assert np.array_equal(s.times(with_state=False), m.phi)
