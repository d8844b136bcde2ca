"""The learned warm start, end to end: training maps from the FIM solver
itself, the per-vertex network trained on the GPU, warm-started solves.

Glue only: features, the network's forward/backward/Adam and the solves run
in the library's CUDA kernels; device buffers are torch tensors (BF16 feature
rows are held as int16 bit patterns).  No counterpart in the reference.
"""
import math

import numpy as np

import fim_api
import fim_mesh


def draw_case(rng, cells, index):
    """A slab of the bench family with random conduction, scar and stimuli."""
    cf = float(rng.uniform(0.4, 0.8))
    ct = cf * float(rng.uniform(0.3, 0.5))
    return fim_mesh.slab_case(cells=cells, size=(20.0 * cells[0] / 266, 7.0 * cells[1] / 93, 3.0 * cells[2] / 40),
                              seed=1000 + index, cf=cf, ct=ct, angle=float(rng.uniform(40.0, 70.0)),
                              scar_radius=float(rng.uniform(0.0, 0.4)) * 20.0 * cells[0] / 266,
                              n_stim=int(rng.integers(1, 9)), t0_max=10.0)


class Map:
    """One solved case: device features, times and the cold solve's statistics."""

    def __init__(self, solver, case, torch):
        nV = case["xyz"].shape[0]
        solver.set_mesh(case["xyz"], case["tets"])
        solver.set_conduction(case["fib"], case["cf"], case["ct"])
        solver.set_stimuli(case["seed_v"], case["seed_t"])
        solver.set_warm_start(None)
        solver.solve()
        self.phi = solver.times(with_state=False)
        self.cold = solver.stats()
        n64 = (nV + 63) // 64 * 64
        self.X = torch.zeros((n64, fim_api.MLP_INPUTS), dtype=torch.int16, device="cuda")
        self.scale = solver.features(self.X.data_ptr())
        self.nV, self.n64, self.case = nV, n64, case
        reached = self.phi < 1e300
        t = np.where(reached, self.phi / self.scale, 0.0).astype(np.float32)
        self.t = torch.from_numpy(t).cuda()
        self.reached = torch.from_numpy(reached).cuda()


def make_maps(n, cells, seed, torch):
    rng = np.random.default_rng(seed)
    maps = []
    with fim_api.Solver() as s:
        for i in range(n):
            maps.append(Map(s, draw_case(rng, cells, seed * 100000 + i), torch))
    return maps


def train(mlp, maps, steps, batch, lr, torch, seed=0):
    """Adam on random vertices of the maps (cosine learning-rate decay); returns the losses."""
    X = torch.cat([m.X[:m.nV][m.reached] for m in maps])
    T = torch.cat([m.t[m.reached] for m in maps])
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    losses = []
    for k in range(steps):
        idx = torch.randint(0, X.shape[0], (batch,), device="cuda", generator=g)
        xb = X[idx].contiguous()
        tb = T[idx].contiguous()
        cur = lr * 0.5 * (1.0 + math.cos(math.pi * k / steps))
        losses.append(mlp.train_step(batch, xb.data_ptr(), tb.data_ptr(), cur))
    return losses


def predict_times(mlp, m, torch):
    y = torch.empty(m.n64, dtype=torch.float32, device="cuda")
    mlp.predict(m.n64, m.X.data_ptr(), y.data_ptr())
    return y[:m.nV].double() * m.scale


def evaluate(mlp, maps, torch):
    """RMS and max of |prediction - cold time| / max(time) over the maps, and
    the same for the distance feature alone (the method without the network)."""
    net, base = [], []
    for m in maps:
        pred = predict_times(mlp, m, torch).cpu().numpy()
        bits = m.X[:m.nV, 3].cpu().numpy().view(np.uint16).astype(np.uint32) << 16
        dist = bits.view(np.float32).astype(np.float64) * m.scale
        r = m.phi < 1e300
        tmax = m.phi[r].max()
        net.append((pred[r] - m.phi[r]) / tmax)
        base.append((dist[r] - m.phi[r]) / tmax)
    net, base = np.concatenate(net), np.concatenate(base)
    return {"net_rms": float(np.sqrt(np.mean(net ** 2))), "net_max": float(np.abs(net).max()),
            "dist_rms": float(np.sqrt(np.mean(base ** 2))), "dist_max": float(np.abs(base).max()),
            "net_below": float(np.mean(net < 0))}


def warm_solve(solver, mlp, m, torch, inflate=1.05):
    """Solve map m from the inflated prediction; returns (times, stats, start).

    The start is clamped to the earliest stimulus time: FIM only ever lowers
    a time, so a start below every stimulus (the network can predict negative
    times near a stimulus) never settles and the solve runs into its
    iteration cap -- the reference's algorithm does the same from such a
    start."""
    c = m.case
    solver.set_mesh(c["xyz"], c["tets"])
    solver.set_conduction(c["fib"], c["cf"], c["ct"])
    solver.set_stimuli(c["seed_v"], c["seed_t"])
    t_first = float(np.min(c["seed_t"]))
    start = torch.clamp(predict_times(mlp, m, torch) * inflate, min=t_first).contiguous()
    solver.set_warm_start(start.data_ptr())
    solver.solve(torch.cuda.current_stream().cuda_stream)  # after the kernels that wrote `start`
    phi = solver.times(with_state=False)
    st = solver.stats()
    solver.set_warm_start(None)
    return phi, st, start.cpu().numpy()
