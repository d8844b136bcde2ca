#!/usr/bin/env python3
"""Benchmark of the GB300 FIM eikonal solver on the anisotropic-slab workload.

One step = one full solve of the slab: the FP64 per-tet metric precompute
from the (HBM-resident) conduction field plus the persistent FIM kernel,
i.e. everything between "conduction + stimuli given" and "activation times
available".  Prints one JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

* value      -- whole-job solves/s with inputs resident in HBM (CUDA events
                on the solver's stream, max over ranks);
* e2e        -- solves/s through the C ABI with pinned host buffers: H2D of
                the conduction field + stimuli, solve, D2H of the times;
* roofline   -- the FIM kernel's algorithmic bytes (vertex updates x
                (40 T/V + 9) B) per launch / launch time vs measured HBM peak;
* cpu_baseline -- the oracle (C restatement of the reference algorithm,
                OpenMP over all host cores) on one full solve of the same slab;
* parity     -- the last GPU result vs that FP64 oracle result.
--gpus N > 1 runs N independent replicas (the path does not shard).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cufim-nvlink_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

SLAB_CELLS = (266, 93, 40)
# DRAM bytes (read + write) of one fim_solve_kernel launch per vertex update,
# from ncu dram__bytes_read.sum + dram__bytes_write.sum on this workload
# (ncu measurement: 4.294 GB for 4,689,493 vertex updates, two-phase kernel, 192x4096 batches)
NCU_DRAM_BYTES_PER_VERTEX_UPDATE = 4.294e9 / 4689493


def metric_launches(nT):
    """fim_metric_kernel launches per conduction upload: the field goes up in
    up to 8 chunks of at least 2^18 tets (fim_solver.cpp, run_metric)."""
    return max(1, min(8, nT >> 18))
METRICS = {
    "slab": "slab solves/s (1.03M-vertex anisotropic FIM, bit-exact vs FP64 oracle)",
    "cube": "cube solves/s (9,261-vertex plain FIM, bit-exact vs FP64 oracle)",
    "shell": "shell solves/s (4.2M-vertex ventricle-like shell FIM, bit-exact vs FP64 oracle)",
    "batch": "batched solves/s (uneven Kuhn boxes, one persistent launch, bit-exact vs FP64 oracle)",
    "warm": "warm-started vs cold FIM solves/s (learned per-vertex start times, slab family)",
    "part": "partitioned slab solves/s (1.03M vertices, 2,964 submeshes, 50 windows, bit-exact vs FP64 oracle)",
    "mlp": "warm-start network forward rows/s (tcgen05 GEMMs over the 1.03M slab vertices)",
}
PART_BLOCKS = (38, 13, 6)   # the slab's geometric partition: ~2,000 tets per submesh
PART_DT, PART_STEPS = 2.0, 50
UNIT = "solves/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--workload", choices=["slab", "cube", "shell", "batch", "warm", "part", "mlp"], default="slab",
                    help="slab: 1M-vertex anisotropic slab (default); cube: 9,261-vertex unit cube, isotropic; "
                         "shell: 4.2M-vertex ventricle-like shell; batch: many uneven solves in one launch; "
                         "warm: learned warm start against the cold start; part: the slab partitioned into "
                         "submeshes, solved in time windows (the reference's own operating mode); mlp: the "
                         "warm-start network's tensor-core GEMMs (forward over the slab's vertices, training steps)")
    ap.add_argument("--batch", type=str, default="32,256,10000,500000",
                    help="batch workload: meshes,solves,min vertices,max vertices")
    ap.add_argument("--cells", type=str, default=None, help="override slab cells, e.g. 66,23,10")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--no-extra", action="store_true", help="skip the short runs of the other workloads")
    ap.add_argument("--precision", choices=["fp64", "fp32"], default="fp64",
                    help="fp32: FP32 local solves wherever their screens are conclusive (not bit-exact; the "
                         "parity block reports the error against the FP64 oracle)")
    ap.add_argument("--e2e-steps", type=int, default=None)
    return ap.parse_args()


def workload(args):
    import fim_mesh
    if args.workload == "cube":
        case = fim_mesh.cube_case(20)
        nV, nT = case["xyz"].shape[0], case["tets"].shape[0]
        return case, {"workload": (f"unit cube, 20^3 Kuhn cells ({nV} vertices, {nT} tets), +-0.2h jitter, "
                                   "isotropic 0.6 mm/ms, one stimulus at (0,0,0) t0 = 0; one endless window"),
                      "vertices": nV, "tets": nT, "seed": 1, "l2": "inputs smaller than L2; L2 not flushed",
                      "parallelism": "replicas"}
    if args.workload == "shell":
        case = fim_mesh.shell_case()
        nV, nT = case["xyz"].shape[0], case["tets"].shape[0]
        return case, {"workload": (f"ventricle-like shell: prolate spheroid wall 20/20/50 -> 30/30/60 mm, base cut at "
                                   f"2/3 height, 21x630x321 structured Kuhn grid ({nV} vertices, {nT} tets), "
                                   "+-0.2h jitter, transmural fibres -60..+60 deg, cf 0.6 / ct 0.24 mm/ms, 8 "
                                   "endocardial stimuli t0~U[0,15] ms; one endless window"),
                      "vertices": nV, "tets": nT, "seed": 5, "l2": "inputs larger than L2",
                      "parallelism": "replicas"}
    cells = tuple(int(x) for x in args.cells.split(",")) if args.cells else SLAB_CELLS
    case = fim_mesh.slab_case(cells=cells)
    nV, nT = case["xyz"].shape[0], case["tets"].shape[0]
    if args.workload == "part":
        blocks = tuple(max(1, round(b * c / s)) for b, c, s in zip(PART_BLOCKS, cells, SLAB_CELLS))
        case["tags"] = fim_mesh.block_tags(case["xyz"], case["tets"], blocks)
        nparts = int(len(np.unique(case["tags"])))
        case["dt"], case["n_steps"] = PART_DT, PART_STEPS
        return case, {"workload": (f"anisotropic slab {cells[0]}x{cells[1]}x{cells[2]} Kuhn cells ({nV} vertices, "
                                   f"{nT} tets) as in the slab workload, partitioned geometrically into {nparts} "
                                   f"submeshes ({blocks[0]}x{blocks[1]}x{blocks[2]} blocks, ~{nT // nparts} tets "
                                   f"each), {PART_STEPS} windows of {PART_DT} ms with the interface sync between "
                                   "them (the reference's compute_step / sync_step2 semantics; APD 3e5, which "
                                   "never fires at these times)"),
                      "vertices": nV, "tets": nT, "submeshes": nparts, "windows": PART_STEPS, "dt_ms": PART_DT,
                      "seed": 2, "l2": "inputs larger than L2", "parallelism": "replicas"}
    cfg = {
        "workload": (f"anisotropic slab 20x7x3 mm, {cells[0]}x{cells[1]}x{cells[2]} Kuhn cells "
                     f"({nV} vertices, {nT} tets), +-0.2h jitter, fibres -60..+60 deg over z, cf 0.6 / "
                     "ct 0.24 mm/ms, 2 mm scar x0.1, 5 surface stimuli t0~U[0,10] ms; one submesh, "
                     "one endless window"),
        "vertices": nV, "tets": nT, "seed": 2,
        "l2": "inputs larger than L2 (corner records 112 B x 4T = 2.7 GB)",
        "parallelism": "replicas",
    }
    return case, cfg


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(pg, value, device=None):
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


# ---------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 3.0 and os.path.getsize(self.path) == 0:
                time.sleep(0.05)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                if int(f[0]) != self.index:
                    continue
                rows.append(f)
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU oracle (checker + CPU baseline): the C restatement of the reference's
# algorithm, OpenMP over every host core
def oracle_solve(case, threads=0):
    from oracle import build as obuild
    obuild.build_oracle()
    from oracle import oracle as O
    nV = case["xyz"].shape[0]
    if "tags" in case:  # submeshes and windows: the reference-semantics restatement
        t0 = time.perf_counter()
        slots, _, _, _ = O.reference_slots(nV, case["tets"], case["tags"])
        geo = O.metric_geo(slots, case["xyz"], case["fib"], case["cf"], case["ct"])
        fw = O.front_width(case["tets"].astype(np.int32), case["xyz"])
        t1 = time.perf_counter()
        phi, st, it = O.solve_reference(nV, case["tets"], case["tags"], geo, case["seed_v"], case["seed_t"],
                                        case["dt"], case["n_steps"], fw, apd_us=3e5)
        return phi, st, {"solve_s": time.perf_counter() - t1, "prep_s": t1 - t0, "iterations": it,
                         "vertex_updates": None}
    t0 = time.perf_counter()
    slots, _, _, _ = O.reference_slots(nV, case["tets"], None)
    t1 = time.perf_counter()
    geo = O.metric_geo(slots, case["xyz"], case["fib"], case["cf"], case["ct"])
    phi, st, it, upd = O.solve_pure(nV, slots, geo, case["seed_v"], case["seed_t"], threads=threads)
    t2 = time.perf_counter()
    return phi, st, {"solve_s": t2 - t1, "prep_s": t1 - t0, "iterations": it, "vertex_updates": upd}


def parity_report(phi, phi_o, tolerance="max |dt| <= 1e-4 max(t); achieved bit-exact"):
    finite = phi_o < 1e300
    tmax = float(phi_o[finite].max()) if finite.any() else 1.0
    d = np.abs(np.where(finite, phi, 0.0) - np.where(finite, phi_o, 0.0))
    same_inf = bool(np.array_equal(phi >= 1e300, ~finite))
    return {"max_abs_err": float(d.max()), "max_rel_err": float(d.max() / tmax),
            "rms_rel_err": float(np.sqrt(np.mean(d ** 2)) / tmax),
            "n_bit_mismatch": int(np.count_nonzero(phi != phi_o)),
            "n_over_1e-4": int(np.count_nonzero(d > 1e-4 * tmax)), "unreached_match": same_inf,
            "tolerance": tolerance}


def run_mine(args):
    import torch
    import fim_api
    world, rank, local, pg = dist_setup(args)
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    case, cfg = workload(args)
    nV, nT = case["xyz"].shape[0], case["tets"].shape[0]
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    s = fim_api.Solver(device=local, fp32_update=1 if args.precision == "fp32" else 0,
                       **({"dt": case["dt"], "n_steps": case["n_steps"], "apd": 3e5} if "tags" in case else {}))
    s.set_mesh(case["xyz"], case["tets"], case.get("tags"))
    stream = torch.cuda.Stream(dev)
    s.set_stream(stream.cuda_stream)
    fib = torch.tensor(case["fib"], dtype=torch.float64, device=dev).contiguous()
    cf = torch.tensor(case["cf"], dtype=torch.float64, device=dev)
    ct = torch.tensor(case["ct"], dtype=torch.float64, device=dev)
    s.set_stimuli(case["seed_v"], case["seed_t"])
    s.set_conduction_device(fib.data_ptr(), cf.data_ptr(), ct.data_ptr())
    tune = s.autotune() if not args.no_autotune else s.tune_info()  # before the timed region
    torch.cuda.synchronize()

    solve_ms, metric_ms = [], []

    def step(record):
        s.set_conduction_device(fib.data_ptr(), cf.data_ptr(), ct.data_ptr())
        s.solve()
        if record:
            st = s.stats()
            solve_ms.append(st["solve_ms"])
            metric_ms.append(st["metric_ms"])

    for _ in range(max(args.warmup, 0)):
        step(False)
    clocks = ClockSampler(index=local)
    clocks.start()
    barrier(pg)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step(True)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(pg)
    clk = clocks.stop()
    dev_ms = ev0.elapsed_time(ev1)
    max_ms = max_over_ranks(pg, dev_ms, dev if pg is not None and torch.cuda.is_available() else None)
    stats = s.stats()
    phi_dev = s.times(with_state=False)

    # end to end through the C ABI from pinned host buffers
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 10))
    h_fib = torch.from_numpy(case["fib"]).pin_memory().numpy()
    h_cf = torch.from_numpy(case["cf"]).pin_memory().numpy()
    h_ct = torch.from_numpy(case["ct"]).pin_memory().numpy()
    h_sv = torch.from_numpy(case["seed_v"].astype(np.int64)).pin_memory().numpy()
    h_st = torch.from_numpy(case["seed_t"]).pin_memory().numpy()
    h_phi = torch.empty(nV, dtype=torch.float64).pin_memory().numpy()
    import ctypes as C
    L = fim_api.lib()
    P = fim_api._ptr

    def e2e_step():
        fim_api._check(L.fim_set_conduction(s.h, P(h_fib, C.c_double), P(h_cf, C.c_double), P(h_ct, C.c_double)), s.h)
        fim_api._check(L.fim_set_stimuli(s.h, h_sv.shape[0], P(h_sv, C.c_int64), P(h_st, C.c_double)), s.h)
        fim_api._check(L.fim_solve(s.h, None), s.h)
        fim_api._check(L.fim_get_times(s.h, P(h_phi, C.c_double), None), s.h)

    e2e_step()
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = max_over_ranks(pg, time.perf_counter() - t0, dev if pg is not None and torch.cuda.is_available() else None)
    barrier(pg)
    h2d = h_fib.nbytes + h_cf.nbytes + h_ct.nbytes + h_sv.nbytes + h_st.nbytes
    d2h = h_phi.nbytes
    assert np.array_equal(h_phi, phi_dev)

    if rank != 0:
        s.close()
        return
    b_vu = 40.0 * nT / nV + 9.0
    cells_default = args.cells is None and args.workload == "slab"
    upd = stats["vertex_updates"]
    mean_solve_ms = float(np.mean(solve_ms))
    achieved = upd * b_vu / (mean_solve_ms * 1e-3) / 1e9
    out = {
        "metric": (METRICS[args.workload] if args.precision == "fp64" else
                   METRICS[args.workload].replace("bit-exact vs FP64 oracle", "FP32 local solves, error vs FP64 oracle")),
        "value": world * args.steps / (max_ms * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32 local solves, f64 where inconclusive",
        "data": "synthetic (seeded slab mesh, conduction field and stimuli)", "config": cfg,
        "solve_ms": mean_solve_ms, "metric_ms": float(np.mean(metric_ms)),
        "iterations": stats["iterations"], "vertex_updates": upd,
        "vertex_updates_per_s": upd / (mean_solve_ms * 1e-3), "corners_screened": stats["corner_evals"],
        "fp64_local_solves": stats["exact_evals"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak,
                     "traffic": NCU_DRAM_BYTES_PER_VERTEX_UPDATE * upd if cells_default else None,
                     "kernel": "fim_solve_kernel", "bytes_per_vertex_update": b_vu,
                     "peak_source": peak_src,
                     "traffic_source": "ncu DRAM bytes per vertex update of the same workload x this run's updates",
                     "note": ("algorithmic bytes = vertex updates x (40 T/V + 9) B; the kernel is bound by the "
                              "latency of its per-batch phase chain (FP64 solves, block barriers), not by HBM")},
        "e2e": {"value": world * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": (metric_launches(nT) + 1) * args.steps,
        "clocks": clk,
        "autotune": {"batch_vertices": tune["batch_slots"], "batch_corners": tune["batch_corners"],
                     "grid_blocks": tune["grid_blocks"], "fp64_tet_warps": tune["dag_warps"],
                     "default_ms": tune["default_ms"], "tuned_ms": tune["tuned_ms"],
                     "gain_vs_default": (tune["default_ms"] / tune["tuned_ms"]) if tune["tuned_ms"] else None,
                     "candidates": tune["candidates"]},
    }
    if world == 1 and (not args.no_cpu_baseline or args.precision == "fp32"):
        phi_o, _, ost = oracle_solve(case)
        cores = os.cpu_count()
        out["cpu_baseline"] = {"value": 1.0 / ost["solve_s"], "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": "one full solve of the same slab (metric + FIM) by the FP64 C oracle"}
        out["parity"] = parity_report(phi_dev, phi_o, "max |dt| <= 1e-4 max(t)" if args.precision == "fp32" else
                                      "max |dt| <= 1e-4 max(t); achieved bit-exact")
        if args.precision == "fp32":
            out["parity"]["within_tolerance"] = out["parity"]["max_rel_err"] <= 1e-4
    s.close()
    if world == 1 and args.workload == "slab" and args.cells is None and not args.no_extra:
        out["other_workloads"] = other_workloads(args)
    print(json.dumps(out), flush=True)


def other_workloads(args):
    """Short measurements of the other workload families in the same run, so
    that they are not only reported by separate invocations: the unit cube
    (bit-exact check against the oracle), the slab partitioned into 2,964
    submeshes with 50 windows, and a scaled batch of 32 uneven solves in one
    launch against the same solves one at a time.  Device time of the solves
    (the conduction is staged once), each configuration autotuned first."""
    import fim_api
    import fim_mesh
    from oracle import build as obuild
    from oracle import oracle as O
    obuild.build_oracle()
    res = {}
    reps = max(3, min(args.steps, 10))

    def timed(solver, n):
        ms = []
        for _ in range(n):
            solver.solve()
            ms.append(solver.stats()["solve_ms"])
        return float(np.median(ms))

    # unit cube (the plain FIM configuration)
    c = fim_mesh.cube_case(20)
    nV = c["xyz"].shape[0]
    with fim_api.Solver() as s:
        s.set_mesh(c["xyz"], c["tets"])
        s.set_conduction(c["fib"], c["cf"], c["ct"])
        s.set_stimuli(c["seed_v"], c["seed_t"])
        tune = s.autotune()
        ms = timed(s, reps)
        phi = s.times(with_state=False)
    slots, _, _, _ = O.reference_slots(nV, c["tets"], None)
    geo = O.metric_geo(slots, c["xyz"], c["fib"], c["cf"], c["ct"])
    phi_o, _, _, _ = O.solve_pure(nV, slots, geo, c["seed_v"], c["seed_t"])
    res["cube"] = {"workload": f"unit cube 20^3 Kuhn cells ({nV} vertices), isotropic 0.6, stimulus at the origin",
                   "solves_per_s": 1e3 / ms, "solve_ms": ms, "n_bit_mismatch_vs_oracle": int(np.count_nonzero(phi != phi_o)),
                   "autotune": {k: tune[k] for k in ("batch_slots", "batch_corners", "grid_blocks", "dag_warps")}}
    # the slab in submeshes and windows (the reference's operating mode)
    p = fim_mesh.slab_case(cells=SLAB_CELLS)
    tags = fim_mesh.block_tags(p["xyz"], p["tets"], PART_BLOCKS)
    with fim_api.Solver(dt=PART_DT, n_steps=PART_STEPS, apd=3e5) as s:
        s.set_mesh(p["xyz"], p["tets"], tags)
        s.set_conduction(p["fib"], p["cf"], p["ct"])
        s.set_stimuli(p["seed_v"], p["seed_t"])
        tune = s.autotune()
        ms = timed(s, max(3, reps // 2))
        st = s.stats()
    res["part"] = {"workload": (f"the 1.03M-vertex slab in {int(len(np.unique(tags)))} submeshes, {PART_STEPS} windows "
                                f"of {PART_DT} ms (bit-exact test: tests/test_gpu_tune.py; full check: bench.py "
                                "--workload part)"),
                   "solves_per_s": 1e3 / ms, "solve_ms": ms, "iterations": st["iterations"],
                   "vertex_updates": st["vertex_updates"], "submesh_sweeps_chosen": tune["submesh_sweeps"]}
    # a scaled batch: 32 solves over 8 uneven boxes in one launch
    meshes, solves = fim_mesh.batch_cases(n_meshes=8, n_solves=32, vmin=12_000, vmax=96_000)
    with fim_api.Batch() as b:
        for sv in solves:
            m = meshes[sv["mesh"]]
            b.add(m["xyz"], m["tets"], sv["fib"], sv["cf"], sv["ct"], sv["seed_v"], sv["seed_t"])
        b.autotune()
        bms = []
        for _ in range(reps):
            b.solve()
            bms.append(b.stats()["solve_ms"])
        bms = float(np.median(bms))
    seq = 0.0
    with fim_api.Solver() as s:
        cur = -1
        for sv in solves:
            m = meshes[sv["mesh"]]
            if sv["mesh"] != cur:
                s.set_mesh(m["xyz"], m["tets"])
                cur = sv["mesh"]
            s.set_conduction(sv["fib"], sv["cf"], sv["ct"])
            s.set_stimuli(sv["seed_v"], sv["seed_t"])
            s.solve()
            seq += s.stats()["solve_ms"]
    res["batch_scaled"] = {"workload": "32 solves over 8 jittered Kuhn boxes of 12k-96k vertices, one launch",
                           "solves_per_s": 32e3 / bms, "batch_ms": bms, "sequential_solves_per_s": 32e3 / seq,
                           "speedup_vs_sequential": seq / bms}
    return res


def run_reference(args):
    """The reference's algorithm on the host cores: the oracle port (the
    reference's own solver is CUDA-only; its CPU twins are commented out and
    its sources are not present on the GPU machine)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    case, cfg = workload(args)
    for _ in range(max(args.warmup, 0)):
        oracle_solve(case)
    t = 0.0
    for _ in range(args.steps):
        _, _, ost = oracle_solve(case)
        t += ost["solve_s"]
    value = args.steps / t
    cores = os.cpu_count()
    print(json.dumps({
        "impl": "reference", "metric": METRICS[args.workload], "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded slab mesh, conduction field and stimuli)", "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "one full solve of the slab per step (metric + FIM), FP64 C oracle, OpenMP"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def batch_workload(args):
    import fim_mesh
    nm, ns, vmin, vmax = (int(x) for x in args.batch.split(","))
    meshes, solves = fim_mesh.batch_cases(n_meshes=nm, n_solves=ns, vmin=vmin, vmax=vmax)
    probs = []
    for sv in solves:
        m = meshes[sv["mesh"]]
        probs.append(dict(mesh=sv["mesh"], xyz=m["xyz"], tets=m["tets"], fib=sv["fib"], cf=sv["cf"], ct=sv["ct"],
                          seed_v=sv["seed_v"], seed_t=sv["seed_t"]))
    nV = sum(p["xyz"].shape[0] for p in probs)
    nT = sum(p["tets"].shape[0] for p in probs)
    sizes = [m["xyz"].shape[0] for m in meshes]
    cfg = {"workload": (f"{ns} solves over {nm} jittered Kuhn boxes of {min(sizes)}-{max(sizes)} vertices "
                        f"(log-uniform in [{vmin}, {vmax}]); per solve cf~U[0.4,0.8], ct=cf*U[0.3,0.5], fibre "
                        "rotation +-U[40,70] deg over z, 1-8 surface stimuli t0~U[0,10] ms; one endless window"),
           "solves": ns, "meshes": nm, "vertices_total": nV, "tets_total": nT, "seed": 3,
           "l2": "inputs larger than L2", "parallelism": "one persistent launch for all solves"}
    return meshes, probs, cfg


def run_batch(args):
    """One step = one fim_batch_solve of every problem (the conduction fields
    are staged once, before the timed region)."""
    import torch
    import fim_api
    torch.cuda.set_device(0)
    meshes, probs, cfg = batch_workload(args)
    ns = len(probs)
    b = fim_api.Batch()
    for p in probs:
        b.add(p["xyz"], p["tets"], p["fib"], p["cf"], p["ct"], p["seed_v"], p["seed_t"])
    tune = b.autotune() if not args.no_autotune else None
    for _ in range(max(args.warmup, 0)):
        b.solve()
    clocks = ClockSampler(index=0)
    clocks.start()
    dev_ms, wall = [], time.perf_counter()
    for _ in range(args.steps):
        b.solve()
        dev_ms.append(b.stats()["solve_ms"])
    wall = time.perf_counter() - wall
    clk = clocks.stop()
    st = b.stats()
    # the same problems one fim_solve each (the plain cold-start GPU FIM)
    seq_ms = 0.0
    with fim_api.Solver() as s:
        cur = -1
        for p in probs:
            if p["mesh"] != cur:
                s.set_mesh(p["xyz"], p["tets"])
                cur = p["mesh"]
            s.set_conduction(p["fib"], p["cf"], p["ct"])
            s.set_stimuli(p["seed_v"], p["seed_t"])
            s.solve()
            seq_ms += s.stats()["solve_ms"]
    mean_ms = float(np.mean(dev_ms))
    out = {
        "metric": METRICS["batch"], "value": ns / (mean_ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Kuhn boxes, conduction draws and stimuli)",
        "config": cfg, "iterations": st["iterations"], "vertex_updates": st["vertex_updates"],
        "vertex_updates_per_s": st["vertex_updates"] / (mean_ms * 1e-3), "fp64_local_solves": st["exact_evals"],
        "sequential": {"value": ns / (seq_ms * 1e-3), "unit": UNIT,
                       "how": "the same problems, one fim_solve each (device time of the solves)"},
        "speedup_vs_sequential": seq_ms / mean_ms,
        "e2e": {"value": ns * args.steps / wall, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(12 * cfg["vertices_total"]),
                "how": "wall time of fim_batch_solve (launch + D2H of every problem's times and states)"},
        "gpu_launches": args.steps, "clocks": clk,
        "autotune": tune,
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        from oracle import build as obuild
        obuild.build_oracle()
        t_cpu, n_cpu, mism = 0.0, 0, 0
        order = sorted(range(ns), key=lambda i: probs[i]["xyz"].shape[0])
        for i in order[::max(1, ns // 16)]:
            p = probs[i]
            nV = p["xyz"].shape[0]
            slots, _, _, _ = O.reference_slots(nV, p["tets"], None)
            t0 = time.perf_counter()
            geo = O.metric_geo(slots, p["xyz"], p["fib"], p["cf"], p["ct"])
            phi_o, _, _, _ = O.solve_pure(nV, slots, geo, p["seed_v"], p["seed_t"])
            t_cpu += time.perf_counter() - t0
            n_cpu += 1
            mism += int(np.count_nonzero(b.times(i, with_state=False) != phi_o))
            if t_cpu > 20.0:
                break
        out["cpu_baseline"] = {"value": n_cpu / t_cpu, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                               "sample": f"{n_cpu} of the {ns} solves (sizes spread), FP64 C oracle, OpenMP"}
        out["parity"] = {"checked_solves": n_cpu, "n_bit_mismatch": mism}
    b.close()
    print(json.dumps(out), flush=True)


def run_mlp(args):
    """The warm-start network's tensor-core workload: the forward pass over
    one row per vertex of the 1M-vertex slab (padded to a multiple of 64
    rows; three tcgen05 GEMMs with fused bias + ReLU, then the output layer)
    and training steps of 4,096 rows (forward, backward with the weight
    gradients, Adam).  Features and targets are seeded synthetic values.
    Each call synchronises its stream, so the times are host wall-clock
    around the call; the GEMM kernels' own durations come from ncu."""
    import torch
    import fim_api
    torch.cuda.set_device(0)
    n = (1029018 + 63) // 64 * 64
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    keep = (torch.arange(64, device="cuda") < 7).to(torch.float32)
    X = (torch.randn(n, 64, device="cuda", generator=g) * keep).to(torch.bfloat16).contiguous()
    tgt = torch.rand(n, device="cuda", generator=g)
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    nb = 4096
    mlp = fim_api.Mlp(seed=5)
    for _ in range(max(args.warmup, 3)):
        mlp.predict(n, X.data_ptr(), y.data_ptr())
        mlp.train_step(nb, X.data_ptr(), tgt.data_ptr(), 1e-3)
    clocks = ClockSampler(index=0)
    clocks.start()
    tf, tt = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        mlp.predict(n, X.data_ptr(), y.data_ptr())
        tf.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        mlp.train_step(nb, X.data_ptr(), tgt.data_ptr(), 1e-3)
        tt.append(time.perf_counter() - t0)
    clk = clocks.stop()
    mlp.close()
    f_s, t_s = float(np.median(tf)), float(np.median(tt))
    gemm_flop = 2.0 * n * (64 * 128 + 2 * 128 * 128)
    # layers 1 and 2 read their input rows and write their BF16 output rows;
    # layer 3 reads H2 and writes only y (4 B per row)
    gemm_bytes = 2.0 * n * (64 + 128) + 2.0 * n * (128 + 128) + n * (2.0 * 128 + 4)
    out = {
        "metric": METRICS["mlp"], "value": n / f_s, "unit": "rows/s", "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": f_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 (FP32 accumulate)", "data": "synthetic (seeded features and targets)",
        "config": {"workload": f"network 7(64)->128->128->128->1, forward over {n} rows (the 1,029,018 slab "
                               f"vertices padded to a multiple of 64); training steps of {nb} rows",
                   "rows": n, "train_rows": nb},
        "forward_ms": f_s * 1e3, "train_step_ms": t_s * 1e3,
        "gemm": {"flop_per_forward": gemm_flop, "bytes_per_forward": gemm_bytes,
                 "tflops_lower_bound": gemm_flop / f_s * 1e-12, "gbs_lower_bound": gemm_bytes / f_s * 1e-9,
                 "note": "wall-clock of the whole synchronised call (3 GEMMs with the output layer fused into the "
                         "last, copy of y); the GEMM kernels are HBM-bound (64-128 FLOP per byte)"},
        "gpu_launches": 25 * args.steps, "clocks": clk,  # per step: forward 3, training step 22
        "e2e": {"value": None, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "how": "report line; the end-to-end number is the slab workload's"},
    }
    print(json.dumps(out), flush=True)


def run_warm(args):
    """Trains the warm-start network on FIM maps of small slabs of the bench
    family (generated by the solver), then solves held-out maps: one at a time
    cold (the plain cold-start GPU FIM), cold in one batched launch, and warm
    in one batched launch (start = 1.05 x the prediction, support-checked).
    Errors are reported against the cold solves and against the oracle's
    fixed point of the local solver (the truth a warm start approaches)."""
    import torch
    import fim_api
    import fim_warm
    from oracle import build as obuild
    from oracle import oracle as O
    obuild.build_oracle()
    torch.cuda.set_device(0)
    cells = (66, 23, 10)
    n_test = max(args.steps, 32)
    t0 = time.perf_counter()
    train_maps = fim_warm.make_maps(400, cells, 7, torch)
    gen_s = time.perf_counter() - t0
    test_maps = fim_warm.make_maps(n_test, cells, 8, torch)
    mlp = fim_api.Mlp(seed=5)
    t0 = time.perf_counter()
    losses = fim_warm.train(mlp, train_maps, steps=3000, batch=4096, lr=1e-3, torch=torch)
    train_s = time.perf_counter() - t0
    ev = fim_warm.evaluate(mlp, test_maps, torch)
    cold_single_ms = float(sum(m.cold["solve_ms"] for m in test_maps))
    starts = [torch.clamp(fim_warm.predict_times(mlp, m, torch) * 1.05, min=float(np.min(m.case["seed_t"])))
              for m in test_maps]
    d_start = torch.cat(starts).contiguous()
    torch.cuda.synchronize()
    b = fim_api.Batch()
    for m in test_maps:
        c = m.case
        b.add(c["xyz"], c["tets"], c["fib"], c["cf"], c["ct"], c["seed_v"], c["seed_t"])
    b.autotune()
    clocks = ClockSampler(index=0)
    clocks.start()
    cold_b, warm_b = [], []
    for _ in range(3):
        b.set_warm_start(None)
        b.solve()
        cold_b.append(b.stats()["solve_ms"])
        b.set_warm_start(d_start.data_ptr())
        b.solve()
        warm_b.append(b.stats()["solve_ms"])
    clk = clocks.stop()
    st_w = b.stats()
    err_cold, err_fp, below_fp = [], [], []
    for i, m in enumerate(test_maps):
        phi = b.times(i, with_state=False)
        c = m.case
        r = m.phi < 1e300
        tmax = m.phi[r].max()
        slots, _, _, _ = O.reference_slots(m.nV, c["tets"], None)
        geo = O.metric_geo(slots, c["xyz"], c["fib"], c["cf"], c["ct"])
        fp, _ = O.fixed_point(m.nV, slots, geo, c["seed_v"], c["seed_t"])
        err_cold.append(np.abs(phi - m.phi)[r] / tmax)
        err_fp.append(np.abs(phi - fp)[r] / tmax)
        below_fp.append(np.max((fp - phi)[r]) / tmax)
    b.close()
    mlp.close()
    ec, ef = np.concatenate(err_cold), np.concatenate(err_fp)
    cold_single = n_test / (cold_single_ms * 1e-3)
    cold_batched = n_test / (min(cold_b) * 1e-3)
    warm_batched = n_test / (min(warm_b) * 1e-3)
    nv = test_maps[0].nV
    out = {
        "metric": METRICS["warm"], "value": warm_batched, "unit": UNIT, "n_gpus": 1,
        "steps": 3, "warmup": 0, "ms_per_step": min(warm_b), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 solve, bf16 network",
        "data": "synthetic (FIM maps of seeded slabs generated by the solver)",
        "config": {"workload": (f"{n_test} held-out slabs {cells[0]}x{cells[1]}x{cells[2]} Kuhn cells ({nv} vertices), "
                                "random cf/ct/fibre/scar/stimuli, solved in one batched launch from the learned start; "
                                "network 7->128->128->128->1 trained on 400 maps, 3000 Adam steps of 4096 vertices; "
                                "start = 1.05 x prediction"), "train_maps": 400, "test_maps": n_test},
        "warm_batched_over_cold_single": {"value": warm_batched / cold_single,
                             "how": "warm-started batched solves/s / plain cold-start single-solve GPU FIM solves/s",
                             "cold_batched_over_cold_single": cold_batched / cold_single,
                             "warm_batched_over_cold_batched": warm_batched / cold_batched},
        "cold_single": {"value": cold_single, "unit": UNIT}, "cold_batched": {"value": cold_batched, "unit": UNIT},
        "warm_support_check": {"reset": st_w["warm_reset"], "rounds": st_w["warm_rounds"]},
        "warm_err_vs_cold": {"max_rel": float(ec.max()), "rms_rel": float(np.sqrt(np.mean(ec ** 2)))},
        "warm_err_vs_fixed_point": {"max_rel": float(ef.max()), "rms_rel": float(np.sqrt(np.mean(ef ** 2))),
                                    "max_below_rel": float(max(below_fp))},
        "network": ev, "train_loss_first_last": [float(np.mean(losses[:10])), float(np.mean(losses[-50:]))],
        "generation_s": gen_s, "training_s": train_s, "gpu_launches": 6, "clocks": clk,
        "e2e": {"value": None, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "how": "report line; the end-to-end number is the slab workload's"},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "warm":
        run_warm(args)
    elif args.workload == "mlp":
        run_mlp(args)
    else:
        run_mine(args)


if __name__ == "__main__":
    main()
