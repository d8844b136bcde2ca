"""The drop-in class tw::CudaSolverFIM against the reference's real types.

oracle/ref_types_driver.cpp runs the reference's own pipeline (tw::run,
src/main.cpp:84-104) -- its load_vtk, read_vector_txt, compute_base_
connectivity, ek_data, load_options and load_plan, compiled from its
sources -- with this repository's drop-in solver class in place of the
reference's.  Needs the reference tree (built here, not on the GPU machine):
  * stage: what the class extracts from the reference's ek_data equals the
    unit mesh, partition and plan as the reference's own readers give them
    (tests/golden/ut_mesh.npz);
  * solve: the same binary goes on into the C ABI (without a GPU it stops
    at fim_create with FIM_ERR_NO_DEVICE, reported as an error, not a
    crash)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.build import reference_root


@pytest.fixture(scope="module")
def driver(built_library):
    from oracle import build as obuild
    ref = reference_root()
    if not os.path.isdir(os.path.join(ref, "src", "eikonal")):
        pytest.skip("reference tree not present")
    path = obuild.build_ref_driver(ref)
    if path is None:
        pytest.skip("driver not built")
    return path


def _inputs():
    d = os.path.join(reference_root(), "data")
    return [os.path.join(d, "ut_mesh", "ut_mesh.vtk"), os.path.join(d, "ut_mesh", "ut_mesh.tags"),
            os.path.join(d, "default.cfg"), os.path.join(d, "ut_mesh", "ut_mesh.plan.json")]


def _read_dump(path):
    b = open(path, "rb").read()
    nV, nT, na, ne, ns, steps = np.frombuffer(b[:48], np.int64)
    dt = float(np.frombuffer(b[48:56], np.float64)[0])
    off = 56
    out = {"n_steps": int(steps), "dt": dt}
    for name, dtype, n in (("xyz", np.float64, 3 * nV), ("tets", np.int64, 4 * nT), ("atags", np.int32, na),
                           ("etags", np.int32, ne), ("fib", np.float64, 3 * nT), ("cf", np.float64, nT),
                           ("ct", np.float64, nT), ("stim", np.int64, ns)):
        a = np.frombuffer(b[off:off + np.dtype(dtype).itemsize * int(n)], dtype)
        out[name] = a
        off += a.nbytes
    assert off == len(b)
    out["xyz"] = out["xyz"].reshape(-1, 3)
    out["tets"] = out["tets"].reshape(-1, 4)
    out["fib"] = out["fib"].reshape(-1, 3)
    return out


def test_shim_stages_the_reference_ek_data(driver, tmp_path):
    dump = str(tmp_path / "stage.bin")
    r = subprocess.run([driver, "stage"] + _inputs() + [dump], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    got = _read_dump(dump)
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    assert np.array_equal(got["xyz"], ut["xyz"])
    # compute_base_connectivity sorts every tet's vertex ids (types.cpp:63-67)
    assert np.array_equal(got["tets"], np.sort(ut["tets"], axis=1))
    assert np.array_equal(got["atags"], ut["tags"]) and np.array_equal(got["etags"], ut["etags"])
    assert got["dt"] == float(ut["plan_dt"]) and got["n_steps"] == int(ut["plan_steps"])
    assert got["stim"].tolist() == ut["stim"].tolist()
    # fibre (1,0,0) per tet (load_vtk, vtk.cpp:99-101); speeds from the plan's CVref
    assert np.array_equal(got["fib"], np.tile([1.0, 0.0, 0.0], (got["tets"].shape[0], 1)))
    assert np.all(got["cf"] == ut["plan_cv"][0]) and np.all(got["ct"] == ut["plan_cv"][1])


def test_shim_solves_through_the_c_abi(driver, tmp_path):
    import torch
    out = str(tmp_path / "out.vtk")
    r = subprocess.run([driver, "solve"] + _inputs() + [out], capture_output=True, text=True, cwd=str(tmp_path))
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
        import fim_api as F
        xyz, tets, _ = F.vtk_read(out)
        assert xyz.shape[0] == 232 and tets.shape[0] == 632
    else:
        assert r.returncode == 1 and "no CUDA device" in r.stderr, (r.returncode, r.stderr)
