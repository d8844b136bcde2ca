"""Host-side checks of the C ABI library that need no GPU: it loads, exports
every symbol include/fim.h declares, its file formats match the reference's
readers/writers, and it reports (not crashes on) a missing device."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from oracle.build import reference_root


@pytest.fixture(scope="module")
def F(built_library):
    import fim_api
    fim_api.lib()
    return fim_api


def test_exports_every_declared_symbol(F):
    header = open(os.path.join(ROOT, "include", "fim.h")).read()
    declared = set(re.findall(r"^(?:const\s+)?\w+\s*\*?\s*(fim_[a-z0-9_]+)\s*\(", header, re.M))
    assert declared, "no declarations found"
    L = F.lib()
    for name in sorted(declared):
        assert hasattr(L, name), name
    assert set(F.EXPORTS) <= declared


def test_vtk_writer_is_byte_compatible(F, tmp_path):
    """fim_vtk_write == the reference's save_vtk (src/io/vtk.cpp:109-211)."""
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    phi = np.where(ut["golden_phi"] < 0, F.INF, ut["golden_phi"])
    out = tmp_path / "w.vtk"
    F.vtk_write(str(out), ut["xyz"], np.sort(ut["tets"], axis=1), ut["etags"], phi, ut["golden_states"])
    assert out.read_bytes() == open(os.path.join(GOLDEN, "ut_mesh_written.vtk"), "rb").read()


def test_vtk_reader_roundtrip(F, tmp_path):
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    out = tmp_path / "m.vtk"
    F.vtk_write(str(out), ut["xyz"], ut["tets"], ut["etags"])
    xyz, tets, et = F.vtk_read(str(out))
    assert np.array_equal(tets, ut["tets"]) and np.array_equal(et, ut["etags"])
    assert np.allclose(xyz, ut["xyz"], atol=1e-3)  # the writer prints %.3f floats


def test_vtk_reader_matches_reference_on_source_mesh(F):
    path = os.path.join(reference_root(), "data", "ut_mesh", "ut_mesh.vtk")
    if not os.path.exists(path):
        pytest.skip("reference data not present")
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    xyz, tets, et = F.vtk_read(path)
    assert np.array_equal(xyz, ut["xyz"]) and np.array_equal(tets, ut["tets"]) and np.array_equal(et, ut["etags"])


def test_vtk_reader_rejects_bad_files(F, tmp_path):
    p = tmp_path / "bad.vtk"
    p.write_text("# vtk DataFile Version 2.0\nx\nASCII\nDATASET UNSTRUCTURED_GRID\nPOINTS 2 double\n0 0 0\n")
    with pytest.raises(F.FimError) as e:
        F.vtk_read(str(p))
    assert e.value.code == 6
    p.write_text("# vtk DataFile Version 2.0\nx\nASCII\nDATASET UNSTRUCTURED_GRID\nPOINTS 1 double\n0 0 0\n"
                 "CELLS 1 4\n3 0 0 0\n")
    with pytest.raises(F.FimError):
        F.vtk_read(str(p))
    with pytest.raises(F.FimError):
        F.vtk_read(str(tmp_path / "missing.vtk"))


def test_tags_reader(F, tmp_path):
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    p = tmp_path / "t.tags"
    p.write_text("\n".join(str(t) for t in ut["tags"]) + "\n")
    assert np.array_equal(F.read_tags(str(p)), ut["tags"])
    p.write_text("1\n2\nx\n")
    with pytest.raises(F.FimError):
        F.read_tags(str(p))


CFG = "true\nfmm\nvol\nconst\ntrue\nfalse\nfrozen\n1.0\n1660\n"


def _plan(stimuli, dt=150.0, steps=4, cv=0.6):
    import json
    return json.dumps({
        "config": {"norm": {"func": "fnorm", "tags": [1, 2, 3, 4]}},
        "functions": {"fnorm": {"CV": {"CVref": {"vf": cv, "vn": cv, "vs": cv * 0.5}}, "EP": {"apd": 300.0}}},
        "simulation": {"deltatime": dt, "timesteps": steps, "stimuli": stimuli},
    })


def _stim(vtx, active=1, start=0.0, npls=1, bcl=1.0):
    return {"active": active, "type": "Transmembrane Current",
            "electrode": {"type": "vtxdata", "vtxdata": vtx},
            "protocol": {"bcl": bcl, "duration": 1.0, "npls": npls, "start": start}}


def test_plan_loader(F, tmp_path):
    cfg = tmp_path / "default.cfg"
    cfg.write_text(CFG)
    plan = tmp_path / "p.json"
    plan.write_text(_plan({"S0": _stim([9, 8, 53]), "S1": _stim([1, 2], active=0), "S2": _stim([4], npls=2)}))
    info = F.load_plan(str(cfg), str(plan))
    assert info["dt"] == 150000.0 and info["n_steps"] == 4
    assert info["n_events"] == 3  # S0 + two pulses of S2
    assert info["stim"].tolist() == [9, 8, 53, 4, 4]
    assert info["cv"] == (0.6, 0.3, 0.6)
    plan.write_text(_plan({"S0": dict(_stim([1]), type="Bogus")}))
    with pytest.raises(F.FimError):
        F.load_plan(str(cfg), str(plan))
    plan.write_text("{ not json")
    with pytest.raises(F.FimError):
        F.load_plan(str(cfg), str(plan))
    cfg.write_text("maybe\n" + CFG[5:])
    with pytest.raises(F.FimError):
        F.load_plan(str(cfg), str(plan))


def test_plan_loader_matches_reference(F):
    ref = reference_root()
    cfg, plan = os.path.join(ref, "data", "default.cfg"), os.path.join(ref, "data", "ut_mesh", "ut_mesh.plan.json")
    if not os.path.exists(plan):
        pytest.skip("reference data not present")
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    info = F.load_plan(cfg, plan)
    assert info["dt"] == float(ut["plan_dt"]) and info["n_steps"] == int(ut["plan_steps"])
    assert info["n_events"] == int(ut["plan_events"]) and info["tstart"] == float(ut["plan_tstart"])
    assert info["stim"].tolist() == ut["stim"].tolist()
    assert info["cv"] == tuple(ut["plan_cv"])


def test_create_reports_missing_device(F):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(F.FimError) as e:
        F.Solver()
    assert e.value.code == 8
