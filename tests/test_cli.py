"""The command line front end (fim_cli, the reference's flags of
src/main.cpp:170-237) on the reference's unit mesh: mesh, partition tags,
config and plan files in, the reference's result file out, byte for byte
equal to the reference's writer output of its golden solve."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG

CFG = "true\nfmm\nvol\nconst\ntrue\nfalse\nfrozen\n1.0\n1660\n"


def _write_mesh(path, xyz, tets, etags):
    """Legacy ASCII VTK with full-precision points (the reader's input format)."""
    n, m = xyz.shape[0], tets.shape[0]
    lines = ["# vtk DataFile Version 3.0", "vtk output", "ASCII", "DATASET UNSTRUCTURED_GRID",
             f"POINTS {n} double"]
    lines += [" ".join(repr(float(c)) for c in p) for p in xyz]
    lines += [f"CELLS {m} {5 * m}"] + ["4 " + " ".join(str(int(v)) for v in t) for t in tets]
    lines += [f"CELL_TYPES {m}"] + ["10"] * m
    lines += [f"CELL_DATA {m}", "SCALARS elemTag int 1", "LOOKUP_TABLE default"] + [str(int(e)) for e in etags]
    open(path, "w").write("\n".join(lines) + "\n")


def _plan(stim, dt_ms, steps):
    return json.dumps({
        "config": {"norm": {"func": "fnorm", "tags": [1]}},
        "functions": {"fnorm": {"CV": {"CVref": {"vf": 0.6, "vn": 0.6, "vs": 0.6}}, "EP": {"apd": 300.0}}},
        "simulation": {"deltatime": dt_ms, "timesteps": steps, "stimuli": {
            "S0": {"active": 1, "type": "Transmembrane Current",
                   "electrode": {"type": "vtxdata", "vtxdata": [int(v) for v in stim]},
                   "protocol": {"bcl": 1.0, "duration": 1.0, "npls": 1, "start": 0.0}}}},
    })


@pytest.mark.gpu
def test_cli_reproduces_golden_file(built_library, tmp_path):
    ut = np.load(os.path.join(GOLDEN, "ut_mesh.npz"))
    mesh, part, plan, cfg = (tmp_path / "m.vtk", tmp_path / "m.tags", tmp_path / "p.json", tmp_path / "d.cfg")
    _write_mesh(mesh, ut["xyz"], ut["tets"], ut["etags"])
    part.write_text("\n".join(str(t) for t in ut["tags"]) + "\n")
    plan.write_text(_plan(ut["stim"], float(ut["golden_dt"]) / 1000.0, int(ut["golden_steps"])))
    cfg.write_text(CFG)
    out = tmp_path / "cuda_fim_res.vtk"
    cli = os.path.join(PKG, "_build", "fim_cli")
    r = subprocess.run([cli, f"--mesh={mesh}", f"--part={part}", f"--plan={plan}", f"--odir={out}", "--reps=1",
                        f"--cfg={cfg}"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert out.read_bytes() == open(os.path.join(GOLDEN, "ut_mesh_written.vtk"), "rb").read()


def test_cli_usage_and_errors(built_library, tmp_path):
    """Without a GPU: usage text, and a clean non-zero exit on a missing mesh."""
    cli = os.path.join(PKG, "_build", "fim_cli")
    r = subprocess.run([cli, "--help"], capture_output=True, text=True, timeout=60)
    assert "usage: fim_cli" in r.stdout
    r = subprocess.run([cli, f"--mesh={tmp_path / 'none.vtk'}", f"--part={tmp_path / 'none.tags'}",
                        f"--plan={tmp_path / 'none.json'}", f"--odir={tmp_path / 'o.vtk'}"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
