"""The multi-process path of bench.py on CPU (gloo, world size 2): replicas
meet at the barrier, the timed value is the maximum over ranks, and the
reference arm prints its one line from rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


WORKER = r"""
import os, sys
sys.path.insert(0, {root!r})
import bench
world, rank, local, pg = bench.dist_setup(None)
assert world == 2 and pg is not None
bench.barrier(pg)
v = bench.max_over_ranks(pg, 1.5 + rank)
open(os.path.join({out!r}, "rank%d.txt" % rank), "w").write("RANK %d MAX %s" % (rank, v))
pg.destroy_process_group()
"""


def test_max_over_ranks_gloo(tmp_path):
    pytest.importorskip("torch")
    w = tmp_path / "w.py"
    w.write_text(WORKER.format(root=ROOT, out=str(tmp_path)))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr=127.0.0.1", f"--master-port={_free_port()}", str(w)],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [(tmp_path / f"rank{k}.txt").read_text() for k in range(2)]
    assert lines == ["RANK 0 MAX 2.5", "RANK 1 MAX 2.5"]


def test_reference_arm_rank0_only(tmp_path):
    """--impl reference under torchrun: one JSON line (rank 0), every rank exits 0."""
    pytest.importorskip("torch")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr=127.0.0.1", f"--master-port={_free_port()}",
                        os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0", "--cells", "8,4,3"],
                       capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    js = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(js) == 1
    line = js[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
