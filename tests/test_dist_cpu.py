"""Multi-rank logic of bench.py on CPU (gloo, world size 2): the barrier and
max/sum reductions used for whole-job timing, the ensemble sharding across
ranks, and the reference arm's single JSON line from rank 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, %r)
import bench
d = bench.Dist()
d.barrier()
out = {"rank": d.rank, "max": d.max(d.rank + 1.5), "sum": d.sum(d.rank + 1),
       "shard": bench.ensemble_shard(96, d.rank, d.world)}
d.barrier()
d.close()
print(json.dumps(out))
""" % ROOT


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def launch(cmd, world=2, timeout=180):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(r), WORLD_SIZE=str(world),
                   LOCAL_RANK=str(r))
        procs.append(subprocess.Popen(cmd, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                                      cwd=ROOT))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=timeout)
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_gloo_reductions_and_ensemble_shards():
    pytest.importorskip("torch")
    outs = [json.loads(o.strip().splitlines()[-1]) for o in launch([sys.executable, "-c", WORKER])]
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["max"] == 2.5
        assert o["sum"] == 3.0
    a, b = outs[0]["shard"], outs[1]["shard"]
    assert not set(a) & set(b)
    assert sorted(a + b) == list(range(96))


def test_reference_arm_prints_one_line_from_rank0():
    pytest.importorskip("torch")
    outs = launch([sys.executable, "bench.py", "--impl", "reference", "--steps", "3", "--warmup", "3", "--gpus", "2"],
                  timeout=300)
    lines = [l for o in outs for l in o.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "site-updates/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
