"""The N > 1 path of bench.py on CPU: two gloo ranks.

Every rank renders its own seeded instances (weak scaling, no exchange of
data); the job's time is the slowest rank's (max over ranks) and its rate
counts the paths of all ranks; the reference arm prints from rank 0 only.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["ROOT"])
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="tcp://127.0.0.1:" + os.environ["PORT"],
                        rank=int(os.environ["RANK"]), world_size=int(os.environ["WORLD_SIZE"]))
rank = dist.get_rank()
insts, desc = bench.workload("batch64", rank)
seeds = [i.seed for i in insts[:4]]
sizes = [(i.camera.width, i.camera.height, i.camera.spp) for i in insts[:4]]
t = bench.max_over_ranks(1.0 + rank, dist)          # rank r took 1 + r seconds
paths = sum(bench.instance_paths(i) for i in insts)
print(json.dumps({"rank": rank, "seeds": seeds, "sizes": sizes, "t": t, "paths": paths,
                  "rate": bench.job_rate(paths, dist.get_world_size(), t)}))
dist.destroy_process_group()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_gloo_ranks_weak_scaling(tmp_path):
    script = tmp_path / "worker.py"
    script.write_text(WORKER)
    port = str(_free_port())
    procs = []
    for r in range(2):
        env = dict(os.environ, ROOT=ROOT, PORT=port, RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    a, b = sorted(outs, key=lambda o: o["rank"])
    # each rank has its own instances
    assert a["seeds"] != b["seeds"] and a["sizes"] != b["sizes"]
    # both ranks see the slowest rank's time; the rate counts both ranks' paths
    assert a["t"] == b["t"] == 2.0
    assert a["rate"] == pytest.approx(a["paths"] * 2 / 2.0 / 1e6)


def test_reference_arm_other_ranks_print_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
