"""The multi-GPU layout is replicas only: under torchrun every rank runs the same apply on its
own GPU and the job time is the slowest rank's.  The host-side logic of that (bench.py's
replica_reduce / replica_value, and the reference arm's rank-0-only rule) runs here on CPU with
world_size 2 over gloo."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

WORKER = r'''
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
ms = 10.0 + 5.0 * rank                      # rank 1 is the slow replica
job = bench.replica_reduce(ms, world)
val = bench.replica_value(6.0e9, world, job)
print(json.dumps({"rank": rank, "job_ms": job, "value": val}), flush=True)
dist.destroy_process_group()
'''


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(script_args, nproc=2):
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    outs = []
    procs = []
    for r in range(nproc):
        e = dict(env, RANK=str(r), WORLD_SIZE=str(nproc), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable] + script_args, env=e, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_replica_job_time_is_the_slowest_rank(tmp_path):
    w = tmp_path / "worker.py"
    w.write_text(WORKER)
    outs = _launch([str(w), str(ROOT)])
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert {r["rank"] for r in res} == {0, 1}
    for r in res:
        assert r["job_ms"] == 15.0                       # max over ranks, on every rank
        assert abs(r["value"] - 2 * 6.0e9 / 15e-3) < 1.0  # all ranks' work / slowest time


def test_reference_arm_runs_on_rank_zero_only(tmp_path):
    """bench.py --impl reference under a 2-rank launch: rank 1 exits 0 without output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--m", "64", "--n", "65", "--k", "2"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=120)
    assert p.returncode == 0 and p.stdout.strip() == ""
