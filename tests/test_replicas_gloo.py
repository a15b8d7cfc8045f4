"""Replicas across ranks (bench.py --gpus N under torchrun): each rank solves
its own batch of solves, nothing is exchanged inside a step, and rank 0
reports the whole job's facet-steps over the slowest rank's device time.  The
rank plumbing of bench.py -- process group set-up, barrier, max and sum over
ranks, the whole-job value, and the reference arm's rule that only rank 0
runs and prints -- runs here as two gloo ranks on the CPU."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

RANK_SCRIPT = r"""
import argparse, contextlib, io, json, sys
sys.path.insert(0, sys.argv[1])
import torch
import bench

bench._cuda = lambda: False  # gloo on the CPU even where a GPU is visible
world, rank, local, dist = bench.dist_setup()
dev = torch.device("cpu")
ms = 100.0 * (rank + 1)      # this rank's device time for its steps
fs = 1.0e9 * (rank + 1)      # the facet-steps it advanced
bench._barrier(dist)
ms_max = bench._max_over_ranks(ms, dist, dev)
fs_all = bench._sum_over_ranks(fs, dist, dev)
out = io.StringIO()
if rank != 0:
    with contextlib.redirect_stdout(out):
        bench.run_reference_arm(argparse.Namespace(steps=1, warmup=0, gpus=world), world, rank)
bench._barrier(dist)
dist.destroy_process_group()
print(json.dumps({"world": world, "rank": rank, "local": local, "ms_max": ms_max, "fs_all": fs_all,
                  "value": fs_all / (ms_max / 1e3), "reference_arm_output": out.getvalue()}))
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_report_the_whole_job_over_the_slowest_rank():
    world, port = 2, _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                   RANK=str(rank), LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, str(ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            so, se = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, se[-2000:]
        outs.append(json.loads(so.strip().splitlines()[-1]))
    for rank, o in enumerate(outs):
        assert (o["world"], o["rank"], o["local"]) == (world, rank, rank)
        assert o["ms_max"] == 200.0            # the slowest rank's time
        assert o["fs_all"] == 3.0e9            # every rank's facet-steps
        assert o["value"] == 3.0e9 / 0.2       # whole job: sum over ranks / max time
    assert outs[1]["reference_arm_output"] == ""  # only rank 0 runs the reference arm
