"""bench.py's multi-rank bookkeeping on CPU with gloo, world size 2: every
rank renders its own replica (the path needs no cross-GPU exchange), the
step time is the maximum over ranks, and only rank 0 reports.  The
reference arm under torchrun: ranks other than 0 exit without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["REPO"])
import torch.distributed as dist
import bench
world, rank, local = bench.dist_setup()
assert world == 2 and dist.get_backend() == "gloo"
t = bench.reduce_max(10.0 + 5.0 * rank, world)
bench.barrier(world)
print(json.dumps({"rank": rank, "max": t}), flush=True)
dist.destroy_process_group()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _launch(code, world=2, extra_env=None):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, REPO=REPO, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=180)
        assert p.returncode == 0, e[-2000:]
        outs.append(o)
    return outs


def test_max_over_ranks_with_gloo():
    outs = _launch(WORKER)
    lines = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(l["rank"] for l in lines) == [0, 1]
    assert all(l["max"] == 15.0 for l in lines)


def test_reference_arm_other_ranks_do_no_work():
    """A rank other than 0 of the reference arm returns at once, printing nothing."""
    code = ("import os, sys; sys.path.insert(0, os.environ['REPO']); import bench; "
            "sys.argv = ['bench.py', '--impl', 'reference', '--gpus', '2', '--steps', '1', '--warmup', '0']; "
            "bench.main()")
    env = dict(os.environ, REPO=REPO, RANK="1", LOCAL_RANK="1", WORLD_SIZE="1", CUDA_VISIBLE_DEVICES="")
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=180)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
