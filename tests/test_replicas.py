"""The multi-GPU form of the benchmark is N independent replicas (the path
has no exchange step): each rank times its own propagations, the job's time is
the maximum over ranks, and the value counts the steps of all replicas.  The
reference arm runs on rank 0 only.  These are checked here with two gloo ranks
on the CPU (127.0.0.1), one process each, as torchrun would start them.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, os, sys, io, contextlib, argparse
sys.path.insert(0, sys.argv[1])
import bench
rank, world, local = bench.dist_init(2)
import torch.distributed as dist
mx = bench.max_over_ranks(10.0 * rank + 1.0, world)
val = bench.replica_value(65536, mx, world)
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    if rank != 0:
        bench.run_reference(argparse.Namespace(steps=1, warmup=0, steps_per_prop=4, gpus=2), rank, world)
dist.barrier()
print(json.dumps({"rank": rank, "world": world, "max": mx, "value": val, "ref_out": buf.getvalue()}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2
        assert o["max"] == 11.0                      # the slower rank's time
        assert abs(o["value"] - 2 * 65536 / 11e-3) < 1e-6 * o["value"]
    assert outs[1]["ref_out"] == ""                  # the reference arm prints on rank 0 only
