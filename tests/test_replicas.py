"""The bench's multi-GPU path is replicas only: under torchrun every rank runs
the same single-GPU workload, the step time is the slowest rank's (an
all-reduce MAX) and the whole-job value counts one circuit per rank per step.
Checked on the CPU with world size 2 over gloo (127.0.0.1 rendezvous), through
bench.py's own functions; and a non-zero rank of the reference arm exits
without work (rank 0 alone times the reference's CPU algorithm)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = """
import json, os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
rank = int(os.environ["RANK"])
values = [1234.5, 2345.25]
m = bench.max_over_ranks(values[rank], 2, "cpu")
print(json.dumps({{"rank": rank, "max": m, "value": bench.whole_job_seconds_per_circuit(m, 2)}}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_world_2_gloo():
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                   LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=180)
            assert p.returncode == 0, err
            outs.append(json.loads(out.strip().splitlines()[-1]))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["max"] == 2345.25  # the slower replica's step time, on every rank
        assert o["value"] == 2345.25 / 1e3 / 2  # two circuits per 2.345 s step


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.whole_job_seconds_per_circuit(4000.0, 1) == 4.0


def test_reference_arm_runs_on_rank_0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
