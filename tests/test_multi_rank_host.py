"""Multi-process host logic of bench.py on CPU: two gloo ranks (world size 2).

The path does not shard a propagation: on N GPUs each rank steps its own shard of the
batched instance list (balanced by Nr x Ntheta, computed alike on every rank), and the only
cross-rank work is the timing barrier and the max-over-ranks of the timed region.  These
tests run that logic, and the reference arm's rank-0-only rule, as real processes."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
world, rank, _ = bench.dist_setup()
bench.barrier(world)
m = bench.allmax(world, float(10 * (rank + 1)))
bench.barrier(world)
import torch.distributed as dist
dist.destroy_process_group()
print(json.dumps({"rank": rank, "world": world, "max": m}))
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch(cmd, world, extra_env=None, timeout=240):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, WORLD_SIZE=str(world), RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), SO_BENCH_GLOO="1", **(extra_env or {}))
        procs.append(subprocess.Popen(cmd, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    outs = []
    for p in procs:
        try:
            o, e = p.communicate(timeout=timeout)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        outs.append((p.returncode, o, e))
    return outs


def test_barrier_and_max_over_ranks_with_gloo():
    outs = launch([sys.executable, "-c", RANK_SCRIPT, ROOT], 2)
    res = []
    for rc, o, e in outs:
        assert rc == 0, e[-2000:]
        res.append(json.loads(o.strip().splitlines()[-1]))
    assert sorted(r["rank"] for r in res) == [0, 1]
    assert all(r["world"] == 2 and r["max"] == 20.0 for r in res)


def test_reference_arm_prints_on_rank_zero_only():
    pytest.importorskip("torch")
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "10", "--warmup", "1",
           "--cpu-seconds", "0.5"]
    outs = launch(cmd, 2)
    (rc0, o0, e0), (rc1, o1, e1) = outs
    assert rc0 == 0, e0[-2000:]
    assert rc1 == 0, e1[-2000:]
    assert o1.strip() == ""
    line = json.loads(o0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


SHARD_SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
from split_operator_gb300 import shards, workloads as W
world, rank, _ = bench.dist_setup()
per_rank = 64
params = W.batched_instance_params(per_rank * world)
mine, total = shards.shard(params, world, rank)
import torch.distributed as dist
got = [None] * world
dist.all_gather_object(got, [p["seed"] for p in mine])

class A:
    workload = "batched"
    instances = per_rank
job = bench.global_points(A, world, sum(p["nr"] * p["nth"] for p in mine))
dist.destroy_process_group()
print(json.dumps({"rank": rank, "seeds": got, "total": total, "job": job,
                  "cost": sum(shards.instance_cost(p) for p in mine)}))
"""


def test_instance_shards_cover_the_list_once_and_balance():
    """Two ranks take disjoint shards whose union is the whole instance list; every rank
    computes the same partition without exchanging it; the costs differ by less than the
    largest instance (longest processing time first); the job's points are the list's."""
    pytest.importorskip("torch")
    outs = launch([sys.executable, "-c", SHARD_SCRIPT, ROOT], 2)
    res = []
    for rc, o, e in outs:
        assert rc == 0, e[-2000:]
        res.append(json.loads(o.strip().splitlines()[-1]))
    res.sort(key=lambda r: r["rank"])
    from split_operator_gb300 import shards, workloads as W
    params = W.batched_instance_params(128)
    assert res[0]["seeds"] == res[1]["seeds"]  # both ranks saw the same gathered partition
    s0, s1 = res[0]["seeds"]
    assert not set(s0) & set(s1) and sorted(s0 + s1) == [p["seed"] for p in params]
    biggest = max(shards.instance_cost(p) for p in params)
    assert abs(res[0]["cost"] - res[1]["cost"]) <= biggest
    assert res[0]["job"] == res[1]["job"] == res[0]["total"] == sum(p["nr"] * p["nth"] for p in params)


def test_partition_is_deterministic_and_balanced():
    from split_operator_gb300 import shards
    costs = [5, 9, 1, 9, 3, 7, 2, 8, 4, 6]
    parts = shards.partition(costs, 3)
    assert parts == shards.partition(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert shards.partition(costs, 1) == [list(range(len(costs)))]
    with pytest.raises(ValueError):
        shards.partition(costs, 0)
