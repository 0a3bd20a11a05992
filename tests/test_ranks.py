"""The N > 1 path of bench.py on the CPU, as world-size-2 gloo process groups
(127.0.0.1).  The sheet does not shard, so N ranks run N independent
replicas with no data-path collective; the only exchange is the reduction of
each rank's timed interval to its maximum, from which rank 0 reports the
whole job's steps/s.  The reference arm runs on rank 0 alone; the other
ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["BENCH_ROOT"])
import torch
import torch.distributed as dist
import bench
rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo")
own = json.loads(os.environ["RANK_MS"])[rank]
total = bench.max_over_ranks(own, world, torch.device("cpu"))
dist.barrier()
print(json.dumps({"rank": rank, "own": own, "total": total,
                  "rate": bench.job_rate(world, 10, total)}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(world, env_extra, argv, timeout=120):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), BENCH_ROOT=ROOT,
                   CUDA_VISIBLE_DEVICES="", **env_extra)
        procs.append(subprocess.Popen(argv, env=env, cwd=ROOT, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
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


def test_timed_interval_is_the_slowest_rank():
    per_rank = [120.0, 80.0]
    outs = _run_ranks(2, {"RANK_MS": json.dumps(per_rank)}, [sys.executable, "-c", WORKER])
    got = []
    for rc, o, e in outs:
        assert rc == 0, e
        got.append(json.loads(o.strip().splitlines()[-1]))
    for g in got:
        assert g["own"] == per_rank[g["rank"]]
        assert g["total"] == max(per_rank)  # every rank sees the maximum
        assert abs(g["rate"] - 2 * 10 / 0.120) < 1e-9  # 20 steps over the slowest 120 ms


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(42.0, 1, None) == 42.0
    assert bench.job_rate(1, 10, 500.0) == 20.0


def test_reference_arm_runs_on_rank_zero_only():
    """Rank 1 of a two-rank reference run returns at once, prints nothing
    and exits 0 (rank 0's sheet-sized oracle step is not run here)."""
    port = _free_port()
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


SHARD_WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["BENCH_ROOT"])
for sub in ("oracle", "tests", "eol-cloth_gb300"):
    sys.path.insert(0, os.path.join(os.environ["BENCH_ROOT"], sub))
import numpy as np
import torch.distributed as dist
import bench, scenes, oracle as O
rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo")
B = scenes.batch(9, lo=3, hi=10, seed=4)
mine = bench.shard_instances([s["n"] for s in B["sheets"]], world)[rank]
S = bench.sub_batch(B, mine)
part = []
for j, k in enumerate(mine):
    s, m = S["sheets"][j], S["mats"][j]
    o = S["node_off"]
    x, v = S["x"][3 * o[j]:3 * o[j + 1]].copy(), S["v"][3 * o[j]:3 * o[j + 1]].copy()
    for _ in range(2):
        O.step(x, s["X"], v, s["tri"], s["hinge"], O.material(**m), scenes.GRAV, scenes.H,
               s["fixed"], s["fixed_vel"], tol=1e-10)
    part.append((k, x.tobytes().hex() + ":" + v.tobytes().hex()))
parts = [None] * world
dist.all_gather_object(parts, part)
merged = bench.merge_shards(len(B["sheets"]), parts)
print(json.dumps({"rank": rank, "mine": mine, "merged": merged}))
dist.destroy_process_group()
"""


def test_batched_instances_shard_across_ranks():
    """World size 2: the batch is split by instance (node-count balanced),
    every instance is stepped exactly once, and the merged states equal a
    single rank stepping every instance, bit for bit (here with the oracle's
    step on the CPU standing in for the GPU's batched step)."""
    outs = _run_ranks(2, {}, [sys.executable, "-c", SHARD_WORKER], timeout=300)
    got = []
    for rc, o, e in outs:
        assert rc == 0, e
        got.append(json.loads(o.strip().splitlines()[-1]))
    mine = [g["mine"] for g in sorted(got, key=lambda g: g["rank"])]
    assert sorted(mine[0] + mine[1]) == list(range(9)) and not set(mine[0]) & set(mine[1])
    assert got[0]["merged"] == got[1]["merged"]
    sys.path.insert(0, ROOT)
    for sub in ("oracle", "tests", "eol-cloth_gb300"):
        sys.path.insert(0, os.path.join(ROOT, sub))
    import oracle as O
    import scenes
    B = scenes.batch(9, lo=3, hi=10, seed=4)
    off = B["node_off"]
    for k, s in enumerate(B["sheets"]):
        x = B["x"][3 * off[k]:3 * off[k + 1]].copy()
        v = B["v"][3 * off[k]:3 * off[k + 1]].copy()
        for _ in range(2):
            O.step(x, s["X"], v, s["tri"], s["hinge"], O.material(**B["mats"][k]), scenes.GRAV,
                   scenes.H, s["fixed"], s["fixed_vel"], tol=1e-10)
        assert got[0]["merged"][k] == x.tobytes().hex() + ":" + v.tobytes().hex()


def test_shard_split_is_balanced_and_deterministic():
    sys.path.insert(0, ROOT)
    import bench
    sizes = [100, 90, 80, 10, 10, 10, 5]
    a = bench.shard_instances(sizes, 2)
    assert a == bench.shard_instances(sizes, 2)
    loads = [sum(sizes[k] for k in part) for part in a]
    assert abs(loads[0] - loads[1]) <= max(sizes)
    assert sorted(a[0] + a[1]) == list(range(len(sizes)))
    assert bench.shard_instances(sizes, 1) == [list(range(len(sizes)))]
    import pytest
    with pytest.raises(ValueError):
        bench.merge_shards(2, [[(0, 1)], [(0, 1), (1, 2)]])
    with pytest.raises(ValueError):
        bench.merge_shards(3, [[(0, 1)], [(1, 2)]])
