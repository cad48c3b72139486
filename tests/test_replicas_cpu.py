"""The N > 1 form of bench.py on CPU (gloo, world size 2, 127.0.0.1).

The path does not shard: a replica run gives every rank its own realisation
(seed + rank) and exchanges nothing on the data path, only the step time
(max over ranks: the slowest rank sets the job's time) and the rods placed
(sum over ranks). These tests run that exchange under torchrun with gloo, and
the reference arm under torchrun, where rank 0 alone runs the CPU path and
prints the one JSON line while the other ranks exit 0 without output.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = """
import json, os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r, w = dist.get_rank(), dist.get_world_size()
params, _ = bench.workload("small", r)
out = {{"rank": r, "world": w, "seed": params["seed"],
        "max": bench.over_ranks(dist, 1.5 + r, "max", "cpu"),
        "sum": bench.over_ranks(dist, 10 + r, "sum", "cpu")}}
dist.barrier()
dist.destroy_process_group()
with open(os.path.join({out!r}, "r%d.json" % r), "w") as f:
    json.dump(out, f)
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, cwd, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=cwd, env=env, capture_output=True, text=True, timeout=timeout)


def test_over_ranks_without_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.over_ranks(None, 3.25, "max", "cpu") == 3.25
    assert bench.over_ranks(None, 7, "sum", "cpu") == 7


def test_replica_exchange_gloo(tmp_path):
    script = tmp_path / "worker.py"
    script.write_text(WORKER.format(root=ROOT, out=str(tmp_path)))
    r = torchrun([str(script)], cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    res = [json.loads((tmp_path / f"r{i}.json").read_text()) for i in range(2)]
    for i, o in enumerate(res):
        assert o["rank"] == i and o["world"] == 2
        assert o["max"] == 2.5  # the slowest rank's time, on every rank
        assert o["sum"] == 21.0  # rods of both replicas
    assert res[1]["seed"] == res[0]["seed"] + 1  # independent realisations


def test_reference_arm_under_torchrun(tmp_path):
    r = torchrun([os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                  "--warmup", "1", "--workload", "small"], cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    o = json.loads(lines[0])
    assert o["impl"] == "reference" and o["n_gpus"] == 2 and o["steps"] == 1
    assert o["value"] > 0 and o["unit"] == "rods/s" and o["higher_is_better"] is True
    assert o["e2e"] == {"value": o["value"], "unit": "rods/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert o["cpu_baseline"]["kind"] == "port" and o["cpu_baseline"]["cores"] >= 1
    assert o["config"]["workload"] == "small"


def test_both_arms_print_the_same_config():
    import bench
    a = bench.workload_config("batched", batch=256)
    assert a["workload"] == "batched" and a["realisations"] == 256 and "parallelism" not in a
    params, _ = bench.workload("medium", 0)
    assert bench.workload_config("medium", params) == bench.workload_config("medium", dict(params))


def test_flip_count_counts_differences():
    import numpy as np

    import bench
    idx = np.array([3, 7, 9], np.uint64)
    ct = dict(I=np.array([0, 1, 2], np.uint32), J=np.array([1, 2, 0xFFFFFFFE], np.uint32),
              image=np.zeros((3, 3), np.int8))
    assert bench.flips(idx, ct, idx, ct) == 0
    idx2 = np.array([3, 7, 11], np.uint64)  # one rod accepted in place of another
    assert bench.flips(idx, ct, idx2, ct) == 2 + 4  # two stream indices, the two contacts of that rod, both ways
    ct2 = dict(ct, image=np.array([[0, 0, 0], [0, 0, 1], [0, 0, 0]], np.int8))
    assert bench.flips(idx, ct, idx, ct2) == 2
