"""The bench's multi-rank (replica) plumbing on CPU with the gloo backend, world size 2:
rendezvous on 127.0.0.1, barrier, max over ranks of the timed region, the whole-job
value, that only rank 0 prints the reference arm's line, and the footprint-balanced split
of the batched and serving workloads over ranks (every rank computes the same split
without communicating; together the shares partition the instances)."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist

    class A:
        pass

    w, r, _ = bench.dist_setup(A())
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    t = bench.max_over_ranks(0.5 + r, w)      # the slowest rank's time
    tests, steps = 1000, 3
    value = w * tests * steps / t              # all ranks' tests over the slowest time
    q.put((r, w, t, value))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_world2_max_over_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == 1.5 for o in out)
    assert all(abs(o[3] - 2 * 1000 * 3 / 1.5) < 1e-9 for o in out)


@pytest.mark.slow
def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    port = free_port()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=900, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]


def _shard_worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    from gpucsl_gb300.shard import discrete_cost, gaussian_cost, my_shard
    from gpucsl_gb300.synthetic import batch_instance_sizes, serving_sizes

    class A:
        pass

    w, r, _ = bench.dist_setup(A())
    sizes = batch_instance_sizes(512)
    costs = [gaussian_cost(p, n) for (p, n, _, _) in sizes]
    mine = my_shard(costs, w, r)
    every = bench.gather_lists(mine, w)             # all ranks' shares, rank order
    loads = bench.gather_lists([sum(costs[k] for k in mine)], w)
    s_sizes = serving_sizes(256, seed=7)
    s_costs = [gaussian_cost(p, n) if kind == "gaussian" else discrete_cost(p, n) for kind, p, n in s_sizes]
    s_every = bench.gather_lists(my_shard(s_costs, w, r), w)
    total = bench.sum_over_ranks(len(mine), w)
    q.put((r, every, loads, max(costs), s_every, total))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_world2_instance_shards_partition_the_workloads():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, every, loads, cmax, s_every, total in out:
        assert sorted(every) == list(range(512))          # a partition of the 512 instances
        assert sorted(s_every) == list(range(256))        # and of the 256 requests
        assert abs(loads[0] - loads[1]) <= cmax           # balanced to within one instance
        assert total == 512
    assert out[0][1] == out[1][1]                          # both ranks agree on the split
