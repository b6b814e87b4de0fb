"""The bench's multi-rank (replica) plumbing on CPU with the gloo backend, world size 2:
rendezvous on 127.0.0.1, barrier, max over ranks of the timed region, the whole-job
value, and that only rank 0 prints the reference arm's line."""
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
