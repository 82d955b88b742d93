"""The multi-rank paths of bench.py on CPU with the gloo backend and world size 2.

The element update does not shard: `bench.py --gpus N` runs N independent replicas, one per rank,
and reports the cell updates of all ranks over the slowest rank's time.  These tests cover the
host side of that on CPU: the rendezvous, the max-over-ranks reduction and the barrier, and the
reference arm under torchrun, where rank 0 alone runs the CPU oracle and prints one JSON line
while the other rank exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    assert dist.get_backend() == "gloo"
    # the timed region ends with the slowest rank: every rank sees the maximum
    slowest = bench.barrier_max(w, 1.5 + rank)
    bench.barrier(w)
    with open(os.path.join(out, f"rank{rank}.json"), "w") as fh:
        json.dump({"max": slowest}, fh)
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        got = json.load(open(tmp_path / f"rank{r}.json"))
        assert got["max"] == 2.5


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_once():
    """torchrun with 2 ranks on CPU: rank 0 prints the reference arm's JSON line, rank 1 exits 0."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus",
           "2", "--steps", "1", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2", CUDA_VISIBLE_DEVICES="")
    res = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout[-2000:]
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
