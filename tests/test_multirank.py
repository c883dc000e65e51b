"""The N > 1 host path of bench.py on CPU: two ranks over gloo (127.0.0.1).
Replicas only: every rank evaluates its own catalogue; the only exchanges are
the barrier around the timed region and the max / sum reductions of the
timing, and the reference arm does its work on rank 0 alone."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    w, r, _ = bench.dist_init()
    assert (w, r) == (world, rank)
    bench.barrier(w)
    res = {"max": bench.reduce(w, float(rank + 1), "max"),
           "sum": bench.reduce(w, float(rank + 1), "sum")}
    if rank != 0:
        # the reference arm: ranks other than 0 exit at once, without work
        class A:
            steps, warmup, gpus, workload = 1, 3, world, bench.DEFAULT
        res["ref_rc"] = bench.run_reference(A(), w, r)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    with open(os.path.join(out, f"rank{rank}.txt"), "w") as f:
        f.write(repr(res))


def test_two_rank_gloo_reductions_and_reference_arm(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = [eval(open(tmp_path / f"rank{r}.txt").read()) for r in range(2)]
    for g in got:
        assert g["max"] == 2.0 and g["sum"] == 3.0
    assert got[1]["ref_rc"] == 0
