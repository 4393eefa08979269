"""Host side of ``bench.py --gpus N`` (replicas: N independent copies of the step, no
data-path collective): process-group set-up from the torchrun environment, the barrier and
the max-over-ranks time, as world-size-2 gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    r, ws, dist = bench.dist_init(None)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.0 + 2.0 * r)  # rank 0: 1.0, rank 1: 3.0
    out.put((r, ws, t, dist.get_backend()))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_time():
    import torch
    if torch.cuda.is_available():
        pytest.skip("the CPU path of the replica harness (gloo) is tested without a GPU")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 3.0, "gloo"), (1, 2, 3.0, "gloo")]


def test_single_process_has_no_group():
    import bench
    os.environ.pop("WORLD_SIZE", None)
    assert bench.dist_init(None) == (0, 1, None)
    assert bench.max_over_ranks(None, 2.5) == 2.5
