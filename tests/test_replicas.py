"""The multi-GPU path (replicas only) on CPU: two gloo ranks agree on the
slowest rank's time and on the whole-job rate; a single process needs no
process group."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bp-layers_gb300"))
    from bpl_gb300 import replicas
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = replicas.env_ranks()
        ms = 10.0 + 5.0 * r  # rank 1 is the slower replica
        mx = replicas.max_over_ranks(ms)
        out[rank] = (r, w, lr, mx, replicas.whole_job_rate(1000.0, 4, w, mx), replicas.replica_seed(1, r))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_agree_on_the_slowest_time():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for rank, (r, w, lr, mx, rate, seed) in res.items():
        assert (r, w, lr) == (rank, world, rank)
        assert mx == 15.0
        assert rate == pytest.approx(1000.0 * 4 * 2 / 0.015)
        assert seed == 1 + rank


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bp-layers_gb300"))
    from bpl_gb300 import replicas
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.whole_job_rate(10.0, 2, 1, 1000.0) == pytest.approx(20.0)
