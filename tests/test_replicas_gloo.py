"""Multi-rank host logic on the CPU: two gloo ranks (no GPU) exercise the
domain partition of the batched ensemble, the max-over-ranks timing and the
gathering of per-rank statistics used by bench.py --gpus N."""
import os
import socket

import pytest

from phasefield_gb300 import replicas


def test_partition_covers_every_item_once():
    for n in (0, 1, 5, 64, 67):
        for w in (1, 2, 3, 8):
            parts = [replicas.partition(n, r, w) for r in range(w)]
            items = [i for p in parts for i in p]
            assert items == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = list(replicas.partition(64, rank, world))
        t = replicas.max_over_ranks(10.0 + rank)
        allv = replicas.gather([rank * 100 + i for i in mine[:2]])
        replicas.barrier()
        q.put((rank, replicas.world(), mine[0], mine[-1], t, allv))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, a0, b0, t0, g0), (r1, w1, a1, b1, t1, g1) = res
    assert w0 == (0, 2) and w1 == (1, 2)
    assert (a0, b0, a1, b1) == (0, 31, 32, 63)
    assert t0 == t1 == 11.0
    assert g0 == g1 == [0, 1, 132, 133]
