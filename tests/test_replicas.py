"""Multi-rank bench path on CPU: two gloo ranks run independent replicas (different seeds) and
reduce their times with a max, as bench.py does under torchrun (replicas only, no data-path
collective)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "idealizedspectralgcm.jl_gb300")]
    import bench
    from jgcm import configs

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    seed = configs.BASE_SEED + r
    noise = configs.normal(seed, 8)
    t = bench.max_over_ranks(1.0 + r, w)
    bench.barrier(w)
    out.put((r, w, local, float(noise[0]), t))
    dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, n0, t0), (r1, w1, l1, n1, t1) = res
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert n0 != n1  # each replica draws its own seeded perturbation
    assert t0 == t1 == 2.0  # max over ranks
