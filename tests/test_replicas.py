"""The multi-GPU path runs independent replicas (one per rank) and reduces
only the timing: job time = max over ranks, job work = sum over ranks.
World size 2 on the gloo backend, on the CPU."""
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


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from cylindrical_epoch_gb300.replicas import reduce_replicas
        # rank r: a replica that took 1 + r seconds for (r + 1) * 1e9 particle-steps
        out[rank] = reduce_replicas(1.0 + rank, (rank + 1) * 1.0e9, dist, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        seconds, psteps, rate = res[r]
        assert seconds == 2.0          # the slowest replica
        assert psteps == 3.0e9         # all replicas' work
        assert rate == 1.5e9


def test_single_process_is_identity():
    from cylindrical_epoch_gb300.replicas import reduce_replicas
    assert reduce_replicas(2.0, 4.0e9) == (2.0, 4.0e9, 2.0e9)
