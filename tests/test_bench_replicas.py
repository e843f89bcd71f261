"""bench.py under torchrun (N > 1): one replica per rank, no collective on
the data path; the per-step time is the max over ranks and only rank 0
prints.  World size 2 over gloo on the CPU (127.0.0.1)."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r = {"ms_step": 10.0 + 5.0 * rank, "e2e_ms": 30.0 - 7.0 * rank, "n": 1000}
    bench.combine_ranks(r, world)
    out[rank] = (r["ms_step"], r["e2e_ms"])
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(i, 2, port, out)) for i in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0] == out[1] == (15.0, 30.0)


def test_single_process_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench

    r = {"ms_step": 3.0, "e2e_ms": 4.0}
    assert bench.combine_ranks(r, 1) == {"ms_step": 3.0, "e2e_ms": 4.0}
