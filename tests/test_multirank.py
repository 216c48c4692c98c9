"""The multi-GPU form of the bench is replicas (weak scaling): every rank
solves its own wavenumber block, the only cross-rank operations are the
barrier and the max of the timed region.  These run as two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from suzerain_gb300 import synth
    ms = bench.max_over_ranks(10.0 + rank, world, "cpu")
    cfg = bench.rank_config(synth.CONFIGS[2], rank, world)
    dist.barrier()
    out.put((rank, ms, cfg.seed, cfg.nsys))
    dist.destroy_process_group()


def test_replicas_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, seed0, n0), (r1, ms1, seed1, n1) = res
    assert ms0 == ms1 == 11.0           # the job's time is the slowest rank's
    assert seed0 != seed1 and n0 == n1  # own block per rank, same shape (weak scaling)
