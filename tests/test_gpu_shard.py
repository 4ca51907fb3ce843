"""The sharded MSM with the engine on both sides of the exchange.

Two ranks run as separate processes on GPU 0 with a gloo process group: each computes the partial
MSM of its slice of the bases with the engine, the partial points go through
``shard.gather_partials`` (one all-gather of a 144-byte point and a status word per rank), and
``shard.combine_on_gpu`` adds them with the engine.  The result is compared with the oracle over
the whole base set.  The ranks' kernels never wait on one another: the only exchange is the
host-side gather.  Multi-GPU hardware is not available here, so this covers the protocol and the
engine calls, not NCCL or scaling.
"""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    sys.path.insert(0, ROOT)
    os.environ["MSM_DEVICE"] = "0"
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import hardcaml_zprize_gb300 as eng
    from hardcaml_zprize_gb300 import shard
    from oracle import cpu as ocpu

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pts = ocpu.gen_bases(71, n)
        sc = ocpu.gen_scalars(72, n)
        ctx = eng.multi_scalar_mult_init(pts)
        try:
            def partial(lo, hi):
                return ctx.mult_uneven([hi - lo], [lo], sc[lo:hi])[0]

            out = shard.sharded_msm(n, rank, world, partial, shard.combine_on_gpu)
        finally:
            ctx.close()
        q.put((rank, "ok", bool(np.array_equal(out, ocpu.msm(pts, sc)))))
    except Exception as e:  # reported to the test, which fails on it
        q.put((rank, "error", repr(e)))
    finally:
        dist.destroy_process_group()


def _run(world, n):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        res = [q.get(timeout=300) for _ in range(world)]
    finally:
        for p in procs:
            p.join(timeout=60)
    return sorted(res)


@pytest.mark.parametrize("world,n", [(2, 1 << 16), (3, 2)])
def test_sharded_msm_on_the_engine(engine, world, n):
    # (3, 2): one rank holds an empty slice and contributes the zero point
    assert _run(world, n) == [(r, "ok", True) for r in range(world)]
