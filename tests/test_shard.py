"""Host logic of the sharded MSM over world-size-2 gloo process groups on CPU; the partial MSMs
and the combine run on the C oracle here (on GPUs they run on the engine)."""
import os
import random
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_partition_balanced():
    from hardcaml_zprize_gb300.shard import partition
    assert partition(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert partition(2, 4) == [(0, 1), (1, 2), (2, 2), (2, 2)]
    with pytest.raises(ValueError):
        partition(5, 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, fail_rank, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from oracle import bls12_377 as ref, cpu as ocpu
    from hardcaml_zprize_gb300 import shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = random.Random(42)
        n = 37
        pts = [ref.mul(ref.GEN, rng.getrandbits(64)) for _ in range(n)]
        ks = [rng.randrange(ref.R_SCALAR) for _ in range(n)]
        recs = np.frombuffer(b"".join(ref.encode_affine(p) for p in pts), dtype=np.uint8).reshape(-1, 104)
        sc = np.frombuffer(b"".join(ref.encode_scalar(k) for k in ks), dtype=np.uint64).reshape(-1, 4)

        def partial(lo, hi):
            if rank == fail_rank:
                raise RuntimeError("injected failure")
            return ocpu.msm(recs[lo:hi], sc[lo:hi])

        def combine(parts):
            aff = shard.projective_to_affine_records(parts)
            ones = np.zeros((len(parts), 4), dtype=np.uint64)
            ones[:, 0] = 1
            return ocpu.msm(aff, ones)

        try:
            out = shard.sharded_msm(n, rank, world, partial, combine)
            q.put((rank, "ok", ref.decode_projective(out.tobytes()) == ref.msm_naive(pts, ks)))
        except shard.ShardError as e:
            q.put((rank, "error", str(e)))
    finally:
        dist.destroy_process_group()


def _run(world, fail_rank):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, fail_rank, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
    return sorted(res)


def test_sharded_msm_gloo_world2():
    res = _run(2, fail_rank=-1)
    assert res == [(0, "ok", True), (1, "ok", True)]


def test_sharded_msm_rank_failure_is_reported():
    res = _run(2, fail_rank=1)
    assert [r[1] for r in res] == ["error", "error"]
    assert "rank(s) [1]" in res[0][2]
