"""The benchmark configurations checked against the oracle at their stated sizes.

Every expected value comes from the C oracle (oracle/cpu_msm.c, the ark-ec 0.3 variable-base
Pippenger restated), never from another form of the engine, so a fault shared by the engine's
plain, batched and served forms (the sort, the final conversion, the top-window split) cannot
pass.  This mirrors the harness, which checks every batch against arkworks
(zprize/msm_pippenger/test_fpga_harness/tests/msm.rs:15-42).

* plain MSM at N = 2^24, on the fixed-base tables the context builds and on the plain
  144-byte-per-base records;
* the uneven batch: 64 MSMs of 2^10..2^20 points over a shared 2^20 base set with the mixed
  scalars, in one pass replayed from a CUDA graph and one pass per MSM;
* served requests of 2^12..2^22 points over a 2^22 base set, submitted while others run, each
  compared with the oracle and with the same request run alone.

The 4 x 2^26 fixed-base configuration is checked against the oracle by bench.py (one of the four
batches, about a minute of CPU time), which the default bench run includes.
"""
import os
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20240601


def _cores():
    return os.cpu_count() or 1


@pytest.fixture(scope="module")
def bench_mod():
    import bench
    return bench


def test_plain_msm_2_24_against_oracle(engine, ocpu, monkeypatch):
    n = 1 << 24
    pts = engine.generate_bases(SEED, n)
    sc = engine.generate_scalars(SEED + 1, n)
    want = ocpu.msm(pts, sc, threads=_cores())
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        assert ctx.info()["table_bits"] > 0  # the headline context keeps fixed-base tables
        got = engine.multi_scalar_mult(ctx, pts, sc)[0]
        assert np.array_equal(got, want), "fixed-base tables"
        assert np.array_equal(ctx.mult(sc, fixed_base=2)[0], want), "windowed on the same context"
    finally:
        ctx.close()
    # the plain resident form: 144 bytes per base, no tables
    monkeypatch.setenv("MSM_FIXED_BASE", "0")
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        info = ctx.info()
        assert info["table_bits"] == 0 and info["resident_bytes"] == n * 144
        assert np.array_equal(engine.multi_scalar_mult(ctx, pts, sc)[0], want), "144 B records"
    finally:
        ctx.close()


def test_uneven_batch_against_oracle(engine, ocpu, bench_mod):
    nbase = 1 << 20
    sizes, offs, sc = bench_mod.uneven_mix(SEED, engine.generate_scalars, 64, nbase)
    pts = engine.generate_bases(SEED, nbase)
    first = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    want = np.stack([ocpu.msm(pts[o:o + s], sc[first[j]:first[j + 1]], threads=_cores())
                     for j, (s, o) in enumerate(zip(sizes, offs))])
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        batched = ctx.mult_uneven(sizes, offs, sc, mode=2, use_graph=1)
        again = ctx.mult_uneven(sizes, offs, sc, mode=2, use_graph=1)  # replayed graph
        plain = ctx.mult_uneven(sizes, offs, sc, mode=1)
        for j in range(len(sizes)):
            assert np.array_equal(batched[j], want[j]), f"batched MSM {j} (n={sizes[j]})"
            assert np.array_equal(again[j], want[j]), f"graph replay MSM {j}"
            assert np.array_equal(plain[j], want[j]), f"plain MSM {j}"
    finally:
        ctx.close()


def test_served_requests_against_oracle(engine, ocpu, bench_mod):
    nbase = 1 << 22
    m = 10
    rng, sizes, offs, reqs = bench_mod.served_mix(SEED, engine.generate_scalars, m, nbase)
    assert max(sizes) > 1 << 21  # the mix reaches the top of its range
    pts = engine.generate_bases(SEED, nbase)
    want = [ocpu.msm(pts[o:o + s], r, threads=_cores()) for s, o, r in zip(sizes, offs, reqs)]
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        alone = [ctx.mult_uneven([s], [o], r)[0] for s, o, r in zip(sizes, offs, reqs)]
        srv = engine.MsmServer(ctx, hbm_budget_bytes=8 << 30, max_inflight=3)
        try:
            ids = []
            for j in range(m):  # arrivals while earlier requests are on the GPU
                ids.append(srv.submit(reqs[j], offs[j]))
                time.sleep(float(rng.exponential(0.002)))
            for j, rid in enumerate(ids):
                got, _lat = srv.poll(rid, wait_ms=600000)
                assert np.array_equal(got, want[j]), f"served request {j} (n={sizes[j]})"
                assert np.array_equal(alone[j], want[j]), f"request {j} alone"
            assert srv.stats()["inflight_peak"] >= 2
        finally:
            srv.close()
    finally:
        ctx.close()
