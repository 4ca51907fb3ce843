"""The GPU NTT (ntt_* entry points) against the oracle, bit-exact, at every size up to 2^24.

Expected values come from oracle/cpu_ntt.c, itself pinned to the reference's root table and
committed transform vectors (tests/test_ntt_oracle.py).  The inputs include the two cases the
reference host's test draws (zprize/ntt/host/test_random.cpp: a vector of ones, and
std::mt19937_64 draws taken modulo p), the reference model's committed vectors, edge values
(0, 1, p - 1) and inputs at or above p, which the engine takes modulo p.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = 0xFFFFFFFF00000001


@pytest.fixture(scope="module")
def ntt_mod(engine):
    from hardcaml_zprize_gb300 import ntt
    return ntt


def random_below_p(rng, n):
    hi = rng.integers(0, 2**32, n, dtype=np.uint64)
    lo = rng.integers(0, 2**32, n, dtype=np.uint64)
    return ((hi << np.uint64(32)) | lo) % np.uint64(P)


def test_field_ops_on_edge_values(ntt_mod):
    rng = np.random.default_rng(5)
    edge = [0, 1, 2, P - 1, P - 2, 2**32 - 1, 2**32, 2**32 + 1, 2**63, P - 2**32, 2**64 - 2**33,
            (P - 1) // 2, 0xFFFFFFFF00000000]
    a = [x for x in edge for _ in edge] + [int(v) for v in random_below_p(rng, 20000)]
    b = [y for _ in edge for y in edge] + [int(v) for v in random_below_p(rng, 20000)]
    A, B = np.array(a, dtype=np.uint64), np.array(b, dtype=np.uint64)
    for op, f in ((0, lambda x, y: (x + y) % P), (1, lambda x, y: (x - y) % P), (2, lambda x, y: x * y % P)):
        got = ntt_mod.field_selftest(op, A, B)
        for i in range(len(a)):
            assert int(got[i]) == f(a[i], b[i]), (op, a[i], b[i])


@pytest.mark.parametrize("log_n", [0, 1, 2, 3, 4, 7, 10, 12, 13, 15, 16, 18, 20, 21])
def test_ntt_matches_oracle(ntt_mod, ocpu, log_n):
    rng = np.random.default_rng(100 + log_n)
    x = random_below_p(rng, 1 << log_n)
    x[0] = P - 1
    if x.size > 2:
        x[1], x[2] = 0, 1
    ctx = ntt_mod.NttContext(log_n)
    try:
        assert ctx.input_vector_size() == 1 << log_n
        want = ocpu.ntt(x)
        assert np.array_equal(ctx.evaluate(x), want)
        assert np.array_equal(ctx.evaluate(x), want)  # a second call on the same context
    finally:
        ctx.close()


def test_reference_model_vectors(ntt_mod):
    with open(os.path.join(ROOT, "tests", "golden", "ntt_kats.json")) as f:
        v = json.load(f)["vectors"]
    ctx = ntt_mod.NttContext(3)
    try:
        for key in ("ntt8_of_1_2", "ntt8_random"):
            x = np.array([int(t, 16) for t in v[key]["input"]], dtype=np.uint64)
            assert [int(t) for t in ctx.evaluate(x)] == [int(t, 16) for t in v[key]["output"]], key
    finally:
        ctx.close()
    ctx = ntt_mod.NttContext(12)
    try:
        x = np.zeros(4096, dtype=np.uint64)
        x[0], x[1] = 1, 2
        got = ctx.evaluate(x)
        assert [int(t) for t in got[:8]] == [int(t, 16) for t in v["ntt4096_of_1_2_first8"]["output_first"]]
    finally:
        ctx.close()


def test_reference_test_inputs_at_2_24(ntt_mod, ocpu):
    """The reference host test's two cases at the contest size: ones, and mt19937_64 % p."""
    n = 1 << 24
    ctx = ntt_mod.NttContext(24)
    try:
        out = ctx.evaluate(np.ones(n, dtype=np.uint64))
        assert int(out[0]) == n and not out[1:].any()
        x = ocpu.mt19937_64(n)
        assert np.array_equal(ctx.evaluate(x), ocpu.ntt(x, threads=os.cpu_count() or 1))
    finally:
        ctx.close()


def test_inputs_at_or_above_p_are_reduced(ntt_mod, ocpu):
    rng = np.random.default_rng(7)
    x = random_below_p(rng, 1 << 14)
    y = x.copy()
    y[::3] += np.uint64(P) * (y[::3] < np.uint64(2**64 - P))  # x + p where it fits in 64 bits
    y[5] = np.uint64(2**64 - 1)
    x[5] = np.uint64((2**64 - 1) % P)
    ctx = ntt_mod.NttContext(14)
    try:
        assert np.array_equal(ctx.evaluate(y), ocpu.ntt(x))
    finally:
        ctx.close()


def test_device_entry_point_and_roundtrip(ntt_mod, ocpu):
    import torch
    log_n = 20
    rng = np.random.default_rng(11)
    x = random_below_p(rng, 1 << log_n)
    ctx = ntt_mod.NttContext(log_n)
    try:
        d_in = torch.from_numpy(x.view(np.int64)).cuda()
        d_out = torch.empty_like(d_in)
        torch.cuda.synchronize()
        ctx.evaluate_device(d_out.data_ptr(), d_in.data_ptr())
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, ctx.evaluate(x))
        assert np.array_equal(ocpu.ntt(got, inverse=True), x)  # the oracle's inverse undoes it
    finally:
        ctx.close()


def test_batch_equals_single_calls(ntt_mod, ocpu):
    rng = np.random.default_rng(17)
    log_n = 18
    xs = np.stack([random_below_p(rng, 1 << log_n) for _ in range(5)])
    ctx = ntt_mod.NttContext(log_n)
    try:
        got = ctx.evaluate_batch(xs)
        again = ctx.evaluate_batch(xs[:3])
        for i in range(5):
            assert np.array_equal(got[i], ocpu.ntt(xs[i])), i
        assert np.array_equal(again, got[:3])
    finally:
        ctx.close()


@pytest.mark.parametrize("log_n", [0, 1, 2, 5, 12, 13, 17, 20])
def test_inverse_ntt_matches_oracle(ntt_mod, ocpu, log_n):
    """ntt_init_inverse against the oracle's inverse (root w^-1, scaled by 1/n), on one pass
    (log_n <= 12) and on two (the 1/n rides in the twist)."""
    rng = np.random.default_rng(300 + log_n)
    x = random_below_p(rng, 1 << log_n)
    x[0] = P - 1
    ctx = ntt_mod.NttContext(log_n, inverse=True)
    try:
        assert ctx.input_vector_size() == 1 << log_n
        assert np.array_equal(ctx.evaluate(x), ocpu.ntt(x, inverse=True))
    finally:
        ctx.close()


@pytest.mark.parametrize("log_n", [12, 24])
def test_round_trip_at_full_size(ntt_mod, log_n):
    """Forward then inverse on device buffers gives the input back (the reference model's
    round-trip property, libs/hardcaml_ntt/test/test_ntt_roundtrip.ml), at 2^24 too."""
    import torch

    rng = np.random.default_rng(400 + log_n)
    x = random_below_p(rng, 1 << log_n)
    fwd, inv = ntt_mod.NttContext(log_n), ntt_mod.NttContext(log_n, inverse=True)
    try:
        d_x = torch.from_numpy(x.view(np.int64)).cuda()
        d_y, d_z = torch.empty_like(d_x), torch.empty_like(d_x)
        torch.cuda.synchronize()
        st = torch.cuda.Stream()  # one stream orders the two contexts' transforms
        fwd.evaluate_device(d_y.data_ptr(), d_x.data_ptr(), st.cuda_stream)
        inv.evaluate_device(d_z.data_ptr(), d_y.data_ptr(), st.cuda_stream)
        torch.cuda.synchronize()
        assert not np.array_equal(d_y.cpu().numpy(), d_x.cpu().numpy())
        assert np.array_equal(d_z.cpu().numpy().view(np.uint64), x)
    finally:
        fwd.close()
        inv.close()
