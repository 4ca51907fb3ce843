"""Parity of the GPU engine (through the C ABI) with the oracle.

Every comparison is bit-exact: both sides write results as (x*R, y*R, R) or (R, R, 0) with
canonical limbs, so the 144-byte records must be identical; the Python oracle additionally checks
the canonical affine point, which is what the reference harness compares
(test_fpga_harness/tests/msm.rs:35-40).
"""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q = None


def recs(ref, pts):
    return np.frombuffer(b"".join(ref.encode_affine(p) for p in pts), dtype=np.uint8).reshape(-1, 104).copy()


def scal(ref, ks):
    return np.frombuffer(b"".join(ref.encode_scalar(k) for k in ks), dtype=np.uint64).reshape(-1, 4).copy()


def msm_gpu(engine, points, scalars, **opts):
    ctx = engine.multi_scalar_mult_init(points)
    try:
        if opts:
            return ctx.mult(scalars, **opts)
        return engine.multi_scalar_mult(ctx, points, scalars)
    finally:
        ctx.close()


# ---- field arithmetic ----------------------------------------------------------------------
def limbs32(v, n=12):
    return [(v >> (32 * i)) & 0xFFFFFFFF for i in range(n)]


def from32(a):
    return sum(int(x) << (32 * i) for i, x in enumerate(a))


def test_field_ops(engine, ref):
    Q = ref.Q
    R = 2**384
    rng = random.Random(1)
    vals = [0, 1, 2, Q - 1, Q, Q + 1, 2 * Q - 1, ref.MONT_R, (R - 1) % (2 * Q)]
    vals += [rng.randrange(2 * Q) for _ in range(500)]
    other = [rng.randrange(2 * Q) for _ in vals]
    a = np.array([limbs32(v) for v in vals], dtype=np.uint32)
    b = np.array([limbs32(v) for v in other], dtype=np.uint32)
    Rinv = pow(R, -1, Q)
    mul = engine.field_selftest(0, a, b)
    add = engine.field_selftest(1, a, b)
    sub = engine.field_selftest(2, a, b)
    can = engine.field_selftest(4, a, b)
    neg = engine.field_selftest(5, a, b)
    inv = engine.field_selftest(3, a, b)
    inv_bgcd = engine.field_selftest(6, a, b)
    for i, (x, y) in enumerate(zip(vals, other)):
        m = from32(mul[i])
        assert m < 2 * Q and m % Q == x * y * Rinv % Q
        s = from32(add[i])
        assert s < 2 * Q and s % Q == (x + y) % Q
        d = from32(sub[i])
        assert d < 2 * Q and d % Q == (x - y) % Q
        c = from32(can[i])
        assert c < Q and c == x % Q
        ng = from32(neg[i])
        assert ng < 2 * Q and ng % Q == (-x) % Q
        for arr in (inv, inv_bgcd):
            iv = from32(arr[i])
            if x % Q:
                assert iv % Q * x % Q == R * R % Q
            else:
                assert iv % Q == 0


# ---- generator -------------------------------------------------------------------------------
def test_generated_bases_match_oracle(engine, ocpu):
    got = engine.generate_bases(99, 300)
    assert np.array_equal(got, ocpu.gen_bases(99, 300))
    got = engine.generate_bases(99, 64, first=1 << 20)
    assert np.array_equal(got, ocpu.gen_bases(99, 64, first=1 << 20))


# ---- MSM parity -------------------------------------------------------------------------------
@pytest.mark.parametrize("form", ["auto", "windowed"])
@pytest.mark.parametrize("n", [1, 2, 3, 17, 64, 1000])
def test_msm_small(engine, ref, ocpu, n, form):
    """Small contexts get fixed-base tables of width 16 (the default form); the windowed form
    with its serial window combine is forced with fixed_base=2."""
    pts = ocpu.gen_bases(7 + n, n)
    sc = engine.generate_scalars(11 + n, 2 * n)
    out = msm_gpu(engine, pts, sc) if form == "auto" else msm_gpu(engine, pts, sc, fixed_base=2)
    for b in range(2):
        want = ocpu.msm(pts, sc[b * n:(b + 1) * n])
        assert np.array_equal(out[b], want), f"batch {b}"


def test_msm_config_2_12(engine, ocpu):
    """Plain single MSM, N = 2^12, seeded bases k_i * G and uniform scalars (4 batches)."""
    n = 1 << 12
    pts = ocpu.gen_bases(2024, n)
    sc = engine.generate_scalars(2025, 4 * n)
    out = msm_gpu(engine, pts, sc)
    for b in range(4):
        assert np.array_equal(out[b], ocpu.msm(pts, sc[b * n:(b + 1) * n]))


@pytest.mark.parametrize("opts", [
    dict(window_bits=6), dict(window_bits=8), dict(window_bits=11), dict(window_bits=13),
    dict(window_bits=16), dict(window_bits=9, signed_digits=2), dict(window_bits=12, signed_digits=2),
    dict(window_bits=10, seg_len=3), dict(window_bits=7, seg_len=1, red_len_log2=2),
    dict(mode=2), dict(mode=2, use_graph=1), dict(use_graph=1),
])
def test_msm_knobs(engine, ocpu, opts):
    n = 1500
    pts = ocpu.gen_bases(31, n)
    sc = engine.generate_scalars(32, 2 * n)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        for rep in range(2):
            out = ctx.mult(sc, **opts)
            for b in range(2):
                assert np.array_equal(out[b], ocpu.msm(pts, sc[b * n:(b + 1) * n])), (opts, rep, b)
    finally:
        ctx.close()


def test_naive_driver_entry_points(engine, ocpu):
    """The naive driver's names (naive_driver.cpp:109-138) bind the same context and MSMs."""
    import ctypes
    lib = engine.load_library()
    n = 700
    pts = ocpu.gen_bases(55, n)
    sc = engine.generate_scalars(56, 3 * n)
    ctx = lib.zprize_msm_fpga_init(pts.ctypes.data, n)
    assert ctx
    try:
        for fn in (lib.zprize_msm_pippenger_mult, lib.zprize_msm_fpga_mult):
            out = np.zeros((3, engine.PROJ_BYTES), dtype=np.uint8)
            fn(ctypes.c_void_p(ctx), out.ctypes.data, 3, sc.ctypes.data)
            for b in range(3):
                assert np.array_equal(out[b], ocpu.msm(pts, sc[b * n:(b + 1) * n])), (fn, b)
    finally:
        lib.msm_free(ctypes.c_void_p(ctx))


def test_trivial_inputs(engine, ref, ocpu):
    """TEST_TRIVIAL_INPUTS of the harness (util.rs:164-183): all bases G, scalar[0] = 1."""
    n = 256
    pts = recs(ref, [ref.GEN] * n)
    sc = np.zeros((4 * n, 4), dtype=np.uint64)
    sc[::n, 0] = 1
    out = msm_gpu(engine, pts, sc)
    for b in range(4):
        assert ref.decode_projective(out[b].tobytes()) == ref.GEN


def test_edge_scalars_and_bases(engine, ref, ocpu):
    rng = random.Random(5)
    n = 777
    pts = [ref.mul(ref.GEN, rng.getrandbits(64)) for _ in range(40)]
    plist = [pts[i % 40] for i in range(n)]
    plist[3] = ref.INF
    plist[100] = ref.INF
    ks = [rng.randrange(ref.R_SCALAR) for _ in range(n)]
    for i in range(0, n, 7):
        ks[i] = 0
    for i in range(1, n, 11):
        ks[i] = ref.R_SCALAR - 1
    for i in range(2, n, 5):
        ks[i] = 0xABCDEF  # one heavy bucket per low window
    ks[5] = (1 << 253) - 1
    ks[6] = ks[7] | (5 << 253)  # bits above 253 are ignored
    P, S = recs(ref, plist), scal(ref, ks)
    out = msm_gpu(engine, P, S)
    assert np.array_equal(out[0], ocpu.msm(P, S))
    for opts in (dict(window_bits=8, seg_len=4), dict(window_bits=16)):
        assert np.array_equal(msm_gpu(engine, P, S, **opts)[0], ocpu.msm(P, S))


def test_all_scalars_zero_and_empty(engine, ref, ocpu):
    pts = ocpu.gen_bases(3, 50)
    out = msm_gpu(engine, pts, np.zeros((50, 4), dtype=np.uint64))
    assert ref.decode_projective(out[0].tobytes()) is ref.INF
    assert np.array_equal(out[0], ocpu.msm(pts, np.zeros((50, 4), dtype=np.uint64)))


# ---- the reference harness's five edge-case tests (tests/msm_unit_tests.rs) ------------------
def special_points(ref, kats):
    return [ref.parse_hex_point(p["x"], p["y"]) for p in kats["non_te_points"]]


def check_case(engine, ref, ocpu, pts, ks, batches=1):
    P = recs(ref, pts)
    S = scal(ref, ks)
    out = msm_gpu(engine, P, S)
    n = len(pts)
    for b in range(batches):
        want = ref.msm_naive(pts, ks[b * n:(b + 1) * n])
        assert ref.decode_projective(out[b].tobytes()) == want
        assert np.array_equal(out[b], ocpu.msm(P, S[b * n:(b + 1) * n]))


def test_intermediate_infinity_non_representable_1(engine, ref, ocpu, kats):
    sp = special_points(ref, kats)  # msm_unit_tests.rs:19-77
    check_case(engine, ref, ocpu, [sp[0], sp[1], sp[2], sp[2]], [1, 1, 1, 1])


def test_intermediate_infinity_non_representable_2(engine, ref, ocpu, kats):
    sp = special_points(ref, kats)  # msm_unit_tests.rs:81-133
    pts = [sp[0], sp[2], ref.neg(ref.add(sp[0], sp[2])), sp[2]]
    check_case(engine, ref, ocpu, pts, [1, 1, 1, 1])


def test_infinity_result(engine, ref, ocpu):
    pts = [ref.GEN if i % 2 == 0 else ref.neg(ref.GEN) for i in range(256)]  # :137-180
    check_case(engine, ref, ocpu, pts, [1] * (4 * 256), batches=4)


def test_unrepresentable_points_at_chunk_boundaries(engine, ref, ocpu, kats):
    sp = special_points(ref, kats)  # :185-240
    n = 1 << 12
    P = ocpu.gen_bases(4242, n)
    for idx, p in ((1024, sp[0]), (2047, sp[2]), (3 * 1024 - 1, sp[1]), (4095, sp[2])):
        P[idx] = np.frombuffer(ref.encode_affine(p), dtype=np.uint8)
    S = engine.generate_scalars(4243, 4 * n)
    out = msm_gpu(engine, P, S)
    for b in range(4):
        assert np.array_equal(out[b], ocpu.msm(P, S[b * n:(b + 1) * n]))


def test_one_unrepresentable_one_regular(engine, ref, ocpu, kats):
    sp = special_points(ref, kats)  # :244-290
    check_case(engine, ref, ocpu, [ref.GEN, sp[0]], [1, 2])


def test_rtl_bucket_kat_through_engine(engine, ref, kats):
    """The single-point case of test_top.ml:148-193 (scalar 82 on a k*G base) end to end."""
    kat = kats["rtl_bucket_kat"]
    px = int(next(e for e in kat["entries"] if e["point"])["point"]["x"], 16)
    k = next(k for k in range(1, 100) if ref.mul(ref.GEN, k)[0] == px)
    P = ref.mul(ref.GEN, k)
    out = msm_gpu(engine, recs(ref, [P]), scal(ref, [82]))
    assert ref.decode_projective(out[0].tobytes()) == ref.mul(P, 82)


# ---- uneven batches, graphs, server, tuner ----------------------------------------------------
def test_uneven_batch_modes(engine, ocpu):
    nb = 1 << 12
    pts = ocpu.gen_bases(77, nb)
    rng = random.Random(9)
    sizes = [1, 0, 5, 64, 1000, 4096, 333, 2048, 17, 4000, 1, 999]
    offs = [rng.randrange(0, nb - s + 1) for s in sizes]
    sc = np.concatenate([engine.generate_scalars(500, s, kind=1, msm_index=j) for j, s in enumerate(sizes)])
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        first = np.concatenate([[0], np.cumsum(sizes)])
        want = [ocpu.msm(pts[o:o + s], sc[first[j]:first[j] + s]) for j, (s, o) in enumerate(zip(sizes, offs))]
        for opts in (dict(mode=1), dict(mode=2), dict(mode=2, use_graph=1), dict(mode=2, use_graph=2),
                     dict(mode=1, fixed_base=2), dict(mode=2, fixed_base=2)):
            for rep in range(2):
                out = ctx.mult_uneven(sizes, offs, sc, **opts)
                for j in range(len(sizes)):
                    assert np.array_equal(out[j], want[j]), (opts, rep, j)
    finally:
        ctx.close()


def test_host_scalar_upload_paths(engine, ocpu, monkeypatch):
    """Host scalars reach the device through the histogram kernel's own reads of host memory (a
    device that reads pageable memory, 16-byte aligned buffer) or through chunked copies
    (MSM_HOST_PULL=0, or a buffer at an address that is 8 mod 16); every path, in both pass modes,
    gives the oracle's results."""
    nb = 1 << 12
    pts = ocpu.gen_bases(31, nb)
    sizes = [4096, 7, 1000, 0, 2500]
    offs = [0, 4000, 17, 5, 1596]
    sc = np.concatenate([engine.generate_scalars(40 + j, s) for j, s in enumerate(sizes)])
    raw = np.empty(sc.size + 2, dtype=np.uint64)
    start = 1 if raw.ctypes.data % 16 == 0 else 0
    mis = raw[start:start + sc.size]
    mis[:] = sc.reshape(-1)
    assert mis.ctypes.data % 16 == 8
    mis = mis.reshape(sc.shape)
    first = np.concatenate([[0], np.cumsum(sizes)])
    want = [ocpu.msm(pts[o:o + s], sc[first[j]:first[j] + s]) for j, (s, o) in enumerate(zip(sizes, offs))]
    for pull in ("1", "0"):
        monkeypatch.setenv("MSM_HOST_PULL", pull)
        ctx = engine.multi_scalar_mult_init(pts)
        try:
            for buf in (sc, mis):
                for mode in (1, 2):
                    out = ctx.mult_uneven(sizes, offs, buf, mode=mode)
                    for j in range(len(sizes)):
                        assert np.array_equal(out[j], want[j]), (pull, buf is mis, mode, j)
        finally:
            ctx.close()


def test_server_results_alone_and_in_the_mix(engine, ocpu):
    nb = 1 << 12
    pts = ocpu.gen_bases(8, nb)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        sizes = [4096, 100, 2000, 1, 3000, 512, 4096, 50]
        offs = [0, 17, 1000, 4095, 500, 3000, 0, 4000]
        reqs = [engine.generate_scalars(600 + j, s) for j, s in enumerate(sizes)]
        alone = [ctx.mult_uneven([s], [o], r)[0] for s, o, r in zip(sizes, offs, reqs)]
        srv = engine.MsmServer(ctx, hbm_budget_bytes=64 << 20, max_inflight=2)
        try:
            ids = [srv.submit(r, o) for r, o in zip(reqs, offs)]
            for j, rid in enumerate(ids):
                res = srv.poll(rid, wait_ms=60000)
                assert res is not None
                out, lat = res
                assert lat >= 0
                assert np.array_equal(out, alone[j])
                assert np.array_equal(out, ocpu.msm(pts[offs[j]:offs[j] + sizes[j]], reqs[j]))
            st = srv.stats()
            assert st["completed"] == len(sizes) and st["passes"] >= 1
        finally:
            srv.close()
        with pytest.raises(engine.MsmError):
            small = engine.MsmServer(ctx, hbm_budget_bytes=1 << 10, max_inflight=1)
            try:
                small.submit(reqs[0], 0)
            finally:
                small.close()
    finally:
        ctx.close()


def test_tuner_keeps_results_exact(engine, ocpu, tmp_path, monkeypatch):
    n = 1 << 12
    pts = ocpu.gen_bases(55, n)
    sc = engine.generate_scalars(56, n)
    cache = str(tmp_path / "tune.txt")
    monkeypatch.setenv("MSM_TUNE_CACHE", cache)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        best = ctx.tune(n, budget_ms=5000)
        assert 6 <= best["window_bits"] <= 21
        assert ctx.config(n)["window_bits"] == best["window_bits"]
        assert np.array_equal(ctx.mult(sc)[0], ocpu.msm(pts, sc))
    finally:
        ctx.close()
    # a new context picks the tuned configuration up from the cache file
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        assert ctx.config(n)["window_bits"] == best["window_bits"]
        assert ctx.config(n)["seg_len"] == best["seg_len"]
    finally:
        ctx.close()


def test_msm_2_18_against_oracle(engine, ocpu):
    n = 1 << 18
    pts = engine.generate_bases(1, n)
    sc = engine.generate_scalars(2, n)
    out = msm_gpu(engine, pts, sc)
    assert np.array_equal(out[0], ocpu.msm(pts, sc))


# ---- fixed-base tables (2^(c w) P_i per window, one shared bucket array) ----------------------
def _ctx_with_fixed_base(engine, pts, c):
    import os
    old = os.environ.get("MSM_FIXED_BASE")
    os.environ["MSM_FIXED_BASE"] = str(c)
    try:
        return engine.multi_scalar_mult_init(pts)
    finally:
        if old is None:
            del os.environ["MSM_FIXED_BASE"]
        else:
            os.environ["MSM_FIXED_BASE"] = old


def test_fixed_base_parity(engine, ref, ocpu, kats):
    nb = 3000
    pts = ocpu.gen_bases(4321, nb)
    sp = special_points(ref, kats)
    pts[17] = np.frombuffer(ref.encode_affine(sp[0]), dtype=np.uint8)   # order-4 point, no TE image
    pts[18] = np.frombuffer(ref.encode_affine(ref.INF), dtype=np.uint8)
    ctx = _ctx_with_fixed_base(engine, pts, 13)
    try:
        assert ctx.config(nb)["fixed_base"] in (1, 2)
        sc = engine.generate_scalars(4322, 2 * nb)
        for opts in (dict(fixed_base=1), dict(fixed_base=1, mode=2), dict(fixed_base=1, seg_len=8),
                     dict(fixed_base=2)):
            out = ctx.mult(sc, **opts)
            for b in range(2):
                assert np.array_equal(out[b], ocpu.msm(pts, sc[b * nb:(b + 1) * nb])), (opts, b)
        sizes = [1, 700, 0, 2999, 64]
        offs = [2999, 5, 0, 1, 2000]
        usc = np.concatenate([engine.generate_scalars(77 + j, s, kind=1, msm_index=j) for j, s in enumerate(sizes)])
        first = np.concatenate([[0], np.cumsum(sizes)])
        for opts in (dict(fixed_base=1, mode=2), dict(fixed_base=1, mode=2, use_graph=1), dict(mode=2)):
            out = ctx.mult_uneven(sizes, offs, usc, **opts)
            for j, (s, o) in enumerate(zip(sizes, offs)):
                assert np.array_equal(out[j], ocpu.msm(pts[o:o + s], usc[first[j]:first[j] + s])), (opts, j)
    finally:
        ctx.close()


@pytest.mark.parametrize("ranges", [3, 8, 32])
def test_staged_sort_key_ranges(engine, ocpu, monkeypatch, ranges):
    """The staged sort with several key ranges (one scatter launch each), which the default rule
    uses only for sorted arrays of hundreds of MB: windowed and fixed-base MSMs, uniform scalars,
    the uneven-batch mix (16-bit values, 0 and r-1, one repeated value) and all-equal scalars."""
    nb = 1 << 13
    pts = ocpu.gen_bases(909, nb)
    sizes = [nb, 3000, 1, 4096]
    offs = [0, 17, 100, 4000]
    sc = np.concatenate([engine.generate_scalars(910, nb), engine.generate_scalars(911, 3000, kind=1),
                         engine.generate_scalars(912, 1),
                         np.repeat(engine.generate_scalars(913, 1), 4096, axis=0)])
    first = np.concatenate([[0], np.cumsum(sizes)])
    want = [ocpu.msm(pts[o:o + s], sc[first[j]:first[j] + s]) for j, (s, o) in enumerate(zip(sizes, offs))]
    monkeypatch.setenv("MSM_SORT_RANGES", str(ranges))
    for ctx in (engine.multi_scalar_mult_init(pts), _ctx_with_fixed_base(engine, pts, 12)):
        try:
            for opts in (dict(mode=1), dict(mode=2), dict(mode=2, use_graph=1), dict(fixed_base=1, mode=1)):
                out = ctx.mult_uneven(sizes, offs, sc, **opts)
                for j in range(len(sizes)):
                    assert np.array_equal(out[j], want[j]), (ranges, opts, j)
        finally:
            ctx.close()


def test_all_equal_scalars_large(engine, ref, ocpu):
    """2^18 equal scalars: every window's entries land in one bucket (2^18 entries, thousands of
    runs merged by blocks of quads); once a random value, once r - 1 (every digit at its most
    negative)."""
    n = 1 << 18
    pts = ocpu.gen_bases(4242, n)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        for k in (ref.uniform_scalar(4243, 0), ref.R_SCALAR - 1):
            sc = np.repeat(scal(ref, [k]), n, axis=0)
            out = ctx.mult(sc)
            assert np.array_equal(out[0], ocpu.msm(pts, sc)), k
            assert ctx.last_pass_stats()["heavy_buckets"] > 0
    finally:
        ctx.close()


@pytest.mark.parametrize("seg_len", [512, 128, 32, 8])
def test_merge_tiers(engine, ocpu, seg_len):
    """A bucket split into few, tens or hundreds of runs is merged by a thread, a warp or a block
    of quads: 4096 equal scalars put 4096 entries in one bucket per window, i.e. 8, 32, 128 or
    512 runs for these run lengths."""
    nb = 1 << 12
    pts = ocpu.gen_bases(515, nb)
    sc = np.concatenate([np.repeat(engine.generate_scalars(516, 1), nb, axis=0)])
    mixed = engine.generate_scalars(517, nb, kind=1)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        for s in (sc, mixed):
            out = ctx.mult_uneven([nb], [0], s, seg_len=seg_len)
            assert np.array_equal(out[0], ocpu.msm(pts, s)), seg_len
    finally:
        ctx.close()


def test_width16_tables_on_a_large_context(engine, ocpu):
    """A context of 2^20 bases holds its main tables (width 20) and a second set of width 16;
    small MSMs over slices take the width-16 set, full-size ones the main set, and every form
    (including windowed) matches the oracle."""
    n = 1 << 20
    pts = engine.generate_bases(4711, n)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        assert ctx.config(4096)["window_bits"] == 16 and ctx.config(4096)["fixed_base"] == 1
        assert ctx.config(n)["window_bits"] == 20 and ctx.config(n)["fixed_base"] == 1
        sizes = [4096, 50000, 1000, 1]
        offs = [0, 123457, n - 1000, n - 1]
        sc = np.concatenate([engine.generate_scalars(4712 + j, s, kind=1, msm_index=j)
                             for j, s in enumerate(sizes)])
        first = np.concatenate([[0], np.cumsum(sizes)])
        want = [ocpu.msm(pts[o:o + s], sc[first[j]:first[j] + s]) for j, (s, o) in enumerate(zip(sizes, offs))]
        for opts in (dict(mode=1), dict(mode=2), dict(mode=2, use_graph=1), dict(fixed_base=2)):
            out = ctx.mult_uneven(sizes, offs, sc, **opts)
            for j in range(len(sizes)):
                assert np.array_equal(out[j], want[j]), (opts, j)
        full = engine.generate_scalars(4720, n)
        assert np.array_equal(ctx.mult(full)[0], ocpu.msm(pts, full))
    finally:
        ctx.close()


@pytest.mark.parametrize("c", [23, 11])
def test_fixed_base_top_window_cap(engine, ref, ocpu, c):
    """The signed top window's buckets stop at the largest top digit of a scalar below r
    (c = 23: 4894097 instead of 2^23).  Scalars up to 2^253 - 1, accepted as plain 253-bit
    integers, can exceed it; such a top digit becomes two entries of the top window.  Edge
    scalars sit at the cap, just above it and at the largest 253-bit values."""
    nb = 2000
    pts = ocpu.gen_bases(991, nb)
    ctx = _ctx_with_fixed_base(engine, pts, c)
    try:
        nwin = -(-253 // c)
        top = c * (nwin - 1)  # first bit of the top window
        cap = ((ref.R_SCALAR - 1) >> top) + 1
        rng = np.random.default_rng(c)
        ks = [int.from_bytes(rng.bytes(32), "little") % ref.R_SCALAR for _ in range(nb)]
        edge = [(1 << 253) - 1, ref.R_SCALAR - 1, 1 << 252, cap << top, (cap + 1) << top,
                ((cap + 1) << top) - 1, (((1 << (253 - top)) - 1) << top) | ((1 << top) - 1) >> 1,
                (1 << 253) - (1 << top), 1]
        ks[:len(edge)] = edge
        for i in range(len(edge), 300):  # 253-bit integers at or above r
            ks[i] = ref.R_SCALAR + int.from_bytes(rng.bytes(32), "little") % ((1 << 253) - ref.R_SCALAR)
        sc = scal(ref, ks)
        for opts in (dict(fixed_base=1), dict(fixed_base=1, mode=2), dict(fixed_base=1, seg_len=8),
                     dict(fixed_base=2), dict(fixed_base=2, window_bits=c)):
            out = ctx.mult(sc, **opts)
            assert np.array_equal(out[0], ocpu.msm(pts, sc)), opts
            if opts == dict(fixed_base=1):  # nonzero digits, and the split top digits
                assert nb * (nwin - 2) < ctx.last_pass_stats()["entries"] <= nb * (nwin + 1)
    finally:
        ctx.close()


def test_fixed_base_with_even_order_bases(engine, ref, ocpu, kats):
    """The reference's second edge case holds a representable base of order 4, whose doubling
    chain reaches the order-two point (0, -1) and then the identity; the tables stay exact.  (A
    chain that left the affine curve would switch the context to the plain table.)"""
    sp = special_points(ref, kats)
    pts_l = [sp[0], sp[2], ref.neg(ref.add(sp[0], sp[2])), sp[2]] + [ref.mul(ref.GEN, k + 2) for k in range(60)]
    P = recs(ref, pts_l)
    ctx = _ctx_with_fixed_base(engine, P, 13)
    try:
        ks = [1] * 4 + [k * 977 + 5 for k in range(60)]
        for fb in (1, 2):
            out = ctx.mult(scal(ref, ks), fixed_base=fb)
            assert ref.decode_projective(out[0].tobytes()) == ref.msm_naive(pts_l, ks), fb
        ks2 = [3, 7, 5, 2] + [(k * 7919) ** 3 % ref.R_SCALAR for k in range(60)]
        out = ctx.mult(scal(ref, ks2), fixed_base=1)
        assert ref.decode_projective(out[0].tobytes()) == ref.msm_naive(pts_l, ks2)
    finally:
        ctx.close()


def test_msm_correctness_from_test_data_files(engine, ref, ocpu, tmp_path):
    """msm_correctness with TEST_LOAD_DATA_FROM (tests/msm.rs:15-42, util.rs:236-257): the data
    directory is written in the harness's format, loaded back, run, and checked batch by batch."""
    from hardcaml_zprize_gb300 import arkworks_io as io
    n, batches = 1 << 10, 4
    pts = ocpu.gen_bases(11, n)
    sc = engine.generate_scalars(12, n * batches)
    expected = np.stack([ocpu.msm(pts, sc[b * n:(b + 1) * n]) for b in range(batches)])
    d = str(tmp_path / "testdata")
    io.save_test_data(d, pts, sc, expected)
    nb, points, scalars, results = io.load_test_data(d)
    ctx = engine.multi_scalar_mult_init(points)
    try:
        out = engine.multi_scalar_mult(ctx, points, scalars)
    finally:
        ctx.close()
    assert nb == batches
    assert np.array_equal(io.projective_to_affine_records(out), results)


@pytest.mark.parametrize("form", ["auto", "windowed"])
def test_equal_bucket_sums_take_the_complete_formula(engine, ref, ocpu, form):
    """The reductions add points with the dedicated twisted-Edwards formula, which fails on a
    doubling; the engine then uses the unified one.  Here every base is the same point P and the
    scalars are 1..n, so window 0's buckets all hold P: the running sums add equal points
    (R + B with R = B, A + R with A = R) and the level-2/3 quad sums meet equal run sums.  The
    second case alternates P and -P under equal scalars, so bucket sums cancel to the identity in
    a form other than the one the code writes, and the third mixes both with uniform scalars."""
    n = 4096
    P = ref.mul(ref.GEN, 0x1234567)
    same = recs(ref, [P] * n)
    alt = recs(ref, [P if i % 2 == 0 else ref.neg(P) for i in range(n)])
    cases = [
        (same, scal(ref, list(range(1, n + 1)))),
        (alt, np.repeat(scal(ref, [ref.uniform_scalar(88, 0)]), n, axis=0)),
        (alt, engine.generate_scalars(89, n)),
    ]
    opts = {} if form == "auto" else {"fixed_base": 2}
    for k, (pts, sc) in enumerate(cases):
        ctx = engine.multi_scalar_mult_init(pts)
        try:
            out = ctx.mult(sc, **opts)
        finally:
            ctx.close()
        assert np.array_equal(out[0], ocpu.msm(pts, sc)), (form, k)
