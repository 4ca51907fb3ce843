"""Pin the oracle to the known answers the reference's own tests and headers hold.

Fixture: tests/golden/reference_kats.json (made by tests/golden/make_golden.py from the
reference's test files read as text); every value carries the reference file:line it came from.
"""
import random

import numpy as np
import pytest


def H(s):
    return int(s, 16) if not s.startswith("-") else -int(s[1:], 16)


def test_field_and_curve_constants(ref, kats):
    assert H(kats["modulus"]["value"]) == ref.Q
    assert H(kats["p"]["value"]) == ref.Q
    assert H(kats["coeff_a"]["value"]) == ref.WEI_A
    assert H(kats["coeff_b"]["value"]) == ref.WEI_B
    assert kats["scalar_bits"]["value"] == ref.SCALAR_BITS == ref.R_SCALAR.bit_length()
    assert H(kats["generator"]["x"]) == ref.GEN_X
    assert H(kats["generator"]["y"]) == ref.GEN_Y
    assert ref.on_curve(ref.GEN)


def test_twisted_edwards_parameters(ref, kats):
    Q = ref.Q
    assert H(kats["weierstrass_s"]["value"]) == ref.S
    assert H(kats["weierstrass_alpha"]["value"]) % Q == ref.ALPHA
    assert H(kats["twisted_scale"]["value"]) == ref.TWISTED_SCALE
    assert H(kats["te_a"]["value"]) == ref.TE_A
    assert H(kats["te_d"]["value"]) == ref.TE_D
    assert H(kats["k"]["value"]) == ref.TE_K == 2 * ref.TE_D % Q
    assert H(kats["k_over_2"]["value"]) == ref.TE_D
    assert H(kats["one_fourth"]["value"]) == ref.inv(4)
    s8 = H(kats["sqrt_k_over_8"]["value"])
    assert s8 * s8 % Q == ref.TE_K * ref.inv(8) % Q
    s3 = H(kats["sqrt3"]["value"])
    assert s3 * s3 % Q == 3
    assert H(kats["c_A"]["value"]) % Q == ref.C_A
    assert H(kats["c_B"]["value"]) == ref.C_B


def test_host_header_words(ref, kats):
    """bls12_377_g1.h:24-54 and constants.h:7-46 against the oracle's constants."""
    w = {k: sum(int(x) << (64 * i) for i, x in enumerate(v["words"])) for k, v in kats["host_words"].items()}
    assert w["COFACTOR"] == ref.MONT_R  # the constant the header calls COFACTOR is R = 2^384 mod q
    assert w["Q"] == ref.Q
    assert w["TWISTED_SCALE"] == ref.TWISTED_SCALE
    assert w["K"] == ref.TE_K
    assert w["S"] == ref.S
    assert w["A"] == ref.TE_A
    assert w["D"] == ref.TE_D
    assert w["C_A"] == ref.C_A
    assert w["C_B"] == ref.C_B
    hx = {k: int(v["value"], 16) for k, v in kats["host_hex"].items()}
    assert hx["Q"] == ref.Q and hx["S"] == ref.S and hx["TWISTED_SCALE"] == ref.TWISTED_SCALE
    assert hx["A"] == ref.TE_A and hx["D"] == ref.TE_D and hx["K"] == ref.TE_K
    assert hx["C_A"] == ref.C_A and hx["C_B"] == ref.C_B


def test_mul_matches_repeated_add_and_zero(ref, kats):
    """test_ark_bls12_377_g1.ml:70-84: mul by 1..10 equals repeated addition; mul by 0 is O."""
    assert kats["mul_by_zero_is_infinity"]["value"]
    assert ref.mul(ref.GEN, 0) is ref.INF
    acc = ref.GEN
    for by in range(1, 11):
        assert ref.mul(ref.GEN, by) == acc
        acc = ref.add(acc, ref.GEN)


def test_points_without_twisted_edwards_image(ref, kats):
    """test_bls12_377_twisted_edwards_form.ml:101-173 and the harness edge points."""
    ix = H(kats["invalid_x"]["value"])
    assert ix == (ref.ALPHA - ref.inv(ref.S)) % ref.Q
    pts = [ref.parse_hex_point(p["x"], p["y"]) for p in kats["non_te_points"]]
    assert len(pts) == 3
    for p in pts:
        assert ref.on_curve(p)
        assert ref.weierstrass_to_te(p) is None
        # every such point has order 2 or 4, so k * P = (k mod 4) * P
        assert ref.mul(p, 4) is ref.INF
    assert ref.neg(pts[0]) == pts[1]
    edge = {ref.parse_hex_point(p["x"], p["y"]) for p in kats["harness_edge_points"]}
    assert edge == set(pts)


def test_te_map_roundtrip_and_addition(ref):
    """Weierstrass <-> twisted Edwards map and the unified addition agree with the Weierstrass
    group law, including P + O, P + P and P + (-P) (the Quickcheck of
    test_bls12_377_twisted_edwards_form.ml:264-323, fewer trials)."""
    rng = random.Random(7)
    for trial in range(60):
        p1 = ref.mul(ref.GEN, rng.getrandbits(64) | 1)
        choice = trial % 5
        p2 = {0: ref.mul(ref.GEN, rng.getrandbits(64) | 1), 1: ref.INF, 2: p1, 3: ref.neg(p1),
              4: ref.mul(ref.GEN, rng.getrandbits(64) | 1)}[choice]
        t1, t2 = ref.weierstrass_to_te(p1), ref.weierstrass_to_te(p2)
        assert ref.te_on_curve(t1) and ref.te_on_curve(t2)
        assert ref.te_to_weierstrass(t1) == p1
        s = ref.te_add_extended(ref.te_extended(t1), ref.te_extended(t2))
        assert ref.te_to_weierstrass(ref.te_affine(s)) == ref.add(p1, p2)
        # precomputed mixed add on the (2(y-x), 2(y+x), 4z, t) bucket form (add_unified_precomputed)
        x1, y1 = t1
        z = rng.randrange(1, ref.Q)
        bucket = (2 * (y1 - x1) * z % ref.Q, 2 * (y1 + x1) * z % ref.Q, 4 * z % ref.Q, x1 * y1 * z % ref.Q)
        for sub in (False, True):
            out = ref.te_madd_fpga(bucket, ref.te_precompute(t2), subtract=sub)
            want = ref.add(p1, ref.neg(p2) if sub else p2)
            assert ref.te_to_weierstrass(ref.te_affine(ref.te_from_fpga(out))) == want


def test_signed_digit_split_reference_config(ref):
    """perform_scalar_reduction / check_scalar_reduction (utils.ml:207-288) on the reference's
    own configuration: 253 bits over 20 windows (config.ml:5-9; 13 x 13-bit then 7 x 12-bit)."""
    sizes = ref.reference_window_sizes(253, 20)
    assert sizes == [13] * 13 + [12] * 7
    assert sum(ref.reference_num_buckets(sizes, w) for w in range(20)) == 69631  # driver.cpp:31
    rng = random.Random(3)
    for _ in range(500):
        k = rng.randrange(ref.R_SCALAR)
        d = ref.signed_digits(k, sizes)
        for w, dw in enumerate(d):
            assert abs(dw) <= ref.reference_num_buckets(sizes, w)
            if w < 19:
                assert -(1 << (sizes[w] - 1)) <= dw < (1 << (sizes[w] - 1)) or dw == 0


def test_engine_digit_layout(ref):
    """The engine's uniform c-bit windows (sequential carry, as utils.ml:243-288): digits
    reconstruct the scalar, lower windows stay within 2^(c-1) buckets and the top window within
    2^(253 - c (W-1)) buckets.  The engine caps the signed top window's buckets at the largest
    top digit of a scalar below r, floor((r-1) / 2^(c (W-1))) + 1, which is at least half of
    2^(253 - c (W-1)): a larger top digit (a 253-bit scalar at or above r) splits into two
    in-range entries."""
    rng = random.Random(5)
    for c in (6, 10, 11, 13, 16, 20, 22, 23):
        sizes = ref.uniform_window_sizes(c)
        assert sum(sizes) == 253 and len(sizes) == -(-253 // c)
        top_off = ref.offsets(sizes)[-1]
        cap = ((ref.R_SCALAR - 1) >> top_off) + 1
        assert 2 * cap >= 1 << sizes[-1] and cap <= 1 << sizes[-1]
        for k in (ref.R_SCALAR - 1, rng.randrange(ref.R_SCALAR), (1 << top_off) - 1):
            assert 0 <= ref.signed_digits(k, sizes)[-1] <= cap
        for _ in range(200):
            k = rng.getrandbits(253) if _ % 4 else (1 << 253) - 1 - rng.getrandbits(8)
            d = ref.signed_digits(k, sizes)
            assert sum(dw << o for dw, o in zip(d, ref.offsets(sizes))) == k
            assert all(abs(dw) <= (1 << (c - 1)) for dw in d[:-1])
            assert 0 <= d[-1] <= (1 << sizes[-1])


def test_rtl_bucket_kat(ref, kats):
    """test_top.ml:148-193: one base k*G (k < 100), 9-bit scalar, 4 windows.  The expected bucket
    contents pin the signed-digit split and the bucket-level result."""
    kat = kats["rtl_bucket_kat"]
    sizes = ref.reference_window_sizes(kat["scalar_bits"], kat["num_windows"])
    offs = ref.offsets(sizes)
    filled = [e for e in kat["entries"] if e["point"]]
    px = H(filled[0]["point"]["x"])
    k = next(k for k in range(1, 100) if ref.mul(ref.GEN, k)[0] == px)
    P = ref.mul(ref.GEN, k)
    digits = [0] * kat["num_windows"]
    for e in filled:
        pt = (H(e["point"]["x"]), H(e["point"]["y"]))
        assert pt in (P, ref.neg(P))
        digits[e["window"]] = e["bucket"] * (1 if pt == P else -1)
    # every (window, bucket) pair of the RTL readout appears, high bucket first
    assert len(kat["entries"]) == sum(ref.reference_num_buckets(sizes, w) for w in range(len(sizes)))
    scalar = sum(d << o for d, o in zip(digits, offs))
    assert 0 <= scalar < (1 << kat["scalar_bits"])
    assert ref.signed_digits(scalar, sizes) == digits
    # calculate_result_from_fpga (utils.ml:137-159): triangle sums, then doublings by offset
    total = ref.INF
    for w in range(len(sizes)):
        cnt1 = cnt2 = ref.INF
        for e in [e for e in kat["entries"] if e["window"] == w]:
            if e["point"]:
                cnt1 = ref.add(cnt1, (H(e["point"]["x"]), H(e["point"]["y"])))
            cnt2 = ref.add(cnt2, cnt1)
        total = ref.add(total, ref.mul(cnt2, 1 << offs[w]) if cnt2 is not ref.INF else ref.INF)
    assert total == ref.mul(P, scalar) == ref.msm_naive([P], [scalar])


def test_python_pippenger_matches_naive(ref):
    rng = random.Random(11)
    pts = [ref.mul(ref.GEN, rng.getrandbits(64)) for _ in range(24)] + [ref.INF]
    ks = [rng.randrange(ref.R_SCALAR) for _ in pts]
    ks[3] = 0
    ks[4] = ref.R_SCALAR - 1
    want = ref.msm_naive(pts, ks)
    for c in (4, 7, 13):
        assert ref.msm_pippenger(pts, ks, c=c) == want
