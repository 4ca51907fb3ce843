"""The C oracle (Jacobian Weierstrass, arkworks-style Pippenger) against the Python oracle."""
import random

import numpy as np
import pytest


def records(ref, pts):
    return np.frombuffer(b"".join(ref.encode_affine(p) for p in pts), dtype=np.uint8).reshape(-1, 104)


def scal(ref, ks):
    return np.frombuffer(b"".join(ref.encode_scalar(k) for k in ks), dtype=np.uint64).reshape(-1, 4)


def test_generated_bases_match(ref, ocpu):
    got = ocpu.gen_bases(1234, 12, first=5)
    want = records(ref, [ref.mul(ref.GEN, ref.base_multiplier(1234, 5 + i)) for i in range(12)])
    assert np.array_equal(got, want)


def test_default_window_rule(ocpu):
    # ark-ec 0.3: 3 below 32 points, else ln_without_floats(n) + 2 = ceil(log2 n) * 69 / 100 + 2
    assert ocpu.default_window(31) == 3
    assert ocpu.default_window(1 << 12) == 12 * 69 // 100 + 2
    assert ocpu.default_window(1 << 24) == 24 * 69 // 100 + 2


@pytest.mark.parametrize("n", [1, 2, 7, 40, 129])
def test_msm_matches_python(ref, ocpu, n):
    rng = random.Random(n)
    pts = [ref.mul(ref.GEN, rng.getrandbits(64)) for _ in range(n)]
    ks = [rng.randrange(ref.R_SCALAR) for _ in range(n)]
    if n > 3:
        pts[1] = ref.INF
        ks[2] = 0
        ks[3] = ref.R_SCALAR - 1
    want = ref.msm_naive(pts, ks)
    for c in (0, 5, 9):
        got = ref.decode_projective(ocpu.msm(records(ref, pts), scal(ref, ks), c=c).tobytes())
        assert got == want


def test_msm_special_points(ref, ocpu, kats):
    """The harness edge cases (msm_unit_tests.rs): points without a twisted-Edwards image."""
    sp = [ref.parse_hex_point(p["x"], p["y"]) for p in kats["non_te_points"]]
    cases = [
        ([sp[0], sp[1], sp[2], sp[2]], [1, 1, 1, 1]),
        ([sp[0], sp[2], ref.neg(ref.add(sp[0], sp[2])), sp[2]], [1, 1, 1, 1]),
        ([ref.GEN, sp[0]], [1, 2]),
        ([ref.GEN if i % 2 == 0 else ref.neg(ref.GEN) for i in range(16)], [1] * 16),
    ]
    for pts, ks in cases:
        got = ref.decode_projective(ocpu.msm(records(ref, pts), scal(ref, ks)).tobytes())
        assert got == ref.msm_naive(pts, ks)


def test_scalar_bits_above_253_ignored(ref, ocpu):
    p = ref.mul(ref.GEN, 99)
    k = ref.R_SCALAR - 5
    got = ref.decode_projective(ocpu.msm(records(ref, [p]), scal(ref, [k | (7 << 253)])).tobytes())
    assert got == ref.mul(p, k)


def test_c_scalar_generator_matches_python(ref, ocpu):
    got = ocpu.gen_scalars(77, 40, kind=0)
    for i in range(40):
        assert ref.from_limbs64(got[i]) == ref.uniform_scalar(77, i)
    mix = ocpu.gen_scalars(77, 300, kind=1, msm_index=3)
    for i in range(300):
        assert ref.from_limbs64(mix[i]) == ref.mixed_scalar(77, 3, i)
