"""Readers/writers of the harness's test-data files (util.rs:126-172) and the conversions
between ark-serialize's canonical encoding and the ABI's Montgomery form (host code, no GPU)."""
import os
import random

import numpy as np
import pytest


def test_field_conversions_match_oracle(engine, ref):
    rng = random.Random(3)
    lib = engine.load_library()
    xs = [0, 1, ref.Q - 1] + [rng.randrange(ref.Q) for _ in range(200)]
    v = np.array([ref.limbs64(x, 6) for x in xs], dtype=np.uint64)
    assert lib.msm_fq_to_montgomery(v.ctypes.data, len(xs)) == 0
    assert [ref.from_limbs64(r) for r in v] == [ref.to_mont(x) for x in xs]
    assert lib.msm_fq_from_montgomery(v.ctypes.data, len(xs)) == 0
    assert [ref.from_limbs64(r) for r in v] == xs
    ks = [0, 1, ref.R_SCALAR - 1] + [rng.randrange(ref.R_SCALAR) for _ in range(200)]
    s = np.array([ref.limbs64(k, 4) for k in ks], dtype=np.uint64)
    assert lib.msm_fr_to_montgomery(s.ctypes.data, len(ks)) == 0
    assert [ref.from_limbs64(r) for r in s] == [k * 2**256 % ref.R_SCALAR for k in ks]
    assert lib.msm_fr_from_montgomery(s.ctypes.data, len(ks)) == 0
    assert [ref.from_limbs64(r) for r in s] == ks
    bad = np.array([ref.limbs64(ref.Q, 6)], dtype=np.uint64)
    assert lib.msm_fq_to_montgomery(bad.ctypes.data, 1) == -3


def test_points_file_roundtrip_and_layout(engine, ref, tmp_path):
    from hardcaml_zprize_gb300 import arkworks_io as io
    pts = [ref.mul(ref.GEN, k) for k in (1, 2, 99, 2**64 - 1)] + [ref.INF]
    recs = np.frombuffer(b"".join(ref.encode_affine(p) for p in pts), dtype=np.uint8).reshape(-1, 104)
    path = os.path.join(tmp_path, "points.bin")
    io.write_points(path, recs)
    raw = open(path, "rb").read()
    assert int.from_bytes(raw[:8], "little") == len(pts)
    assert len(raw) == 8 + 97 * len(pts)
    # canonical little-endian coordinates, then the infinity byte
    assert int.from_bytes(raw[8:56], "little") == ref.GEN_X
    assert int.from_bytes(raw[56:104], "little") == ref.GEN_Y
    assert raw[104] == 0 and raw[8 + 97 * 4 + 96] == 1
    back = io.read_points(path)
    assert np.array_equal(back[:4], recs[:4])
    assert back[4, 96] == 1


def test_scalars_file_matches_harness_transmute(engine, ref, tmp_path):
    """A scalar the harness builds as Fp256::new(BigInteger256::from(1)) (raw integer 1, as in
    msm_unit_tests.rs:52) is stored canonically as 2^-256 mod r and read back as 1."""
    from hardcaml_zprize_gb300 import arkworks_io as io
    rng = random.Random(8)
    ks = [1, 0, ref.R_SCALAR - 1] + [rng.randrange(ref.R_SCALAR) for _ in range(50)]
    s = np.array([ref.limbs64(k, 4) for k in ks], dtype=np.uint64)
    path = os.path.join(tmp_path, "scalars.bin")
    io.write_scalars(path, s)
    raw = open(path, "rb").read()
    assert int.from_bytes(raw[8:40], "little") == pow(2, -256, ref.R_SCALAR)
    assert np.array_equal(io.read_scalars(path), s)


def test_test_data_directory_roundtrip(engine, ref, ocpu, tmp_path):
    from hardcaml_zprize_gb300 import arkworks_io as io
    n, batches = 24, 2
    pts = ocpu.gen_bases(5, n)
    sc = engine.generate_scalars(6, n * batches)
    res = np.stack([ocpu.msm(pts, sc[b * n:(b + 1) * n]) for b in range(batches)])
    d = os.path.join(tmp_path, "data")
    io.save_test_data(d, pts, sc, res)
    b2, p2, s2, r2 = io.load_test_data(d)
    assert b2 == batches and np.array_equal(p2, pts) and np.array_equal(s2, sc)
    for b in range(batches):
        want = ref.decode_projective(res[b].tobytes())
        got = r2[b]
        assert (want is ref.INF) == bool(got[96])
        if want is not ref.INF:
            assert ref.from_mont(ref.from_limbs64(got[:48].view(np.uint64))) == want[0]
