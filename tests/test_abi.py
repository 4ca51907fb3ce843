"""The C ABI library: builds, loads, exports what include/msm_gb300.h declares, and its host-only
logic (generators, argument checks) behaves.  No GPU compute here."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "msm_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:zprize_)?msm_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol(engine):
    lib = engine.load_library()
    names = header_functions()
    assert "msm_init" in names and "msm_mult" in names and "zprize_msm_pippenger_mult" in names
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(engine.EXPORTED) == names


def test_ntt_exports_every_declared_symbol(engine):
    from hardcaml_zprize_gb300 import ntt
    text = open(os.path.join(ROOT, "include", "ntt_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(ntt_[a-z_0-9]+)\s*\(", text)))
    assert "ntt_init" in names and "ntt_evaluate" in names
    lib = engine.load_library()
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(ntt.EXPORTED) == names


def test_ntt_argument_errors(engine):
    from hardcaml_zprize_gb300 import ntt
    with pytest.raises(engine.MsmError, match="maximum"):
        ntt.NttContext(25)


def test_struct_layout_matches_harness(engine):
    # rust_types.h:8-83; the library static_asserts the same sizes
    assert engine.AFFINE_BYTES == 104 and engine.PROJ_BYTES == 144 and engine.SCALAR_BYTES == 32


def test_host_scalar_generator_matches_oracle(engine, ref):
    got = engine.generate_scalars(77, 40, kind=0)
    for i in range(40):
        assert ref.from_limbs64(got[i]) == ref.uniform_scalar(77, i)
    mix = engine.generate_scalars(77, 300, kind=1, msm_index=3)
    vals = [ref.from_limbs64(mix[i]) for i in range(300)]
    for i, v in enumerate(vals):
        assert v == ref.mixed_scalar(77, 3, i)
        assert v < ref.R_SCALAR
    assert 0 in vals and ref.R_SCALAR - 1 in vals
    assert any(0 < v < 65536 for v in vals)
    dup = ref.uniform_scalar(77, (3 << 32) | 0xFFFFFFFF)
    assert vals.count(dup) >= 10


def test_host_scalar_generator_matches_c_oracle(engine, ocpu):
    # the reference arm of bench.py draws its scalars with the C oracle, the GPU arm with the
    # engine: both must produce the same inputs for the same seed
    assert np.array_equal(engine.generate_scalars(20240602, 5000), ocpu.gen_scalars(20240602, 5000))
    assert np.array_equal(engine.generate_scalars(9, 3000, kind=1, msm_index=5),
                          ocpu.gen_scalars(9, 3000, kind=1, msm_index=5))


def test_length_mismatch_error(engine):
    ctx = engine.MultiScalarMultContext(None, 4)
    pts = np.zeros((4, 104), dtype=np.uint8)
    with pytest.raises(ValueError, match="length mismatch"):
        engine.multi_scalar_mult(ctx, pts, np.zeros((6, 4), dtype=np.uint64))
    with pytest.raises(ValueError):
        engine.as_points(np.zeros(100, dtype=np.uint8))


def test_bad_arguments_are_errors_not_crashes(engine):
    lib = engine.load_library()
    assert lib.msm_init(None, 0, None, -1) is None
    assert "bad point array" in engine.last_error()
    rc = lib.msm_mult_ex(None, None, 1, None, None)
    assert rc < 0
    assert lib.msm_generate_scalars(1, 4, 9, 0, None) < 0
