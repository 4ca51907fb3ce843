"""MSM results pinned by tests/golden/msm_vectors.json (made by the pure-Python oracle with
tests/golden/make_msm_vectors.py): the C oracle on the CPU and the engine on the GPU must
reproduce every vector byte for byte."""
import json
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cases():
    with open(os.path.join(ROOT, "tests", "golden", "msm_vectors.json")) as f:
        return json.load(f)["cases"]


def _inputs(ref, case):
    if case["kind"] == "explicit":
        pts = np.frombuffer(b"".join(bytes.fromhex(h) for h in case["points"]), dtype=np.uint8)
        sc = np.frombuffer(b"".join(bytes.fromhex(h) for h in case["scalars"]), dtype="<u8")
        return pts.reshape(-1, 104).copy(), sc.reshape(-1, 4).astype(np.uint64)
    n = case["n"]
    pts = np.frombuffer(b"".join(ref.encode_affine(p) for p in ref.gen_bases(case["base_seed"], n)),
                        dtype=np.uint8).reshape(-1, 104).copy()
    if case["scalar_kind"] == "uniform":
        ks = ref.gen_scalars(case["scalar_seed"], n)
    else:
        ks = [ref.mixed_scalar(case["scalar_seed"], 0, i) for i in range(n)]
    sc = np.frombuffer(b"".join(ref.encode_scalar(k) for k in ks), dtype="<u8")
    return pts, sc.reshape(-1, 4).astype(np.uint64)


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_cpu_oracle_reproduces_golden(ref, ocpu, case):
    pts, sc = _inputs(ref, case)
    assert ocpu.msm(pts, sc).tobytes().hex() == case["expected"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_engine_reproduces_golden(engine, ref, case):
    pts, sc = _inputs(ref, case)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        out = engine.multi_scalar_mult(ctx, pts, sc)
        assert out.shape[0] == 1
        assert out[0].tobytes().hex() == case["expected"]
        # the same MSM as one job of a shared pass
        out2 = ctx.mult_uneven([sc.shape[0]], [0], sc, mode=2)
        assert out2[0].tobytes().hex() == case["expected"]
    finally:
        ctx.close()
