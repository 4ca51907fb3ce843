"""The NTT oracle (oracle/cpu_ntt.c) against the reference's own values: the modulus and root
table of zprize/ntt/host/gf.h, the committed transform vectors of the reference C++ model
(libs/hardcaml_ntt/reference_code/ntt_test.cpp), the all-ones input of the reference host's test
(zprize/ntt/host/test_random.cpp: its special first case) and a Python transform by definition.
When a reference checkout is present, the reference's gf.h itself is compiled (oracle/_ref) and
its field operations and roots are compared with the oracle's."""
import json
import os
import random
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = 0xFFFFFFFF00000001


@pytest.fixture(scope="module")
def nkats():
    with open(os.path.join(ROOT, "tests", "golden", "ntt_kats.json")) as f:
        return json.load(f)


def dft(x, logn):
    """X[k] = sum_j x[j] w^(j k), w the reference's 2^logn-th root (by definition, Python ints)."""
    from oracle import cpu as ocpu
    w = ocpu.gl_omega(logn)
    n = 1 << logn
    return [sum(int(x[j]) * pow(w, j * k, P) for j in range(n)) % P for k in range(n)]


def test_modulus_and_root_table(ocpu, nkats):
    assert int(nkats["modulus"]["value"], 16) == P == ocpu.GL_P
    om = [int(v, 16) for v in nkats["omega"]["value"]]
    for i, w in enumerate(om):
        assert ocpu.gl_omega(i) == w
        assert pow(w, 1 << i, P) == 1
        if i:
            assert pow(w, 1 << (i - 1), P) == P - 1  # primitive
        if i < 32:
            assert pow(om[i + 1], 2, P) == w


def test_reference_model_vectors(ocpu, nkats):
    v = nkats["vectors"]
    for key in ("ntt8_of_1_2", "ntt8_random"):
        x = np.array([int(t, 16) for t in v[key]["input"]], dtype=np.uint64)
        want = [int(t, 16) for t in v[key]["output"]]
        assert [int(t) for t in ocpu.ntt(x)] == want, key
    x = np.zeros(4096, dtype=np.uint64)
    x[0], x[1] = 1, 2
    got = ocpu.ntt(x)
    assert [int(t) for t in got[:8]] == [int(t, 16) for t in v["ntt4096_of_1_2_first8"]["output_first"]]


@pytest.mark.parametrize("logn", [0, 1, 2, 3, 5, 8])
def test_oracle_matches_definition(ocpu, logn):
    rng = random.Random(logn)
    x = [rng.randrange(P) for _ in range(1 << logn)]
    x[0] = P - 1
    assert [int(t) for t in ocpu.ntt(np.array(x, dtype=np.uint64))] == dft(x, logn)


@pytest.mark.parametrize("logn", [0, 1, 2, 3, 5, 7])
def test_oracle_inverse_matches_definition(ocpu, logn):
    """The oracle's inverse, x[j] = (1/n) sum_k X[k] w^(-j k), which the GPU's ntt_init_inverse is
    checked against (the reference model's transform with the other root table,
    libs/hardcaml_ntt/src/reference_model.ml:54-55, scaled as its round-trip test scales)."""
    rng = random.Random(50 + logn)
    n = 1 << logn
    X = [rng.randrange(P) for _ in range(n)]
    winv, ninv = pow(ocpu.gl_omega(logn), P - 2, P), pow(n, P - 2, P)
    want = [sum(X[k] * pow(winv, j * k, P) for k in range(n)) * ninv % P for j in range(n)]
    assert [int(t) for t in ocpu.ntt(np.array(X, dtype=np.uint64), inverse=True)] == want


def test_all_ones_and_roundtrip(ocpu):
    n = 1 << 12
    out = ocpu.ntt(np.ones(n, dtype=np.uint64))
    assert int(out[0]) == n and not out[1:].any()
    rng = np.random.default_rng(3)
    x = (rng.integers(0, 2**63, 1 << 16, dtype=np.uint64) * 2 + rng.integers(0, 2, 1 << 16, dtype=np.uint64)) % np.uint64(P)
    assert np.array_equal(ocpu.ntt(ocpu.ntt(x), inverse=True), x)


def test_field_ops_match_the_reference_header(ocpu):
    from oracle import build as ob
    probe = ob.build_ref()
    if not probe:
        pytest.skip("no reference checkout on this machine")
    om = struct.unpack("<33Q", subprocess.run([probe, "omega"], capture_output=True, check=True).stdout)
    assert list(om) == [ocpu.gl_omega(i) for i in range(33)]
    rng = random.Random(9)
    pairs = [(0, 0), (P - 1, P - 1), (P - 1, 1), (1, P - 1), (2**32, 2**32), (2**63, 2**63)]
    pairs += [(rng.randrange(P), rng.randrange(P)) for _ in range(2000)]
    inp = b"".join(struct.pack("<2Q", a, b) for a, b in pairs)
    out = subprocess.run([probe], input=inp, capture_output=True, check=True).stdout
    for k, (a, b) in enumerate(pairs):
        m, s, d = struct.unpack("<3Q", out[24 * k:24 * (k + 1)])
        assert m == a * b % P == ocpu.gl_mul(a, b)
        assert s == (a + b) % P and d == (a - b) % P


def test_mt19937_64_matches_the_standard_library(ocpu, tmp_path):
    # the C++ standard requires the 10000th draw of a default-constructed mt19937_64 to be
    # 9981545732273789042
    raw = ocpu.mt19937_64(10000, mod_p=False)
    assert int(raw[-1]) == 9981545732273789042
    import shutil
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    src = tmp_path / "mt.cpp"
    src.write_text("#include <random>\n#include <cstdio>\nint main(){std::mt19937_64 r;"
                   "for(int i=0;i<1000;i++){unsigned long long v=r();fwrite(&v,8,1,stdout);}}\n")
    exe = tmp_path / "mt"
    subprocess.run(["g++", "-O1", str(src), "-o", str(exe)], check=True)
    got = np.frombuffer(subprocess.run([str(exe)], capture_output=True, check=True).stdout, dtype=np.uint64)
    assert np.array_equal(got, raw[:1000])
    assert np.array_equal(ocpu.mt19937_64(1000), raw[:1000] % np.uint64(P))
