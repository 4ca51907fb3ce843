"""Extract the known-answer values that fyquah/hardcaml_zprize's own tests hold for the MSM path
and write them to ``reference_kats.json`` beside this script.

Run it with the path of a checkout of the reference tree, given as the first argument or in
the environment variable HARDCAML_ZPRIZE_REF (there is no default):

    python tests/golden/make_golden.py REF

It reads the reference's test and header files as text (nothing of the reference is executed)
and records, with the file:line each value came from:

* the base-field modulus, the G1 generator and the curve coefficients
  (libs/ark_bls12_377_g1/test/test_ark_bls12_377_g1.ml),
* the Weierstrass/Montgomery/twisted-Edwards parameters and derived constants
  (libs/twisted_edwards/test/test_bls12_377_twisted_edwards_form.ml),
* the three listed points without a twisted-Edwards image (same file),
* the 64-bit word constants of the host driver (host/msm_compute/include/bls12_377_g1/
  bls12_377_g1.h) and the hex constants (constants.h),
* the bucket-level expect test of the RTL top (hardcaml/test/top/test_top.ml),
* the hard-coded points of the harness's edge-case tests (test_fpga_harness/tests/
  msm_unit_tests.rs).
"""
from __future__ import annotations

import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HARDCAML_ZPRIZE_REF", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: make_golden.py REF  (REF = a checkout of fyquah/hardcaml_zprize; "
             "or set HARDCAML_ZPRIZE_REF)")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read().splitlines()


def find(lines, pattern, start=0):
    rx = re.compile(pattern)
    for i in range(start, len(lines)):
        m = rx.search(lines[i])
        if m:
            return i, m
    raise KeyError(pattern)


def hexval(s):
    s = s.strip()
    neg = s.startswith("0x-")
    v = int(s.replace("0x-", "").replace("0x", ""), 16)
    return -v if neg else v


kats = {"source": "fyquah/hardcaml_zprize test and header files, read as text"}

# --- ark shim test: modulus, a, b, generator -------------------------------------------------
f = "libs/ark_bls12_377_g1/test/test_ark_bls12_377_g1.ml"
L = read(f)
i, m = find(L, r"\(\(a (0x[0-9a-f]+)\) \(b (0x[0-9a-f]+)\)")
kats["coeff_a"] = {"value": hex(hexval(m.group(1))), "at": f"{f}:{i + 1}"}
kats["coeff_b"] = {"value": hex(hexval(m.group(2))), "at": f"{f}:{i + 1}"}
i, _ = find(L, r"\(modulus", i)
kats["modulus"] = {"value": L[i + 1].strip().rstrip(")"), "at": f"{f}:{i + 2}"}
i, _ = find(L, r"Display subgroup generator")
j, _ = find(L, r"\(\(x", i)
kats["generator"] = {
    "x": L[j + 1].strip().rstrip(")"),
    "y": L[j + 3].strip().rstrip(")").rstrip(")"),
    "at": f"{f}:{j + 1}-{j + 4}",
}
i, m = find(L, r"\(\(x 0x0\) \(y 0x1\) \(infinity true\)\)")
kats["mul_by_zero_is_infinity"] = {"value": True, "at": f"{f}:{i + 1}"}

# --- twisted Edwards form test: parameters, derived constants, invalid points ------------------
f = "libs/twisted_edwards/test/test_bls12_377_twisted_edwards_form.ml"
L = read(f)
i, _ = find(L, r'let%expect_test "Modulo square root"')
j, m = find(L, r"\{\| (0x[0-9a-f]+) \|\}", i)
kats["sqrt3"] = {"value": m.group(1), "at": f"{f}:{j + 1}"}
for name in ("k", "k_over_2", "one_fourth", "sqrt_k_over_8"):
    j, _ = find(L, r"\(\(?%s$" % name)
    kats[name] = {"value": L[j + 1].strip().rstrip(")").rstrip(")"), "at": f"{f}:{j + 2}"}
j, _ = find(L, r"^\s+\(p$")
kats["p"] = {"value": L[j + 1].strip().rstrip(")"), "at": f"{f}:{j + 2}"}
j, _ = find(L, r"\(\(a 0x0\) \(b 0x1\)")
kats["weierstrass_s"] = {"value": L[j + 2].strip().rstrip(")"), "at": f"{f}:{j + 3}"}
k2, m = find(L, r"\(alpha (0x-?[0-9a-f]+)\)", j)
kats["weierstrass_alpha"] = {"value": hex(hexval(m.group(1))), "at": f"{f}:{k2 + 1}"}
k3, _ = find(L, r"\(twisted_scale$", j)
kats["twisted_scale"] = {"value": L[k3 + 1].strip().rstrip(")").rstrip(")"), "at": f"{f}:{k3 + 2}"}
j, _ = find(L, r"\(\(a$", k3)
kats["te_a"] = {"value": L[j + 1].strip().rstrip(")"), "at": f"{f}:{j + 2}"}
j2, _ = find(L, r"\(d$", j)
kats["te_d"] = {"value": L[j2 + 1].strip().rstrip(")"), "at": f"{f}:{j2 + 2}"}
j, _ = find(L, r"\(\(c_A$", j2)
kats["c_A"] = {"value": hex(hexval(L[j + 1].strip().rstrip(")"))), "at": f"{f}:{j + 2}"}
j2, _ = find(L, r"\(c_B$", j)
kats["c_B"] = {"value": L[j2 + 1].strip().rstrip(")"), "at": f"{f}:{j2 + 2}"}
j, m = find(L, r"^\s+x = (0x[0-9a-f]+)$")
kats["invalid_x"] = {"value": m.group(1), "at": f"{f}:{j + 1}"}
pts = []
j, _ = find(L, r"All points that can't be represented")
for _ in range(3):
    j, mx = find(L, r"- x = (0x[0-9a-f]+)", j + 1)
    _, my = find(L, r"y = (0x[0-9a-f]+)", j + 1)
    pts.append({"x": mx.group(1), "y": my.group(1), "at": f"{f}:{j + 1}-{j + 2}"})
kats["non_te_points"] = pts

# --- host header word constants ---------------------------------------------------------------
f = "zprize/msm_pippenger/host/msm_compute/include/bls12_377_g1/bls12_377_g1.h"
L = read(f)
words = {}
for name in ("COFACTOR", "Q", "TWISTED_SCALE", "K", "S", "A", "D", "C_A", "C_B"):
    j, _ = find(L, r"const uint64_t %s_WORDS\[NUM_64B_WORDS\] = \{" % name)
    text = " ".join(L[j:j + 4])
    body = text[text.index("{") + 1:text.index("}")]
    vals = [int(x.strip().rstrip("ULL")) for x in body.split(",")]
    words[name] = {"words": [str(v) for v in vals], "at": f"{f}:{j + 1}"}
kats["host_words"] = words
j, m = find(L, r"SCALAR_NUM_BITS = (\d+)")
kats["scalar_bits"] = {"value": int(m.group(1)), "at": f"{f}:{j + 1}"}

f = "zprize/msm_pippenger/host/msm_compute/include/bls12_377_g1/constants.h"
L = read(f)
hx = {}
for name in ("Q", "S", "TWISTED_SCALE", "A", "D", "K", "C_A", "C_B"):
    j, _ = find(L, r"const char %s_STR\[\] =" % name)
    parts = []
    k = j + 1
    while True:
        parts += re.findall(r'"([0-9a-fx]+)"', L[k])
        if L[k].rstrip().endswith(";"):
            break
        k += 1
    hx[name] = {"value": "".join(parts), "at": f"{f}:{j + 1}-{k + 1}"}
kats["host_hex"] = hx

# --- RTL top expect test: bucket-level output for scalar_bits = 9, 4 windows, 1 point ---------
f = "zprize/msm_pippenger/hardcaml/test/top/test_top.ml"
L = read(f)
j, _ = find(L, r'let%expect_test "Test over small input size')
s0, _ = find(L, r"\(result\.points", j)
s1, _ = find(L, r"\|\}\]", s0)
blob = " ".join(x.strip() for x in L[s0:s1 + 1])
entries = []
for m in re.finditer(r"\(\(point (\(\)|\(\(\(x (0x[0-9a-f]+)\) \(y (0x[0-9a-f]+)\)\)\))\) "
                     r"\(bucket (\d+)\) \(window (\d+)\)\)", blob):
    pt = None if m.group(1) == "()" else {"x": m.group(2), "y": m.group(3)}
    entries.append({"bucket": int(m.group(4)), "window": int(m.group(5)), "point": pt})
sb = find(L, r"let scalar_bits = (\d+)", j)[1].group(1)
nw = find(L, r"let num_windows = (\d+)", j)[1].group(1)
kats["rtl_bucket_kat"] = {
    "scalar_bits": int(sb),
    "num_windows": int(nw),
    "num_inputs": 1,
    "base_is_generator_times_k_below": 100,
    "entries": entries,
    "at": f"{f}:{s0 + 1}-{s1 + 1}",
}

# --- harness edge-case tests: hard-coded points -------------------------------------------------
f = "zprize/msm_pippenger/test_fpga_harness/tests/msm_unit_tests.rs"
L = read(f)
hp = []
for idx, line in enumerate(L):
    m = re.search(r'b"([0-9A-Fa-f]+)",?', line)
    if m and "create_g1_affine_from_string" in L[idx - 1]:
        m2 = re.search(r'b"([0-9A-Fa-f]+)"', L[idx + 1])
        hp.append({"x": "0x" + m.group(1).lower(), "y": "0x" + m2.group(1).lower(),
                   "at": f"{f}:{idx + 1}-{idx + 2}"})
kats["harness_edge_points"] = hp

def _clean(o):
    """Keep only the hex literal of each extracted value (the expect blocks end in ')) |}]')."""
    if isinstance(o, dict):
        return {k: (_clean_hex(v) if k in ("value", "x", "y") and isinstance(v, str) else _clean(v))
                for k, v in o.items()}
    if isinstance(o, list):
        return [_clean(v) for v in o]
    return o


def _clean_hex(s):
    m = re.search(r"-?0x-?[0-9a-f]+", s)
    return m.group(0) if m else s


kats = _clean(kats)
with open(OUT, "w") as fh:
    json.dump(kats, fh, indent=1)
print("wrote", OUT, "with", len(kats), "groups")
