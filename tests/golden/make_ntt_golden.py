"""Extract the known-answer values that fyquah/hardcaml_zprize's own code holds for its NTT track
and write them to ``ntt_kats.json`` beside this script.

Run it with the path of a checkout of the reference tree, given as the first argument or in the
environment variable HARDCAML_ZPRIZE_REF (there is no default):

    python tests/golden/make_ntt_golden.py REF

It reads the files as text (nothing of the reference is executed) and records, with the
file:line each value came from:

* the Goldilocks modulus and the table of 2^i-th roots of unity the host driver uses
  (zprize/ntt/host/gf.h),
* the NTT test vectors of the reference C++ model (libs/hardcaml_ntt/reference_code/
  ntt_test.cpp): the 8-point transforms of (1, 2, 0, ...) and of eight given values, and the
  first eight outputs of the 4096-point transform of (1, 2, 0, ...).
"""
from __future__ import annotations

import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HARDCAML_ZPRIZE_REF", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: make_ntt_golden.py REF  (REF = a checkout of fyquah/hardcaml_zprize; "
             "or set HARDCAML_ZPRIZE_REF)")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ntt_kats.json")


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read().splitlines()


kats = {"source": "fyquah/hardcaml_zprize NTT host header and reference-model test, read as text"}

f = "zprize/ntt/host/gf.h"
L = read(f)
for i, ln in enumerate(L):
    m = re.search(r"MODULUS\s*=\s*(0x[0-9A-Fa-f]+)", ln)
    if m:
        kats["modulus"] = {"value": hex(int(m.group(1), 16)), "at": f"{f}:{i + 1}"}
omega, start = [], None
for i, ln in enumerate(L):
    if "OMEGA[33]" in ln:
        start = i
    elif start is not None:
        m = re.search(r"GF\((\d+)ull\)", ln)
        if m:
            omega.append(int(m.group(1)))
        if ln.strip().startswith("};"):
            kats["omega"] = {"value": [hex(v) for v in omega], "at": f"{f}:{start + 1}-{i + 1}",
                             "meaning": "omega[i] is the 2^i-th root of unity used for a domain of 2^i"}
            break
assert len(omega) == 33

f = "libs/hardcaml_ntt/reference_code/ntt_test.cpp"
L = read(f)
text = "\n".join(L)


def gf_list(chunk):
    return [hex(int(x, 16)) for x in re.findall(r"GF\(\s*(0x[0-9a-fA-F]+)\s*\)", chunk)]


def func_span(name):
    a = next(i for i, ln in enumerate(L) if re.match(rf"int {name}\(\)", ln))
    b = next(i for i in range(a + 1, len(L)) if L[i].startswith("}"))
    return a, b


vec = {}
a, b = func_span("test_2_3_linear")
body = "\n".join(L[a:b + 1])
vec["ntt8_of_1_2"] = {"log_n": 3, "input": ["0x1", "0x2"] + ["0x0"] * 6,
                      "output": gf_list(body.split("expected_out")[1]), "at": f"{f}:{a + 1}-{b + 1}"}
a, b = func_span("test_2_12_linear")
body = "\n".join(L[a:b + 1])
vec["ntt4096_of_1_2_first8"] = {"log_n": 12, "input_nonzero": {"0": "0x1", "1": "0x2"},
                                "output_first": gf_list(body.split("expected_out")[1]),
                                "at": f"{f}:{a + 1}-{b + 1}"}
a, b = func_span("test_2_3_fully_random")
body = "\n".join(L[a:b + 1])
parts = body.split("expected_out")
vec["ntt8_random"] = {"log_n": 3, "input": gf_list(parts[0]), "output": gf_list(parts[1]),
                      "at": f"{f}:{a + 1}-{b + 1}"}
for k, v in vec.items():
    assert len(v.get("output", v.get("output_first"))) == 8, k
kats["vectors"] = vec
with open(OUT, "w") as fh:
    json.dump(kats, fh, indent=1)
print(f"wrote {OUT}")
