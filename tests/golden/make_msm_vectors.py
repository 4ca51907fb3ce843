"""Write ``msm_vectors.json`` beside this script: MSM results of the pure-Python big-int oracle
(oracle/bls12_377.py, affine and Jacobian Weierstrass arithmetic, no code shared with the C
oracle or the device) on seeded inputs and on explicit edge-case inputs.  The reference commits
no MSM-level outputs; these vectors pin the engine's results against regressions.

    python tests/golden/make_msm_vectors.py

Each case lists how its inputs are made (seeds into the oracle's SplitMix64 generators, or the
encoded points and scalars themselves) and the expected g1_projective_t as hex.
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import bls12_377 as ref  # noqa: E402

OUT = os.path.join(HERE, "msm_vectors.json")


def result_hex(points, scalars):
    return ref.encode_projective(ref.msm_pippenger(points, scalars, c=8)).hex()


def main():
    cases = []
    for n in (1, 2, 17, 256, 1000):
        pts = ref.gen_bases(101, n)
        ks = ref.gen_scalars(202, n)
        cases.append({"name": f"uniform_{n}", "kind": "seeded", "n": n, "base_seed": 101,
                      "scalar_seed": 202, "scalar_kind": "uniform",
                      "expected": result_hex(pts, ks)})
    n = 512
    pts = ref.gen_bases(303, n)
    ks = [ref.mixed_scalar(404, 0, i) for i in range(n)]
    cases.append({"name": "mixed_512", "kind": "seeded", "n": n, "base_seed": 303,
                  "scalar_seed": 404, "scalar_kind": "mixed", "expected": result_hex(pts, ks)})
    # explicit edge cases: the identity, the generator's multiples with scalars 0, 1, r - 1 and
    # the 253-bit maximum (bits 253..255 set as well, which the engine ignores), and the three
    # points without a twisted-Edwards image listed by the reference's tests
    with open(os.path.join(HERE, "reference_kats.json")) as f:
        kats = json.load(f)
    special = [ref.parse_hex_point(p["x"], p["y"]) for p in kats["non_te_points"]]
    g = ref.GEN
    pts = [ref.INF, g, ref.mul(g, 2), ref.mul(g, 3), ref.mul(g, 5), ref.neg(g)] + special
    ks = [7, 0, 1, ref.R_SCALAR - 1, (1 << 256) - 1, 12345, 3, 2, 1]
    cases.append({"name": "edges", "kind": "explicit",
                  "points": [ref.encode_affine(p).hex() for p in pts],
                  "scalars": [ref.encode_scalar(k).hex() for k in ks],
                  "expected": result_hex(pts, ks)})
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_msm_vectors.py (oracle/bls12_377.py)",
                   "cases": cases}, f, indent=1)
        f.write("\n")
    print(f"wrote {OUT}: {len(cases)} cases")


if __name__ == "__main__":
    main()
