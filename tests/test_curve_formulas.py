"""The addition formulas the reductions use, checked on the CPU against the oracle's group law.

The bucket reduction, the merges and the window combine add extended twisted-Edwards points with
the dedicated formula (add-2008-hwcd-4, a = -1; Hisil, Wong, Carter, Dawson, "Twisted Edwards
curves revisited", 2008): 8 products instead of the unified formula's 9
(oracle.bls12_377.te_add_extended, which restates bls12_377_g1.h:449-491).  The dedicated formula
is not complete, and the engine relies on two facts tested here:

* wherever its Z3 is nonzero it gives the same projective point as the unified formula;
* wherever it fails (doubling, the identity plus a point with T = 0, ...) every output coordinate
  is zero, so a test of Z3 alone finds every failure and the engine uses the unified formula.
"""
import random

import pytest

from oracle import bls12_377 as b

Q = b.Q


def dedicated(p1, p2):
    """add-2008-hwcd-4 with a = -1, in the order the device computes it (curve.cuh te_add_fast)."""
    X1, Y1, Z1, T1 = p1
    X2, Y2, Z2, T2 = p2
    A = (Y1 - X1) * (Y2 + X2) % Q
    B = (Y1 + X1) * (Y2 - X2) % Q
    C = 2 * Z1 * T2 % Q
    D = 2 * T1 * Z2 % Q
    E, F, G, H = (D + C) % Q, (B - A) % Q, (B + A) % Q, (D - C) % Q
    return (E * F % Q, G * H % Q, F * G % Q, E * H % Q)


def same_point(p, q):
    X1, Y1, Z1, T1 = p
    X2, Y2, Z2, T2 = q
    return all((a * Z2 - c * Z1) % Q == 0 for a, c in ((X1, X2), (Y1, Y2), (T1, T2)))


def extended_points(seed, count):
    rng = random.Random(seed)
    out = []
    while len(out) < count:
        te = b.weierstrass_to_te(b.mul(b.GEN, rng.getrandbits(64) + 1))
        if te is None:
            continue
        z = rng.randrange(1, Q)  # a random projective representative
        out.append(tuple(v * z % Q for v in b.te_extended(te)))
    return out


IDENTITY = (0, 1, 1, 0)
ORDER_TWO = (0, Q - 1, 1, 0)  # (0, -1)


def neg(p):
    X, Y, Z, T = p
    return ((-X) % Q, Y, Z, (-T) % Q)


def test_dedicated_equals_unified_on_distinct_points():
    pts = extended_points(11, 24)
    for p in pts[:12]:
        for q in pts[12:]:
            d = dedicated(p, q)
            assert d[2] % Q != 0
            assert same_point(d, b.te_add_extended(p, q))


@pytest.mark.parametrize("case", ["double", "inverse", "identity_left", "identity_right",
                                  "identity_twice", "order_two", "order_two_twice"])
def test_every_failure_is_all_zero_and_every_success_is_right(case):
    pts = extended_points(12, 6)
    pairs = {
        "double": [(p, p) for p in pts],
        "inverse": [(p, neg(p)) for p in pts],
        "identity_left": [(IDENTITY, p) for p in pts],
        "identity_right": [(p, IDENTITY) for p in pts],
        "identity_twice": [(IDENTITY, IDENTITY), (ORDER_TWO, IDENTITY), (IDENTITY, ORDER_TWO)],
        "order_two": [(ORDER_TWO, p) for p in pts] + [(p, ORDER_TWO) for p in pts],
        "order_two_twice": [(ORDER_TWO, ORDER_TWO)],
    }[case]
    for p, q in pairs:
        d = dedicated(p, q)
        u = b.te_add_extended(p, q)
        assert u[2] % Q != 0  # the unified formula is complete here
        if d[2] % Q == 0:
            assert all(v % Q == 0 for v in d), "a failure must zero every coordinate"
        else:
            assert same_point(d, u)
    if case == "double":
        assert all(dedicated(p, q)[2] == 0 for p, q in pairs)
    if case in ("inverse", "identity_left", "identity_right", "order_two"):
        assert all(dedicated(p, q)[2] != 0 for p, q in pairs)
