"""CPU oracle for the BLS12-377 G1 multi-scalar multiplication (test infrastructure only).

This module is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg import it.  Everything is plain Python big-int arithmetic,
written from the reference's math and sized for small cases (N up to a few thousand).

What it restates (citations are paths inside the fyquah/hardcaml_zprize tree):

* field and curve constants -- ``zprize/msm_pippenger/host/msm_compute/include/bls12_377_g1/
  bls12_377_g1.h:17-54`` and ``constants.h:7-46``; the G1 generator from
  ``libs/ark_bls12_377_g1/test/test_ark_bls12_377_g1.ml:45-58``;
* the Weierstrass -> Montgomery -> twisted-Edwards map and back --
  ``bls12_377_g1.h:343-447`` (and ``libs/twisted_edwards/model/conversions.ml``);
* the host precompute ((y-x)/2, (y+x)/2, 4d*t) and the precomputed mixed add --
  ``bls12_377_g1.h:606-618`` and ``libs/twisted_edwards/model/twisted_edwards_curve.ml:100-170``;
* the strongly-unified extended addition (add-2008-hwcd-3, k = 2d) -- ``bls12_377_g1.h:449-491``;
* the signed-digit scalar split -- ``zprize/msm_pippenger/hardcaml/test/top/utils.ml:243-288``
  with window sizes from ``hardcaml/src/config_utils.ml:7-41``;
* bucket triangle sums and the window combine -- ``host/msm_compute/include/bls12_377_g1/
  pippenger.h:7-45`` and ``host/driver/driver.cpp:306-375``;
* the Weierstrass fallback for points without a twisted-Edwards image --
  ``bls12_377_g1.h:493-566, 701-742`` and ``driver.cpp:349-372``;
* the ABI of the harness -- ``rust_types.h:73-83`` (g1_affine_t / g1_projective_t, Fq limbs in
  arkworks Montgomery form, R = 2^384) and ``test_fpga_harness/src/lib.rs:18-85``.

The MSM result itself is the unique group element sum k_i * P_i; arkworks' ``into_affine()``
(the harness's comparison, ``test_fpga_harness/tests/msm.rs:35-40``) compares canonical affine
coordinates, so "bit-exact vs arkworks" means equal canonical affine (x, y) or both infinity.
"""
from __future__ import annotations

import struct
from typing import Iterable, List, Optional, Sequence, Tuple

# ---------------------------------------------------------------------------------------------
# constants (bls12_377_g1.h:17-54, constants.h:7-46)
# ---------------------------------------------------------------------------------------------
Q = 0x1AE3A4617C510EAC63B05C06CA1493B1A22D9F300F5138F1EF3622FBA094800170B5D44300000008508C00000000001
R_SCALAR = 0x12AB655E9A2CA55660B44D1E5C37B00159AA76FED00000010A11800000000001
SCALAR_BITS = 253
FIELD_BITS = 377
MONT_R = pow(2, 384, Q)  # the constant the reference names COFACTOR (bls12_377_g1.h:24-26)

# Weierstrass y^2 = x^3 + 1 (a = 0, b = 1)
WEI_A = 0
WEI_B = 1
# Weierstrass -> Montgomery scale s and alpha = -1 (bls12_377_g1.h:40-45, 243-245)
S = 0x19D47D415B5FF60A87A8B7BBAB25EB6427DD58CA38E47030EFD1E6310AC7BF3079221BF2B4BD72C5106E9E70FCC6156
ALPHA = Q - 1
TWISTED_SCALE = 0x363B01DF81A0405E86206F2CC504D147752B91B664D91D4C82FED217902EE874354485836FA3CCBA3AF539C173857B
# twisted Edwards a = -1 and d (bls12_377_g1.h:43-48)
TE_A = Q - 1
TE_D = 0xE2DCEDFF103E7161354A88156E4B00FE66A526A0237CFE5F683497C9AFB7635D5C9307F78E160E14F2B6D4BD949004
TE_K = 0x177F95E65B6BF7FC2F8F4FBE3B4CC6E2AA705A3F51E66D9FDD06FFD95626C6A3ADC8CBBF1C2C1BA4DCADA97B292007
# Montgomery-curve c_A, c_B (bls12_377_g1.h:49-54)
C_A = 0x32D756062D349E59416ECE15CCBF8E86EF0D33183465A42FE2CB65FC1664272E6BB28F0E1C7A7C9C05824AD09ADC01
C_B = S

GEN_X = 0x8848DEFE740A67C8FC6225BF87FF5485951E2CAA9D41BB188282C8BD37CB5CD5481512FFCD394EEAB9B16EB21BE9EF
GEN_Y = 0x1914A69C5102EFF1F674F5D30AFEEC4BD7FB348CA3E52D96D182AD44FB82305C2FE3D3634A9591AFD82DE55559C8EA6

INF = None  # affine point at infinity


def inv(a: int) -> int:
    a %= Q
    if a == 0:
        raise ZeroDivisionError("inverse of 0 mod q")
    return pow(a, Q - 2, Q)


# ---------------------------------------------------------------------------------------------
# affine Weierstrass group law (the arithmetic arkworks' into_affine() results live in;
# the reference's host fallback is bls12_377_g1.h:493-566)
# ---------------------------------------------------------------------------------------------
def on_curve(p) -> bool:
    if p is INF:
        return True
    x, y = p
    return (y * y - x * x * x - WEI_B) % Q == 0


def neg(p):
    if p is INF:
        return INF
    return (p[0], (-p[1]) % Q)


def add(p, q2):
    if p is INF:
        return q2
    if q2 is INF:
        return p
    x1, y1 = p
    x2, y2 = q2
    if x1 == x2:
        if (y1 + y2) % Q == 0:
            return INF
        lam = (3 * x1 * x1 + WEI_A) * inv(2 * y1) % Q
    else:
        lam = (y2 - y1) * inv(x2 - x1) % Q
    x3 = (lam * lam - x1 - x2) % Q
    y3 = (lam * (x1 - x3) - y1) % Q
    return (x3, y3)


def double(p):
    return add(p, p)


# Jacobian coordinates (a = 0) for speed in the Pippenger oracle ------------------------------
JINF = (1, 1, 0)


def to_jac(p):
    return JINF if p is INF else (p[0], p[1], 1)


def from_jac(p):
    X, Y, Z = p
    if Z % Q == 0:
        return INF
    zi = inv(Z)
    zi2 = zi * zi % Q
    return (X * zi2 % Q, Y * zi2 * zi % Q)


def jdouble(p):
    X, Y, Z = p
    if Z == 0 or Y == 0:
        return JINF
    A = X * X % Q
    B = Y * Y % Q
    C = B * B % Q
    D = 2 * ((X + B) * (X + B) - A - C) % Q
    E = 3 * A % Q
    F = E * E % Q
    X3 = (F - 2 * D) % Q
    Y3 = (E * (D - X3) - 8 * C) % Q
    Z3 = 2 * Y * Z % Q
    return (X3, Y3, Z3)


def jadd(p, q2):
    X1, Y1, Z1 = p
    X2, Y2, Z2 = q2
    if Z1 == 0:
        return q2
    if Z2 == 0:
        return p
    Z1Z1 = Z1 * Z1 % Q
    Z2Z2 = Z2 * Z2 % Q
    U1 = X1 * Z2Z2 % Q
    U2 = X2 * Z1Z1 % Q
    S1 = Y1 * Z2 * Z2Z2 % Q
    S2 = Y2 * Z1 * Z1Z1 % Q
    if U1 == U2:
        if S1 == S2:
            return jdouble(p)
        return JINF
    H = (U2 - U1) % Q
    I = (2 * H) * (2 * H) % Q
    J = H * I % Q
    rr = 2 * (S2 - S1) % Q
    V = U1 * I % Q
    X3 = (rr * rr - J - 2 * V) % Q
    Y3 = (rr * (V - X3) - 2 * S1 * J) % Q
    Z3 = ((Z1 + Z2) * (Z1 + Z2) - Z1Z1 - Z2Z2) * H % Q
    return (X3, Y3, Z3)


def mul(p, k: int):
    """k*P by double-and-add (Weierstrass; bls12_377_g1.h:701-724 does the same over bits)."""
    acc = JINF
    base = to_jac(p)
    while k > 0:
        if k & 1:
            acc = jadd(acc, base)
        base = jdouble(base)
        k >>= 1
    return from_jac(acc)


GEN = (GEN_X, GEN_Y)


# ---------------------------------------------------------------------------------------------
# twisted-Edwards map and arithmetic (bls12_377_g1.h:343-491, 582-618)
# ---------------------------------------------------------------------------------------------
def weierstrass_to_te(p) -> Optional[Tuple[int, int]]:
    """affineWeierstrassToExtendedTwistedEdwards (bls12_377_g1.h:361-415); None if unmappable."""
    if p is INF:
        return (0, 1)
    x, y = p
    u = (x - ALPHA) * S % Q        # affineWeierstrassToMontgomery (:361-365)
    v = S * y % Q
    if v == 0 or (u + 1) % Q == 0:  # affineMontgomeryToTwistedEdwards fails (:382-384)
        return None
    xe = TWISTED_SCALE * u * inv(v) % Q
    ye = (u - 1) * inv(u + 1) % Q
    return (xe, ye)


def te_to_weierstrass(p):
    """extendedTwistedEdwardsToWeierstrass (bls12_377_g1.h:389-402, 366-374, 417-425).

    The reference maps both x = 0 points to infinity (:393-396).  (0, -1) is a genuine point of
    order two; the oracle maps it to its Weierstrass image so that results stay group-correct.
    """
    xe, ye = p
    if xe % Q == 0:
        if ye % Q == 1:
            return INF
        # (0, -1) <-> Montgomery (0, 0) <-> Weierstrass (c_A / (3 c_B), 0)
        return (C_A * inv(3 * C_B) % Q, 0)
    u = (1 + ye) * inv(1 - ye) % Q
    v = u * TWISTED_SCALE * inv(xe) % Q
    xw = (u * inv(C_B) + C_A * inv(3 * C_B)) % Q
    yw = v * inv(C_B) % Q
    return (xw, yw)


def te_on_curve(p) -> bool:
    x, y = p
    return (TE_A * x * x + y * y - 1 - TE_D * x * x * y * y) % Q == 0


def te_add_extended(p1, p2):
    """generalUnifiedAddInto, add-2008-hwcd-3 with k = 2d (bls12_377_g1.h:449-491)."""
    X1, Y1, Z1, T1 = p1
    X2, Y2, Z2, T2 = p2
    A = (Y1 - X1) * (Y2 - X2) % Q
    B = (Y1 + X1) * (Y2 + X2) % Q
    C = T1 * TE_K % Q * T2 % Q
    D = Z1 * 2 * Z2 % Q
    E, F, G, H = (B - A) % Q, (D - C) % Q, (D + C) % Q, (B + A) % Q
    return (E * F % Q, G * H % Q, F * G % Q, E * H % Q)


def te_extended(p):
    x, y = p
    return (x, y, 1, x * y % Q)


def te_affine(pe):
    X, Y, Z, T = pe
    zi = inv(Z)
    return (X * zi % Q, Y * zi % Q)


def te_precompute(p):
    """preComputeFPGA (bls12_377_g1.h:606-618): (x, y) -> ((y-x)/2, (y+x)/2, 4d*x*y)."""
    x, y = p
    h = inv(2)
    return ((y - x) * h % Q, (y + x) * h % Q, 4 * TE_D * x * y % Q)


def te_madd_fpga(acc, pre, subtract=False):
    """add_unified_precomputed (twisted_edwards_curve.ml:142-170): (2x,2y,4z,t)-form bucket
    plus a precomputed host point; subtract swaps the first two coordinates and negates t."""
    x1, y1, z1, t1 = acc
    xh, yh, th = pre
    if subtract:
        xh, yh, th = yh, xh, (-th) % Q
    cA = x1 * xh % Q
    cB = y1 * yh % Q
    cC = t1 * th % Q
    cD = z1
    cE, cF, cG, cH = (cB - cA) % Q, (cD - cC) % Q, (cD + cC) % Q, (cB + cA) % Q
    px = cE * cF % Q
    py = cG * cH % Q
    return ((py - px) % Q, (py + px) % Q, cF * cG % Q, cE * cH % Q)


def te_fpga_identity():
    """bucket RAM initial value (2, 2, 4, 0) (hardcaml/src/top.ml:115-128)."""
    return (2, 2, 4, 0)


def te_from_fpga(pe):
    """postComputeFPGA (bls12_377_g1.h:582-599): (2(y-x),2(y+x),4z,t) -> extended."""
    X, Y, Z, T = pe
    q4 = inv(4)
    return ((Y - X) * q4 % Q, (Y + X) * q4 % Q, Z * q4 % Q, T)


# ---------------------------------------------------------------------------------------------
# scalar split (hardcaml/test/top/utils.ml:243-288; config_utils.ml:7-41)
# ---------------------------------------------------------------------------------------------
def reference_window_sizes(scalar_bits: int, num_windows: int) -> List[int]:
    lower = scalar_bits // num_windows
    higher = scalar_bits - lower * num_windows
    return [lower + 1 if i < higher else lower for i in range(num_windows)]


def reference_num_buckets(sizes: Sequence[int], w: int) -> int:
    if w == len(sizes) - 1:
        return (1 << sizes[w]) - 1
    return 1 << (sizes[w] - 1)


def signed_digits(scalar: int, sizes: Sequence[int]) -> List[int]:
    """perform_scalar_reduction: slice + carry; if >= 2^(b-1) subtract 2^b and carry; the top
    window stays unsigned.  Returns signed digits d_w with scalar = sum d_w 2^offset_w."""
    out = []
    carry = 0
    off = 0
    for i, b in enumerate(sizes):
        sl = ((scalar >> off) & ((1 << b) - 1)) + carry
        if i == len(sizes) - 1:
            out.append(sl)
        elif sl >= (1 << b):
            carry = 1
            out.append(0)
        elif sl >= (1 << (b - 1)):
            carry = 1
            out.append(sl - (1 << b))
        else:
            carry = 0
            out.append(sl)
        off += b
    assert sum(d << o for d, o in zip(out, offsets(sizes))) == scalar
    return out


def offsets(sizes: Sequence[int]) -> List[int]:
    o, acc = [], 0
    for b in sizes:
        o.append(acc)
        acc += b
    return o


def uniform_window_sizes(c: int, scalar_bits: int = SCALAR_BITS) -> List[int]:
    """The GPU engine's layout: ceil(253/c) windows of c bits, the top one holding the rest."""
    w = -(-scalar_bits // c)
    return [c] * (w - 1) + [scalar_bits - c * (w - 1)]


# ---------------------------------------------------------------------------------------------
# MSM oracles
# ---------------------------------------------------------------------------------------------
def msm_naive(points: Sequence, scalars: Sequence[int]):
    acc = JINF
    for p, k in zip(points, scalars):
        k &= (1 << SCALAR_BITS) - 1
        if k and p is not INF:
            acc = jadd(acc, to_jac(mul(p, k)))
    return from_jac(acc)


def msm_pippenger(points: Sequence, scalars: Sequence[int], c: int = 8):
    """Signed-window Pippenger in Jacobian Weierstrass coordinates: bucket sums, the running
    (triangle) sum of pippenger.h:25-33 and a Horner window combine (pippenger.h:36-45)."""
    sizes = uniform_window_sizes(c)
    offs = offsets(sizes)
    nwin = len(sizes)
    digits = [signed_digits(k & ((1 << SCALAR_BITS) - 1), sizes) for k in scalars]
    total = JINF
    for w in reversed(range(nwin)):
        nb = max(1 << (c - 1), 1 << sizes[w]) if w == nwin - 1 else 1 << (c - 1)
        buckets = [JINF] * (nb + 1)
        for p, dg in zip(points, digits):
            d = dg[w]
            if d == 0 or p is INF:
                continue
            pj = to_jac(p if d > 0 else neg(p))
            buckets[abs(d)] = jadd(buckets[abs(d)], pj)
        running = JINF
        acc = JINF
        for b in range(nb, 0, -1):
            running = jadd(running, buckets[b])
            acc = jadd(acc, running)
        if w < nwin - 1:
            for _ in range(offs[w + 1] - offs[w]):
                total = jdouble(total)
        total = jadd(total, acc)
    return from_jac(total)


# ---------------------------------------------------------------------------------------------
# deterministic generators (SplitMix64, counter-based so every element is independent)
# ---------------------------------------------------------------------------------------------
M64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def splitmix64(x: int) -> int:
    """One SplitMix64 output for state x (Steele, Lea, Flood 2014)."""
    z = (x + GOLDEN) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def rand_u64(seed: int, stream: int, index: int, word: int) -> int:
    """Counter-based 64-bit draw: word `word` of element `index` in stream `stream`."""
    s = splitmix64((seed ^ ((stream * 0xD1B54A32D192ED03) & M64)) & M64)
    h = splitmix64(s ^ splitmix64(index & M64))
    return splitmix64((h + word) & M64)


STREAM_BASE_K = 1
STREAM_SCALAR = 2
STREAM_MIX = 3


def base_multiplier(seed: int, i: int) -> int:
    """k_i for base i = k_i * G: a uniform 64-bit value."""
    return rand_u64(seed, STREAM_BASE_K, i, 0)


def uniform_scalar(seed: int, i: int, stream: int = STREAM_SCALAR) -> int:
    """Uniform in [0, r): 253-bit draws (words 4a..4a+3 for attempt a), rejected while >= r."""
    a = 0
    while True:
        w = [rand_u64(seed, stream, i, 4 * a + j) for j in range(4)]
        v = w[0] | (w[1] << 64) | (w[2] << 128) | ((w[3] & ((1 << 61) - 1)) << 192)
        if v < R_SCALAR:
            return v
        a += 1


def gen_bases(seed: int, n: int):
    return [mul(GEN, base_multiplier(seed, i)) for i in range(n)]


def gen_scalars(seed: int, n: int):
    return [uniform_scalar(seed, i) for i in range(n)]


def mixed_scalar(seed: int, msm: int, i: int) -> int:
    """Scalar mix of the uneven-batch workload: 70% uniform 253-bit, 10% uniform 16-bit,
    10% edge (0 or r-1, half each), 10% one repeated value per MSM."""
    sel = rand_u64(seed, STREAM_MIX, (msm << 32) | i, 0) % 10
    if sel < 7:
        return uniform_scalar(seed, (msm << 32) | i)
    if sel == 7:
        return rand_u64(seed, STREAM_MIX, (msm << 32) | i, 1) & 0xFFFF
    if sel == 8:
        return 0 if rand_u64(seed, STREAM_MIX, (msm << 32) | i, 2) & 1 == 0 else R_SCALAR - 1
    return uniform_scalar(seed, (msm << 32) | 0xFFFFFFFF)


# ---------------------------------------------------------------------------------------------
# harness ABI encoding (rust_types.h:8-9, 73-83)
# ---------------------------------------------------------------------------------------------
def limbs64(v: int, n: int) -> List[int]:
    return [(v >> (64 * i)) & M64 for i in range(n)]


def from_limbs64(ws: Iterable[int]) -> int:
    return sum(int(w) << (64 * i) for i, w in enumerate(ws))


def to_mont(v: int) -> int:
    return v * MONT_R % Q


def from_mont(v: int) -> int:
    return v * inv(MONT_R) % Q


def encode_affine(p) -> bytes:
    """g1_affine_t {u64 x[6]; u64 y[6]; bool infinity;} padded to 104 bytes, arkworks
    Montgomery form; infinity is (0, 1, true) as arkworks' zero()."""
    if p is INF:
        return struct.pack("<6Q6Q?7x", *limbs64(0, 6), *limbs64(to_mont(1), 6), True)
    return struct.pack("<6Q6Q?7x", *limbs64(to_mont(p[0]), 6), *limbs64(to_mont(p[1]), 6), False)


def encode_scalar(k: int) -> bytes:
    return struct.pack("<4Q", *limbs64(k, 4))


def encode_projective(p) -> bytes:
    """An affine result as the engine writes it (bls12_377_g1.h:667-690): g1_projective_t with
    Z = 1 in Montgomery form, (x R, y R, R); infinity as arkworks' zero(), (R, R, 0)."""
    if p is INF:
        return struct.pack("<18Q", *limbs64(to_mont(1), 6), *limbs64(to_mont(1), 6), *limbs64(0, 6))
    return struct.pack("<18Q", *limbs64(to_mont(p[0]), 6), *limbs64(to_mont(p[1]), 6),
                       *limbs64(to_mont(1), 6))


def decode_projective(b: bytes):
    """g1_projective_t {x[6], y[6], z[6]} as an arkworks Jacobian point in Montgomery form ->
    canonical affine (what into_affine() returns)."""
    w = struct.unpack("<18Q", b)
    X = from_mont(from_limbs64(w[0:6]))
    Y = from_mont(from_limbs64(w[6:12]))
    Z = from_mont(from_limbs64(w[12:18]))
    return from_jac((X, Y, Z))


def parse_hex_point(xh: str, yh: str):
    return (int(xh, 16) % Q, int(yh, 16) % Q)
