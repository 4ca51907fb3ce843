// Base field of BLS12-377 (q, 377 bits) on sm_103a: twelve 32-bit limbs, Montgomery form with
// R = 2^384 -- the same R as arkworks' six 64-bit limbs, so a device element is bit-for-bit the
// arkworks Fq representation once it is fully reduced.
//
// Values are kept "lazy" in [0, 2q): 4q < 2^384, so the CIOS product of two such values is again
// below 2q without a final subtraction.  Addition/subtraction reduce by 2q.  fq_canon() brings a
// value to [0, q) for comparisons and for the ABI.
//
// The multiplier is operand-scanning CIOS with 32 x 32 -> 64 wide multiplies: 12 + 11 limb
// products per row (q's lowest limb is 1), 276 wide IMADs per product.  The algorithmic count for
// the roofline stays 588 32-bit IMAD per product (lo and hi halves of 12 x 12 + 12 x 12).
// The field is the one the reference computes in with GMP (host/msm_compute/include/
// bls12_377_g1/bls12_377_g1.h:31-33, 90-219); the limb layout is new.
#pragma once
#include <stdint.h>

#include "fq_divstep.cuh"

#define FQ_LIMBS 12

// q and 2q, little-endian 32-bit limbs
#define BLS_Q {0x00000001u, 0x8508c000u, 0x30000000u, 0x170b5d44u, 0xba094800u, 0x1ef3622fu, 0x00f5138fu, 0x1a22d9f3u, 0x6ca1493bu, 0xc63b05c0u, 0x17c510eau, 0x01ae3a46u}
#define BLS_Q2 {0x00000002u, 0x0a118000u, 0x60000001u, 0x2e16ba88u, 0x74129000u, 0x3de6c45fu, 0x01ea271eu, 0x3445b3e6u, 0xd9429276u, 0x8c760b80u, 0x2f8a21d5u, 0x035c748cu}
// -q^-1 mod 2^32 (q = 1 mod 2^46)
#define BLS_QINV 0xffffffffu
// Montgomery-form constants (value * 2^384 mod q)
#define BLS_ONE {0xffffff68u, 0x02cdffffu, 0x7fffffb1u, 0x51409f83u, 0x8a7d3ff2u, 0x9f7db3a9u, 0x6e7c6305u, 0x7b4e97b7u, 0x803c84e8u, 0x4cf495bfu, 0xe2fdf49au, 0x008d6661u}
#define BLS_INV2 {0xffffffb4u, 0x8166ffffu, 0xbfffffd8u, 0x28a04fc1u, 0xc53e9ff9u, 0xcfbed9d4u, 0xb73e3182u, 0x3da74bdbu, 0xc01e4274u, 0x267a4adfu, 0xf17efa4du, 0x0046b330u}
// twisted Edwards k = 2d and d (bls12_377_g1.h:37-39, 46-48)
#define BLS_TE_K {0xbb58e892u, 0x33f6817bu, 0xff054e5du, 0x3fd664cau, 0xd6752edau, 0x6ad7181au, 0x47ff7cfeu, 0x55eabefau, 0x93fe9656u, 0xacf17111u, 0x199ed6ffu, 0x008d1a81u}
#define BLS_TE_D {0xddac7449u, 0x99fb40bdu, 0x7f82a72eu, 0x1feb3265u, 0x6b3a976du, 0x356b8c0du, 0x23ffbe7fu, 0x2af55f7du, 0xc9ff4b2bu, 0xd678b888u, 0x8ccf6b7fu, 0x00468d40u}
// Weierstrass -> Montgomery scale s (bls12_377_g1.h:40-42) and the twisted scale (:34-36)
#define BLS_WS {0x27ce5f5fu, 0x171ef565u, 0x214ae372u, 0x6e5b6922u, 0x26a8cea6u, 0xc47c7b6au, 0x2d74b055u, 0xc22f509cu, 0xcbda4b0au, 0x0134cecbu, 0x229913d6u, 0x001ef3f3u}
#define BLS_TWISTED_SCALE {0xe4aeaf1eu, 0x432a25c1u, 0xcd4c9661u, 0x5b39d21fu, 0xcd09455du, 0x692669ecu, 0x0f74f6bbu, 0xddae3345u, 0xabb65d37u, 0x76cbfeebu, 0x517df4cdu, 0x0143462fu}
// 1/c_B and c_A/(3 c_B) of the Montgomery -> Weierstrass map (bls12_377_g1.h:366-374)
#define BLS_INV_CB {0x776b1e1du, 0x455ce02fu, 0x63e0aa56u, 0x4b123b66u, 0x73fa6bf3u, 0x4d75723eu, 0x885e1101u, 0x468df1d4u, 0x638ee120u, 0x039e6c63u, 0x67cb3b82u, 0x005cdbd9u}
#define BLS_CA_OVER_3CB {0x00000099u, 0x823ac000u, 0xb000004fu, 0xc5cabdc0u, 0x2f8c080du, 0x7f75ae86u, 0x9278b089u, 0x9ed4423bu, 0xec64c452u, 0x79467000u, 0x34c71c50u, 0x0120d3e4u}
// R^3 mod q: turns a plain inverse of a Montgomery-form value into the Montgomery-form inverse
#define BLS_R3 {0x8815de20u, 0x581f532fu, 0xbe329585u, 0xe50f4148u, 0x0449f513u, 0x2be8b118u, 0xc804a20eu, 0x6a2a9516u, 0x13590cb9u, 0x3f725407u, 0xc0e7dda5u, 0x01065ab4u}
// q - 2, the Fermat inversion exponent
#define BLS_QM2 {0xffffffffu, 0x8508bfffu, 0x30000000u, 0x170b5d44u, 0xba094800u, 0x1ef3622fu, 0x00f5138fu, 0x1a22d9f3u, 0x6ca1493bu, 0xc63b05c0u, 0x17c510eau, 0x01ae3a46u}

struct fq_t {
  uint32_t v[FQ_LIMBS];
};

// ---- carry-chain primitives (one PTX instruction each; the carry flag lives between them) ----
__device__ __forceinline__ uint32_t madlo_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("mad.lo.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t madclo_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("madc.lo.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t madhi_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("mad.hi.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t madchi_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("madc.hi.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t madchi(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("madc.hi.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t add_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("add.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t addc_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t addc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("addc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t sub_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t subc_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t subc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("subc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}

// ---- constructors ----
__device__ __forceinline__ fq_t fq_from(const uint32_t (&c)[FQ_LIMBS]) {
  fq_t r;
#pragma unroll
  for (int i = 0; i < FQ_LIMBS; i++) r.v[i] = c[i];
  return r;
}
__device__ __forceinline__ fq_t fq_zero() {
  fq_t r;
#pragma unroll
  for (int i = 0; i < FQ_LIMBS; i++) r.v[i] = 0;
  return r;
}
__device__ __forceinline__ fq_t fq_one() {
  const uint32_t c[FQ_LIMBS] = BLS_ONE;
  return fq_from(c);
}

// ---- a * b * 2^-384 mod q (CIOS; inputs and output in [0, 2q)) ----
// Each row adds b_i * a and then m * q to the running value t, m = -t0 (q = 1 mod 2^32 and
// -q^-1 = -1 mod 2^32, so the row factor needs no product and m * q0 + t0 = 0 with a carry of
// (t0 != 0)).  The limb products are wide multiplies with no addend: a wide multiply whose 64-bit
// addend is a 32-bit carry needs that carry moved into an aligned register pair with a zero high
// half, and a carry folded in before the multiply needs an add-with-carry that the compiler puts
// on the multiply pipe.  Instead each row sums four word vectors -- the products' low words, their
// high words one word up, and the same two of m * q -- in four add.cc/addc.cc chains, which run on
// the integer ALU pipe.  Per product (ncu, sm_103a): 276 wide multiplies and about 50 other
// multiply-pipe instructions, against 276 and 336 for a 64-bit-accumulator CIOS; the two pipes
// are then about equally busy.
// Bound: at the start of a row t < 4q < 2^384 (so t[12] = 0) and no row sum leaves 13 words, for
// any a < 2^383 and any b.
__device__ __forceinline__ fq_t fq_mul(const fq_t &a, const fq_t &b) {
  const uint32_t q[FQ_LIMBS] = BLS_Q;
  uint32_t t[FQ_LIMBS + 1];
#pragma unroll
  for (int i = 0; i < FQ_LIMBS; i++) {
    const uint32_t bi = b.v[i];
    uint32_t lo[FQ_LIMBS], hi[FQ_LIMBS];
#pragma unroll
    for (int j = 0; j < FQ_LIMBS; j++) {
      const uint64_t p = (uint64_t)a.v[j] * bi;
      lo[j] = (uint32_t)p;
      hi[j] = (uint32_t)(p >> 32);
    }
    if (i == 0) {
#pragma unroll
      for (int j = 0; j < FQ_LIMBS; j++) t[j] = lo[j];
      t[FQ_LIMBS] = 0;
    } else {
      t[0] = add_cc(t[0], lo[0]);
#pragma unroll
      for (int j = 1; j < FQ_LIMBS; j++) t[j] = addc_cc(t[j], lo[j]);
      t[FQ_LIMBS] = addc(0u, 0u);
    }
    t[1] = add_cc(t[1], hi[0]);
#pragma unroll
    for (int j = 2; j < FQ_LIMBS; j++) t[j] = addc_cc(t[j], hi[j - 1]);
    t[FQ_LIMBS] = addc(t[FQ_LIMBS], hi[FQ_LIMBS - 1]);
    const uint32_t m = 0u - t[0];
#pragma unroll
    for (int j = 1; j < FQ_LIMBS; j++) {
      const uint64_t p = (uint64_t)m * q[j];
      lo[j] = (uint32_t)p;
      hi[j] = (uint32_t)(p >> 32);
    }
    add_cc(t[0], m);  // t0 + m = 0 mod 2^32 with a carry of (t0 != 0)
#pragma unroll
    for (int j = 1; j < FQ_LIMBS; j++) t[j] = addc_cc(t[j], lo[j]);
    t[FQ_LIMBS] = addc(t[FQ_LIMBS], 0u);
    t[2] = add_cc(t[2], hi[1]);
#pragma unroll
    for (int j = 3; j < FQ_LIMBS; j++) t[j] = addc_cc(t[j], hi[j - 1]);
    t[FQ_LIMBS] = addc(t[FQ_LIMBS], hi[FQ_LIMBS - 1]);
#pragma unroll
    for (int j = 0; j < FQ_LIMBS; j++) t[j] = t[j + 1];
  }
  fq_t r;
#pragma unroll
  for (int j = 0; j < FQ_LIMBS; j++) r.v[j] = t[j];
  return r;
}

__device__ __forceinline__ fq_t fq_sqr(const fq_t &a) { return fq_mul(a, a); }

// r = x - 2q if x >= 2q else x   (x < 4q < 2^384)
__device__ __forceinline__ fq_t fq_reduce_2q(const uint32_t (&x)[FQ_LIMBS]) {
  const uint32_t q2[FQ_LIMBS] = BLS_Q2;
  uint32_t d[FQ_LIMBS];
  d[0] = sub_cc(x[0], q2[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS; j++) d[j] = subc_cc(x[j], q2[j]);
  const uint32_t borrow = subc(0u, 0u);  // 0xffffffff if x < 2q
  fq_t r;
#pragma unroll
  for (int j = 0; j < FQ_LIMBS; j++) r.v[j] = borrow ? x[j] : d[j];
  return r;
}

__device__ __forceinline__ fq_t fq_add(const fq_t &a, const fq_t &b) {
  uint32_t s[FQ_LIMBS];
  s[0] = add_cc(a.v[0], b.v[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS - 1; j++) s[j] = addc_cc(a.v[j], b.v[j]);
  s[FQ_LIMBS - 1] = addc(a.v[FQ_LIMBS - 1], b.v[FQ_LIMBS - 1]);
  return fq_reduce_2q(s);
}

__device__ __forceinline__ fq_t fq_sub(const fq_t &a, const fq_t &b) {
  const uint32_t q2[FQ_LIMBS] = BLS_Q2;
  uint32_t d[FQ_LIMBS];
  d[0] = sub_cc(a.v[0], b.v[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS; j++) d[j] = subc_cc(a.v[j], b.v[j]);
  const uint32_t mask = subc(0u, 0u);  // all ones on borrow
  fq_t r;
  r.v[0] = add_cc(d[0], q2[0] & mask);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS - 1; j++) r.v[j] = addc_cc(d[j], q2[j] & mask);
  r.v[FQ_LIMBS - 1] = addc(d[FQ_LIMBS - 1], q2[FQ_LIMBS - 1] & mask);
  return r;
}

// Unreduced forms for operands that only feed products: for a, b < 2q, a + b and a - b + 2q are
// below 4q, and a product of two values below 4q is again below 2q (16q < 2^384).
__device__ __forceinline__ fq_t fq_add_lazy(const fq_t &a, const fq_t &b) {
  fq_t r;
  r.v[0] = add_cc(a.v[0], b.v[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS - 1; j++) r.v[j] = addc_cc(a.v[j], b.v[j]);
  r.v[FQ_LIMBS - 1] = addc(a.v[FQ_LIMBS - 1], b.v[FQ_LIMBS - 1]);
  return r;
}
__device__ __forceinline__ fq_t fq_sub_lazy(const fq_t &a, const fq_t &b) {
  const uint32_t q2[FQ_LIMBS] = BLS_Q2;
  uint32_t d[FQ_LIMBS];
  d[0] = add_cc(a.v[0], q2[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS; j++) d[j] = addc_cc(a.v[j], q2[j]);
  fq_t r;
  r.v[0] = sub_cc(d[0], b.v[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS - 1; j++) r.v[j] = subc_cc(d[j], b.v[j]);
  r.v[FQ_LIMBS - 1] = subc(d[FQ_LIMBS - 1], b.v[FQ_LIMBS - 1]);
  return r;
}

__device__ __forceinline__ fq_t fq_neg(const fq_t &a) { return fq_sub(fq_zero(), a); }

__device__ __forceinline__ fq_t fq_dbl(const fq_t &a) { return fq_add(a, a); }

// [0, 2q) -> [0, q)
__device__ __forceinline__ fq_t fq_canon(const fq_t &a) {
  const uint32_t q[FQ_LIMBS] = BLS_Q;
  uint32_t d[FQ_LIMBS];
  d[0] = sub_cc(a.v[0], q[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS; j++) d[j] = subc_cc(a.v[j], q[j]);
  const uint32_t borrow = subc(0u, 0u);
  fq_t r;
#pragma unroll
  for (int j = 0; j < FQ_LIMBS; j++) r.v[j] = borrow ? a.v[j] : d[j];
  return r;
}

__device__ __forceinline__ bool fq_is_zero(const fq_t &a) {
  const fq_t c = fq_canon(a);
  uint32_t acc = 0;
#pragma unroll
  for (int j = 0; j < FQ_LIMBS; j++) acc |= c.v[j];
  return acc == 0;
}

__device__ __forceinline__ bool fq_eq(const fq_t &a, const fq_t &b) {
  const fq_t x = fq_canon(a), y = fq_canon(b);
  uint32_t acc = 0;
#pragma unroll
  for (int j = 0; j < FQ_LIMBS; j++) acc |= x.v[j] ^ y.v[j];
  return acc == 0;
}

__device__ __forceinline__ fq_t fq_select(bool c, const fq_t &a, const fq_t &b) {
  fq_t r;
#pragma unroll
  for (int j = 0; j < FQ_LIMBS; j++) r.v[j] = c ? a.v[j] : b.v[j];
  return r;
}

// a^(q-2) = a^-1 (0 -> 0): left-to-right 4-bit fixed windows over the exponent.
static __device__ __noinline__ fq_t fq_inv(const fq_t &a) {
  const uint32_t e[FQ_LIMBS] = BLS_QM2;
  fq_t tbl[16];
  tbl[0] = fq_one();
  tbl[1] = a;
#pragma unroll 1
  for (int i = 2; i < 16; i++) tbl[i] = fq_mul(tbl[i - 1], a);
  fq_t r = fq_one();
  bool started = false;
#pragma unroll 1
  for (int w = FQ_LIMBS * 8 - 1; w >= 0; w--) {
    const uint32_t nib = (e[w >> 3] >> ((w & 7) * 4)) & 15u;
    if (started) {
      r = fq_sqr(r);
      r = fq_sqr(r);
      r = fq_sqr(r);
      r = fq_sqr(r);
    }
    if (nib) {
      r = started ? fq_mul(r, tbl[nib]) : tbl[nib];
      started = true;
    }
  }
  return r;
}

// ---- variable-time inversion by Bernstein-Yang divsteps (fq_divstep.cuh) ----
// Montgomery-form inverse (0 -> 0).  With a = xR, the integer inverse of a times R^3 through one
// Montgomery product gives x^-1 R.  One thread; about 25 batches of 30 divsteps replace the
// ~750 serial rounds of a binary extended Euclid (k_final of a 2^12-point MSM: 97 -> 71 us).
static __device__ __noinline__ fq_t fq_inv_vartime(const fq_t &a) {
  const fq_t c = fq_canon(a);
  const uint32_t q[FQ_LIMBS] = BLS_Q;
  fq_t inv;
  ds_inverse(c.v, q, inv.v);
  const uint32_t r3[FQ_LIMBS] = BLS_R3;
  return fq_mul(inv, fq_from(r3));
}

// The same inverse computed by the four lanes of a quad together (all four hold `a`; `mask`
// covers them).  Every batch's four combinations (f, g, d, e) run one per lane through one code
// path and are exchanged by shuffles, so a batch costs one combination instead of four on one
// thread.  All four lanes return the inverse.
static __device__ __noinline__ fq_t fq_inv_quad(const fq_t &a, uint32_t mask) {
  const int l = (int)(threadIdx.x & 3);
  const fq_t c = fq_canon(a);
  const uint32_t q12[FQ_LIMBS] = BLS_Q;
  uint32_t f[DS_LIMBS], g[DS_LIMBS], d[DS_LIMBS], e[DS_LIMBS], q[DS_LIMBS];
  uint32_t nz = 0;
#pragma unroll
  for (int i = 0; i < FQ_LIMBS; i++) {
    f[i] = q[i] = q12[i];
    g[i] = c.v[i];
    d[i] = e[i] = 0;
    nz |= c.v[i];
  }
  f[12] = g[12] = d[12] = e[12] = q[12] = 0;
  e[0] = 1;
  if (!nz) return fq_zero();
  int delta = 1;
#pragma unroll 1
  for (int batch = 0; batch < 64; batch++) {
    int32_t u, v, qq, r;
    delta = ds_batch30(delta, f[0], g[0], u, v, qq, r);
    // lane 0: f' = (u f + v g) / 2^30, lane 1: g' = (qq f + r g) / 2^30, lanes 2, 3: d', e' mod q
    uint32_t x[DS_LIMBS], y[DS_LIMBS], res[DS_LIMBS];
#pragma unroll
    for (int i = 0; i < DS_LIMBS; i++) {
      x[i] = l < 2 ? f[i] : d[i];
      y[i] = l < 2 ? g[i] : e[i];
    }
    ds_combine_any(res, (l & 1) ? qq : u, x, (l & 1) ? r : v, y, q, l >= 2);
    uint32_t gz = 0;
#pragma unroll
    for (int i = 0; i < DS_LIMBS; i++) {
      f[i] = __shfl_sync(mask, res[i], 0, 4);
      g[i] = __shfl_sync(mask, res[i], 1, 4);
      d[i] = __shfl_sync(mask, res[i], 2, 4);
      e[i] = __shfl_sync(mask, res[i], 3, 4);
      gz |= g[i];
    }
    if (gz == 0) break;  // the same on all four lanes
  }
  if (ds_is_neg(f)) {  // f = -1: the inverse is q - d
    int64_t acc = 0;
#pragma unroll
    for (int i = 0; i < DS_LIMBS; i++) {
      acc += (int64_t)q[i] - (int64_t)d[i];
      d[i] = (uint32_t)acc;
      acc >>= 32;
    }
  }
  fq_t inv;
#pragma unroll
  for (int i = 0; i < FQ_LIMBS; i++) inv.v[i] = d[i];
  const uint32_t r3[FQ_LIMBS] = BLS_R3;
  return fq_mul(inv, fq_from(r3));
}

// ---- 16-byte vector loads/stores of field elements ----
__device__ __forceinline__ void fq_load(fq_t &r, const uint4 *p) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const uint4 u = p[k];
    r.v[4 * k + 0] = u.x;
    r.v[4 * k + 1] = u.y;
    r.v[4 * k + 2] = u.z;
    r.v[4 * k + 3] = u.w;
  }
}
__device__ __forceinline__ void fq_store(uint4 *p, const fq_t &a) {
#pragma unroll
  for (int k = 0; k < 3; k++) p[k] = make_uint4(a.v[4 * k], a.v[4 * k + 1], a.v[4 * k + 2], a.v[4 * k + 3]);
}
