// Inversion modulo q by Bernstein-Yang divsteps ("Fast constant-time gcd computation and modular
// inversion", D. J. Bernstein and B.-Y. Yang, TCHES 2019), in the variable-time form: the loop
// stops as soon as g reaches zero, which is fine here because nothing in an MSM is secret.
//
// State (delta, f, g) with f odd, started at (1, q, a).  One divstep is
//   delta > 0 and g odd:  (delta, f, g) <- (1 - delta, g, (g - f) / 2)
//   g odd:                (delta, f, g) <- (1 + delta, f, (g + f) / 2)
//   g even:               (delta, f, g) <- (1 + delta, f, g / 2)
// and ends with g = 0, f = +-gcd(a, q) = +-1.  d and e follow f and g modulo q (f = d a, g = e a),
// so a^-1 = +-d.  The steps only look at the low bits of f and g, so they run in batches of 30
// on the low 32-bit words, which yields a 2 x 2 matrix with entries below 2^30 in magnitude
// (each row's |entries| sum to at most 2^30); the matrix is then applied once to the full f, g
// (exact division by 2^30) and to d, e (division by 2^30 modulo q: q = 1 mod 2^46, so adding
// (-t mod 2^30) q makes t divisible).  About 25 batches for a 377-bit input, against about 750
// serial shift/subtract rounds of a binary extended Euclid.
//
// Plain integer code (host and device): signed values are 13 limbs of 32 bits, two's complement.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define FQ_HD __host__ __device__ __forceinline__
#else
#define FQ_HD inline
#endif

#define DS_LIMBS 13

FQ_HD int ds_ctz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __ffs((int)x) - 1;
#else
  return __builtin_ctz(x);
#endif
}

// 30 divsteps on the low words of f and g; returns delta and the transition matrix
// [u v; q r] with 2^30 (f', g') = (u f + v g, q f + r g).
FQ_HD int ds_batch30(int delta, uint32_t f, uint32_t g, int32_t &u, int32_t &v, int32_t &q,
                     int32_t &r) {
  int32_t uu = 1, vv = 0, qq = 0, rr = 1;
  int left = 30;
  while (left > 0) {
    if (g == 0) {  // the rest of the batch is halvings
      uu = (int32_t)((uint32_t)uu << left);
      vv = (int32_t)((uint32_t)vv << left);
      delta += left;
      break;
    }
    int z = ds_ctz32(g);
    if (z > left) z = left;
    if (z) {  // a run of even g: halve z times at once
      g >>= z;
      uu = (int32_t)((uint32_t)uu << z);
      vv = (int32_t)((uint32_t)vv << z);
      delta += z;
      left -= z;
      if (left == 0) break;
    }
    // g is odd
    if (delta > 0) {
      delta = 1 - delta;
      const uint32_t nf = g;
      g = (g - f) >> 1;
      f = nf;
      const int32_t nu = 2 * qq, nv = 2 * rr;
      qq -= uu;
      rr -= vv;
      uu = nu;
      vv = nv;
    } else {
      delta = 1 + delta;
      g = (g + f) >> 1;
      qq += uu;
      rr += vv;
      uu *= 2;
      vv *= 2;
    }
    left--;
  }
  u = uu;
  v = vv;
  q = qq;
  r = rr;
  return delta;
}

// limb i of a signed 13-limb value as a signed 64-bit number (the top limb carries the sign)
FQ_HD int64_t ds_limb(const uint32_t (&x)[DS_LIMBS], int i) {
  return i == DS_LIMBS - 1 ? (int64_t)(int32_t)x[i] : (int64_t)x[i];
}

// out = (a x + b y) / 2^30 for signed x, y (the division is exact)
FQ_HD void ds_combine(uint32_t (&out)[DS_LIMBS], int32_t a, const uint32_t (&x)[DS_LIMBS], int32_t b,
                      const uint32_t (&y)[DS_LIMBS]) {
  uint32_t w[DS_LIMBS];
  int64_t acc = 0;
  for (int i = 0; i < DS_LIMBS; i++) {
    acc += (int64_t)a * ds_limb(x, i) + (int64_t)b * ds_limb(y, i);
    w[i] = (uint32_t)acc;
    acc >>= 32;  // arithmetic: the carry keeps its sign
  }
  for (int i = 0; i < DS_LIMBS - 1; i++) out[i] = (w[i] >> 30) | (w[i + 1] << 2);
  out[DS_LIMBS - 1] = (w[DS_LIMBS - 1] >> 30) | ((uint32_t)acc << 2);
}

FQ_HD bool ds_is_neg(const uint32_t (&x)[DS_LIMBS]) { return (int32_t)x[DS_LIMBS - 1] < 0; }

// x += s * q (s = +1 or -1), q as 13 limbs (top limb 0)
FQ_HD void ds_add_q(uint32_t (&x)[DS_LIMBS], const uint32_t (&q)[DS_LIMBS], int s) {
  int64_t acc = 0;
  for (int i = 0; i < DS_LIMBS; i++) {
    acc += ds_limb(x, i) + (int64_t)s * (int64_t)q[i];
    x[i] = (uint32_t)acc;
    acc >>= 32;
  }
}

// true when x >= q for 0 <= x (unsigned compare of the limbs)
FQ_HD bool ds_geq(const uint32_t (&x)[DS_LIMBS], const uint32_t (&q)[DS_LIMBS]) {
  for (int i = DS_LIMBS - 1; i >= 0; i--) {
    if (x[i] != q[i]) return x[i] > q[i];
  }
  return true;
}

// out = (a x + b y) / 2^30 mod q, for x, y in [0, q); result in [0, q)
FQ_HD void ds_combine_mod(uint32_t (&out)[DS_LIMBS], int32_t a, const uint32_t (&x)[DS_LIMBS], int32_t b,
                          const uint32_t (&y)[DS_LIMBS], const uint32_t (&q)[DS_LIMBS]) {
  uint32_t w[DS_LIMBS + 1];
  int64_t acc = 0;
  for (int i = 0; i < DS_LIMBS; i++) {
    acc += (int64_t)a * (int64_t)x[i] + (int64_t)b * (int64_t)y[i];
    w[i] = (uint32_t)acc;
    acc >>= 32;
  }
  w[DS_LIMBS] = (uint32_t)acc;  // sign word: |a x + b y| < 2^30 q < 2^407 fits 13 limbs and a sign
  // add m q with m = -t mod 2^30 (q = 1 mod 2^30), so that the sum is divisible by 2^30
  const uint32_t m = (0u - w[0]) & 0x3fffffffu;
  int64_t acc2 = 0;
  for (int i = 0; i < DS_LIMBS; i++) {
    acc2 += (int64_t)w[i] + (int64_t)m * (int64_t)q[i];
    w[i] = (uint32_t)acc2;
    acc2 >>= 32;
  }
  w[DS_LIMBS] = (uint32_t)((int64_t)(int32_t)w[DS_LIMBS] + acc2);
  for (int i = 0; i < DS_LIMBS - 1; i++) out[i] = (w[i] >> 30) | (w[i + 1] << 2);
  out[DS_LIMBS - 1] = (w[DS_LIMBS - 1] >> 30) | (w[DS_LIMBS] << 2);
  // the result lies in [-q, 2q): one correction each way
  if (ds_is_neg(out)) ds_add_q(out, q, 1);
  if (ds_geq(out, q)) ds_add_q(out, q, -1);
}

// One code path for all four combinations of a batch, so that four lanes of a warp can each take
// one without diverging: out = (a x + b y) / 2^30, and modulo q when `mod` (x, y in [0, q), result
// in [0, q)); without `mod`, x and y are signed and the division is exact.
FQ_HD void ds_combine_any(uint32_t (&out)[DS_LIMBS], int32_t a, const uint32_t (&x)[DS_LIMBS], int32_t b,
                          const uint32_t (&y)[DS_LIMBS], const uint32_t (&q)[DS_LIMBS], bool mod) {
  uint32_t w[DS_LIMBS + 1];
  int64_t acc = 0;
  for (int i = 0; i < DS_LIMBS; i++) {
    acc += (int64_t)a * ds_limb(x, i) + (int64_t)b * ds_limb(y, i);
    w[i] = (uint32_t)acc;
    acc >>= 32;
  }
  w[DS_LIMBS] = (uint32_t)acc;
  const uint32_t m = mod ? (0u - w[0]) & 0x3fffffffu : 0u;  // a zero multiple of q otherwise
  int64_t acc2 = 0;
  for (int i = 0; i < DS_LIMBS; i++) {
    acc2 += (int64_t)w[i] + (int64_t)m * (int64_t)q[i];
    w[i] = (uint32_t)acc2;
    acc2 >>= 32;
  }
  w[DS_LIMBS] = (uint32_t)((int64_t)(int32_t)w[DS_LIMBS] + acc2);
  for (int i = 0; i < DS_LIMBS - 1; i++) out[i] = (w[i] >> 30) | (w[i + 1] << 2);
  out[DS_LIMBS - 1] = (w[DS_LIMBS - 1] >> 30) | (w[DS_LIMBS] << 2);
  if (mod && ds_is_neg(out)) ds_add_q(out, q, 1);
  if (mod && ds_geq(out, q)) ds_add_q(out, q, -1);
}

// a^-1 mod q as plain integers (12 limbs of 32 bits; a < q; 0 -> 0).  Returns false only if
// the batch guard ran out, which the divstep bound (at most about 1100 steps for 377 bits,
// Bernstein-Yang theorem 11.2) rules out.
FQ_HD bool ds_inverse(const uint32_t (&a)[12], const uint32_t (&q12)[12], uint32_t (&out)[12]) {
  uint32_t f[DS_LIMBS], g[DS_LIMBS], d[DS_LIMBS], e[DS_LIMBS], q[DS_LIMBS];
  uint32_t nz = 0;
  for (int i = 0; i < 12; i++) {
    f[i] = q12[i];
    q[i] = q12[i];
    g[i] = a[i];
    d[i] = 0;
    e[i] = 0;
    nz |= a[i];
  }
  f[12] = g[12] = d[12] = e[12] = q[12] = 0;
  e[0] = 1;
  for (int i = 0; i < 12; i++) out[i] = 0;
  if (!nz) return true;
  int delta = 1;
  bool done = false;
  for (int batch = 0; batch < 64 && !done; batch++) {
    int32_t u, v, qq, r;
    delta = ds_batch30(delta, f[0], g[0], u, v, qq, r);
    uint32_t nf[DS_LIMBS], ng[DS_LIMBS], nd[DS_LIMBS], ne[DS_LIMBS];
    ds_combine(nf, u, f, v, g);
    ds_combine(ng, qq, f, r, g);
    ds_combine_mod(nd, u, d, v, e, q);
    ds_combine_mod(ne, qq, d, r, e, q);
    uint32_t gz = 0;
    for (int i = 0; i < DS_LIMBS; i++) {
      f[i] = nf[i];
      g[i] = ng[i];
      d[i] = nd[i];
      e[i] = ne[i];
      gz |= ng[i];
    }
    done = gz == 0;
  }
  if (!done) return false;
  // f = +-1: a^-1 = d or q - d
  if (ds_is_neg(f)) {
    uint32_t z[DS_LIMBS];
    for (int i = 0; i < DS_LIMBS; i++) z[i] = 0;
    ds_add_q(z, q, 1);  // z = q
    int64_t acc = 0;
    for (int i = 0; i < DS_LIMBS; i++) {
      acc += (int64_t)z[i] - (int64_t)d[i];
      d[i] = (uint32_t)acc;
      acc >>= 32;
    }
  }
  for (int i = 0; i < 12; i++) out[i] = d[i];
  return true;
}
