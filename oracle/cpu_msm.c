/* CPU oracle and CPU baseline for the BLS12-377 G1 MSM -- test infrastructure only.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library; the
 * product path never does.  It deliberately shares no code and no coordinate system with the GPU
 * engine: arithmetic is six 64-bit limbs in Montgomery form (R = 2^384, the arkworks Fq layout),
 * points are Jacobian Weierstrass y^2 = x^3 + 1, and the MSM is the variable-base Pippenger of
 * ark-ec 0.3.0 (`VariableBaseMSM::multi_scalar_mul`, the oracle the reference's harness calls in
 * zprize/msm_pippenger/test_fpga_harness/src/util.rs:115-118 and tests/msm_unit_tests.rs:58-61):
 * unsigned c-bit windows with c = ln_without_floats(n) + 2 (3 below 32 points), one bucket array
 * per window filled by mixed additions, a running-sum reduction per window
 * (host/msm_compute/include/bls12_377_g1/pippenger.h:25-33 is the same triangle sum) and a
 * doubling combine of the windows (pippenger.h:36-45).  Windows run in parallel with OpenMP, as
 * ark-ec's "parallel" feature runs them with rayon (test_fpga_harness/Cargo.toml: ark-ec
 * features = ["parallel"]).  ark-ec's crate source is not in the reference tree; the structure
 * above is its published algorithm, restated.
 *
 * Scalars are the raw 4 x u64 integers of the harness ABI, taken modulo 2^253 as the reference's
 * 253-bit scalar path does (host/driver/driver.cpp:15; bls12_377_g1.h:17, 714-721).
 * Base-field constants: bls12_377_g1.h:24-54.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;
typedef struct { uint64_t v[6]; } fp;
typedef struct { fp x, y, z; } jac;               /* z == 0: infinity */
typedef struct { fp x, y; int inf; } aff;

static const fp P = {{0x8508c00000000001ull, 0x170b5d4430000000ull, 0x1ef3622fba094800ull,
                      0x1a22d9f300f5138full, 0xc63b05c06ca1493bull, 0x01ae3a4617c510eaull}};
static const uint64_t PINV = 0x8508bfffffffffffull; /* -p^-1 mod 2^64 */
static const fp ONE = {{0x02cdffffffffff68ull, 0x51409f837fffffb1ull, 0x9f7db3a98a7d3ff2ull,
                        0x7b4e97b76e7c6305ull, 0x4cf495bf803c84e8ull, 0x008d6661e2fdf49aull}};
static const fp GX = {{0x260f33b9772451f4ull, 0xc54dd773169d5658ull, 0x5c1551c469a510ddull,
                       0x761662e4425e1698ull, 0xc97d78cc6f065272ull, 0x00a41206b361fd4dull}};
static const fp GY = {{0x8193961fb8cb81f3ull, 0x00638d4c5f44adb8ull, 0xfafaf3dad4daf54aull,
                       0xc27849e2d655cd18ull, 0x2ec3ddb401d52814ull, 0x007da93326303c71ull}};

static int fp_is_zero(const fp *a) {
  return (a->v[0] | a->v[1] | a->v[2] | a->v[3] | a->v[4] | a->v[5]) == 0;
}
static int fp_eq(const fp *a, const fp *b) { return memcmp(a, b, sizeof(fp)) == 0; }

static int geq_p(const uint64_t *a) {
  for (int i = 5; i >= 0; i--) {
    if (a[i] > P.v[i]) return 1;
    if (a[i] < P.v[i]) return 0;
  }
  return 1;
}
static void sub_p(uint64_t *a) {
  u128 br = 0;
  for (int i = 0; i < 6; i++) {
    u128 d = (u128)a[i] - P.v[i] - br;
    a[i] = (uint64_t)d;
    br = (d >> 64) & 1;
  }
}

static fp fp_add(fp a, const fp *b) {
  u128 c = 0;
  for (int i = 0; i < 6; i++) {
    c += (u128)a.v[i] + b->v[i];
    a.v[i] = (uint64_t)c;
    c >>= 64;
  }
  if (geq_p(a.v)) sub_p(a.v);
  return a;
}
static fp fp_sub(fp a, const fp *b) {
  u128 br = 0;
  for (int i = 0; i < 6; i++) {
    u128 d = (u128)a.v[i] - b->v[i] - br;
    a.v[i] = (uint64_t)d;
    br = (d >> 64) & 1;
  }
  if (br) {
    u128 c = 0;
    for (int i = 0; i < 6; i++) {
      c += (u128)a.v[i] + P.v[i];
      a.v[i] = (uint64_t)c;
      c >>= 64;
    }
  }
  return a;
}
static fp fp_dbl(const fp *a) { return fp_add(*a, a); }

/* Montgomery product, CIOS over 64-bit limbs */
static fp fp_mul(const fp *a, const fp *b) {
  uint64_t t[8] = {0};
  for (int i = 0; i < 6; i++) {
    u128 c = 0;
    for (int j = 0; j < 6; j++) {
      c += (u128)a->v[j] * b->v[i] + t[j];
      t[j] = (uint64_t)c;
      c >>= 64;
    }
    c += t[6];
    t[6] = (uint64_t)c;
    t[7] = (uint64_t)(c >> 64);
    const uint64_t m = t[0] * PINV;
    c = (u128)m * P.v[0] + t[0];
    c >>= 64;
    for (int j = 1; j < 6; j++) {
      c += (u128)m * P.v[j] + t[j];
      t[j - 1] = (uint64_t)c;
      c >>= 64;
    }
    c += t[6];
    t[5] = (uint64_t)c;
    t[6] = t[7] + (uint64_t)(c >> 64);
  }
  fp r;
  memcpy(r.v, t, 48);
  if (t[6] || geq_p(r.v)) sub_p(r.v);
  return r;
}
static fp fp_sqr(const fp *a) { return fp_mul(a, a); }

static fp fp_inv(const fp *a) { /* a^(p-2) */
  static const uint64_t e[6] = {0x8508bfffffffffffull, 0x170b5d4430000000ull, 0x1ef3622fba094800ull,
                                0x1a22d9f300f5138full, 0xc63b05c06ca1493bull, 0x01ae3a4617c510eaull};
  fp r = ONE, b = *a;
  for (int i = 0; i < 6; i++)
    for (int k = 0; k < 64; k++) {
      if ((e[i] >> k) & 1) r = fp_mul(&r, &b);
      b = fp_sqr(&b);
    }
  return r;
}

/* ---- Jacobian arithmetic, a = 0 ---- */
static jac jac_inf(void) {
  jac r;
  r.x = ONE;
  r.y = ONE;
  memset(&r.z, 0, sizeof(fp));
  return r;
}

static jac jac_dbl(const jac *p) { /* dbl-2009-l */
  if (fp_is_zero(&p->z) || fp_is_zero(&p->y)) return jac_inf();
  fp A = fp_sqr(&p->x), B = fp_sqr(&p->y), C = fp_sqr(&B);
  fp t = fp_add(p->x, &B);
  t = fp_sqr(&t);
  t = fp_sub(t, &A);
  t = fp_sub(t, &C);
  fp D = fp_dbl(&t);
  fp E = fp_add(fp_dbl(&A), &A);
  fp F = fp_sqr(&E);
  jac r;
  r.x = fp_sub(F, &D);
  r.x = fp_sub(r.x, &D);
  fp C8 = fp_dbl(&C);
  C8 = fp_dbl(&C8);
  C8 = fp_dbl(&C8);
  fp dmx = fp_sub(D, &r.x);
  r.y = fp_mul(&E, &dmx);
  r.y = fp_sub(r.y, &C8);
  fp yz = fp_mul(&p->y, &p->z);
  r.z = fp_dbl(&yz);
  return r;
}

static jac jac_madd(const jac *p, const aff *q) { /* madd-2007-bl, complete by cases */
  if (q->inf) return *p;
  if (fp_is_zero(&p->z)) {
    jac r = {q->x, q->y, ONE};
    return r;
  }
  fp Z1Z1 = fp_sqr(&p->z);
  fp U2 = fp_mul(&q->x, &Z1Z1);
  fp S2 = fp_mul(&q->y, &p->z);
  S2 = fp_mul(&S2, &Z1Z1);
  fp H = fp_sub(U2, &p->x);
  fp rr = fp_sub(S2, &p->y);
  if (fp_is_zero(&H)) {
    if (fp_is_zero(&rr)) return jac_dbl(p);
    return jac_inf();
  }
  rr = fp_dbl(&rr);
  fp HH = fp_sqr(&H);
  fp I = fp_dbl(&HH);
  I = fp_dbl(&I);
  fp J = fp_mul(&H, &I);
  fp V = fp_mul(&p->x, &I);
  jac r;
  r.x = fp_sqr(&rr);
  r.x = fp_sub(r.x, &J);
  r.x = fp_sub(r.x, &V);
  r.x = fp_sub(r.x, &V);
  fp t = fp_sub(V, &r.x);
  r.y = fp_mul(&rr, &t);
  fp yj = fp_mul(&p->y, &J);
  yj = fp_dbl(&yj);
  r.y = fp_sub(r.y, &yj);
  fp zh = fp_add(p->z, &H);
  zh = fp_sqr(&zh);
  zh = fp_sub(zh, &Z1Z1);
  r.z = fp_sub(zh, &HH);
  return r;
}

static jac jac_add(const jac *p, const jac *q) { /* add-2007-bl, complete by cases */
  if (fp_is_zero(&p->z)) return *q;
  if (fp_is_zero(&q->z)) return *p;
  fp Z1Z1 = fp_sqr(&p->z), Z2Z2 = fp_sqr(&q->z);
  fp U1 = fp_mul(&p->x, &Z2Z2), U2 = fp_mul(&q->x, &Z1Z1);
  fp S1 = fp_mul(&p->y, &q->z);
  S1 = fp_mul(&S1, &Z2Z2);
  fp S2 = fp_mul(&q->y, &p->z);
  S2 = fp_mul(&S2, &Z1Z1);
  if (fp_eq(&U1, &U2)) {
    if (fp_eq(&S1, &S2)) return jac_dbl(p);
    return jac_inf();
  }
  fp H = fp_sub(U2, &U1);
  fp I = fp_dbl(&H);
  I = fp_sqr(&I);
  fp J = fp_mul(&H, &I);
  fp rr = fp_sub(S2, &S1);
  rr = fp_dbl(&rr);
  fp V = fp_mul(&U1, &I);
  jac r;
  r.x = fp_sqr(&rr);
  r.x = fp_sub(r.x, &J);
  r.x = fp_sub(r.x, &V);
  r.x = fp_sub(r.x, &V);
  fp t = fp_sub(V, &r.x);
  r.y = fp_mul(&rr, &t);
  fp sj = fp_mul(&S1, &J);
  sj = fp_dbl(&sj);
  r.y = fp_sub(r.y, &sj);
  fp zz = fp_add(p->z, &q->z);
  zz = fp_sqr(&zz);
  zz = fp_sub(zz, &Z1Z1);
  zz = fp_sub(zz, &Z2Z2);
  r.z = fp_mul(&zz, &H);
  return r;
}

/* g1_affine_t: 6 u64 x, 6 u64 y, bool at byte 96, 104 bytes */
static aff load_aff(const uint8_t *rec) {
  aff a;
  memcpy(a.x.v, rec, 48);
  memcpy(a.y.v, rec + 48, 48);
  a.inf = rec[96] != 0;
  return a;
}

/* Jacobian -> g1_projective_t (x*R, y*R, R) or arkworks' zero (R, R, 0) */
static void store_proj(const jac *p, uint64_t *out) {
  if (fp_is_zero(&p->z)) {
    memcpy(out, ONE.v, 48);
    memcpy(out + 6, ONE.v, 48);
    memset(out + 12, 0, 48);
    return;
  }
  fp zi = fp_inv(&p->z), zi2 = fp_sqr(&zi), zi3 = fp_mul(&zi2, &zi);
  fp x = fp_mul(&p->x, &zi2), y = fp_mul(&p->y, &zi3);
  memcpy(out, x.v, 48);
  memcpy(out + 6, y.v, 48);
  memcpy(out + 12, ONE.v, 48);
}

static unsigned ceil_log2(uint64_t n) {
  unsigned k = 0;
  while ((1ull << k) < n) k++;
  return k;
}

/* ark-ec 0.3 window width: ln_without_floats(n) + 2, or 3 below 32 points */
int oracle_default_window(uint64_t n) { return n < 32 ? 3 : (int)(ceil_log2(n) * 69 / 100) + 2; }

/* window bits [start, start + c) of a scalar, masked to 253 bits */
static uint64_t window_of(const uint64_t *s, unsigned start, unsigned c) {
  uint64_t v = 0;
  for (unsigned b = 0; b < c; b++) {
    const unsigned bit = start + b;
    if (bit >= 253) break;
    v |= ((s[bit >> 6] >> (bit & 63)) & 1ull) << b;
  }
  return v;
}

/* Variable-base MSM: out = sum scalars[i] * points[i].  c <= 0 picks ark-ec's default window.
 * threads <= 0 uses every core OpenMP offers.  Returns 0. */
int oracle_msm(const void *points, const uint64_t *scalars, uint64_t n, int c, int threads,
               uint64_t *out) {
  const uint8_t *pts = (const uint8_t *)points;
  if (c <= 0) c = oracle_default_window(n);
  const unsigned nwin = (253 + c - 1) / c;
  const uint64_t nb = (1ull << c) - 1;
  jac *wsum = (jac *)malloc(sizeof(jac) * nwin);
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int w = 0; w < (int)nwin; w++) {
    jac *buckets = (jac *)malloc(sizeof(jac) * nb);
    for (uint64_t b = 0; b < nb; b++) buckets[b] = jac_inf();
    for (uint64_t i = 0; i < n; i++) {
      const uint64_t d = window_of(scalars + 4 * i, (unsigned)w * c, c);
      if (!d) continue;
      const aff a = load_aff(pts + 104 * i);
      buckets[d - 1] = jac_madd(&buckets[d - 1], &a);
    }
    jac running = jac_inf(), acc = jac_inf();
    for (uint64_t b = nb; b-- > 0;) {
      running = jac_add(&running, &buckets[b]);
      acc = jac_add(&acc, &running);
    }
    wsum[w] = acc;
    free(buckets);
  }
  jac total = jac_inf();
  for (int w = (int)nwin - 1; w >= 0; w--) {
    if (w != (int)nwin - 1)
      for (int k = 0; k < c; k++) total = jac_dbl(&total);
    total = jac_add(&total, &wsum[w]);
  }
  free(wsum);
  store_proj(&total, out);
  return 0;
}

/* ---- seeded bases k_i * G (SplitMix64 counter-based draws, as the engine's generator) ---- */
static uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t oracle_rand_u64(uint64_t seed, uint64_t stream, uint64_t index, uint64_t word) {
  const uint64_t s = splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull));
  const uint64_t h = splitmix64(s ^ splitmix64(index));
  return splitmix64(h + word);
}

/* out[i] = k_i * G as g1_affine_t, k_i = oracle_rand_u64(seed, 1, first + i, 0) */
int oracle_gen_bases(uint64_t seed, uint64_t first, uint64_t n, void *out, int threads) {
  uint8_t *o = (uint8_t *)out;
  const aff g = {GX, GY, 0};
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static)
#endif
  for (int64_t i = 0; i < (int64_t)n; i++) {
    uint64_t k = oracle_rand_u64(seed, 1, first + (uint64_t)i, 0);
    jac acc = jac_inf();
    for (int b = 63; b >= 0; b--) {
      acc = jac_dbl(&acc);
      if ((k >> b) & 1) acc = jac_madd(&acc, &g);
    }
    uint8_t *rec = o + 104 * (size_t)i;
    memset(rec, 0, 104);
    if (fp_is_zero(&acc.z)) {
      memcpy(rec + 48, ONE.v, 48);
      rec[96] = 1;
    } else {
      uint64_t proj[18];
      store_proj(&acc, proj);
      memcpy(rec, proj, 96);
    }
  }
  return 0;
}

/* scalar-multiple check used by tests: out = k * P (k as 4 x u64, all 256 bits) */
int oracle_mul(const void *point, const uint64_t *k, uint64_t *out) {
  const aff a = load_aff((const uint8_t *)point);
  jac acc = jac_inf();
  for (int b = 255; b >= 0; b--) {
    acc = jac_dbl(&acc);
    if ((k[b >> 6] >> (b & 63)) & 1) acc = jac_madd(&acc, &a);
  }
  store_proj(&acc, out);
  return 0;
}

/* ---- seeded scalars (the same SplitMix64 draws as oracle/bls12_377.py uniform_scalar and
 *      mixed_scalar), so the CPU baseline makes its inputs without the engine ---- */
static const uint64_t R_SCALAR_WORDS[4] = {0x0a11800000000001ull, 0x59aa76fed0000001ull,
                                           0x60b44d1e5c37b001ull, 0x12ab655e9a2ca556ull};
static int lt_r_scalar(const uint64_t *v) {
  for (int k = 3; k >= 0; k--) {
    if (v[k] < R_SCALAR_WORDS[k]) return 1;
    if (v[k] > R_SCALAR_WORDS[k]) return 0;
  }
  return 0;
}
/* uniform in [0, r): 253-bit draws, words 4a..4a+3 for attempt a, rejected while >= r */
static void uniform_scalar(uint64_t seed, uint64_t i, uint64_t *out) {
  for (uint64_t a = 0;; a++) {
    for (int j = 0; j < 4; j++) out[j] = oracle_rand_u64(seed, 2, i, 4 * a + (uint64_t)j);
    out[3] &= (1ull << 61) - 1;
    if (lt_r_scalar(out)) return;
  }
}
/* the uneven-batch mix: 70% uniform, 10% 16-bit, 10% 0 or r - 1, 10% one value per MSM */
static void mixed_scalar(uint64_t seed, uint64_t msm, uint64_t i, uint64_t *out) {
  const uint64_t key = (msm << 32) | i;
  const uint64_t sel = oracle_rand_u64(seed, 3, key, 0) % 10;
  if (sel < 7) {
    uniform_scalar(seed, key, out);
  } else if (sel == 7) {
    out[0] = oracle_rand_u64(seed, 3, key, 1) & 0xffff;
    out[1] = out[2] = out[3] = 0;
  } else if (sel == 8) {
    if ((oracle_rand_u64(seed, 3, key, 2) & 1) == 0) {
      out[0] = out[1] = out[2] = out[3] = 0;
    } else {
      for (int k = 0; k < 4; k++) out[k] = R_SCALAR_WORDS[k];
      out[0] -= 1;
    }
  } else {
    uniform_scalar(seed, (msm << 32) | 0xffffffffull, out);
  }
}
/* kind 0: n uniform scalars of element indices 0..n-1; kind 1: the mix for MSM msm_index */
int oracle_gen_scalars(uint64_t seed, uint64_t n, int kind, uint64_t msm_index, uint64_t *out,
                       int threads) {
  if (kind != 0 && kind != 1) return -1;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static)
#endif
  for (int64_t i = 0; i < (int64_t)n; i++) {
    if (kind == 0) uniform_scalar(seed, (uint64_t)i, out + 4 * i);
    else mixed_scalar(seed, msm_index, (uint64_t)i, out + 4 * i);
  }
  return 0;
}
