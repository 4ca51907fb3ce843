/* CPU oracle for the NTT track (Goldilocks field, p = 2^64 - 2^32 + 1) -- test infrastructure only.
 *
 * Only tests/ and bench.py's CPU-baseline leg load this code; the GPU engine never does.  It
 * restates the reference's host-side model of the transform (zprize/ntt/host/reference.cpp:94-139,
 * ntt_reference_inplace): bit-reverse the input, then log2(n) radix-2 decimation-in-time stages
 * whose stage-i twiddle is the 2^i-th root of unity of the reference's table
 * (zprize/ntt/host/gf.h:65-99), so X[k] = sum_j x[j] w^(j k) with w = omega[log2 n], natural order
 * in and out.  Field arithmetic follows the modulus of gf.h:6; the multiplication reduces the
 * 128-bit product with 2^64 = 2^32 - 1 and 2^96 = -1 (mod p), written here with 128-bit integers.
 * The root table restates gf.h's constants (it must: another primitive root gives another
 * transform) and tests/golden/ntt_kats.json pins it to the reference's file.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;
static const uint64_t GL_P = 0xffffffff00000001ull;

/* 2^i-th roots of unity, i = 0..32 (gf.h:65-99) */
static const uint64_t GL_OMEGA[33] = {
    0x0000000000000001ull,
    0xffffffff00000000ull,
    0x0001000000000000ull,
    0xfffffffeff000001ull,
    0xefffffff00000001ull,
    0x00003fffffffc000ull,
    0x0000008000000000ull,
    0xf80007ff08000001ull,
    0xbf79143ce60ca966ull,
    0x1905d02a5c411f4eull,
    0x9d8f2ad78bfed972ull,
    0x0653b4801da1c8cfull,
    0xf2c35199959dfcb6ull,
    0x1544ef2335d17997ull,
    0xe0ee099310bba1e2ull,
    0xf6b2cffe2306baacull,
    0x54df9630bf79450eull,
    0xabd0a6e8aa3d8a0eull,
    0x81281a7b05f9beacull,
    0xfbd41c6b8caa3302ull,
    0x30ba2ecd5e93e76dull,
    0xf502aef532322654ull,
    0x4b2a18ade67246b5ull,
    0xea9d5a1336fbc98bull,
    0x86cdcc31c307e171ull,
    0x4bbaf5976ecfefd8ull,
    0xed41d05b78d6e286ull,
    0x10d78dd8915a171dull,
    0x59049500004a4485ull,
    0xdfa8c93ba46d2666ull,
    0x7e9bd009b86a0845ull,
    0x400a7f755588e659ull,
    0x185629dcda58878cull
};

static uint64_t gl_add(uint64_t a, uint64_t b) {
  u128 s = (u128)a + b;
  return (uint64_t)(s >= GL_P ? s - GL_P : s);
}
static uint64_t gl_sub(uint64_t a, uint64_t b) { return a >= b ? a - b : (uint64_t)((u128)a + GL_P - b); }
static uint64_t gl_mul(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * b) % GL_P); }
static uint64_t gl_pow(uint64_t a, uint64_t e) {
  uint64_t r = 1;
  while (e) {
    if (e & 1) r = gl_mul(r, a);
    a = gl_mul(a, a);
    e >>= 1;
  }
  return r;
}

uint64_t oracle_gl_mul(uint64_t a, uint64_t b) { return gl_mul(a, b); }
uint64_t oracle_gl_omega(int i) { return (i >= 0 && i <= 32) ? GL_OMEGA[i] : 0; }

static uint64_t bitrev(uint64_t x, int bits) {
  uint64_t r = 0;
  for (int i = 0; i < bits; i++) r = (r << 1) | ((x >> i) & 1);
  return r;
}

/* in-place transform of 2^logn values in [0, p) with root w (w = omega[logn] forward) */
static void ntt_with_root(uint64_t *a, int logn, uint64_t w_n, int threads) {
  const uint64_t n = 1ull << logn;
  for (uint64_t k = 0; k < n; k++) {
    const uint64_t r = bitrev(k, logn);
    if (k < r) {
      const uint64_t t = a[k];
      a[k] = a[r];
      a[r] = t;
    }
  }
  uint64_t *tw = (uint64_t *)malloc(sizeof(uint64_t) * (n / 2 + 1));
  for (int s = 1; s <= logn; s++) {
    const uint64_t m = 1ull << (s - 1);  /* half size of this stage's butterflies */
    /* the stage's root is w_n^(n / 2m), a primitive 2m-th root */
    const uint64_t wm = gl_pow(w_n, n >> s);
    tw[0] = 1;
    for (uint64_t j = 1; j < m; j++) tw[j] = gl_mul(tw[j - 1], wm);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static) if (n >= (1u << 14))
#endif
    for (int64_t k = 0; k < (int64_t)n; k += 2 * (int64_t)m) {
      for (uint64_t j = 0; j < m; j++) {
        const uint64_t t = gl_mul(a[k + j + m], tw[j]);
        const uint64_t u = a[k + j];
        a[k + j] = gl_add(u, t);
        a[k + j + m] = gl_sub(u, t);
      }
    }
  }
  free(tw);
}

/* forward NTT, out-of-place (dst may equal src); inputs must be below p */
int oracle_ntt(uint64_t *dst, const uint64_t *src, int logn, int threads) {
  if (logn < 0 || logn > 32) return -1;
  const uint64_t n = 1ull << logn;
  if (dst != src) memcpy(dst, src, n * sizeof(uint64_t));
  ntt_with_root(dst, logn, GL_OMEGA[logn], threads);
  return 0;
}

/* inverse NTT: the transform with w^-1, scaled by n^-1 */
int oracle_intt(uint64_t *dst, const uint64_t *src, int logn, int threads) {
  if (logn < 0 || logn > 32) return -1;
  const uint64_t n = 1ull << logn;
  if (dst != src) memcpy(dst, src, n * sizeof(uint64_t));
  ntt_with_root(dst, logn, gl_pow(GL_OMEGA[logn], GL_P - 2), threads);
  const uint64_t ninv = gl_pow(n % GL_P, GL_P - 2);
  for (uint64_t i = 0; i < n; i++) dst[i] = gl_mul(dst[i], ninv);
  return 0;
}

/* ---- the random inputs of the reference host's NTT test (zprize/ntt/host/test_random.cpp:
 * std::mt19937_64 with its default seed, each draw taken modulo p).  MT19937-64 as published by
 * Nishimura and Matsumoto (2000/2004), the generator std::mt19937_64 specifies. ---- */
#define MT_NN 312
#define MT_MM 156
int oracle_mt19937_64(uint64_t seed, uint64_t *out, uint64_t n, int mod_p) {
  static const uint64_t MATRIX_A = 0xB5026F5AA96619E9ull, UM = 0xFFFFFFFF80000000ull,
                        LM = 0x7FFFFFFFull;
  uint64_t mt[MT_NN];
  mt[0] = seed;
  for (int i = 1; i < MT_NN; i++) mt[i] = 6364136223846793005ull * (mt[i - 1] ^ (mt[i - 1] >> 62)) + (uint64_t)i;
  int idx = MT_NN;
  for (uint64_t k = 0; k < n; k++) {
    if (idx >= MT_NN) {
      for (int i = 0; i < MT_NN; i++) {
        const uint64_t x = (mt[i] & UM) | (mt[(i + 1) % MT_NN] & LM);
        mt[i] = mt[(i + MT_MM) % MT_NN] ^ (x >> 1) ^ ((x & 1ull) ? MATRIX_A : 0ull);
      }
      idx = 0;
    }
    uint64_t x = mt[idx++];
    x ^= (x >> 29) & 0x5555555555555555ull;
    x ^= (x << 17) & 0x71D67FFFEDA60000ull;
    x ^= (x << 37) & 0xFFF7EEE000000000ull;
    x ^= x >> 43;
    out[k] = mod_p ? x % GL_P : x;
  }
  return 0;
}
