// Host-side conversions for the data formats either side of the MSM path.
//
// The reference harness stores test data with ark-serialize (`serialize_unchecked`, canonical
// little-endian field elements; test_fpga_harness/src/util.rs:126-172) while the C ABI carries
// arkworks' in-memory Montgomery form: Fq elements as x * 2^384 mod q and scalars as the raw
// Montgomery integer of Fr, v * 2^256 mod r, which the harness transmutes into BigInteger256
// (tests/msm.rs:30-32).  These routines convert between the two, in place, on all host cores.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "../../include/msm_gb300.h"

namespace {

typedef unsigned __int128 u128;

template <int N>
struct Field {
  uint64_t p[N];
  uint64_t pinv;  // -p^-1 mod 2^64
  uint64_t r2[N]; // 2^(128 N) mod p

  bool geq_p(const uint64_t *a) const {
    for (int i = N - 1; i >= 0; i--) {
      if (a[i] > p[i]) return true;
      if (a[i] < p[i]) return false;
    }
    return true;
  }
  void sub_p(uint64_t *a) const {
    u128 br = 0;
    for (int i = 0; i < N; i++) {
      const u128 d = (u128)a[i] - p[i] - br;
      a[i] = (uint64_t)d;
      br = (d >> 64) & 1;
    }
  }
  // a * b * 2^(-64 N) mod p, CIOS; a, b < p
  void mont_mul(uint64_t *out, const uint64_t *a, const uint64_t *b) const {
    uint64_t t[N + 2];
    memset(t, 0, sizeof(t));
    for (int i = 0; i < N; i++) {
      u128 c = 0;
      for (int j = 0; j < N; j++) {
        c += (u128)a[j] * b[i] + t[j];
        t[j] = (uint64_t)c;
        c >>= 64;
      }
      c += t[N];
      t[N] = (uint64_t)c;
      t[N + 1] = (uint64_t)(c >> 64);
      const uint64_t m = t[0] * pinv;
      c = ((u128)m * p[0] + t[0]) >> 64;
      for (int j = 1; j < N; j++) {
        c += (u128)m * p[j] + t[j];
        t[j - 1] = (uint64_t)c;
        c >>= 64;
      }
      c += t[N];
      t[N - 1] = (uint64_t)c;
      t[N] = t[N + 1] + (uint64_t)(c >> 64);
    }
    if (t[N] || geq_p(t)) sub_p(t);
    memcpy(out, t, sizeof(uint64_t) * N);
  }
  bool reduced(const uint64_t *a) const { return !geq_p(a); }
};

const Field<6> kFq = {
    {0x8508c00000000001ull, 0x170b5d4430000000ull, 0x1ef3622fba094800ull, 0x1a22d9f300f5138full,
     0xc63b05c06ca1493bull, 0x01ae3a4617c510eaull},
    0x8508bfffffffffffull,
    {0xb786686c9400cd22ull, 0x0329fcaab00431b1ull, 0x22a5f11162d6b46dull, 0xbfdf7d03827dc3acull,
     0x837e92f041790bf9ull, 0x006dfccb1e914b88ull}};

const Field<4> kFr = {
    {0x0a11800000000001ull, 0x59aa76fed0000001ull, 0x60b44d1e5c37b001ull, 0x12ab655e9a2ca556ull},
    0x0a117fffffffffffull,
    {0x25d577bab861857bull, 0xcc2c27b58860591full, 0xa7cc008fe5dc8593ull, 0x011fdae7eff1c939ull}};

template <int N, class F>
int convert_all(uint64_t *v, uint64_t n, F fn) {
  if (n == 0) return 0;
  if (!v) return -1;
  const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  std::vector<int> bad(nt, 0);
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([=, &bad] {
      const uint64_t a = n * t / nt, b = n * (t + 1) / nt;
      for (uint64_t i = a; i < b; i++)
        if (!fn(v + (size_t)N * i)) bad[t] = 1;
    });
  for (auto &x : th) x.join();
  for (int b : bad)
    if (b) return -3;
  return 0;
}

}  // namespace

extern "C" {

int msm_fq_to_montgomery(uint64_t *v, uint64_t n) {
  return convert_all<6>(v, n, [](uint64_t *x) {
    if (!kFq.reduced(x)) return false;
    kFq.mont_mul(x, x, kFq.r2);
    return true;
  });
}

int msm_fq_from_montgomery(uint64_t *v, uint64_t n) {
  const uint64_t one[6] = {1, 0, 0, 0, 0, 0};
  return convert_all<6>(v, n, [&](uint64_t *x) {
    if (!kFq.reduced(x)) return false;
    kFq.mont_mul(x, x, one);
    return true;
  });
}

int msm_fr_to_montgomery(uint64_t *v, uint64_t n) {
  return convert_all<4>(v, n, [](uint64_t *x) {
    if (!kFr.reduced(x)) return false;
    kFr.mont_mul(x, x, kFr.r2);
    return true;
  });
}

int msm_fr_from_montgomery(uint64_t *v, uint64_t n) {
  const uint64_t one[4] = {1, 0, 0, 0};
  return convert_all<4>(v, n, [&](uint64_t *x) {
    if (!kFr.reduced(x)) return false;
    kFr.mont_mul(x, x, one);
    return true;
  });
}

}  // extern "C"
