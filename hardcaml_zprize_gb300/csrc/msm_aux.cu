// Device kernels around the pipeline: the one-time base precompute of msm_init, the seeded base
// generator used by the benchmark and tests, self-test hooks of the field arithmetic, and the
// IMAD-pipe peak microbenchmark that serves as the roofline denominator.
#include "engine.h"
#include "curve.cuh"

#define BLS_GEN_X {0x772451f4u, 0x260f33b9u, 0x169d5658u, 0xc54dd773u, 0x69a510ddu, 0x5c1551c4u, 0x425e1698u, 0x761662e4u, 0x6f065272u, 0xc97d78ccu, 0xb361fd4du, 0x00a41206u}
#define BLS_GEN_Y {0xb8cb81f3u, 0x8193961fu, 0x5f44adb8u, 0x00638d4cu, 0xd4daf54au, 0xfafaf3dau, 0xd655cd18u, 0xc27849e2u, 0x01d52814u, 0x2ec3ddb4u, 0x26303c71u, 0x007da933u}

namespace {

__device__ __forceinline__ bool fq_lt_q(const fq_t &a) {  // a < q as integers
  const uint32_t q[FQ_LIMBS] = BLS_Q;
  sub_cc(a.v[0], q[0]);
#pragma unroll
  for (int j = 1; j < FQ_LIMBS; j++) subc_cc(a.v[j], q[j]);
  return subc(0u, 0u) != 0u;
}

__device__ __forceinline__ void load_u64x6(fq_t &r, const uint64_t *p) {
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const uint64_t w = p[k];
    r.v[2 * k] = (uint32_t)w;
    r.v[2 * k + 1] = (uint32_t)(w >> 32);
  }
}
__device__ __forceinline__ void store_u64x6(uint64_t *p, const fq_t &a) {
#pragma unroll
  for (int k = 0; k < 6; k++) p[k] = ((uint64_t)a.v[2 * k + 1] << 32) | a.v[2 * k];
}

// Affine Weierstrass (Montgomery form) -> precomputed twisted Edwards, following
// affineWeierstrassToExtendedTwistedEdwards and preComputeFPGA (bls12_377_g1.h:361-415,
// 606-618) with one inversion: u = s(x+1), v = s y, x_e = ts u / v, y_e = (u-1)/(u+1).
// Returns false when v = 0 or u = -1 (no twisted-Edwards image, bls12_377_g1.h:382-384).
__device__ __forceinline__ bool weierstrass_to_pre(const fq_t &x, const fq_t &y, pre_t &out,
                                                   xyzt_t *ext) {
  const uint32_t ws[FQ_LIMBS] = BLS_WS, ts[FQ_LIMBS] = BLS_TWISTED_SCALE;
  const uint32_t inv2[FQ_LIMBS] = BLS_INV2, dd[FQ_LIMBS] = BLS_TE_D;
  const fq_t one = fq_one();
  const fq_t u = fq_mul_ool(fq_from(ws), fq_add(x, one));
  const fq_t v = fq_mul_ool(fq_from(ws), y);
  const fq_t up1 = fq_add(u, one);
  if (fq_is_zero(v) || fq_is_zero(up1)) return false;
  const fq_t inv = fq_inv_vartime(fq_mul_ool(v, up1));
  const fq_t xe = fq_mul_ool(fq_mul_ool(fq_mul_ool(fq_from(ts), u), up1), inv);
  const fq_t ye = fq_mul_ool(fq_mul_ool(fq_sub(u, one), v), inv);
  out.ymx = fq_canon(fq_mul_ool(fq_sub(ye, xe), fq_from(inv2)));
  out.ypx = fq_canon(fq_mul_ool(fq_add(ye, xe), fq_from(inv2)));
  out.kt = fq_canon(fq_mul_ool(fq_mul_ool(xe, ye), fq_from(dd)));
  if (ext) {
    ext->x = xe;
    ext->y = ye;
    ext->z = one;
    ext->t = fq_mul_ool(xe, ye);
  }
  return true;
}

__global__ void k_precompute(const uint64_t *affine, size_t n, uint4 *bases, uint8_t *flags,
                             uint32_t *special_idx, uint32_t *special_count, uint32_t index_offset) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t *rec = affine + i * 13;  // 104-byte g1_affine_t
  const uint8_t inf = (uint8_t)(rec[12] & 0xff);
  pre_t p;
  p.ymx = fq_zero();
  p.ypx = fq_zero();
  p.kt = fq_zero();
  uint8_t flag = BASE_OK;
  if (inf) {
    flag = BASE_INFINITY;
  } else {
    fq_t x, y;
    load_u64x6(x, rec);
    load_u64x6(y, rec + 6);
    if (!fq_lt_q(x) || !fq_lt_q(y)) {
      flag = BASE_BAD_INPUT;
    } else if (!weierstrass_to_pre(x, y, p, nullptr)) {
      flag = BASE_SPECIAL;
      const uint32_t k = atomicAdd(special_count, 1u);
      special_idx[k] = index_offset + (uint32_t)i;
    }
  }
  pre_store(bases + i * 9, p);
  flags[i] = flag;
}

// 4 * P == infinity for every class point (affine x, y in Montgomery form)
__global__ void k_check_classes(const uint4 *pts, uint32_t n, uint32_t *ok) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  wpt_t p;
  fq_load(p.x, pts + 6 * i);
  fq_load(p.y, pts + 6 * i + 3);
  p.z = fq_one();
  const fq_t lhs = fq_sqr_ool(p.y);
  const fq_t rhs = fq_add(fq_mul_ool(fq_sqr_ool(p.x), p.x), fq_one());
  const wpt_t q = w_dbl(w_dbl(p));
  ok[i] = (fq_eq(lhs, rhs) && fq_is_zero(q.z)) ? 1u : 0u;
}

// Fixed-base tables: for every base P_i (window 0 of the table), the multiples 2^(c w) P_i for
// w = 1 .. nwin - 1 in the same precomputed form.  One thread per base walks the doubling chain
// and converts all windows to affine with one batched inversion (Montgomery's trick).
constexpr int kMaxFbWindows = 24;

__global__ void __launch_bounds__(128) k_fixed_base(uint4 *bases, const uint8_t *flags, uint64_t n,
                                                    uint64_t first, uint64_t count, uint32_t c,
                                                    uint32_t nwin, uint32_t *fail) {
  const uint64_t i = first + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= first + count || i >= n || nwin > kMaxFbWindows) return;
  if (flags[i] != BASE_OK) {
    pre_t z;
    z.ymx = fq_zero();
    z.ypx = fq_zero();
    z.kt = fq_zero();
    for (uint32_t w = 1; w < nwin; w++) pre_store(bases + ((size_t)w * n + i) * 9, z);
    return;
  }
  pre_t p0;
  pre_load(p0, bases + i * 9);
  xyzt_t P;
  P.x = fq_sub(p0.ypx, p0.ymx);  // (y+x)/2 - (y-x)/2
  P.y = fq_add(p0.ypx, p0.ymx);
  P.z = fq_one();
  P.t = fq_mul_ool(P.x, P.y);
  fq_t X[kMaxFbWindows], Y[kMaxFbWindows], Z[kMaxFbWindows], pre[kMaxFbWindows];
  fq_t acc = fq_one();
#pragma unroll 1
  for (uint32_t w = 1; w < nwin; w++) {
#pragma unroll 1
    for (uint32_t k = 0; k < c; k++) P = te_dbl_ool(P);
    X[w] = P.x;
    Y[w] = P.y;
    Z[w] = P.z;
    pre[w] = acc;  // product of Z[1 .. w-1]
    acc = fq_mul_ool(acc, P.z);
  }
  if (fq_is_zero(acc)) {  // some 2^j P left the affine curve: P has 2-power order
    atomicAdd(fail, 1u);
    return;
  }
  fq_t inv = fq_inv_vartime(acc);
  const uint32_t inv2[FQ_LIMBS] = BLS_INV2, dd[FQ_LIMBS] = BLS_TE_D;
#pragma unroll 1
  for (uint32_t w = nwin - 1; w >= 1; w--) {
    const fq_t zi = fq_mul_ool(inv, pre[w]);
    inv = fq_mul_ool(inv, Z[w]);
    const fq_t x = fq_mul_ool(X[w], zi), y = fq_mul_ool(Y[w], zi);
    pre_t q;
    q.ymx = fq_canon(fq_mul_ool(fq_sub(y, x), fq_from(inv2)));
    q.ypx = fq_canon(fq_mul_ool(fq_add(y, x), fq_from(inv2)));
    q.kt = fq_canon(fq_mul_ool(fq_mul_ool(x, y), fq_from(dd)));
    pre_store(bases + ((size_t)w * n + i) * 9, q);
  }
}

// ---- seeded generator: SplitMix64 (Steele, Lea, Flood 2014), counter-based ----
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t rand_u64(uint64_t seed, uint64_t stream, uint64_t index,
                                             uint64_t word) {
  const uint64_t s = splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull));
  const uint64_t h = splitmix64(s ^ splitmix64(index));
  return splitmix64(h + word);
}

// table[w][v] = v * 2^(8w) * G in precomputed form, w < 8, v < 256 (entry v = 0 unused)
__global__ void k_gen_table(uint4 *table) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2048) return;
  const uint32_t w = t >> 8, v = t & 255;
  const uint32_t gx[FQ_LIMBS] = BLS_GEN_X, gy[FQ_LIMBS] = BLS_GEN_Y;
  pre_t gp;
  xyzt_t g;
  weierstrass_to_pre(fq_from(gx), fq_from(gy), gp, &g);
  xyzt_t acc = xyzt_identity();
  if (v != 0) {
    // v * 2^(8w) * G by double-and-add over the (8w + 8)-bit multiplier
    bool started = false;
#pragma unroll 1
    for (int bit = 8 * (int)w + 7; bit >= 0; bit--) {
      if (started) acc = te_dbl_ool(acc);
      const bool set = bit >= 8 * (int)w && ((v >> (bit - 8 * w)) & 1u);
      if (set) {
        acc = started ? te_add_ool(acc, g) : g;
        started = true;
      }
    }
  }
  // affine twisted Edwards, then the precomputed form
  const uint32_t inv2[FQ_LIMBS] = BLS_INV2, dd[FQ_LIMBS] = BLS_TE_D;
  const fq_t zi = fq_inv_vartime(acc.z);
  const fq_t x = fq_mul_ool(acc.x, zi), y = fq_mul_ool(acc.y, zi);
  pre_t p;
  p.ymx = fq_canon(fq_mul_ool(fq_sub(y, x), fq_from(inv2)));
  p.ypx = fq_canon(fq_mul_ool(fq_add(y, x), fq_from(inv2)));
  p.kt = fq_canon(fq_mul_ool(fq_mul_ool(x, y), fq_from(dd)));
  pre_store(table + (size_t)t * 9, p);
}

// base i = k_i * G with k_i = rand_u64(seed, 1, first + i, 0), written as g1_affine_t
__global__ void k_gen_bases(uint64_t seed, uint64_t first, size_t n, uint64_t *out,
                            const uint4 *table) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = rand_u64(seed, 1, first + i, 0);
  xyzt_t acc = xyzt_identity();
#pragma unroll 1
  for (int w = 0; w < 8; w++) {
    const uint32_t byte = (uint32_t)(k >> (8 * w)) & 255u;
    if (!byte) continue;
    pre_t p;
    pre_load(p, table + ((size_t)w * 256 + byte) * 9);
    acc = te_madd(acc, p, false);
  }
  uint64_t *rec = out + i * 13;
  if (k == 0) {
    store_u64x6(rec, fq_zero());
    store_u64x6(rec + 6, fq_canon(fq_one()));
    rec[12] = 1;
    return;
  }
  const wpt_t a = te_to_weierstrass(acc);
  store_u64x6(rec, fq_canon(a.x));
  store_u64x6(rec + 6, fq_canon(a.y));
  rec[12] = 0;
}

// ---- self-test hooks ----
__global__ void k_field_test(int op, const uint32_t *a, const uint32_t *b, uint32_t *out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fq_t x, y, r;
#pragma unroll
  for (int k = 0; k < FQ_LIMBS; k++) {
    x.v[k] = a[i * FQ_LIMBS + k];
    y.v[k] = b[i * FQ_LIMBS + k];
  }
  switch (op) {
    case 0: r = fq_mul(x, y); break;
    case 1: r = fq_add(x, y); break;
    case 2: r = fq_sub(x, y); break;
    case 3: r = fq_inv(x); break;
    case 4: r = fq_canon(x); break;
    case 5: r = fq_neg(x); break;
    case 6: r = fq_inv_vartime(x); break;
    default: r = fq_zero(); break;
  }
#pragma unroll
  for (int k = 0; k < FQ_LIMBS; k++) out[i * FQ_LIMBS + k] = r.v[k];
}

// Peak IMAD rates: 8 independent chains per thread of mad.lo/mad.hi pairs (mode 0), mad.lo only
// (mode 1) or mad.hi only (mode 2); 16 IMAD per chain step.
template <int MODE>
__global__ void k_imad_peak(uint32_t *sink, int iters) {
  uint32_t a[8], b = threadIdx.x | 1u, c = blockIdx.x * 2654435761u;
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = c + k * 0x9e3779b9u;
#pragma unroll 1
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (MODE == 0) {
        asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(b), "r"(c));
        asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(b), "r"(c));
      } else if (MODE == 1) {
        asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(b), "r"(c));
        asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(b), "r"(c));
      } else {
        asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(b), "r"(c));
        asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(b), "r"(c));
      }
    }
  }
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s ^= a[k];
  if (s == 0x12345678u) sink[0] = s;
}

// te_madd throughput on L2-resident bases (arithmetic ceiling of the accumulate loop)
__global__ void __launch_bounds__(256) k_madd_bench(const uint4 *bases, uint32_t nb, uint4 *out, int iters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  xyzt_t acc = xyzt_identity();
  uint32_t idx = tid % nb;
#pragma unroll 1
  for (int it = 0; it < iters; it++) {
    pre_t b;
    pre_load(b, bases + (size_t)idx * 9);
    acc = te_madd(acc, b, (it & 1) != 0);
    idx = (idx * 1103515245u + 12345u) % nb;
  }
  xyzt_store(out + (size_t)tid * 12, acc);
}

}  // namespace

cudaError_t msm_launch_precompute(const void *d_affine, size_t n, uint4 *d_bases, uint8_t *d_flags,
                                  uint32_t *d_special_idx, uint32_t *d_special_count,
                                  uint32_t index_offset, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_precompute<<<(unsigned)((n + 127) / 128), 128, 0, st>>>((const uint64_t *)d_affine, n, d_bases,
                                                             d_flags, d_special_idx,
                                                             d_special_count, index_offset);
  return cudaGetLastError();
}

cudaError_t msm_launch_fixed_base(uint4 *d_bases, const uint8_t *d_flags, uint64_t n, uint64_t first,
                                  uint64_t count, uint32_t c, uint32_t nwin, uint32_t *d_fail,
                                  cudaStream_t st) {
  if (count == 0 || nwin <= 1) return cudaSuccess;
  if (nwin > kMaxFbWindows) return cudaErrorInvalidValue;
  k_fixed_base<<<(unsigned)((count + 127) / 128), 128, 0, st>>>(d_bases, d_flags, n, first, count, c,
                                                               nwin, d_fail);
  return cudaGetLastError();
}

cudaError_t msm_launch_check_classes(const uint4 *d_pts, uint32_t n, uint32_t *d_ok, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_check_classes<<<1, 32, 0, st>>>(d_pts, n, d_ok);
  return cudaGetLastError();
}

cudaError_t msm_build_gen_table(uint4 *d_table, cudaStream_t st) {
  k_gen_table<<<16, 128, 0, st>>>(d_table);
  return cudaGetLastError();
}

cudaError_t msm_launch_gen_bases(uint64_t seed, uint64_t first, size_t n, void *d_affine,
                                 const uint4 *d_table, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_gen_bases<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(seed, first, n, (uint64_t *)d_affine, d_table);
  return cudaGetLastError();
}

cudaError_t msm_launch_field_test(int op, const uint32_t *a, const uint32_t *b, uint32_t *out,
                                  size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_field_test<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(op, a, b, out, n);
  return cudaGetLastError();
}

cudaError_t msm_launch_imad_peak(uint32_t *sink, int blocks, int threads, int iters, int mode,
                                 cudaStream_t st) {
  if (mode == 1) k_imad_peak<1><<<blocks, threads, 0, st>>>(sink, iters);
  else if (mode == 2) k_imad_peak<2><<<blocks, threads, 0, st>>>(sink, iters);
  else k_imad_peak<0><<<blocks, threads, 0, st>>>(sink, iters);
  return cudaGetLastError();
}

cudaError_t msm_launch_madd_bench(const uint4 *bases, uint32_t nbases, uint4 *out, int blocks,
                                  int threads, int iters, cudaStream_t st) {
  k_madd_bench<<<blocks, threads, 0, st>>>(bases, nbases, out, iters);
  return cudaGetLastError();
}
