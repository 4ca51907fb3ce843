// NTT over the Goldilocks field (p = 2^64 - 2^32 + 1) on sm_103a: the GPU form of the reference's
// NTT track (zprize/ntt).  The transform is the reference's (zprize/ntt/host/reference.cpp:94-139):
// X[k] = sum_j x[j] w^(j k) with w = OMEGA[log2 n] of zprize/ntt/host/gf.h:65-99, natural order in
// and out.  The reference evaluates 2^24 points on the FPGA with the 4-step decomposition into
// 2^12-point transforms (zprize/ntt/docs/zprize_ntt_top.mld:6-31); this engine does the same split,
// n = n1 n2 with n1, n2 <= 2^12:
//   pass A: for every column j1 of the n2 x n1 row-major input, the n2-point transform over j2,
//           times w^(j1 k2), written to Z[k2][j1];
//   pass B: for every row k2 of Z, the n1-point transform over j1, written to X[k2 + n2 k1].
// One kernel (k_ntt_pass8) does both passes: a block holds C <= 4 of the short transforms in
// shared memory, runs them as radix-8 decimation-in-frequency rounds (three stages per round in
// registers), and gathers the outputs in natural order, optionally twisted.  With C = 4 every row
// of a column load and every output group of a store is 32 contiguous bytes, one DRAM sector.
// HBM traffic: n x 8 B read and written per pass.  k_ntt_pass, the first form (radix-2
// decimation-in-time stages on bit-reversed positions), stays for comparison (NTT_RADIX2=1).
// Transforms of at most 2^12 points are one pass.  An inverse context (ntt_init_inverse) runs the
// same kernels with the inverse roots and multiplies by 1/n: the factor sits in pass A's twist
// table, or in the store of a transform of one pass.
//
// Field arithmetic: elements in [0, p).  The 128-bit product hi 2^64 + lo reduces with
// 2^64 = 2^32 - 1 and 2^96 = -1 (mod p): hi = hh 2^32 + hl gives lo - hh + hl (2^32 - 1).
#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/ntt_gb300.h"

namespace {

constexpr uint64_t GL_P = 0xffffffff00000001ull;
constexpr uint32_t NTT_MAX_LOG_M = 12;      // longest transform of one block
constexpr uint32_t NTT_THREADS = 1024;

// 2^i-th roots of unity of the reference's table (gf.h:65-99); OMEGA[i+1]^2 = OMEGA[i]
const uint64_t GL_OMEGA[33] = {
    0x0000000000000001ull, 0xffffffff00000000ull, 0x0001000000000000ull, 0xfffffffeff000001ull,
    0xefffffff00000001ull, 0x00003fffffffc000ull, 0x0000008000000000ull, 0xf80007ff08000001ull,
    0xbf79143ce60ca966ull, 0x1905d02a5c411f4eull, 0x9d8f2ad78bfed972ull, 0x0653b4801da1c8cfull,
    0xf2c35199959dfcb6ull, 0x1544ef2335d17997ull, 0xe0ee099310bba1e2ull, 0xf6b2cffe2306baacull,
    0x54df9630bf79450eull, 0xabd0a6e8aa3d8a0eull, 0x81281a7b05f9beacull, 0xfbd41c6b8caa3302ull,
    0x30ba2ecd5e93e76dull, 0xf502aef532322654ull, 0x4b2a18ade67246b5ull, 0xea9d5a1336fbc98bull,
    0x86cdcc31c307e171ull, 0x4bbaf5976ecfefd8ull, 0xed41d05b78d6e286ull, 0x10d78dd8915a171dull,
    0x59049500004a4485ull, 0xdfa8c93ba46d2666ull, 0x7e9bd009b86a0845ull, 0x400a7f755588e659ull,
    0x185629dcda58878cull};

// ---- host-side field arithmetic (table set-up) ----
uint64_t h_mul(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) % GL_P); }

// ---- device field arithmetic ----
// Carry-chain forms on 32-bit halves: every correction is driven by a carry or borrow flag, so no
// 64-bit comparison or select chain is needed.  Inputs and outputs are canonical (below p).
__device__ __forceinline__ uint64_t gl_pack(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }

// a + b: S = a + b < 2p; S >= p exactly when S + (2^32 - 1) carries out of 64 bits (counting
// the first carry), and then S - p = (S + 2^32 - 1) mod 2^64
__device__ __forceinline__ uint64_t gl_add(uint64_t a, uint64_t b) {
  uint32_t s0, s1, t0, t1, c;
  asm("{\n\t.reg .u32 c1;\n\t"
      "add.cc.u32 %0, %5, %7;\n\t"
      "addc.cc.u32 %1, %6, %8;\n\t"
      "addc.u32 c1, 0, 0;\n\t"
      "add.cc.u32 %2, %0, 0xffffffff;\n\t"
      "addc.cc.u32 %3, %1, 0;\n\t"
      "addc.u32 %4, c1, 0;\n\t}"
      : "=&r"(s0), "=&r"(s1), "=&r"(t0), "=&r"(t1), "=&r"(c)
      : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"((uint32_t)b), "r"((uint32_t)(b >> 32)));
  return c ? gl_pack(t0, t1) : gl_pack(s0, s1);
}

// a - b: on a borrow the wrapped difference d = a - b + 2^64 >= 2^32, and d - (2^32 - 1) is
// a - b + p
__device__ __forceinline__ uint64_t gl_sub(uint64_t a, uint64_t b) {
  uint32_t d0, d1;
  asm("{\n\t.reg .u32 bw;\n\t"
      "sub.cc.u32 %0, %2, %4;\n\t"
      "subc.cc.u32 %1, %3, %5;\n\t"
      "subc.u32 bw, 0, 0;\n\t"
      "sub.cc.u32 %0, %0, bw;\n\t"
      "subc.u32 %1, %1, 0;\n\t}"
      : "=&r"(d0), "=&r"(d1)
      : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"((uint32_t)b), "r"((uint32_t)(b >> 32)));
  return gl_pack(d0, d1);
}

// a b: the 128-bit product (r3 r2 r1 r0) from four wide multiplies whose 64-bit addends carry
// the partial products' overflow (the carries ride in the multiplies, which run on the multiply
// pipe, and not in add chains on the integer ALU, which bounded the passes), then
// lo + hl (2^32 - 1) - hh with
// lo = r1 r0, hl = r2, hh = r3 (2^64 = 2^32 - 1, 2^96 = -1 mod p): hl (2^32 - 1) is a fifth wide
// multiply, each step is corrected by its own carry or borrow, and a last conditional
// subtraction of p makes the value canonical.
//   s = lo + hl (2^32 - 1) < 2^65; a carry out adds 2^32 - 1, and then s < 2^64 - 2^32;
//   t = s - hh; a borrow subtracts 2^32 - 1 more (t + p), which stays above zero.
__device__ __forceinline__ uint64_t gl_mul(uint64_t a, uint64_t b) {
  const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  const uint64_t x = (uint64_t)a0 * b0;
  const uint64_t y = (uint64_t)a0 * b1 + (x >> 32);
  const uint64_t z = (uint64_t)a1 * b0 + (uint32_t)y;
  const uint64_t w = (uint64_t)a1 * b1 + (y >> 32) + (z >> 32);
  const uint64_t u = (uint64_t)(uint32_t)w * 0xffffffffu;  // hl (2^32 - 1)
  uint32_t t0, t1, q0, q1, c;
  asm("{\n\t.reg .u32 m;\n\t"
      "add.cc.u32 %0, %5, %7;\n\t"       // s = lo + u
      "addc.cc.u32 %1, %6, %8;\n\t"
      "addc.u32 m, 0, 0;\n\t"
      "neg.s32 m, m;\n\t"                // 2^32 - 1 on a carry
      "add.cc.u32 %0, %0, m;\n\t"
      "addc.u32 %1, %1, 0;\n\t"
      "sub.cc.u32 %0, %0, %9;\n\t"       // t = s - hh
      "subc.cc.u32 %1, %1, 0;\n\t"
      "subc.u32 m, 0, 0;\n\t"            // 2^32 - 1 on a borrow
      "sub.cc.u32 %0, %0, m;\n\t"
      "subc.u32 %1, %1, 0;\n\t"
      "add.cc.u32 %2, %0, 0xffffffff;\n\t"  // t >= p exactly when t + 2^32 - 1 carries
      "addc.cc.u32 %3, %1, 0;\n\t"
      "addc.u32 %4, 0, 0;\n\t}"
      : "=&r"(t0), "=&r"(t1), "=&r"(q0), "=&r"(q1), "=&r"(c)
      : "r"((uint32_t)x), "r"((uint32_t)z), "r"((uint32_t)u), "r"((uint32_t)(u >> 32)),
        "r"((uint32_t)(w >> 32)));
  return c ? gl_pack(q0, q1) : gl_pack(t0, t1);
}

__device__ __forceinline__ uint32_t bit_reverse(uint32_t x, uint32_t bits) {
  return bits ? __brev(x) >> (32 - bits) : 0u;
}

struct NttPass {
  const uint64_t *src;
  uint64_t *dst;
  uint32_t log_m;  // transform length of this pass
  uint32_t cols;   // transforms per block (1, 2 or 4)
  uint32_t log_cols;  // log2 cols: the block's index splits are shifts and masks, not divisions
  uint64_t in_c, in_i;    // element i of transform g: src[g in_c + i in_i]
  uint64_t out_c, out_k;  // output k of transform g: dst[g out_c + k out_k]
  const uint64_t *tw_m;   // w_m^j, j < m/2
  // twist (pass A): output k of transform g times w_n^(g k mod n), from w_n^e = hi[e >> 12] lo[e & 4095]
  const uint64_t *tw_lo, *tw_hi;
  uint64_t n_mask;  // n - 1 when twisting, 0 otherwise
  uint64_t scale;   // outputs of an untwisted pass times this (0: none), the inverse's 1/n
};

__global__ void __launch_bounds__(NTT_THREADS) k_ntt_pass(NttPass ps) {
  extern __shared__ uint64_t sm[];
  const uint32_t m = 1u << ps.log_m, C = ps.cols, half = m >> 1;
  uint64_t *tw = sm + (size_t)C * m;
  const uint64_t g0 = (uint64_t)blockIdx.x * C;
  for (uint32_t j = threadIdx.x; j < half; j += blockDim.x) tw[j] = ps.tw_m[j];
  // load C transforms, element i to its bit-reversed slot; the unit-stride index runs fastest
  const bool c_fast = ps.in_c == 1;
  for (uint32_t t = threadIdx.x; t < C * m; t += blockDim.x) {
    const uint32_t c = c_fast ? t & (C - 1) : t >> ps.log_m, i = c_fast ? t >> ps.log_cols : t & (m - 1);
    uint64_t v = __ldcs(ps.src + (g0 + c) * ps.in_c + (uint64_t)i * ps.in_i);
    if (v >= GL_P) v -= GL_P;  // inputs are taken modulo p
    sm[(size_t)c * m + bit_reverse(i, ps.log_m)] = v;
  }
  __syncthreads();
  for (uint32_t s = 1; s <= ps.log_m; s++) {
    const uint32_t h = 1u << (s - 1);
    for (uint32_t t = threadIdx.x; t < C * half; t += blockDim.x) {
      const uint32_t c = t >> (ps.log_m - 1), r = t & (half - 1);
      const uint32_t j = r & (h - 1), k0 = ((r >> (s - 1)) << s) + j;
      uint64_t *a = sm + (size_t)c * m;
      const uint64_t w = tw[j << (ps.log_m - s)];  // w_m^(j m / 2h), a primitive 2h-th root
      const uint64_t u = a[k0], v = gl_mul(a[k0 + h], w);
      a[k0] = gl_add(u, v);
      a[k0 + h] = gl_sub(u, v);
    }
    __syncthreads();
  }
  // store, output groups of C consecutive transforms together
  for (uint32_t t = threadIdx.x; t < C * m; t += blockDim.x) {
    const uint32_t c = t & (C - 1), k = t >> ps.log_cols;
    uint64_t v = sm[(size_t)c * m + k];
    if (ps.n_mask) {
      const uint64_t e = ((g0 + c) * (uint64_t)k) & ps.n_mask;
      v = gl_mul(v, gl_mul(ps.tw_hi[e >> 12], ps.tw_lo[e & 4095]));
    } else if (ps.scale) {
      v = gl_mul(v, ps.scale);
    }
    __stcs(ps.dst + (g0 + c) * ps.out_c + (uint64_t)k * ps.out_k, v);
  }
}

// ---- radix-8 decimation in frequency (the pass kernel) ----
// Natural order in, bit-reversed order in shared memory out: stage H (half size) turns the pair
// (k, k + H) of each block of 2H into (u + v, (u - v) w_2H^(k mod H)).  Three consecutive stages
// only mix the 8 elements {b 2H0 + j + t h : t < 8} (h = H0 / 4), so each round of three stages
// runs in registers: one shared-memory load and store per element per round instead of one per
// stage, and the first round reads global memory directly (natural order: coalesced).  The last
// step gathers X[k] = a[rev(k)].  Slots are swizzled (low four bits XOR bits 4..7 and 8..11) and
// transforms sit 8 slots apart, which makes the rounds' and the gather's 64-bit accesses free of
// bank conflicts for m = 4096.
__device__ __forceinline__ uint32_t slot(uint32_t q) { return q ^ ((q >> 4) & 15u) ^ ((q >> 8) & 15u); }

// LAST: the round ending at half size 1, where every unit has j = 0 and the twiddle of a pair
// whose position within the half is 0 is 1 (7 of the 12 of a radix-8 round): no product there.
template <int R, bool LAST>
__device__ __forceinline__ void dif_unit(uint64_t (&x)[8], uint32_t j, uint32_t log_hmin,
                                         uint32_t log_m, const uint64_t *tw) {
#pragma unroll
  for (int l = 0; l < R; l++) {
    const int d = 1 << (R - 1 - l);                    // partner distance within the unit
    const uint32_t log_h = log_hmin + (R - 1 - l);     // this stage's half size
#pragma unroll
    for (int t = 0; t < (1 << R); t++) {
      if (t & d) continue;
      const uint64_t u = x[t], v = x[t + d];
      x[t] = gl_add(u, v);
      if (LAST && (t & (d - 1)) == 0) {
        x[t + d] = gl_sub(u, v);
      } else {
        const uint32_t jp = j + ((uint32_t)(t & (d - 1)) << log_hmin);  // position within the half
        const uint64_t w = tw[jp << (log_m - 1 - log_h)];              // w_2H^jp = w_m^(jp m / 2H)
        x[t + d] = gl_mul(gl_sub(u, v), w);
      }
    }
  }
}

// One round of R stages over every unit of the block's transforms; the first round reads the
// transforms from global memory (natural order), the others from shared memory.
template <int R, bool LAST>
__device__ __forceinline__ void dif_round(const NttPass &ps, uint64_t *sm, uint32_t pitch,
                                          const uint64_t *tw, uint32_t log_hmin, bool from_global) {
  const uint32_t m = 1u << ps.log_m, C = ps.cols, units = m >> R;
  const uint64_t g0 = (uint64_t)blockIdx.x * C;
  const bool c_fast = from_global && ps.in_c == 1;  // consecutive lanes on consecutive transforms
  // q0 holds no bit of t << log_hmin, so q = q0 ^ (t << log_hmin), and the swizzle is linear over
  // XOR: slot(q) = slot(q0) ^ slot(t << log_hmin), the second term fixed for the round
  uint32_t st[1 << R];
#pragma unroll
  for (int t = 0; t < (1 << R); t++) st[t] = slot((uint32_t)t << log_hmin);
  for (uint32_t w = threadIdx.x; w < C * units; w += blockDim.x) {
    const uint32_t c = c_fast ? w & (C - 1) : w >> (ps.log_m - R);
    const uint32_t u = c_fast ? w >> ps.log_cols : w & (units - 1);
    const uint32_t j = u & ((1u << log_hmin) - 1), b = u >> log_hmin;
    const uint32_t q0 = (b << (log_hmin + R)) + j;
    const uint32_t s0 = slot(q0);
    uint64_t x[8];
    uint64_t *a = sm + (size_t)c * pitch;
#pragma unroll
    for (int t = 0; t < (1 << R); t++) {
      if (from_global) {
        const uint32_t q = q0 + ((uint32_t)t << log_hmin);
        uint64_t v = __ldcs(ps.src + (g0 + c) * ps.in_c + (uint64_t)q * ps.in_i);
        x[t] = v >= GL_P ? v - GL_P : v;  // inputs are taken modulo p
      } else {
        x[t] = a[s0 ^ st[t]];
      }
    }
    dif_unit<R, LAST>(x, j, log_hmin, ps.log_m, tw);
#pragma unroll
    for (int t = 0; t < (1 << R); t++) a[s0 ^ st[t]] = x[t];
  }
}

__global__ void __launch_bounds__(NTT_THREADS) k_ntt_pass8(NttPass ps) {
  extern __shared__ uint64_t sm[];
  const uint32_t m = 1u << ps.log_m, C = ps.cols, half = m >> 1, pitch = m + 8;
  uint64_t *tw = sm + (size_t)C * pitch;
  const uint64_t g0 = (uint64_t)blockIdx.x * C;
  for (uint32_t j = threadIdx.x; j < half; j += blockDim.x) tw[j] = ps.tw_m[j];
  __syncthreads();
  int log_h0 = (int)ps.log_m - 1;  // half size of the next stage
  bool first = true;
  while (log_h0 >= 0) {
    const int r = log_h0 + 1 >= 3 ? 3 : log_h0 + 1;
    const uint32_t log_hmin = (uint32_t)(log_h0 - (r - 1));
    if (log_hmin == 0) {  // the last round
      if (r == 3) dif_round<3, true>(ps, sm, pitch, tw, 0, first);
      else if (r == 2) dif_round<2, true>(ps, sm, pitch, tw, 0, first);
      else dif_round<1, true>(ps, sm, pitch, tw, 0, first);
    } else {
      if (r == 3) dif_round<3, false>(ps, sm, pitch, tw, log_hmin, first);
      else if (r == 2) dif_round<2, false>(ps, sm, pitch, tw, log_hmin, first);
      else dif_round<1, false>(ps, sm, pitch, tw, log_hmin, first);
    }
    __syncthreads();
    first = false;
    log_h0 -= r;
  }
  if (first) {  // m = 1: no stage, the value itself
    for (uint32_t c = threadIdx.x; c < C; c += blockDim.x) {
      const uint64_t v = __ldcs(ps.src + (g0 + c) * ps.in_c);
      sm[(size_t)c * pitch] = v >= GL_P ? v - GL_P : v;
    }
    __syncthreads();
  }
  // gather in natural order, output groups of C consecutive transforms together
  for (uint32_t t = threadIdx.x; t < C * m; t += blockDim.x) {
    const uint32_t c = t & (C - 1), k = t >> ps.log_cols;
    uint64_t v = sm[(size_t)c * pitch + slot(bit_reverse(k, ps.log_m))];
    if (ps.n_mask) {
      const uint64_t e = ((g0 + c) * (uint64_t)k) & ps.n_mask;
      v = gl_mul(v, gl_mul(ps.tw_hi[e >> 12], ps.tw_lo[e & 4095]));
    } else if (ps.scale) {
      v = gl_mul(v, ps.scale);
    }
    __stcs(ps.dst + (g0 + c) * ps.out_c + (uint64_t)k * ps.out_k, v);
  }
}

// self-test hook: element-wise a op b (0 add, 1 sub, 2 mul)
__global__ void k_gl_test(int op, const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = op == 0 ? gl_add(a[i], b[i]) : op == 1 ? gl_sub(a[i], b[i]) : gl_mul(a[i], b[i]);
}

// Linear copy of n values in 16-byte vectors; the source may be host memory that the device
// reads through the host's page tables (Grace over NVLink-C2C).
__global__ void __launch_bounds__(256) k_ntt_copy(const uint4 *src, uint4 *dst, uint64_t nvec) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvec;
       i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// ---- host context ----
thread_local int g_err = 0;
thread_local char g_msg[512] = "";

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  g_err = code;
  return code;
}

#define NCK(x)                                                                            \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) return fail(NTT_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
  } while (0)

struct NttCtx {
  int device = 0;
  uint32_t log_n = 0, log_n1 = 0, log_n2 = 0, cols = 4;
  uint64_t n = 0;
  uint64_t *d_in = nullptr, *d_out = nullptr, *d_tmp = nullptr;
  uint64_t *d_tw1 = nullptr, *d_tw2 = nullptr, *d_twlo = nullptr, *d_twhi = nullptr;
  // the device reads pageable host memory through the host's page tables: the input vector
  // moves by a copy kernel instead of a driver copy
  bool host_direct = false;
  bool radix2 = false;  // the radix-2 pass kernel (comparison)
  bool inverse = false;   // roots w^-1 and outputs times 1/n
  uint64_t scale_single = 0;  // 1/n for an inverse of one pass (the twist carries it otherwise)
  int num_sms = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev[5] = {};
  bool timing = false;
  double last_ms[4] = {0, 0, 0, 0};
  // batches: a second input and output vector, and one stream each for uploads and downloads
  uint64_t *d_in2 = nullptr, *d_out2 = nullptr;
  cudaStream_t st_up = nullptr, st_down = nullptr;
  cudaEvent_t up_done[2] = {}, comp_done[2] = {}, down_done[2] = {};
  ~NttCtx() {
    for (uint64_t *p : {d_in, d_out, d_tmp, d_tw1, d_tw2, d_twlo, d_twhi, d_in2, d_out2})
      if (p) cudaFree(p);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    for (int k = 0; k < 2; k++)
      for (cudaEvent_t e : {up_done[k], comp_done[k], down_done[k]})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t x : {st, st_up, st_down})
      if (x) cudaStreamDestroy(x);
  }
};

uint64_t h_pow(uint64_t b, uint64_t e) {
  uint64_t r = 1;
  for (; e; e >>= 1, b = h_mul(b, b))
    if (e & 1) r = h_mul(r, b);
  return r;
}
uint64_t h_inv(uint64_t a) { return h_pow(a, GL_P - 2); }  // Fermat; a != 0

// the 2^k-th root the context transforms with: the reference's, or its inverse
uint64_t ctx_root(const NttCtx *cx, uint32_t k) {
  return cx->inverse ? h_inv(GL_OMEGA[k]) : GL_OMEGA[k];
}

// w^0 .. w^(count - 1)
std::vector<uint64_t> powers(uint64_t w, uint64_t count) {
  std::vector<uint64_t> v(std::max<uint64_t>(count, 1));
  v[0] = 1;
  for (uint64_t i = 1; i < count; i++) v[i] = h_mul(v[i - 1], w);
  return v;
}

int upload(uint64_t **dst, const std::vector<uint64_t> &v) {
  NCK(cudaMalloc(dst, v.size() * 8));
  NCK(cudaMemcpy(*dst, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
  return 0;
}

size_t pass_smem(uint32_t log_m, uint32_t cols) {
  return ((size_t)cols * ((1u << log_m) + 8) + (1u << log_m) / 2 + 1) * 8;
}

// one pass: `count` transforms of 2^log_m points, `cols` per block
cudaError_t launch_pass(const NttCtx *cx, const uint64_t *src, uint64_t *dst, uint32_t log_m,
                        uint64_t count, uint64_t in_c, uint64_t in_i, uint64_t out_c, uint64_t out_k,
                        const uint64_t *tw_m, bool twist, cudaStream_t st, uint64_t scale = 0) {
  NttPass ps;
  ps.src = src;
  ps.dst = dst;
  ps.log_m = log_m;
  ps.cols = (uint32_t)std::min<uint64_t>(cx->cols, count);  // powers of two
  ps.log_cols = (uint32_t)__builtin_ctz(ps.cols);
  ps.in_c = in_c;
  ps.in_i = in_i;
  ps.out_c = out_c;
  ps.out_k = out_k;
  ps.tw_m = tw_m;
  ps.tw_lo = cx->d_twlo;
  ps.tw_hi = cx->d_twhi;
  ps.n_mask = twist ? cx->n - 1 : 0;
  ps.scale = twist ? 0 : scale;
  const uint32_t blocks = (uint32_t)(count / ps.cols);
  const uint32_t threads = std::min<uint32_t>(NTT_THREADS, std::max<uint32_t>(32, ps.cols << (log_m - (log_m ? 1 : 0))));
  if (cx->radix2)
    k_ntt_pass<<<blocks, threads, pass_smem(log_m, ps.cols), st>>>(ps);
  else
    k_ntt_pass8<<<blocks, threads, pass_smem(log_m, ps.cols), st>>>(ps);
  return cudaGetLastError();
}

// the transform of cx->n points from d_src to d_dst (device memory), enqueued on st
int enqueue_ntt(NttCtx *cx, uint64_t *d_dst, const uint64_t *d_src, cudaStream_t st, bool marks) {
  if (cx->log_n <= NTT_MAX_LOG_M) {
    NCK(launch_pass(cx, d_src, d_dst, cx->log_n, 1, 0, 1, 0, 1, cx->d_tw1, false, st,
                    cx->scale_single));
    if (marks) NCK(cudaEventRecord(cx->ev[2], st));
    return 0;
  }
  const uint64_t n1 = 1ull << cx->log_n1, n2 = 1ull << cx->log_n2;
  // pass A: n1 columns of n2 points (stride n1), twisted, to Z[k2][j1]
  NCK(launch_pass(cx, d_src, cx->d_tmp, cx->log_n2, n1, 1, n1, 1, n1, cx->d_tw2, true, st));
  if (marks) NCK(cudaEventRecord(cx->ev[2], st));
  // pass B: n2 rows of n1 points, to X[k2 + n2 k1]
  NCK(launch_pass(cx, cx->d_tmp, d_dst, cx->log_n1, n2, n1, 1, 1, n2, cx->d_tw1, false, st));
  return 0;
}

}  // namespace

extern "C" {

int ntt_last_error(char *buf, size_t len) {
  if (buf && len) {
    strncpy(buf, g_msg, len - 1);
    buf[len - 1] = 0;
  }
  return g_err;
}

}  // extern "C"

namespace {

// a context of either direction (ntt_init, ntt_init_inverse)
void *ntt_create(uint32_t log_n, bool inverse) {
  g_err = 0;
  if (log_n > 2 * NTT_MAX_LOG_M) {
    fail(NTT_ERR_ARG, "ntt_init: 2^%u points is over the maximum of 2^%u", log_n, 2 * NTT_MAX_LOG_M);
    return nullptr;
  }
  auto *cx = new NttCtx();
  cx->inverse = inverse;
  const char *dev = getenv("MSM_DEVICE");
  cx->device = dev ? atoi(dev) : 0;
  if (const char *c = getenv("NTT_COLS")) {  // transforms per block: 1, 2 or 4
    const int v = atoi(c);
    cx->cols = v >= 4 ? 4 : v >= 2 ? 2 : 1;
  }
  cx->log_n = log_n;
  cx->n = 1ull << log_n;
  cx->log_n2 = log_n / 2;
  cx->log_n1 = log_n - cx->log_n2;
  int rc = 0;
  auto step = [&](cudaError_t e, const char *what) {
    if (!rc && e != cudaSuccess) rc = fail(NTT_ERR_CUDA, "ntt_init: %s: %s", what, cudaGetErrorString(e));
  };
  step(cudaSetDevice(cx->device), "cudaSetDevice");
  int pageable = 0, host_tables = 0;
  step(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, cx->device), "attribute");
  step(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                              cx->device), "attribute");
  step(cudaDeviceGetAttribute(&cx->num_sms, cudaDevAttrMultiProcessorCount, cx->device), "attribute");
  const char *hd = getenv("NTT_HOST_DIRECT");
  cx->host_direct = pageable && host_tables && !(hd && strcmp(hd, "0") == 0);
  step(cudaStreamCreateWithFlags(&cx->st, cudaStreamNonBlocking), "stream");
  for (auto &e : cx->ev) step(cudaEventCreate(&e), "event");
  step(cudaFuncSetAttribute(k_ntt_pass, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)pass_smem(NTT_MAX_LOG_M, 4)),
       "shared memory size");
  step(cudaFuncSetAttribute(k_ntt_pass8, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)pass_smem(NTT_MAX_LOG_M, 4)),
       "shared memory size");
  if (const char *r2 = getenv("NTT_RADIX2")) cx->radix2 = strcmp(r2, "1") == 0;
  step(cudaMalloc(&cx->d_in, cx->n * 8), "input buffer");
  step(cudaMalloc(&cx->d_out, cx->n * 8), "output buffer");
  if (log_n > NTT_MAX_LOG_M) step(cudaMalloc(&cx->d_tmp, cx->n * 8), "intermediate buffer");
  if (!rc) {
    // short-transform roots: w_m = w_n^(n/m), from the reference's table (inverted for the
    // inverse transform)
    const uint32_t l1 = log_n > NTT_MAX_LOG_M ? cx->log_n1 : log_n;
    rc = upload(&cx->d_tw1, powers(ctx_root(cx, l1), (1ull << l1) / 2));
    // the inverse's 1/n: in the twist of pass A (every entry of the high table), or in the
    // store of a transform of one pass
    const uint64_t inv_n = h_inv(cx->n % GL_P);
    if (inverse && log_n <= NTT_MAX_LOG_M) cx->scale_single = inv_n;
    if (!rc && log_n > NTT_MAX_LOG_M) {
      rc = upload(&cx->d_tw2, powers(ctx_root(cx, cx->log_n2), (1ull << cx->log_n2) / 2));
      const uint64_t w = ctx_root(cx, log_n);
      if (!rc) rc = upload(&cx->d_twlo, powers(w, std::min<uint64_t>(cx->n, 4096)));
      uint64_t w4096 = w;
      for (int i = 0; i < 12; i++) w4096 = h_mul(w4096, w4096);
      std::vector<uint64_t> hi = powers(w4096, std::max<uint64_t>(cx->n >> 12, 1));
      if (inverse)
        for (uint64_t &v : hi) v = h_mul(v, inv_n);
      if (!rc) rc = upload(&cx->d_twhi, hi);
    }
  }
  if (rc) {
    delete cx;
    return nullptr;
  }
  return cx;
}

}  // namespace

extern "C" {

void *ntt_init(uint32_t log_n) { return ntt_create(log_n, false); }

void *ntt_init_inverse(uint32_t log_n) { return ntt_create(log_n, true); }

void ntt_free(void *context) { delete (NttCtx *)context; }

uint64_t ntt_input_vector_size(void *context) {
  return context ? ((NttCtx *)context)->n : 0;
}

int ntt_evaluate_device(void *context, uint64_t *d_out, const uint64_t *d_in, void *stream) {
  g_err = 0;
  auto *cx = (NttCtx *)context;
  if (!cx || !d_out || !d_in) return fail(NTT_ERR_ARG, "ntt_evaluate_device: null argument");
  if (d_out == d_in && cx->log_n <= NTT_MAX_LOG_M)
    return fail(NTT_ERR_ARG, "ntt_evaluate_device: the transform is out of place");
  NCK(cudaSetDevice(cx->device));
  return enqueue_ntt(cx, d_out, d_in, stream ? (cudaStream_t)stream : cx->st, false);
}

int ntt_evaluate(void *context, uint64_t *out, const uint64_t *in, uint64_t len) {
  g_err = 0;
  auto *cx = (NttCtx *)context;
  if (!cx || !out || !in) return fail(NTT_ERR_ARG, "ntt_evaluate: null argument");
  if (len != cx->n)
    return fail(NTT_ERR_ARG, "ntt_evaluate: %llu values for a transform of %llu points",
                (unsigned long long)len, (unsigned long long)cx->n);
  NCK(cudaSetDevice(cx->device));
  // A copy kernel reads the input when the device reaches pageable memory and the buffer is
  // 16-byte aligned (GB300 at 2^24: 0.67 ms against 0.77 ms for the driver's copy); otherwise the
  // driver copies it.  The output always goes back through the driver: a kernel writing into
  // pages the host has not touched yet takes a fault per page (29 ms at 2^24 against 4.9 ms).
  const bool direct = cx->host_direct && cx->n >= 2 && ((uintptr_t)in & 15) == 0;
  const uint32_t cblocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)cx->num_sms * 8, cx->n / 512));
  NCK(cudaEventRecord(cx->ev[0], cx->st));
  if (direct) {
    k_ntt_copy<<<cblocks, 256, 0, cx->st>>>((const uint4 *)in, (uint4 *)cx->d_in, cx->n / 2);
    NCK(cudaGetLastError());
  } else {
    NCK(cudaMemcpyAsync(cx->d_in, in, cx->n * 8, cudaMemcpyHostToDevice, cx->st));
  }
  NCK(cudaEventRecord(cx->ev[1], cx->st));
  if (int rc = enqueue_ntt(cx, cx->d_out, cx->d_in, cx->st, true)) return rc;
  NCK(cudaEventRecord(cx->ev[3], cx->st));
  NCK(cudaMemcpyAsync(out, cx->d_out, cx->n * 8, cudaMemcpyDeviceToHost, cx->st));
  NCK(cudaEventRecord(cx->ev[4], cx->st));
  NCK(cudaStreamSynchronize(cx->st));
  float ms[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; k++) cudaEventElapsedTime(&ms[k], cx->ev[k], cx->ev[k + 1]);
  for (int k = 0; k < 4; k++) cx->last_ms[k] = ms[k];
  return 0;
}

int ntt_field_selftest(int32_t op, const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n) {
  g_err = 0;
  if (n && (!a || !b || !out)) return fail(NTT_ERR_ARG, "ntt_field_selftest: null argument");
  if (op < 0 || op > 2) return fail(NTT_ERR_ARG, "ntt_field_selftest: unknown operation %d", op);
  if (n == 0) return 0;
  const char *dev = getenv("MSM_DEVICE");
  NCK(cudaSetDevice(dev ? atoi(dev) : 0));
  uint64_t *d = nullptr;
  NCK(cudaMalloc(&d, n * 24));
  int rc = 0;
  if (cudaMemcpy(d, a, n * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d + n, b, n * 8, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = fail(NTT_ERR_CUDA, "ntt_field_selftest: upload failed");
  if (!rc) {
    k_gl_test<<<(unsigned)((n + 255) / 256), 256>>>(op, d, d + n, d + 2 * n, n);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(out, d + 2 * n, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(NTT_ERR_CUDA, "ntt_field_selftest: %s", cudaGetErrorString(cudaGetLastError()));
  }
  cudaFree(d);
  return rc;
}

int ntt_evaluate_batch(void *context, uint64_t *out, const uint64_t *in, uint64_t count) {
  g_err = 0;
  auto *cx = (NttCtx *)context;
  if (!cx || (count && (!out || !in))) return fail(NTT_ERR_ARG, "ntt_evaluate_batch: null argument");
  if (count == 0) return 0;
  NCK(cudaSetDevice(cx->device));
  if (!cx->d_in2) {  // the second buffer pair and the copy streams, on first use
    NCK(cudaMalloc(&cx->d_in2, cx->n * 8));
    NCK(cudaMalloc(&cx->d_out2, cx->n * 8));
    NCK(cudaStreamCreateWithFlags(&cx->st_up, cudaStreamNonBlocking));
    NCK(cudaStreamCreateWithFlags(&cx->st_down, cudaStreamNonBlocking));
    for (int k = 0; k < 2; k++) {
      NCK(cudaEventCreateWithFlags(&cx->up_done[k], cudaEventDisableTiming));
      NCK(cudaEventCreateWithFlags(&cx->comp_done[k], cudaEventDisableTiming));
      NCK(cudaEventCreateWithFlags(&cx->down_done[k], cudaEventDisableTiming));
    }
  }
  uint64_t *din[2] = {cx->d_in, cx->d_in2}, *dout[2] = {cx->d_out, cx->d_out2};
  const size_t bytes = cx->n * 8;
  // Uploads go through the driver; the copy kernel (NTT_BATCH_DIRECT=1) does not block this
  // thread but competes with the transform for the SMs (2^24, 8 vectors: 1.57 against 1.37 ms
  // per transform on GB300).
  const char *bd = getenv("NTT_BATCH_DIRECT");
  const bool direct_up = cx->host_direct && cx->n >= 2 && bd && strcmp(bd, "1") == 0;
  const uint32_t cblocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)cx->num_sms * 8, cx->n / 512));
  // A copy from or into pageable memory blocks its calling thread until it is done, so the
  // downloads run on a worker thread while this thread uploads and enqueues transforms.
  // Vector i uses slot i % 2.  Handshakes on the host: the worker takes vector i once its
  // transform is enqueued (and its completion event recorded); this thread enqueues the
  // transform of i + 2 only once the download of i is done, so no slot is overwritten while in
  // use and no event is recorded again before the worker has waited on it.
  std::mutex mu;
  std::condition_variable cv;
  uint64_t enqueued = 0, downloaded = 0;
  int worker_rc = 0;
  std::thread worker([&] {
    cudaSetDevice(cx->device);
    for (uint64_t i = 0; i < count; i++) {
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return enqueued > i || worker_rc < 0; });
        if (worker_rc < 0) return;
      }
      const int k = (int)(i & 1);
      cudaError_t e = cudaStreamWaitEvent(cx->st_down, cx->comp_done[k], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(out + i * cx->n, dout[k], bytes, cudaMemcpyDeviceToHost, cx->st_down);
      if (e == cudaSuccess) e = cudaStreamSynchronize(cx->st_down);
      std::lock_guard<std::mutex> lk(mu);
      if (e != cudaSuccess) {
        worker_rc = -1;
        cv.notify_all();
        return;
      }
      downloaded = i + 1;
      cv.notify_all();
    }
  });
  int rc = 0;
  for (uint64_t i = 0; i < count && !rc; i++) {
    const int k = (int)(i & 1);
    if (i >= 2) {  // the download of i - 2 has emptied the output slot
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return downloaded >= i - 1 || worker_rc < 0; });
      if (worker_rc < 0) break;
    }
    cudaError_t e = cudaSuccess;
    if (i >= 2) e = cudaStreamWaitEvent(cx->st_up, cx->comp_done[k], 0);  // the input slot is free
    if (e == cudaSuccess) {
      const uint64_t *src = in + i * cx->n;
      if (direct_up && ((uintptr_t)src & 15) == 0) {  // asynchronous: this thread does not block
        k_ntt_copy<<<cblocks, 256, 0, cx->st_up>>>((const uint4 *)src, (uint4 *)din[k], cx->n / 2);
        e = cudaGetLastError();
      } else {
        e = cudaMemcpyAsync(din[k], src, bytes, cudaMemcpyHostToDevice, cx->st_up);
      }
    }
    if (e == cudaSuccess) e = cudaEventRecord(cx->up_done[k], cx->st_up);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cx->st, cx->up_done[k], 0);
    if (e != cudaSuccess) {
      rc = fail(NTT_ERR_CUDA, "ntt_evaluate_batch: %s", cudaGetErrorString(e));
      break;
    }
    if ((rc = enqueue_ntt(cx, dout[k], din[k], cx->st, false))) break;
    if ((e = cudaEventRecord(cx->comp_done[k], cx->st)) != cudaSuccess) {
      rc = fail(NTT_ERR_CUDA, "ntt_evaluate_batch: %s", cudaGetErrorString(e));
      break;
    }
    std::lock_guard<std::mutex> lk(mu);
    enqueued = i + 1;
    cv.notify_all();
  }
  if (rc) {
    std::lock_guard<std::mutex> lk(mu);
    worker_rc = -1;
    cv.notify_all();
  }
  worker.join();
  if (!rc && worker_rc < 0) rc = fail(NTT_ERR_CUDA, "ntt_evaluate_batch: a download failed");
  cudaStreamSynchronize(cx->st);
  return rc;
}

int ntt_last_timings(void *context, double *ms, int32_t max_stages) {
  auto *cx = (NttCtx *)context;
  if (!cx || !ms) return fail(NTT_ERR_ARG, "ntt_last_timings: null argument");
  const int k = std::min<int32_t>(max_stages, 4);
  for (int i = 0; i < k; i++) ms[i] = cx->last_ms[i];
  return k;
}

}  // extern "C"
