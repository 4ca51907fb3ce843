// BLS12-377 G1 point arithmetic on sm_103a.
//
// Buckets and all partial sums live in extended twisted-Edwards coordinates (X:Y:Z:T), a = -1,
// the representation the reference's FPGA pipeline uses (bls12_377_g1.h:291-491).  Resident
// bases are affine twisted-Edwards points in the reference's "host precomputed" form
// ((y-x)/2, (y+x)/2, d*x*y) (bls12_377_g1.h:606-618, twisted_edwards_curve.ml:100-119; the
// reference scales t by 4d for its (2x,2y,4z,t) bucket form, this engine keeps plain (X,Y,Z,T)
// buckets and scales t by d).  Adding such a base costs 7 multiplications and returns the sum
// scaled by 1/4, which is the same projective point.
//
// Subtraction of a base swaps its first two coordinates and negates the third
// (twisted_edwards_curve.ml:152), so a signed bucket digit costs no extra multiplication.
#pragma once
#include "fq.cuh"

struct xyzt_t {  // extended twisted Edwards, x = X/Z, y = Y/Z, T = XY/Z
  fq_t x, y, z, t;
};

struct pre_t {  // precomputed affine base: ((y-x)/2, (y+x)/2, d*x*y)
  fq_t ymx, ypx, kt;
};

struct wpt_t {  // Weierstrass point, Jacobian (X/Z^2, Y/Z^3); z = 0 is infinity
  fq_t x, y, z;
};

// Out-of-line Montgomery product with operands by value.  The point formulas call it instead of
// inlining seven or nine copies of the fully unrolled product: the hot loop then fits the
// instruction cache (inlined, instruction-fetch stalls dominated k_accumulate) and runs ~20%
// faster on GB300.
static __device__ __noinline__ fq_t fq_mul_nv(fq_t a, fq_t b) { return fq_mul(a, b); }

__device__ __forceinline__ xyzt_t xyzt_identity() {
  xyzt_t r;
  r.x = fq_zero();
  r.y = fq_one();
  r.z = fq_one();
  r.t = fq_zero();
  return r;
}

// acc + (neg ? -b : b), madd-2008-hwcd-3 with the 1/2 scaling folded into the base
__device__ __forceinline__ xyzt_t te_madd(const xyzt_t &p, const pre_t &b, bool neg) {
  const fq_t p0 = fq_select(neg, b.ypx, b.ymx);
  const fq_t p1 = fq_select(neg, b.ymx, b.ypx);
  const fq_t A = fq_mul_nv(fq_sub(p.y, p.x), p0);
  const fq_t B = fq_mul_nv(fq_add(p.y, p.x), p1);
  fq_t C = fq_mul_nv(p.t, b.kt);
  C = fq_select(neg, fq_neg(C), C);
  const fq_t E = fq_sub(B, A);
  const fq_t H = fq_add(B, A);
  const fq_t F = fq_sub(p.z, C);
  const fq_t G = fq_add(p.z, C);
  xyzt_t r;
  r.x = fq_mul_nv(E, F);
  r.y = fq_mul_nv(G, H);
  r.t = fq_mul_nv(E, H);
  r.z = fq_mul_nv(F, G);
  return r;
}

// general unified addition, add-2008-hwcd-3 with k = 2d (bls12_377_g1.h:449-491)
__device__ __forceinline__ xyzt_t te_add(const xyzt_t &p, const xyzt_t &q) {
  const uint32_t kc[FQ_LIMBS] = BLS_TE_K;
  const fq_t A = fq_mul_nv(fq_sub(p.y, p.x), fq_sub(q.y, q.x));
  const fq_t B = fq_mul_nv(fq_add(p.y, p.x), fq_add(q.y, q.x));
  const fq_t C = fq_mul_nv(fq_mul_nv(p.t, fq_from(kc)), q.t);
  const fq_t D = fq_dbl(fq_mul_nv(p.z, q.z));
  const fq_t E = fq_sub(B, A);
  const fq_t F = fq_sub(D, C);
  const fq_t G = fq_add(D, C);
  const fq_t H = fq_add(B, A);
  xyzt_t r;
  r.x = fq_mul_nv(E, F);
  r.y = fq_mul_nv(G, H);
  r.t = fq_mul_nv(E, H);
  r.z = fq_mul_nv(F, G);
  return r;
}

// dedicated doubling, dbl-2008-hwcd with a = -1 (does not read T)
__device__ __forceinline__ xyzt_t te_dbl(const xyzt_t &p) {
  const fq_t A = fq_mul_nv(p.x, p.x);
  const fq_t B = fq_mul_nv(p.y, p.y);
  const fq_t C = fq_dbl(fq_mul_nv(p.z, p.z));
  const fq_t D = fq_neg(A);
  const fq_t E = fq_sub(fq_sub(fq_mul_nv(fq_add(p.x, p.y), fq_add(p.x, p.y)), A), B);
  const fq_t G = fq_add(D, B);
  const fq_t F = fq_sub(G, C);
  const fq_t H = fq_sub(D, B);
  xyzt_t r;
  r.x = fq_mul_nv(E, F);
  r.y = fq_mul_nv(G, H);
  r.t = fq_mul_nv(E, H);
  r.z = fq_mul_nv(F, G);
  return r;
}

// Out-of-line copies for the cold kernels (reductions, combine, generators): one body each
// keeps compile time and code size down; the hot accumulate loop inlines te_madd instead.
static __device__ __noinline__ xyzt_t te_add_ool(const xyzt_t &p, const xyzt_t &q) { return te_add(p, q); }
static __device__ __noinline__ xyzt_t te_dbl_ool(const xyzt_t &p) { return te_dbl(p); }
static __device__ __noinline__ fq_t fq_mul_ool(const fq_t &a, const fq_t &b) { return fq_mul(a, b); }
static __device__ __noinline__ fq_t fq_sqr_ool(const fq_t &a) { return fq_mul(a, a); }

// p + q by the dedicated addition, add-2008-hwcd-4 with a = -1: 8 products, no multiple of d.
//   A = (Y1 - X1)(Y2 + X2), B = (Y1 + X1)(Y2 - X2), C = 2 Z1 T2, D = 2 T1 Z2,
//   E = D + C, F = B - A, G = B + A, H = D - C;  X3 = E F, Y3 = G H, T3 = E H, Z3 = F G.
// In affine terms x3 = E / G = (x1 y1 + x2 y2) / (y1 y2 - x1 x2) and y3 = H / F =
// (x1 y1 - x2 y2) / (x1 y2 - y1 x2), the twisted-Edwards sum wherever F G != 0.  This formula and
// the unified one are polynomial maps that agree on a dense set of pairs, so their 2 x 2 minors
// vanish everywhere: wherever F G != 0 the result is the unified formula's point.  F G = 0
// (doubling, the identity plus a point with T = 0, ...) is tested right after the first two
// products, and the unified formula (9 products) is used then.  E and H feed products only, so
// they stay unreduced (below 4q).
__device__ __forceinline__ xyzt_t te_add_fast(const xyzt_t &p, const xyzt_t &q) {
  const fq_t A = fq_mul_nv(fq_sub_lazy(p.y, p.x), fq_add_lazy(q.y, q.x));
  const fq_t B = fq_mul_nv(fq_add_lazy(p.y, p.x), fq_sub_lazy(q.y, q.x));
  const fq_t F = fq_sub(B, A);
  const fq_t G = fq_add(B, A);
  if (fq_is_zero(F) || fq_is_zero(G)) return te_add_ool(p, q);
  const fq_t C = fq_dbl(fq_mul_nv(p.z, q.t));
  const fq_t D = fq_dbl(fq_mul_nv(p.t, q.z));
  const fq_t E = fq_add_lazy(D, C);
  const fq_t H = fq_sub_lazy(D, C);
  xyzt_t r;
  r.x = fq_mul_nv(E, F);
  r.y = fq_mul_nv(G, H);
  r.t = fq_mul_nv(E, H);
  r.z = fq_mul_nv(F, G);
  return r;
}
static __device__ __noinline__ xyzt_t te_add_fast_ool(const xyzt_t &p, const xyzt_t &q) {
  return te_add_fast(p, q);
}

// small scalar multiple k*p (k >= 0) by double-and-add from the top bit
static __device__ __noinline__ xyzt_t te_mul_small(const xyzt_t &p, uint32_t k) {
  xyzt_t r = xyzt_identity();
  bool started = false;
#pragma unroll 1
  for (int i = 31; i >= 0; i--) {
    if (started) r = te_dbl_ool(r);
    if ((k >> i) & 1u) {
      r = started ? te_add_ool(r, p) : p;
      started = true;
    }
  }
  return r;
}

__device__ __forceinline__ void xyzt_load(xyzt_t &r, const uint4 *p) {
  fq_load(r.x, p + 0);
  fq_load(r.y, p + 3);
  fq_load(r.z, p + 6);
  fq_load(r.t, p + 9);
}
__device__ __forceinline__ void xyzt_store(uint4 *p, const xyzt_t &a) {
  fq_store(p + 0, a.x);
  fq_store(p + 3, a.y);
  fq_store(p + 6, a.z);
  fq_store(p + 9, a.t);
}
__device__ __forceinline__ void pre_load(pre_t &r, const uint4 *p) {
  fq_load(r.ymx, p + 0);
  fq_load(r.ypx, p + 3);
  fq_load(r.kt, p + 6);
}
__device__ __forceinline__ void pre_store(uint4 *p, const pre_t &a) {
  fq_store(p + 0, a.ymx);
  fq_store(p + 3, a.ypx);
  fq_store(p + 6, a.kt);
}

// ---- Weierstrass y^2 = x^3 + 1, Jacobian coordinates (a = 0); used for the points without a
// twisted-Edwards image (bls12_377_g1.h:493-566 does the same in affine form) ----
__device__ __forceinline__ wpt_t w_infinity() {
  wpt_t r;
  r.x = fq_one();
  r.y = fq_one();
  r.z = fq_zero();
  return r;
}

static __device__ __noinline__ wpt_t w_dbl(const wpt_t &p) {  // dbl-2009-l
  if (fq_is_zero(p.z) || fq_is_zero(p.y)) return w_infinity();
  const fq_t A = fq_sqr_ool(p.x);
  const fq_t B = fq_sqr_ool(p.y);
  const fq_t C = fq_sqr_ool(B);
  fq_t D = fq_sub(fq_sub(fq_sqr_ool(fq_add(p.x, B)), A), C);
  D = fq_dbl(D);
  const fq_t E = fq_add(fq_dbl(A), A);
  const fq_t F = fq_sqr_ool(E);
  wpt_t r;
  r.x = fq_sub(F, fq_dbl(D));
  fq_t C8 = fq_dbl(fq_dbl(fq_dbl(C)));
  r.y = fq_sub(fq_mul_ool(E, fq_sub(D, r.x)), C8);
  r.z = fq_dbl(fq_mul_ool(p.y, p.z));
  return r;
}

static __device__ __noinline__ wpt_t w_add(const wpt_t &p, const wpt_t &q) {  // add-2007-bl, complete by cases
  if (fq_is_zero(p.z)) return q;
  if (fq_is_zero(q.z)) return p;
  const fq_t Z1Z1 = fq_sqr_ool(p.z);
  const fq_t Z2Z2 = fq_sqr_ool(q.z);
  const fq_t U1 = fq_mul_ool(p.x, Z2Z2);
  const fq_t U2 = fq_mul_ool(q.x, Z1Z1);
  const fq_t S1 = fq_mul_ool(fq_mul_ool(p.y, q.z), Z2Z2);
  const fq_t S2 = fq_mul_ool(fq_mul_ool(q.y, p.z), Z1Z1);
  if (fq_eq(U1, U2)) {
    if (fq_eq(S1, S2)) return w_dbl(p);
    return w_infinity();
  }
  const fq_t H = fq_sub(U2, U1);
  const fq_t I = fq_sqr_ool(fq_dbl(H));
  const fq_t J = fq_mul_ool(H, I);
  const fq_t rr = fq_dbl(fq_sub(S2, S1));
  const fq_t V = fq_mul_ool(U1, I);
  wpt_t r;
  r.x = fq_sub(fq_sub(fq_sqr_ool(rr), J), fq_dbl(V));
  r.y = fq_sub(fq_mul_ool(rr, fq_sub(V, r.x)), fq_dbl(fq_mul_ool(S1, J)));
  r.z = fq_mul_ool(fq_sub(fq_sub(fq_sqr_ool(fq_add(p.z, q.z)), Z1Z1), Z2Z2), H);
  return r;
}

// Extended twisted Edwards -> Weierstrass Jacobian with Z = 1 (affine), following
// extendedTwistedEdwardsToWeierstrass (bls12_377_g1.h:389-402, 366-374, 417-425) with one
// inversion: u = (Z+Y)/(Z-Y), v = ts*u*Z/X, x_w = u/c_B + c_A/(3 c_B), y_w = v/c_B.
// The identity maps to infinity; the order-two point (0, -1) maps to its Weierstrass image
// (c_A/(3 c_B), 0) (the reference sends both x = 0 points to infinity, :393-396).
template <bool QUAD>
__device__ __forceinline__ wpt_t te_to_weierstrass_t(const xyzt_t &p, uint32_t mask) {
  const uint32_t ts[FQ_LIMBS] = BLS_TWISTED_SCALE;
  const uint32_t icb[FQ_LIMBS] = BLS_INV_CB;
  const uint32_t ca3[FQ_LIMBS] = BLS_CA_OVER_3CB;
  wpt_t r;
  if (fq_is_zero(p.x)) {
    if (fq_eq(p.y, p.z)) return w_infinity();
    r.x = fq_from(ca3);
    r.y = fq_zero();
    r.z = fq_one();
    return r;
  }
  const fq_t zpy = fq_add(p.z, p.y);
  const fq_t zmy = fq_sub(p.z, p.y);
  const fq_t den = fq_mul_ool(zmy, p.x);
  const fq_t inv = QUAD ? fq_inv_quad(den, mask) : fq_inv_vartime(den);
  const fq_t u = fq_mul_ool(fq_mul_ool(zpy, p.x), inv);
  const fq_t v = fq_mul_ool(fq_mul_ool(fq_mul_ool(zpy, p.z), inv), fq_from(ts));
  r.x = fq_add(fq_mul_ool(u, fq_from(icb)), fq_from(ca3));
  r.y = fq_mul_ool(v, fq_from(icb));
  r.z = fq_one();
  return r;
}

static __device__ __noinline__ wpt_t te_to_weierstrass(const xyzt_t &p) {
  return te_to_weierstrass_t<false>(p, 0u);
}
// The same map run by the four lanes of a quad that all hold p (`mask` covers them): the
// inversion is shared between the lanes (fq_inv_quad); every lane returns the result.
static __device__ __noinline__ wpt_t te_to_weierstrass_quad(const xyzt_t &p, uint32_t mask) {
  return te_to_weierstrass_t<true>(p, mask);
}

// Jacobian -> affine with z in {0, 1}, all coordinates canonical in [0, q)
static __device__ __noinline__ wpt_t w_normalize(const wpt_t &p) {
  if (fq_is_zero(p.z)) {
    wpt_t r = w_infinity();
    r.x = fq_canon(r.x);
    r.y = fq_canon(r.y);
    return r;
  }
  const fq_t zi = fq_inv_vartime(p.z);
  const fq_t zi2 = fq_sqr_ool(zi);
  wpt_t r;
  r.x = fq_canon(fq_mul_ool(p.x, zi2));
  r.y = fq_canon(fq_mul_ool(fq_mul_ool(p.y, zi2), zi));
  r.z = fq_canon(fq_one());
  return r;
}
