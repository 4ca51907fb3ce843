// The MSM pipeline of one pass (one or many MSMs sharing one sort), all on the device:
//
//   1. k_count     signed c-bit digits of every scalar, histogram of (MSM, window, |digit|) keys;
//                  stages each block's entries by key range (and uploads host scalars)
//   2. k_scan_*    exclusive scans -> bucket offsets in the sorted array and task offsets
//   3. k_scatter_staged  counting-sort scatter of (base index | sign) into bucket order, one
//                  launch per key range (k_scatter: the same from the scalars, for passes
//                  without a stage)
//   4. k_tasks     split every bucket into runs of <= seg_len entries (load balance under skew)
//   5. k_accumulate persistent: each thread sums one run of bases into a partial bucket sum
//                  (the run's first base taken as is, then a 7-product mixed add per base)
//   6. k_merge_*   buckets split over several runs: sum of their partials (a thread, a warp or
//                  a block per bucket, by the number of runs)
//   7. k_reduce1   per run of buckets: running sum R and triangle sum A (pippenger.h:25-33),
//                  by the dedicated addition (8 products; the unified one where it fails)
//   8. k_reduce2/3 combine runs into groups, groups into window sums (k_reduce3_small: one
//                  quad per window of few groups), by quad additions of two product latencies
//   9. k_final     per MSM: Horner window combine (pippenger.h:36-45), map back to affine
//                  Weierstrass, add the bases without a twisted-Edwards image
//                  (driver.cpp:349-372), write g1_projective_t (bls12_377_g1.h:427-439, 667-690)
//
// Every launch has a shape fixed by the host plan; data-dependent sizes (tasks, heavy buckets)
// are read from device counters, so a pass can be captured in a CUDA graph and replayed.
#include "engine.h"
#include "curve.cuh"

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ void set_error(uint32_t *counters, uint32_t code, uint32_t info) {
  if (atomicCAS(&counters[CNT_ERROR], 0u, code) == 0u) counters[CNT_ERROR_INFO] = info;
}

__device__ __forceinline__ uint32_t find_job(const JobDesc *jobs, uint32_t n_jobs, uint64_t g) {
  uint32_t lo = 0, hi = n_jobs;  // last job with point_begin <= g
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (jobs[mid].point_begin <= g) lo = mid; else hi = mid;
  }
  return lo;
}

// The scalar bits not yet consumed, least significant first, masked to 253 bits on load.
// Windows are taken in order: each take shifts the whole scalar right by c (funnel shifts in
// registers; a runtime word index into the scalar would compile to select chains).
struct ScalarBits {
  uint32_t w[8];
};

__device__ __forceinline__ ScalarBits scalar_bits(const uint4 &a, const uint4 &b) {
  ScalarBits s;
  s.w[0] = a.x; s.w[1] = a.y; s.w[2] = a.z; s.w[3] = a.w;
  s.w[4] = b.x; s.w[5] = b.y; s.w[6] = b.z; s.w[7] = b.w & 0x1fffffffu;
  return s;
}

__device__ __forceinline__ ScalarBits load_scalar(const uint4 *p) { return scalar_bits(p[0], p[1]); }

// the next c bits (1 <= c <= 31); bits past 253 read as zero
__device__ __forceinline__ uint32_t take_bits(ScalarBits &s, uint32_t c) {
  const uint32_t v = s.w[0] & ((1u << c) - 1u);
#pragma unroll
  for (int k = 0; k < 7; k++) s.w[k] = __funnelshift_r(s.w[k], s.w[k + 1], c);
  s.w[7] >>= c;
  return v;
}

// Digit of window w, the windows taken in order from 0, given the running carry
// (hardcaml/test/top/utils.ml:243-288): slice + carry; below the top window a value >= 2^(c-1)
// becomes value - 2^c with carry 1.  Returns the signed digit and updates carry.  Unsigned mode
// returns the plain slice.
__device__ __forceinline__ int32_t next_digit(ScalarBits &s, const JobDesc &jd, uint32_t w,
                                              uint32_t &carry) {
  int32_t d = (int32_t)(take_bits(s, jd.c) + carry);
  if (!jd.signed_digits) return d;
  if (w + 1 < jd.nwin && d >= (int32_t)(1u << (jd.c - 1))) {
    d -= (int32_t)(1u << jd.c);
    carry = 1;
  } else {
    carry = 0;
  }
  return d;
}

// Global bucket id of digit magnitude `mag` in window w.  Fixed-base jobs keep one bucket array
// for all windows: their entries point at the window's own table of 2^(c w) P_i instead.
__device__ __forceinline__ uint32_t bucket_key(const JobDesc &jd, uint32_t w, uint32_t mag) {
  return jd.bucket_begin + (jd.fixed ? 0u : w * jd.nb) + (mag - 1u);
}

// The part of a digit's magnitude above its window's bucket range.  Only the top window of a
// signed layout can have one: its range is capped at the largest top digit of a scalar below r,
// and a 253-bit scalar at or above r can exceed it.  That digit becomes two entries of the same
// window, nb_top and the excess (at most nb_top: the cap is at least half of 2^c_top).
__device__ __forceinline__ uint32_t top_excess(const JobDesc &jd, uint32_t w, uint32_t mag) {
  return (w + 1 == jd.nwin && mag > jd.nb_top) ? mag - jd.nb_top : 0u;
}

// ---------------------------------------------------------------------------------------------
// 1. histogram
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void count_key(const PassBuffers &pb, uint32_t key, uint32_t *sh_bins) {
  if (sh_bins) atomicAdd(&sh_bins[key >> pb.bin_shift], 1u);
  if (pb.stage_rank) return;  // the bucket counts come with the ranks in stage_digits
  // a warp whose active lanes all hit one bucket (e.g. equal scalars) adds once; otherwise
  // every lane adds on its own (distinct buckets for uniform scalars)
  const uint32_t active = __activemask();
  const int leader = __ffs(active) - 1;
  const uint32_t k0 = __shfl_sync(active, key, leader);
  if (__all_sync(active, key == k0)) {
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&pb.count[key], (uint32_t)__popc(active));
  } else {
    atomicAdd(&pb.count[key], 1u);
  }
}

// Round 1: the global bucket histogram (and, for the staged sort, the block's key-range counts).
__device__ __forceinline__ void count_digits(const PassBuffers &pb, const JobDesc &jd, ScalarBits s,
                                             uint32_t *sh_bins) {
  uint32_t carry = 0;
  for (uint32_t w = 0; w < jd.nwin; w++) {
    const int32_t d = next_digit(s, jd, w, carry);
    if (d == 0) continue;
    const uint32_t mag = (uint32_t)abs(d);
    const uint32_t extra = top_excess(jd, w, mag);
    count_key(pb, bucket_key(jd, w, mag - extra), sh_bins);
    if (extra) count_key(pb, bucket_key(jd, w, extra), sh_bins);
  }
}

// Round 2 of the staged sort: one entry into the block's chunk, at the cursor of its key range.
__device__ __forceinline__ void stage_key(const PassBuffers &pb, uint32_t key, uint32_t val,
                                          uint32_t *sh_cur, uint2 *chunk, uint32_t *ranks) {
  uint32_t rank = 0;
  if (ranks) {
    // the bucket count's old value is the entry's rank in its bucket (one atomic per warp
    // when its active lanes share the bucket)
    const uint32_t active = __activemask();
    const int leader = __ffs(active) - 1;
    const int lane = threadIdx.x & 31;
    const uint32_t k0 = __shfl_sync(active, key, leader);
    if (__all_sync(active, key == k0)) {
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(&pb.count[key], (uint32_t)__popc(active));
      rank = __shfl_sync(active, base, leader) + __popc(active & ((1u << lane) - 1u));
    } else {
      rank = atomicAdd(&pb.count[key], 1u);
    }
  }
  const uint32_t pos = atomicAdd(&sh_cur[key >> pb.bin_shift], 1u);
  if (pos < pb.stage_cap) {
    chunk[pos] = make_uint2(key, val);
    if (ranks) ranks[pos] = rank;
  } else {
    set_error(pb.counters, 6, pos);
  }
}

// The entries of one point, in window order.
__device__ __forceinline__ void stage_digits(const PassBuffers &pb, const JobDesc &jd, ScalarBits s,
                                             uint64_t bidx, uint32_t *sh_cur, uint2 *chunk,
                                             uint32_t *ranks) {
  uint32_t carry = 0;
  for (uint32_t w = 0; w < jd.nwin; w++) {
    const int32_t d = next_digit(s, jd, w, carry);
    if (d == 0) continue;
    const uint32_t mag = (uint32_t)abs(d);
    const uint32_t extra = top_excess(jd, w, mag);
    const uint64_t tidx = jd.tab_base + (jd.fixed ? (uint64_t)w * jd.fb_stride : 0) + bidx;
    const uint32_t val = (uint32_t)tidx | (d < 0 ? 0x80000000u : 0u);
    stage_key(pb, bucket_key(jd, w, mag - extra), val, sh_cur, chunk, ranks);
    if (extra) stage_key(pb, bucket_key(jd, w, extra), val, sh_cur, chunk, ranks);
  }
}

// One thread per point, 256 points per block.  With host_scalars set, the kernel also uploads
// the pass's scalars; with stage set, the block also writes its entries to its chunk of the
// stage, grouped by key range.
__global__ void __launch_bounds__(MSM_POINTS_PER_CHUNK) k_count(PassBuffers pb, uint64_t g_begin,
                                                                uint64_t g_end) {
  __shared__ uint32_t sh_cur[MSM_MAX_BINS];
  const uint32_t tid = threadIdx.x;
  const bool staged = pb.stage != nullptr;
  const uint64_t g = g_begin + (uint64_t)blockIdx.x * blockDim.x + tid;
  bool ok = false;
  JobDesc jd{};
  ScalarBits s{};
  uint64_t bidx = 0;
  if (g < g_end && g < pb.n_points) {
    jd = pb.jobs[find_job(pb.jobs, pb.n_jobs, g)];
    const uint64_t i = g - jd.point_begin;
    const uint64_t si = 2 * (jd.scalar_off + i);
    uint4 a, b;
    if (pb.host_scalars) {
      // fused upload: every scalar of the pass (bases without a bucket entry included, k_final
      // reads theirs) goes from host memory to the device copy the later kernels read
      a = pb.host_scalars[si];
      b = pb.host_scalars[si + 1];
      uint4 *dst = const_cast<uint4 *>(pb.scalars) + si;
      dst[0] = a;
      dst[1] = b;
    } else {
      a = pb.scalars[si];
      b = pb.scalars[si + 1];
    }
    bidx = jd.base_off + i;
    ok = pb.flags[bidx] == BASE_OK;
    s = scalar_bits(a, b);
  }
  if (staged) {
    if (tid < MSM_MAX_BINS) sh_cur[tid] = 0;
    __syncthreads();
  }
  if (ok) count_digits(pb, jd, s, staged ? sh_cur : nullptr);
  if (!staged) return;
  __syncthreads();
  const uint64_t chunk = g_begin / MSM_POINTS_PER_CHUNK + blockIdx.x;
  if (tid == 0) {  // key-range counts -> starts (n_bins <= 32)
    uint32_t *bo = pb.blk_off + chunk * (pb.n_bins + 1);
    uint32_t acc = 0;
    for (uint32_t r = 0; r < pb.n_bins; r++) {
      const uint32_t c = sh_cur[r];
      sh_cur[r] = acc;
      bo[r] = acc;
      acc += c;
    }
    bo[pb.n_bins] = acc;
  }
  __syncthreads();
  if (ok)
    stage_digits(pb, jd, s, bidx, sh_cur, pb.stage + chunk * pb.stage_cap,
                 pb.stage_rank ? pb.stage_rank + chunk * pb.stage_cap : nullptr);
}

// ---------------------------------------------------------------------------------------------
// 2. scans of (count, ceil(count / seg_len))
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint2 warp_incl_scan2(uint2 v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t a = __shfl_up_sync(0xffffffffu, v.x, o);
    const uint32_t b = __shfl_up_sync(0xffffffffu, v.y, o);
    if ((int)(threadIdx.x & 31) >= o) { v.x += a; v.y += b; }
  }
  return v;
}

// block-wide exclusive scan of pairs; returns this thread's exclusive prefix and the block total
__device__ __forceinline__ uint2 block_excl_scan2(uint2 v, uint2 &total) {
  __shared__ uint2 warp_tot[32];
  __shared__ uint2 tot_sh;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const uint2 inc = warp_incl_scan2(v);
  if (lane == 31) warp_tot[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const uint2 t = lane < nw ? warp_tot[lane] : make_uint2(0, 0);
    const uint2 ti = warp_incl_scan2(t);
    if (lane < nw) warp_tot[lane] = make_uint2(ti.x - t.x, ti.y - t.y);
    if (lane == 31) tot_sh = ti;
  }
  __syncthreads();
  total = tot_sh;
  const uint2 base = warp_tot[wid];
  __syncthreads();  // the shared words are reused by the next call
  return make_uint2(base.x + inc.x - v.x, base.y + inc.y - v.y);
}

__device__ __forceinline__ uint32_t ntask_of(uint32_t cnt, uint32_t seg_len) {
  return (cnt + seg_len - 1) / seg_len;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(PassBuffers pb) {
  const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint2 v = make_uint2(0, 0);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < pb.n_buckets) {
      const uint32_t c = pb.count[base + k];
      v.x += c;
      v.y += ntask_of(c, pb.seg_len);
    }
  }
  uint2 total;
  block_excl_scan2(v, total);
  if (threadIdx.x == 0) {
    pb.scan_tmp[2 * blockIdx.x] = total.x;
    pb.scan_tmp[2 * blockIdx.x + 1] = total.y;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(PassBuffers pb, uint32_t nblk) {
  // one block: exclusive scan of the per-block totals, in chunks of kScanThreads
  __shared__ uint2 carry_sh;
  if (threadIdx.x == 0) carry_sh = make_uint2(0, 0);
  __syncthreads();
  for (uint32_t c0 = 0; c0 < nblk; c0 += kScanThreads) {
    const uint32_t i = c0 + threadIdx.x;
    const uint2 v = i < nblk ? make_uint2(pb.scan_tmp[2 * i], pb.scan_tmp[2 * i + 1]) : make_uint2(0, 0);
    uint2 total;
    const uint2 ex = block_excl_scan2(v, total);
    const uint2 cr = carry_sh;
    if (i < nblk) {
      pb.scan_tmp[2 * i] = cr.x + ex.x;
      pb.scan_tmp[2 * i + 1] = cr.y + ex.y;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry_sh = make_uint2(cr.x + total.x, cr.y + total.y);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const uint2 t = carry_sh;
    if ((uint64_t)t.x > pb.max_entries) set_error(pb.counters, 1, t.x);
    if (t.y > pb.max_tasks) set_error(pb.counters, 2, t.y);
    pb.counters[CNT_TASKS] = min(t.y, pb.max_tasks);
    pb.counters[CNT_ENTRIES] = t.x;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(PassBuffers pb) {
  const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint32_t c[kScanItems];
  uint2 v = make_uint2(0, 0);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    c[k] = base + k < pb.n_buckets ? pb.count[base + k] : 0u;
    v.x += c[k];
    v.y += ntask_of(c[k], pb.seg_len);
  }
  uint2 total;
  uint2 ex = block_excl_scan2(v, total);
  ex.x += pb.scan_tmp[2 * blockIdx.x];
  ex.y += pb.scan_tmp[2 * blockIdx.x + 1];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < pb.n_buckets) {
      pb.offset[base + k] = ex.x;
      pb.fill[base + k] = ex.x;  // the scatter's slot cursor starts at the bucket's offset
      pb.taskoff[base + k] = ex.y;
    }
    ex.x += c[k];
    ex.y += ntask_of(c[k], pb.seg_len);
  }
}

// ---------------------------------------------------------------------------------------------
// 3. scatter into bucket order, one launch per range of bucket keys [key_lo, key_hi).  A range's
//    slice of the sorted array is a few hundred MB, so its random 4-byte stores mostly merge in
//    L2 instead of each costing a DRAM read-modify-write of a whole sector; every launch
//    recomputes the digits and keeps only the entries in its range.
// ---------------------------------------------------------------------------------------------
__global__ void k_scatter(PassBuffers pb, uint32_t key_lo, uint32_t key_hi) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= pb.n_points) return;
  if (pb.counters[CNT_ERROR]) return;
  const uint32_t j = find_job(pb.jobs, pb.n_jobs, g);
  const JobDesc jd = pb.jobs[j];
  const uint64_t i = g - jd.point_begin;
  const uint64_t bidx = jd.base_off + i;
  if (pb.flags[bidx] != BASE_OK) return;
  ScalarBits s = load_scalar(pb.scalars + 2 * (jd.scalar_off + i));
  const int lane = threadIdx.x & 31;
  uint32_t carry = 0;
  // four windows per step: their slot atomics are independent, so the four round trips
  // overlap instead of running one after another.  fill[key] starts at the bucket's offset in
  // the sorted array, so the atomic returns the entry's position directly.
  uint32_t extra_key = 0, extra_val = 0;  // a split top digit's second entry (see top_excess)
  bool extra = false;
#pragma unroll 1
  for (uint32_t w0 = 0; w0 < jd.nwin; w0 += 4) {
    uint32_t key[4], val[4], pos[4];
    bool ok[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint32_t w = w0 + k;
      ok[k] = false;
      key[k] = 0;
      val[k] = 0;
      if (w < jd.nwin) {
        const int32_t d = next_digit(s, jd, w, carry);
        if (d != 0) {
          const uint32_t mag = (uint32_t)abs(d);
          const uint32_t ex = top_excess(jd, w, mag);
          key[k] = bucket_key(jd, w, mag - ex);
          ok[k] = key[k] >= key_lo && key[k] < key_hi;
          const uint64_t tidx = jd.tab_base + (jd.fixed ? (uint64_t)w * jd.fb_stride : 0) + bidx;
          val[k] = (uint32_t)tidx | (d < 0 ? 0x80000000u : 0u);
          if (ex) {
            extra_key = bucket_key(jd, w, ex);
            extra_val = val[k];
            extra = extra_key >= key_lo && extra_key < key_hi;
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      pos[k] = 0;
      if (ok[k]) {
        const uint32_t active = __activemask();
        const int leader = __ffs(active) - 1;
        const uint32_t k0 = __shfl_sync(active, key[k], leader);
        if (__all_sync(active, key[k] == k0)) {  // one bucket for the whole warp: one atomic
          uint32_t bp = 0;
          if (lane == leader) bp = atomicAdd(&pb.fill[key[k]], (uint32_t)__popc(active));
          pos[k] = __shfl_sync(active, bp, leader) + __popc(active & ((1u << lane) - 1u));
        } else {
          pos[k] = atomicAdd(&pb.fill[key[k]], 1u);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (!ok[k]) continue;
      if (pos[k] < pb.max_entries) {
        pb.vals[pos[k]] = val[k];
      } else {
        set_error(pb.counters, 3, pos[k]);
      }
    }
  }
  if (extra) {
    const uint32_t p = atomicAdd(&pb.fill[extra_key], 1u);
    if (p < pb.max_entries) {
      pb.vals[p] = extra_val;
    } else {
      set_error(pb.counters, 3, p);
    }
  }
}

// Staged sort: the entries of key range `bin`, chunk by chunk (one block per histogram block),
// each to the position its bucket's slot cursor returns.  The range's slice of the sorted array
// stays in L2 while the launch runs.
__global__ void __launch_bounds__(256) k_scatter_staged(PassBuffers pb, uint32_t bin) {
  if (pb.counters[CNT_ERROR]) return;
  const uint64_t chunk = blockIdx.x;
  const uint32_t *bo = pb.blk_off + chunk * (pb.n_bins + 1);
  const uint32_t lo = bo[bin], hi = min(bo[bin + 1], pb.stage_cap);
  const uint2 *st = pb.stage + chunk * pb.stage_cap;
  const uint32_t *rk = pb.stage_rank ? pb.stage_rank + chunk * pb.stage_cap : nullptr;
  const int lane = threadIdx.x & 31;
  for (uint32_t e = lo + threadIdx.x; e < hi; e += blockDim.x) {
    const uint2 kv = st[e];
    if (kv.x >= pb.n_buckets) {  // cannot happen for a consistent stage; never write out of bounds
      set_error(pb.counters, 7, kv.x);
      continue;
    }
    if (rk) {  // position known from the rank: no atomic
      const uint32_t p = pb.offset[kv.x] + rk[e];
      if (p < pb.max_entries) {
        pb.vals[p] = kv.y;
      } else {
        set_error(pb.counters, 3, p);
      }
      continue;
    }
    uint32_t pos;
    const uint32_t active = __activemask();
    const int leader = __ffs(active) - 1;
    const uint32_t k0 = __shfl_sync(active, kv.x, leader);
    if (__all_sync(active, kv.x == k0)) {  // one bucket for the whole warp: one atomic
      uint32_t bp = 0;
      if (lane == leader) bp = atomicAdd(&pb.fill[kv.x], (uint32_t)__popc(active));
      pos = __shfl_sync(active, bp, leader) + __popc(active & ((1u << lane) - 1u));
    } else {
      pos = atomicAdd(&pb.fill[kv.x], 1u);
    }
    if (pos < pb.max_entries) {
      pb.vals[pos] = kv.y;
    } else {
      set_error(pb.counters, 3, pos);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// 4. tasks: runs of <= seg_len entries, and a processing order with the longest runs first.
//    Lanes of one warp then get runs of (almost) equal length, so no lane idles while another
//    finishes a longer bucket; long runs also start first, which evens out the tail.
// ---------------------------------------------------------------------------------------------
__global__ void k_len_hist(PassBuffers pb) {
  extern __shared__ uint32_t h[];
  for (uint32_t i = threadIdx.x; i <= pb.seg_len; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < pb.n_buckets; b += gridDim.x * blockDim.x) {
    const uint32_t cnt = pb.count[b];
    if (!cnt) continue;
    const uint32_t nt = ntask_of(cnt, pb.seg_len);
    atomicAdd(&h[cnt - (nt - 1) * pb.seg_len], 1u);
    if (nt > 1) atomicAdd(&h[pb.seg_len], nt - 1);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i <= pb.seg_len; i += blockDim.x)
    if (h[i]) atomicAdd(&pb.len_hist[i], h[i]);
}

// cursor[len] = number of tasks longer than len (longest first); one thread, seg_len + 1 bins
__global__ void k_len_scan(PassBuffers pb) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t acc = 0;
  for (uint32_t l = pb.seg_len + 1; l-- > 0;) {
    const uint32_t c = pb.len_hist[l];
    pb.len_hist[l] = acc;
    acc += c;
  }
}

// One thread per bucket writes the bucket's runs and their slots in the processing order: the
// last run takes a slot in the bin of its length, the full runs of a split bucket a block of
// slots in the seg_len bin.  The block ranks its runs per bin in shared memory and reserves each
// bin's slots with one global atomic, so the few hot bin cursors (lengths cluster around the mean
// bucket load) see one atomic per block and bin.
__global__ void __launch_bounds__(256) k_tasks(PassBuffers pb) {
  extern __shared__ uint32_t sh_bins[];  // [seg_len + 1] counts, then [seg_len + 1] slot bases
  uint32_t *bin_cnt = sh_bins, *bin_base = sh_bins + pb.seg_len + 1;
  for (uint32_t i = threadIdx.x; i <= pb.seg_len; i += blockDim.x) bin_cnt[i] = 0;
  __syncthreads();
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  bool live = b < pb.n_buckets && !pb.counters[CNT_ERROR];
  uint32_t cnt = 0, nt = 0, t0 = 0, last = 0, r_last = 0, r_full = 0;
  if (live) {
    cnt = pb.count[b];
    live = cnt != 0;
  }
  if (live) {
    nt = ntask_of(cnt, pb.seg_len);
    t0 = pb.taskoff[b];
    if (t0 + nt > pb.max_tasks) {
      set_error(pb.counters, 4, t0 + nt);
      live = false;
    }
  }
  if (live) {
    const uint32_t off = pb.offset[b];
    for (uint32_t k = 0; k < nt; k++) {
      Task tk;
      tk.start = off + k * pb.seg_len;
      tk.len = min(pb.seg_len, cnt - k * pb.seg_len);
      tk.bucket = b;
      tk.pad = 0;
      pb.tasks[t0 + k] = tk;
    }
    last = cnt - (nt - 1) * pb.seg_len;
    r_last = atomicAdd(&bin_cnt[last], 1u);
    if (nt > 1) {
      r_full = atomicAdd(&bin_cnt[pb.seg_len], nt - 1);
      pb.heavy[atomicAdd(&pb.counters[CNT_HEAVY], 1u)] = b;
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i <= pb.seg_len; i += blockDim.x) {
    const uint32_t c = bin_cnt[i];
    bin_base[i] = c ? atomicAdd(&pb.len_hist[i], c) : 0u;
  }
  __syncthreads();
  if (live) {
    if (nt > 1) {
      const uint32_t base = bin_base[pb.seg_len] + r_full;
      for (uint32_t k = 0; k + 1 < nt; k++) pb.order[base + k] = t0 + k;
    }
    pb.order[bin_base[last] + r_last] = t0 + nt - 1;
  }
}

// ---------------------------------------------------------------------------------------------
// 5. bucket accumulation (persistent; warps fetch 32 tasks at a time)
// ---------------------------------------------------------------------------------------------
// The base of the current entry sits in shared memory, transposed (uint4 k of thread t at
// sh[k * 128 + t], no bank conflicts), and each operand is read right before its product.  With
// all nine words held in registers across the first three products the kernel spilled; staged,
// it fits 128 registers and runs 1.4% faster.
__device__ __forceinline__ fq_t staged_fq(const uint4 *sh, int part) {
  const uint4 a = sh[(part * 3 + 0) * 128 + threadIdx.x];
  const uint4 b = sh[(part * 3 + 1) * 128 + threadIdx.x];
  const uint4 c = sh[(part * 3 + 2) * 128 + threadIdx.x];
  fq_t r;
  r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
  r.v[4] = b.x; r.v[5] = b.y; r.v[6] = b.z; r.v[7] = b.w;
  r.v[8] = c.x; r.v[9] = c.y; r.v[10] = c.z; r.v[11] = c.w;
  return r;
}

// te_madd with the base ((y-x)/2, (y+x)/2, d x y) read from the staging slots.  Sums and
// differences that only feed products stay unreduced (below 4q; every product is again below
// 2q), and a negative digit swaps F and G instead of negating C: with C' = -C, Z - C' = Z + C
// and Z + C' = Z - C.  Measured in the mixed-add loop on GB300: 3.00e9 against 2.92e9 madd/s.
__device__ __forceinline__ xyzt_t te_madd_staged(const xyzt_t &p, const uint4 *sh, bool neg) {
  const fq_t A = fq_mul_nv(fq_sub_lazy(p.y, p.x), staged_fq(sh, neg ? 1 : 0));
  const fq_t B = fq_mul_nv(fq_add_lazy(p.y, p.x), staged_fq(sh, neg ? 0 : 1));
  const fq_t C = fq_mul_nv(p.t, staged_fq(sh, 2));
  const fq_t E = fq_sub_lazy(B, A);
  const fq_t H = fq_add_lazy(B, A);
  const fq_t Zm = fq_sub_lazy(p.z, C);
  const fq_t Zp = fq_add_lazy(p.z, C);
  const fq_t F = fq_select(neg, Zp, Zm);
  const fq_t G = fq_select(neg, Zm, Zp);
  xyzt_t r;
  r.x = fq_mul_nv(E, F);
  r.y = fq_mul_nv(G, H);
  r.t = fq_mul_nv(E, H);
  r.z = fq_mul_nv(F, G);
  return r;
}

// The first entry of a run starts the sum from the base itself instead of adding it to the
// identity: x = (y+x)/2 - (y-x)/2, y = (y+x)/2 + (y-x)/2 (x negated for a negative digit), z = 1,
// t = x y -- one product instead of seven.  The warp fetches its 32 runs together, so every lane
// is at its run's first entry in the same iteration and the branch is the same on every lane.
__device__ __forceinline__ xyzt_t te_from_staged(const uint4 *sh, bool neg) {
  const fq_t ymx = staged_fq(sh, 0), ypx = staged_fq(sh, 1);
  xyzt_t r;
  r.x = neg ? fq_sub(ymx, ypx) : fq_sub(ypx, ymx);
  r.y = fq_add(ypx, ymx);
  r.z = fq_one();
  r.t = fq_mul_nv(r.x, r.y);
  return r;
}

__global__ void __launch_bounds__(128, 4) k_accumulate(PassBuffers pb) {
  __shared__ uint4 sh[9 * 128];
  const int lane = threadIdx.x & 31;
  const uint32_t ntasks = pb.counters[CNT_TASKS];
  if (pb.counters[CNT_ERROR]) return;
  for (;;) {
    uint32_t first = 0;
    if (lane == 0) first = atomicAdd(&pb.counters[CNT_TASK_CURSOR], 32u);
    first = __shfl_sync(0xffffffffu, first, 0);
    if (first >= ntasks) break;
    const uint32_t i = first + lane;
    if (i < ntasks) {
      const uint32_t t = pb.order[i];
      const Task tk = pb.tasks[t];
      xyzt_t acc = xyzt_identity();
      for (uint32_t e = 0; e < tk.len; e++) {
        const uint32_t v = pb.vals[tk.start + e];
        const uint32_t idx = v & 0x7fffffffu;
        if (idx >= pb.n_bases) {  // cannot happen for a consistent sort; never read out of bounds
          set_error(pb.counters, 5, idx);
          break;
        }
        const uint4 *src = pb.bases + (size_t)idx * 9;
#pragma unroll
        for (int k = 0; k < 9; k++) sh[k * 128 + threadIdx.x] = src[k];
        const bool neg = (v >> 31) != 0;
        if (e == 0) acc = te_from_staged(sh, neg);
        else acc = te_madd_staged(acc, sh, neg);
      }
      xyzt_store(pb.partials + (size_t)t * 12, acc);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// 6. buckets spread over several tasks: one warp sums the partials
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ xyzt_t shfl_down_xyzt(const xyzt_t &p, int off) {
  xyzt_t r;
#pragma unroll
  for (int k = 0; k < FQ_LIMBS; k++) {
    r.x.v[k] = __shfl_down_sync(0xffffffffu, p.x.v[k], off);
    r.y.v[k] = __shfl_down_sync(0xffffffffu, p.y.v[k], off);
    r.z.v[k] = __shfl_down_sync(0xffffffffu, p.z.v[k], off);
    r.t.v[k] = __shfl_down_sync(0xffffffffu, p.t.v[k], off);
  }
  return r;
}

__device__ __forceinline__ xyzt_t warp_sum_xyzt(xyzt_t acc) {
#pragma unroll 1
  for (int off = 16; off > 0; off >>= 1) {
    const xyzt_t o = shfl_down_xyzt(acc, off);
    acc = te_add_ool(acc, o);  // lanes >= 32 - off add garbage-free copies; only lane 0 is used
  }
  return acc;
}

// Split buckets of at most kMergeThreadMax runs (the common case: a few more entries than
// seg_len) are summed by one thread each, larger ones by a warp (k_merge) or a block
// (k_merge_big).  Lanes of a warp
// execute one instruction stream, so a warp's tree over three partials costs as much as the
// thread version summing 32 such buckets.
constexpr uint32_t kMergeThreadMax = 16;

__global__ void __launch_bounds__(128) k_merge_small(PassBuffers pb) {
  if (pb.counters[CNT_ERROR]) return;
  const uint32_t nheavy = pb.counters[CNT_HEAVY];
  for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nheavy; h += gridDim.x * blockDim.x) {
    const uint32_t b = pb.heavy[h];
    const uint32_t nt = ntask_of(pb.count[b], pb.seg_len);
    if (nt > kMergeThreadMax) continue;
    const uint32_t t0 = pb.taskoff[b];
    xyzt_t acc;
    xyzt_load(acc, pb.partials + (size_t)t0 * 12);
    for (uint32_t k = 1; k < nt; k++) {
      xyzt_t p;
      xyzt_load(p, pb.partials + (size_t)(t0 + k) * 12);
      acc = te_add_fast_ool(acc, p);  // partials of disjoint runs: the dedicated formula
    }
    xyzt_store(pb.partials + (size_t)t0 * 12, acc);
  }
}

// Buckets of more than kMergeWarpMax runs (a value repeated across many scalars) get a block of
// 64 quads each (k_merge_big, after the quad arithmetic below).
constexpr uint32_t kMergeWarpMax = 64;

__global__ void __launch_bounds__(256) k_merge(PassBuffers pb) {
  if (pb.counters[CNT_ERROR]) return;
  const int lane = threadIdx.x & 31;
  const uint32_t nheavy = pb.counters[CNT_HEAVY];
  const uint32_t warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t h = warp_global; h < nheavy; h += nwarps) {
    const uint32_t b = pb.heavy[h];
    const uint32_t nt = ntask_of(pb.count[b], pb.seg_len);
    if (nt <= kMergeThreadMax || nt > kMergeWarpMax) continue;  // k_merge_small's, k_merge_big's
    const uint32_t t0 = pb.taskoff[b];
    xyzt_t acc = xyzt_identity();
    for (uint32_t k = lane; k < nt; k += 32) {
      xyzt_t p;
      xyzt_load(p, pb.partials + (size_t)(t0 + k) * 12);
      acc = te_add_ool(acc, p);
    }
    acc = warp_sum_xyzt(acc);
    __syncwarp();
    if (lane == 0) xyzt_store(pb.partials + (size_t)t0 * 12, acc);
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
// 7-8. bucket reduction: window sum = sum_b (b + 1) B_b over the window's buckets (digit
//    magnitude b + 1), the triangle sum of pippenger.h:25-33 computed in three parallel levels.
//    A run of items summarised as (R, A) -- R = sum of the items' point sums, A = sum of
//    (local position + 1) * point -- combines exactly: a run of runs has
//    A = sum_i A_i + len * sum_i i R_i, and len is a power of two (doublings only).
//    level 1: runs of 2^red_len_log2 buckets, one thread each (throughput part);
//    level 2: groups of 2^grp_len_log2 level-1 runs, one block each;
//    level 3: the groups of one window, one block per window.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t find_win(const WinDesc *wins, uint32_t n_wins, uint32_t s) {
  uint32_t lo = 0, hi = n_wins;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (wins[mid].seg_begin <= s) lo = mid; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ uint32_t find_win_grp(const WinDesc *wins, uint32_t n_wins, uint32_t g) {
  uint32_t lo = 0, hi = n_wins;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (wins[mid].grp_begin <= g) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(128) k_reduce1(PassBuffers pb) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= pb.n_segs) return;
  if (pb.counters[CNT_ERROR]) return;
  const WinDesc wd = pb.wins[find_win(pb.wins, pb.n_wins, s)];
  const uint32_t L = 1u << pb.red_len_log2;
  const uint32_t lo = (s - wd.seg_begin) * L;
  const uint32_t hi = min(lo + L, wd.nb);
  xyzt_t R = xyzt_identity(), A = xyzt_identity();
  bool r_live = false, a_live = false;
  bool a_is_r = false;  // A was set to R at the first live bucket and R has not changed since
#pragma unroll 1
  for (uint32_t b = hi; b-- > lo;) {
    const uint32_t gb = wd.bucket_begin + b;
    if (pb.count[gb] != 0) {
      xyzt_t B;
      xyzt_load(B, pb.partials + (size_t)pb.taskoff[gb] * 12);
      R = r_live ? te_add_fast(R, B) : B;
      r_live = true;
      a_is_r = false;
    }
    if (r_live) {
      if (!a_live) {
        A = R;
        a_live = true;
        a_is_r = true;
      } else {
        // with A = R (an empty bucket right after the first live one) A + R is a doubling, the
        // dedicated formula's failure; a warp holding such a lane takes the unified formula for
        // this step instead of running both
        if (__any_sync(__activemask(), a_is_r)) A = te_add(A, R);
        else A = te_add_fast(A, R);
        a_is_r = false;
      }
    }
  }
  xyzt_store(pb.seg_out + (size_t)s * 24, R);
  xyzt_store(pb.seg_out + (size_t)s * 24 + 12, A);
}

// ---- 4-lane cooperative point operations on distributed points ----
// The four lanes of a quad (lanes 4k..4k+3 of a warp) hold one extended point, one coordinate
// each: lane 0 X, lane 1 T, lane 2 Y, lane 3 Z.  Each lane computes one of the four independent
// products of a step and the lanes exchange what the next step needs, so a doubling costs two
// product latencies instead of eight and an addition three instead of nine, and a point takes 12
// registers per lane.  `mask` names the lanes executing the call (whole quads).
__device__ __forceinline__ int dq_lane() { return (int)(threadIdx.x & 3); }

// offset (uint4) of this lane's coordinate in an (X, Y, Z, T) record of 12 uint4
__device__ __forceinline__ int dq_off() {
  const int l = dq_lane();
  return l == 0 ? 0 : l == 1 ? 9 : l == 2 ? 3 : 6;
}
__device__ __forceinline__ fq_t dq_load(const uint4 *p) {
  fq_t r;
  fq_load(r, p + dq_off());
  return r;
}
__device__ __forceinline__ void dq_store(uint4 *p, const fq_t &v) { fq_store(p + dq_off(), v); }
__device__ __forceinline__ fq_t dq_identity() { return dq_lane() >= 2 ? fq_one() : fq_zero(); }

// the value of lane (this lane ^ x) of the quad
__device__ __forceinline__ fq_t dq_xchg(const fq_t &a, int x, uint32_t mask) {
  fq_t r;
#pragma unroll
  for (int k = 0; k < FQ_LIMBS; k++) r.v[k] = __shfl_xor_sync(mask, a.v[k], x, 4);
  return r;
}
__device__ __forceinline__ fq_t pick4(int l, const fq_t &a, const fq_t &b, const fq_t &c, const fq_t &d) {
  return fq_select(l == 0, a, fq_select(l == 1, b, fq_select(l == 2, c, d)));
}

// dbl-2008-hwcd, a = -1: A = X^2, B = Y^2, C = 2 Z^2, S = (X + Y)^2, E = S - A - B, G = B - A,
// F = G - C, H = -A - B; X3 = E F, Y3 = G H, T3 = E H, Z3 = F G
static __device__ __noinline__ fq_t dq_dbl(fq_t p, uint32_t mask) {
  const int l = dq_lane();
  const fq_t o1 = dq_xchg(p, 1, mask), o3 = dq_xchg(p, 3, mask);  // lane 1 gets X and Y
  const fq_t sq = fq_sqr(l == 1 ? fq_add(o1, o3) : p);              // A, S, B, Z^2 on lanes 0..3
  const fq_t s1 = dq_xchg(sq, 1, mask), s2 = dq_xchg(sq, 2, mask), s3 = dq_xchg(sq, 3, mask);
  // the square of lane j sits in sq, s1, s2 or s3 as j ^ l is 0, 1, 2 or 3
  const fq_t A = pick4(l, sq, s1, s2, s3), S = pick4(l, s1, sq, s3, s2);
  const fq_t B = pick4(l, s2, s3, sq, s1), ZZ = pick4(l, s3, s2, s1, sq);
  const fq_t C = fq_dbl(ZZ);
  const fq_t E = fq_sub(fq_sub(S, A), B);
  const fq_t G = fq_sub(B, A);
  const fq_t F = fq_sub(G, C);
  const fq_t H = fq_sub(fq_neg(A), B);
  return fq_mul(pick4(l, E, E, G, F), pick4(l, F, H, H, G));
}

// add-2008-hwcd-3 with k = 2d (the same formula as te_add): three product latencies
static __device__ __noinline__ fq_t dq_add_unified(fq_t p, fq_t q, uint32_t mask) {
  const uint32_t kc[FQ_LIMBS] = BLS_TE_K;
  const int l = dq_lane();
  const fq_t po = dq_xchg(p, 2, mask), qo = dq_xchg(q, 2, mask);  // lanes 0, 2 swap X and Y
  // lane 0: (Y1 - X1)(Y2 - X2) = A, lane 2: (Y1 + X1)(Y2 + X2) = B, lane 1: T1 T2, lane 3: Z1 Z2
  const fq_t m1 = l == 0 ? fq_sub(po, p) : l == 2 ? fq_add(p, po) : p;
  const fq_t m2 = l == 0 ? fq_sub(qo, q) : l == 2 ? fq_add(q, qo) : q;
  fq_t pr = fq_mul(m1, m2);
  const fq_t kpr = fq_mul(pr, fq_from(kc));
  pr = l == 1 ? kpr : l == 3 ? fq_dbl(pr) : pr;  // lane 1: C = k T1 T2, lane 3: D = 2 Z1 Z2
  // pairs {0, 2} (A, B) and {1, 3} (C, D): E = B - A, H = B + A on lanes 0, 2; F = D - C,
  // G = D + C on lanes 1, 3
  const fq_t o = dq_xchg(pr, 2, mask);
  const fq_t lo = l < 2 ? pr : o, hi = l < 2 ? o : pr;
  const fq_t u = fq_sub(hi, lo), w = fq_add(hi, lo);
  const fq_t u1 = dq_xchg(u, 1, mask);  // lane 0 gets F, lane 1 gets E
  const fq_t w3 = dq_xchg(w, 3, mask);  // lane 1 gets H, lane 2 gets G
  // X3 = E F (lane 0), T3 = E H (lane 1), Y3 = G H (lane 2), Z3 = F G (lane 3)
  return fq_mul(pick4(l, u, u1, w3, u), pick4(l, u1, w3, w, w));
}

// this lane's coordinate equals the identity's as dq_identity() writes it, on all four lanes
__device__ __forceinline__ bool dq_is_identity_bits(const fq_t &p, uint32_t mask) {
  const uint32_t one[FQ_LIMBS] = BLS_ONE;
  const bool unit = dq_lane() >= 2;  // Y and Z are one, X and T zero
  uint32_t acc = 0;
#pragma unroll
  for (int j = 0; j < FQ_LIMBS; j++) acc |= p.v[j] ^ (unit ? one[j] : 0u);
  int ok = acc == 0;
  ok &= __shfl_xor_sync(mask, ok, 1, 4);
  ok &= __shfl_xor_sync(mask, ok, 2, 4);
  return ok != 0;
}

// p + q by the dedicated formula (curve.cuh te_add_fast): two product latencies instead of three.
//   lane 0: A = (Y1 - X1)(Y2 + X2), lane 2: B = (Y1 + X1)(Y2 - X2), lane 1: C = 2 Z1 T2,
//   lane 3: D = 2 T1 Z2; then X3 = E F (lane 0), T3 = E H (1), Y3 = G H (2), Z3 = F G (3).
// Where it gives Z3 = 0 the quad takes the unified formula; an operand that is the identity as
// dq_identity() writes it (padding, empty runs) returns the other one unchanged.  Every lane of
// `mask` calls this, and the branch to the unified formula is uniform over `mask`.
static __device__ __noinline__ fq_t dq_add(fq_t p, fq_t q, uint32_t mask) {
  const int l = dq_lane();
  const bool pid = dq_is_identity_bits(p, mask), qid = dq_is_identity_bits(q, mask);
  const fq_t po = dq_xchg(p, 2, mask), qo = dq_xchg(q, 2, mask);  // X <-> Y on 0, 2; T <-> Z on 1, 3
  const fq_t m1 = l == 0 ? fq_sub_lazy(po, p) : l == 2 ? fq_add_lazy(p, po) : po;
  const fq_t m2 = l == 0 ? fq_add_lazy(qo, q) : l == 2 ? fq_sub_lazy(q, qo) : q;
  fq_t pr = fq_mul(m1, m2);  // A, C' = Z1 T2, B, D' = T1 Z2 on lanes 0..3
  if (l & 1) pr = fq_dbl(pr);
  // pairs {0, 2}: F = B - A, G = B + A; pairs {1, 3}: H = D - C, E = D + C
  const fq_t o = dq_xchg(pr, 2, mask);
  const fq_t lo = l < 2 ? pr : o, hi = l < 2 ? o : pr;
  const fq_t u = fq_sub_lazy(hi, lo), w = fq_add_lazy(hi, lo);
  const fq_t u1 = dq_xchg(u, 1, mask), w1 = dq_xchg(w, 1, mask);
  fq_t r = fq_mul(pick4(l, w1, w, w, u1), pick4(l, u, u, u1, w1));
  const int zero = fq_is_zero(r);
  const bool need = __shfl_sync(mask, zero, 3, 4) != 0 && !pid && !qid;  // Z3 = 0 on lane 3
  if (__any_sync(mask, need)) {
    const fq_t ru = dq_add_unified(p, q, mask);
    if (need) r = ru;
  }
  return pid ? q : qid ? p : r;
}

constexpr int kRedThreads = 256;
constexpr uint32_t kRedQuads = kRedThreads / 4;
constexpr uint32_t kAllLanes = 0xffffffffu;

// Levels 2 and 3 are chains of dependent additions, so they run on quads: every quad of the
// block executes every addition (a quad with nothing to add adds the identity), which keeps the
// warps converged for the quad shuffles.  Blocks of NT threads (NT / 4 quads): with 128 each
// SMSP runs one warp, so a step of the block's trees is shorter, but each quad sums twice as
// many items in sequence as with 256.

// Three independent sums over the block's quads at once (sh holds 3 x NT / 4 points): at each
// tree level the 3 x stride additions are spread over the quads, so the three trees take
// log2(NT / 4) + 1 rounds of dependent additions instead of 3 log2(NT / 4).  Only warps holding an
// active quad add (whole warps, so their shuffles stay converged).  The sums are valid in quad 0.
template <int NT>
__device__ __forceinline__ void block_sum3(fq_t (&X)[3], uint4 *sh) {
  constexpr uint32_t Q = NT / 4;
  const uint32_t q = threadIdx.x >> 2;
  const uint32_t warp_q0 = (threadIdx.x >> 5) * 8;  // first quad of this warp
  for (int k = 0; k < 3; k++) dq_store(sh + (k * Q + q) * 12, X[k]);
  __syncthreads();
#pragma unroll 1
  for (uint32_t stride = Q / 2; stride > 0; stride >>= 1) {
#pragma unroll 1
    for (uint32_t u0 = 0; u0 < 3 * stride; u0 += Q) {
      const uint32_t u = u0 + q;  // item u: array u / stride, element u % stride
      const bool act = u < 3 * stride;
      const uint32_t slot = act ? (u / stride) * Q + u % stride : 0;
      fq_t a = dq_identity(), o = dq_identity();
      if (act) {
        a = dq_load(sh + slot * 12);
        o = dq_load(sh + (slot + stride) * 12);
      }
      if (u0 + warp_q0 < 3 * stride) a = dq_add(a, o, kAllLanes);
      __syncthreads();
      if (act) dq_store(sh + slot * 12, a);
      __syncthreads();
    }
  }
  for (int k = 0; k < 3; k++) X[k] = dq_load(sh + k * Q * 12);
}

// Inclusive suffix sums over the quads: quad u gets sum_{v >= u} X_v (Hillis-Steele).
template <int NT>
__device__ __forceinline__ fq_t block_suffix_scan(fq_t X, uint4 *sh) {
  constexpr uint32_t Q = NT / 4;
  const uint32_t q = threadIdx.x >> 2;
  dq_store(sh + q * 12, X);
  __syncthreads();
#pragma unroll 1
  for (uint32_t d = 1; d < Q; d <<= 1) {
    fq_t o = dq_identity();
    if (q + d < Q) o = dq_load(sh + (q + d) * 12);
    __syncthreads();
    X = dq_add(X, o, kAllLanes);
    dq_store(sh + q * 12, X);
    __syncthreads();
  }
  return X;
}

// Combine `cnt` runs (R, A) of 2^lin_log2 buckets each into one run (result in quad 0).
// Quad u takes runs [u per, u per + per) (per a power of two) and forms SA = sum A_i,
// RR = sum R_i and T = sum (i - u per) R_i.  Then
//   A = sum_u SA_u + 2^lin_log2 (sum_u T_u + per sum_u u RR_u),  R = sum_u RR_u,
// where sum_u u RR_u = sum_{u >= 1} (suffix sum of RR at u): one block scan and three block
// sums (run together), and only quad 0 doubles.
template <int NT>
__device__ void block_combine(const uint4 *items, uint32_t cnt, uint32_t lin_log2, bool want_r,
                              uint4 *sh, fq_t &A_out, fq_t &R_out) {
  constexpr uint32_t Q = NT / 4;
  const uint32_t q = threadIdx.x >> 2;
  uint32_t per = 1, per_log2 = 0;
  while (per * Q < cnt) {
    per <<= 1;
    per_log2++;
  }
  const uint32_t i0 = q * per;
  // the last run of the quad's share starts the sums (T = 0 R, RR = R, SA = A: no additions)
  fq_t SA = dq_identity(), T = dq_identity(), RR = dq_identity();
  if (i0 + per - 1 < cnt) {  // runs past cnt are the identity
    RR = dq_load(items + (size_t)(i0 + per - 1) * 24);
    SA = dq_load(items + (size_t)(i0 + per - 1) * 24 + 12);
  }
#pragma unroll 1
  for (uint32_t k = per - 1; k-- > 0;) {
    const uint32_t i = i0 + k;
    T = dq_add(T, RR, kAllLanes);
    fq_t R = dq_identity(), A = dq_identity();
    if (i < cnt) {
      R = dq_load(items + (size_t)i * 24);
      A = dq_load(items + (size_t)i * 24 + 12);
    }
    RR = dq_add(RR, R, kAllLanes);
    SA = dq_add(SA, A, kAllLanes);
  }
  const fq_t suf = block_suffix_scan<NT>(RR, sh);
  if (want_r && q == 0) R_out = suf;  // suffix at 0 is the total
  fq_t S[3] = {q ? suf : dq_identity(), T, SA};
  block_sum3<NT>(S, sh);
  if (q == 0) {  // lanes 0..3 of warp 0
    fq_t X = S[0];
#pragma unroll 1
    for (uint32_t k = 0; k < per_log2; k++) X = dq_dbl(X, 0xfu);
    X = dq_add(S[1], X, 0xfu);
#pragma unroll 1
    for (uint32_t k = 0; k < lin_log2; k++) X = dq_dbl(X, 0xfu);
    A_out = dq_add(X, S[2], 0xfu);
  }
}

template <int NT>
__global__ void __launch_bounds__(NT) k_reduce2(PassBuffers pb) {
  if (pb.counters[CNT_ERROR]) return;
  const uint32_t g = blockIdx.x;
  if (g >= pb.n_grps) return;
  __shared__ uint4 sh[3 * (NT / 4) * 12];
  const WinDesc wd = pb.wins[find_win_grp(pb.wins, pb.n_wins, g)];
  const uint32_t G = 1u << pb.grp_len_log2;
  const uint32_t first = (g - wd.grp_begin) * G;
  const uint32_t cnt = min(G, wd.nseg - first);
  fq_t A, R;
  block_combine<NT>(pb.seg_out + (size_t)(wd.seg_begin + first) * 24, cnt, pb.red_len_log2, true,
                    sh, A, R);
  if (threadIdx.x < 4) {  // quad 0: one coordinate per lane
    dq_store(pb.grp_out + (size_t)g * 24, R);
    dq_store(pb.grp_out + (size_t)g * 24 + 12, A);
  }
}

// Windows of at most kRed3SmallMax groups (windowed MSMs: 2^(c-1) buckets make a few groups)
// are combined by one quad each, in order:
//   A = sum_i A_i + 2^lin sum_i i R_i,  sum_i i R_i = sum_{i >= 1} (suffix sum of R at i),
// so hundreds of windows run side by side instead of one block each.  The quads of a warp work
// on different windows, so each shuffles under its own 4-lane mask.
constexpr uint32_t kRed3SmallMax = 16;

__global__ void __launch_bounds__(128) k_reduce3_small(PassBuffers pb) {
  if (pb.counters[CNT_ERROR]) return;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;  // one window per quad
  if (gw >= pb.n_wins) return;
  const WinDesc wd = pb.wins[gw];
  const uint32_t n = wd.ngrp;
  if (n == 0 || n > kRed3SmallMax) return;
  const uint32_t mask = 0xfu << (threadIdx.x & 28);
  const uint32_t lin = pb.red_len_log2 + pb.grp_len_log2;
  const uint4 *items = pb.grp_out + (size_t)wd.grp_begin * 24;
  fq_t RR = dq_load(items + (size_t)(n - 1) * 24);
  fq_t SA = dq_load(items + (size_t)(n - 1) * 24 + 12);
  fq_t T = n >= 2 ? RR : dq_identity();
#pragma unroll 1
  for (uint32_t i = n - 1; i-- > 0;) {
    const fq_t R = dq_load(items + (size_t)i * 24);
    const fq_t A = dq_load(items + (size_t)i * 24 + 12);
    SA = dq_add(SA, A, mask);
    if (i >= 1) {
      RR = dq_add(RR, R, mask);
      T = dq_add(T, RR, mask);
    }
  }
  fq_t out = SA;
  if (n >= 2) {
#pragma unroll 1
    for (uint32_t k = 0; k < lin; k++) T = dq_dbl(T, mask);
    out = dq_add(T, SA, mask);
  }
  dq_store(pb.win_sum + (size_t)gw * 12, out);
}

template <int NT>
__global__ void __launch_bounds__(NT) k_reduce3(PassBuffers pb) {
  if (pb.counters[CNT_ERROR]) return;
  const uint32_t gw = blockIdx.x;
  if (gw >= pb.n_wins) return;
  __shared__ uint4 sh[3 * (NT / 4) * 12];
  const WinDesc wd = pb.wins[gw];
  if (wd.ngrp <= kRed3SmallMax) return;  // k_reduce3_small's
  fq_t A, R;
  block_combine<NT>(pb.grp_out + (size_t)wd.grp_begin * 24, wd.ngrp,
                    pb.red_len_log2 + pb.grp_len_log2, false, sh, A, R);
  if (threadIdx.x < 4) dq_store(pb.win_sum + (size_t)gw * 12, A);
}

// Buckets split into more than kMergeWarpMax runs: a block of 64 quads per bucket, each quad
// summing a strided share of the partials, then a tree over the quads in shared memory.
__global__ void __launch_bounds__(kRedThreads) k_merge_big(PassBuffers pb) {
  if (pb.counters[CNT_ERROR]) return;
  __shared__ uint4 sh[kRedQuads * 12];
  const uint32_t q = threadIdx.x >> 2;
  const uint32_t warp_q0 = (threadIdx.x >> 5) * 8;  // first quad of this warp
  const uint32_t nheavy = pb.counters[CNT_HEAVY];
  for (uint32_t h = blockIdx.x; h < nheavy; h += gridDim.x) {
    const uint32_t b = pb.heavy[h];
    const uint32_t nt = ntask_of(pb.count[b], pb.seg_len);
    if (nt <= kMergeWarpMax) continue;  // block-uniform
    const uint32_t t0 = pb.taskoff[b];
    fq_t acc = dq_identity();
#pragma unroll 1
    for (uint32_t k0 = 0; k0 < nt; k0 += kRedQuads) {  // the same trip count for every quad
      const fq_t p = k0 + q < nt ? dq_load(pb.partials + (size_t)(t0 + k0 + q) * 12) : dq_identity();
      acc = dq_add(acc, p, kAllLanes);
    }
    dq_store(sh + q * 12, acc);
    __syncthreads();
#pragma unroll 1
    for (uint32_t stride = kRedQuads / 2; stride > 0; stride >>= 1) {
      fq_t o = dq_identity();
      if (q < stride) o = dq_load(sh + (q + stride) * 12);
      if (warp_q0 < stride) acc = dq_add(acc, o, kAllLanes);
      __syncthreads();
      if (q < stride) dq_store(sh + q * 12, acc);
      __syncthreads();
    }
    if (threadIdx.x < 4) dq_store(pb.partials + (size_t)t0 * 12, acc);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// 9. per MSM: window combine, Weierstrass map, special bases, ABI output
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void load_class_point(wpt_t &p, const uint4 *cp) {
  fq_load(p.x, cp);
  fq_load(p.y, cp + 3);
  p.z = fq_one();
}

__global__ void __launch_bounds__(128) k_final(PassBuffers pb) {
  const uint32_t j = blockIdx.x;
  if (j >= pb.n_jobs) return;
  const JobDesc jd = pb.jobs[j];
  __shared__ uint32_t cls_sum[8];
  if (threadIdx.x < 8) cls_sum[threadIdx.x] = 0;
  __syncthreads();
  // multiples of the special bases: every special base has order 2 or 4 (y = 0, or
  // Montgomery u = -1), so k * P = (k mod 4) * P
  for (uint32_t s = threadIdx.x; s < pb.n_special; s += blockDim.x) {
    const uint32_t idx = pb.special_idx[s];
    if (idx < jd.base_off || idx >= jd.base_off + jd.n) continue;
    const uint4 w0 = pb.scalars[2 * (jd.scalar_off + (idx - jd.base_off))];
    atomicAdd(&cls_sum[pb.special_cls[s] & 7], w0.x & 3u);
  }
  __syncthreads();
  if (threadIdx.x >= 4) return;  // lanes 0..3 of warp 0 run the combine together
  uint64_t *out = pb.results + (size_t)jd.result_slot * 18;
  if (pb.counters[CNT_ERROR]) {
    if (threadIdx.x == 0)
      for (int k = 0; k < 18; k++) out[k] = 0;
    return;
  }
  // Horner over the windows: acc = 2^c * acc + WS_w (pippenger.h:36-45 doubles per offset)
  fq_t dacc = dq_identity();
  if (jd.n > 0 && jd.nred > 0) {
    dacc = dq_load(pb.win_sum + (size_t)(jd.win_begin + jd.nred - 1) * 12);
#pragma unroll 1
    for (int w = (int)jd.nred - 2; w >= 0; w--) {
#pragma unroll 1
      for (uint32_t k = 0; k < jd.c; k++) dacc = dq_dbl(dacc, 0xfu);
      dacc = dq_add(dacc, dq_load(pb.win_sum + (size_t)(jd.win_begin + w) * 12), 0xfu);
    }
  }
  // gather the point on lane 0 (lane 1 holds T, lane 2 Y, lane 3 Z)
  xyzt_t acc;
  // every lane of the quad takes the whole point (lane 0 holds X, 1 T, 2 Y, 3 Z), and the four
  // share the inversion of the map to Weierstrass
#pragma unroll
  for (int k = 0; k < FQ_LIMBS; k++) {
    acc.x.v[k] = __shfl_sync(0xfu, dacc.v[k], 0, 4);
    acc.t.v[k] = __shfl_sync(0xfu, dacc.v[k], 1, 4);
    acc.y.v[k] = __shfl_sync(0xfu, dacc.v[k], 2, 4);
    acc.z.v[k] = __shfl_sync(0xfu, dacc.v[k], 3, 4);
  }
  wpt_t res = te_to_weierstrass_quad(acc, 0xfu);  // z is 1, or 0 for infinity
  if (threadIdx.x != 0) return;
  bool added = false;
  for (uint32_t c = 0; c < pb.n_classes && c < 8; c++) {
    const uint32_t m = cls_sum[c] & 3u;
    if (m == 0) continue;
    wpt_t p;
    load_class_point(p, pb.class_pts + c * 6);
    for (uint32_t k = 0; k < m; k++) res = w_add(res, p);
    added = true;
  }
  if (added) res = w_normalize(res);
  // g1_projective_t {x[6], y[6], z[6]}: (x*R, y*R, R) or arkworks' zero() (R, R, 0)
  const fq_t one = fq_canon(fq_one());
  const bool inf = fq_is_zero(res.z);
  const fq_t ox = inf ? one : fq_canon(res.x);
  const fq_t oy = inf ? one : fq_canon(res.y);
  const fq_t oz = inf ? fq_zero() : one;
  for (int k = 0; k < 6; k++) {
    out[k] = ((uint64_t)ox.v[2 * k + 1] << 32) | ox.v[2 * k];
    out[6 + k] = ((uint64_t)oy.v[2 * k + 1] << 32) | oy.v[2 * k];
    out[12 + k] = ((uint64_t)oz.v[2 * k + 1] << 32) | oz.v[2 * k];
  }
}

}  // namespace

// Scatter launches per pass: one per ~200 MB of sorted array, at most 8 (on GB300 the best
// counts measured were 4 for 2^24 points x 12 windows and 8 for 2^26 x 11 windows).
uint32_t msm_scatter_passes(uint64_t max_entries) {
  const uint64_t bytes = max_entries * 4, per = 200ull << 20;
  const uint64_t p = (bytes + per / 2) / per;
  return (uint32_t)(p < 1 ? 1 : p > 8 ? 8 : p);
}

// Key ranges of the staged sort, as a shift of the bucket key (ranges of 2^shift keys, at most
// MSM_MAX_BINS of them): one per ~150 MB of sorted array, and, for a scatter with slot cursors,
// no more than 2^19 keys per range while that keeps MSM_MAX_BINS ranges or fewer.  The keys a
// scatter launch touches bound its slot-cursor footprint: measured on GB300 at 2^24 points (4.9 M buckets), ranges of 2^20 keys
// (5 launches) took 3.86 ms, 2^19 (10) 2.42 ms and 2^18 (19) 2.49 ms; 2^26 points use 2^18.
// `ranges` > 0 asks for that many ranges instead (rounded to a shift).
uint32_t msm_bin_shift(uint32_t n_buckets, uint64_t max_entries, uint32_t ranges, bool cursors) {
  const uint64_t per = 150ull << 20;
  const uint64_t want = ranges ? ranges : (max_entries * 4 + per / 2) / per;
  const uint32_t target = (uint32_t)(want < 1 ? 1 : want > MSM_MAX_BINS ? MSM_MAX_BINS : want);
  uint32_t shift = 0;
  while (shift < 31 && (((uint64_t)n_buckets + (1ull << shift) - 1) >> shift) > target) shift++;
  if (!ranges && cursors)
    while (shift > 19 &&
           (((uint64_t)n_buckets + (1ull << (shift - 1)) - 1) >> (shift - 1)) <= MSM_MAX_BINS)
      shift--;
  return shift;
}

// Points per chunk of a chunked scalar upload: a multiple of the histogram block, so every block
// of a chunk's histogram launch is a whole chunk of the stage.
uint64_t msm_upload_chunk_points(uint64_t n_points, int nchunks) {
  const uint64_t per = (n_points + nchunks - 1) / nchunks;
  return (per + MSM_POINTS_PER_CHUNK - 1) / MSM_POINTS_PER_CHUNK * MSM_POINTS_PER_CHUNK;
}

size_t msm_scan_tmp_words(uint32_t n_buckets) {
  return 2ull * ((n_buckets + kScanBlock - 1) / kScanBlock) + 2;
}

cudaError_t msm_launch_pass(const PassBuffers &pb, int num_sms, cudaStream_t st, cudaEvent_t *ev,
                            const cudaEvent_t *chunk_ready, int nchunks, uint32_t *n_kernels) {
  cudaError_t e;
  uint32_t launched = 0;
  auto mark = [&](int k) {
    if (ev) cudaEventRecord(ev[k], st);
  };
  if ((e = cudaMemsetAsync(pb.count, 0, (size_t)pb.n_buckets * 4, st))) return e;
  if ((e = cudaMemsetAsync(pb.counters, 0, CNT_WORDS * 4, st))) return e;
  if ((e = cudaMemsetAsync(pb.len_hist, 0, (size_t)(pb.seg_len + 1) * 4, st))) return e;
  mark(0);
  const uint32_t pts_blocks = (uint32_t)((pb.n_points + 255) / 256);
  if (pb.n_points > 0) {
    if (chunk_ready && nchunks > 0) {
      // the scalars arrive in chunks on another stream: count each chunk as soon as it lands
      const uint64_t per = msm_upload_chunk_points(pb.n_points, nchunks);
      for (int c = 0; c < nchunks; c++) {
        const uint64_t g0 = (uint64_t)c * per, g1 = g0 + per < pb.n_points ? g0 + per : pb.n_points;
        if ((e = cudaStreamWaitEvent(st, chunk_ready[c], 0))) return e;
        if (g1 > g0) {
          k_count<<<(uint32_t)((g1 - g0 + 255) / 256), 256, 0, st>>>(pb, g0, g1);
          launched++;
        }
      }
    } else {
      k_count<<<pts_blocks, 256, 0, st>>>(pb, 0, pb.n_points);
      launched++;
    }
  }
  mark(1);
  const uint32_t nblk = (pb.n_buckets + kScanBlock - 1) / kScanBlock;
  if (nblk > 0) {
    k_scan_reduce<<<nblk, kScanThreads, 0, st>>>(pb);
    launched++;
    k_scan_blocks<<<1, kScanThreads, 0, st>>>(pb, nblk);
    launched++;
    k_scan_apply<<<nblk, kScanThreads, 0, st>>>(pb);
    launched++;
  }
  mark(2);
  if (pb.n_points > 0 && pb.stage) {
    for (uint32_t r = 0; r < pb.n_bins; r++) {
      k_scatter_staged<<<pts_blocks, 256, 0, st>>>(pb, r);
      launched++;
    }
  } else if (pb.n_points > 0) {
    const uint32_t passes = msm_scatter_passes(pb.max_entries);
    for (uint32_t p = 0; p < passes; p++) {
      const uint32_t lo = (uint32_t)((uint64_t)pb.n_buckets * p / passes);
      const uint32_t hi = (uint32_t)((uint64_t)pb.n_buckets * (p + 1) / passes);
      k_scatter<<<pts_blocks, 256, 0, st>>>(pb, lo, hi);
      launched++;
    }
  }
  mark(3);
  if (pb.n_buckets > 0) {
    k_len_hist<<<num_sms * 4, 256, (pb.seg_len + 1) * 4, st>>>(pb);
    launched++;
    k_len_scan<<<1, 32, 0, st>>>(pb);
    launched++;
    k_tasks<<<(pb.n_buckets + 255) / 256, 256, 2 * (pb.seg_len + 1) * 4, st>>>(pb);
    launched++;
  }
  mark(4);
  k_accumulate<<<num_sms * (pb.acc_blocks_per_sm ? pb.acc_blocks_per_sm : 4), 128, 0, st>>>(pb);
  launched++;
  mark(5);
  k_merge_small<<<num_sms * 4, 128, 0, st>>>(pb);
  launched++;
  k_merge<<<num_sms, 256, 0, st>>>(pb);
  launched++;
  k_merge_big<<<num_sms * 3, kRedThreads, 0, st>>>(pb);
  launched++;
  mark(6);
  if (pb.n_segs > 0) {
    k_reduce1<<<(pb.n_segs + 127) / 128, 128, 0, st>>>(pb);
    launched++;
  }
  mark(7);
  // Level 2 in blocks of 256 threads; level 3 (one block per window) in blocks of 128 while
  // they fit on the SMs in one wave.  Measured on GB300 (ms, 256 against 128 threads): level 3
  // of one fixed-base MSM of 2^12 / 2^16 / 2^20 / 2^24 points 0.130 / 0.145 / 0.171 / 0.215
  // against 0.107 / 0.123 / 0.154 / 0.206; level 2, groups of 512 runs at 2^20 / 2^24,
  // 0.188 / 0.268 against 0.214 / 0.348 (each quad then sums twice as many runs in sequence).
  if (pb.n_grps > 0) {
    k_reduce2<256><<<pb.n_grps, 256, 0, st>>>(pb);
    launched++;
  }
  mark(8);
  if (pb.n_wins > 0) {
    k_reduce3_small<<<(pb.n_wins + 31) / 32, 128, 0, st>>>(pb);
    launched++;
    if (pb.n_wins <= (uint32_t)num_sms)
      k_reduce3<128><<<pb.n_wins, 128, 0, st>>>(pb);
    else
      k_reduce3<256><<<pb.n_wins, 256, 0, st>>>(pb);
    launched++;
  }
  mark(9);
  if (pb.n_jobs > 0) {
    k_final<<<pb.n_jobs, 128, 0, st>>>(pb);
    launched++;
  }
  mark(10);
  if (n_kernels) *n_kernels = launched;
  return cudaGetLastError();
}
