// Host side of libdriver.so: the C ABI of include/msm_gb300.h over the device pipeline.
//
// It mirrors the reference host driver (zprize/msm_pippenger/host/driver/driver.cpp):
//   msm_init  -> Driver::Driver + load_xclbin (driver.cpp:137-304): bases converted once to the
//                precomputed twisted-Edwards form, here on the GPU, and kept resident in HBM,
//                with fixed-base tables 2^(c w) P_i when HBM allows (a second set of width 16
//                for large contexts); bases without a twisted-Edwards image are listed for the
//                Weierstrass path (driver.cpp:158-171);
//   msm_mult  -> run_asynchronous (driver.cpp:495-600): the first MSM's scalars are read from
//                host memory by the histogram kernel itself (Grace: over NVLink-C2C) and those of
//                batch b+1 are copied while batch b computes; everything after the scalars (sort,
//                buckets, reduction, window combine, affine map) runs on the device and only
//                144 B per MSM return.
// Additions: uneven batches in one pass with one shared sort, CUDA-graph replay, an autotuner,
// a continuous-batching server, per-stage timing and data generators for tests and benchmarks.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/msm_gb300.h"
#include "engine.h"

static_assert(sizeof(biginteger256_t) == 32, "biginteger256_t is 32 bytes");
static_assert(sizeof(g1_affine_t) == 104, "g1_affine_t is 104 bytes");
static_assert(offsetof(g1_affine_t, infinity) == 96, "g1_affine_t.infinity at byte 96");
static_assert(sizeof(g1_projective_t) == 144, "g1_projective_t is 144 bytes");

// ---------------------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------------------
namespace {

thread_local int g_err = 0;
thread_local char g_msg[512] = {0};

enum {
  ERR_ARG = -1,
  ERR_CUDA = -2,
  ERR_INPUT = -3,
  ERR_DEVICE = -4,
  ERR_BUDGET = -5,
  ERR_STATE = -6,
};

int fail(int code, const char *fmt, ...) {
  g_err = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  return code;
}

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
                  __FILE__, __LINE__);                                                \
  } while (0)

// ---------------------------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // grow-only; returns true if the address changed
  cudaError_t ensure(size_t want, bool *moved = nullptr) {
    if (want <= bytes && p) return cudaSuccess;
    release();
    size_t sz = std::max<size_t>(want, 256);
    cudaError_t e = cudaMalloc(&p, sz);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    bytes = sz;
    if (moved) *moved = true;
    return cudaSuccess;
  }
  template <class T> T *as() const { return (T *)p; }
};

struct HostPinned {
  void *p = nullptr;
  size_t bytes = 0;
  ~HostPinned() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t ensure(size_t want) {
    if (want <= bytes && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost(&p, std::max<size_t>(want, 256));
    if (e == cudaSuccess) bytes = std::max<size_t>(want, 256);
    return e;
  }
};

// ---------------------------------------------------------------------------------------------
// configuration
// ---------------------------------------------------------------------------------------------
struct Cfg {
  uint32_t c = 16;
  uint32_t signed_digits = 1;
  uint32_t seg_len = 1024;
  uint32_t red_log2 = 0;  // level-1 reduction run length (log2); 0: chosen from the pass's buckets
  uint32_t fixed = 0;  // 1: the context's main fixed-base tables, 2: its width-16 tables (c is
                       // then the tables' width); 0: windowed over the plain bases
};

// Level-1 reduction runs of 2^red buckets, 4 to 64.  Small passes are latency-bound: each thread
// adds 2 x 2^red points in sequence.  Passes of 2^22 buckets or more take runs of 64 (about 2^16
// of them still keep k_reduce1 near the product throughput), which leaves fewer groups for the
// latency-bound levels 2 and 3.  Measured on GB300:
//   2^15 buckets (one MSM on tables of width 16): 4 beats 8 by 0.1 ms (2^12 points: 0.76 against
//   0.87 ms per MSM), and 16 is 0.33 ms worse;
//   2^21 buckets: 16 is best (8 and 16 tie at 2^19);
//   4.9 M shared buckets (tables of width 23): 64 beats 32 by 0.3 ms (level 1 +0.08 ms, levels 2
//   and 3 -0.37 ms), and 64 is best at 2^23.
uint32_t red_log2_for(uint64_t buckets) {
  int lg = 0;
  while (lg < 63 && (2ull << lg) <= buckets) lg++;  // floor(log2(buckets))
  return lg <= 15 ? 2u : lg <= 18 ? 3u : lg <= 21 ? 4u : 6u;
}


// the scalar field's modulus r, little-endian 64-bit words
const uint64_t R_WORDS[4] = {0x0a11800000000001ull, 0x59aa76fed0000001ull, 0x60b44d1e5c37b001ull,
                             0x12ab655e9a2ca556ull};

uint32_t windows_of(uint32_t c) { return (MSM_SCALAR_BITS + c - 1) / c; }

uint32_t log2_ceil(uint64_t n) {
  uint32_t k = 0;
  while ((1ull << k) < n) k++;
  return k;
}

// Bucket counts of a window layout: signed 2^(c-1) per window, unsigned 2^c - 1.  The top window
// holds the c_top = 253 - c (W-1) bits left over: unsigned 2^c_top - 1 buckets; signed (its
// digit also takes the carry out of the window below) 2^c_top, capped at the largest top digit a
// scalar below r produces, floor((r-1) / 2^(c (W-1))) + 1.  A 253-bit scalar at or above r whose
// top digit is larger gets it as two entries (see entries_per_point).
void layout(uint32_t c, uint32_t sgn, uint32_t &nwin, uint32_t &nb, uint32_t &nb_top) {
  nwin = windows_of(c);
  const uint32_t shift = c * (nwin - 1);  // >= 222: (r-1) >> shift is r's top word shifted
  const uint32_t ctop = MSM_SCALAR_BITS - shift;
  if (sgn) {
    nb = 1u << (c - 1);
    nb_top = (uint32_t)std::min<uint64_t>(1ull << ctop, (R_WORDS[3] >> (shift - 192)) + 1);
  } else {
    nb = (1u << c) - 1;
    nb_top = (1u << ctop) - 1;
  }
}

// Sorted entries one point can produce: one per window, plus one when the top window's bucket
// range is capped below 2^c_top (its digit then splits into nb_top and the rest, which is at most
// nb_top since the cap is at least 2^(c_top - 1)).
uint32_t entries_per_point(uint32_t c, uint32_t sgn) {
  uint32_t nwin, nb, nbt;
  layout(c, sgn, nwin, nb, nbt);
  const uint32_t ctop = MSM_SCALAR_BITS - c * (nwin - 1);
  return nwin + (sgn && nbt < (1u << ctop) ? 1u : 0u);
}

// Cost model in 12-limb products at throughput: 7 per bucket add, 18 per bucket in the
// reduction, and the serial window combine of the standard layout, c doublings per window at
// two product latencies each (one product latency ~ 12.6k products of throughput on GB300).
double model_cost(uint64_t n, uint32_t c, uint32_t sgn) {
  uint32_t nwin, nb, nbt;
  layout(c, sgn, nwin, nb, nbt);
  const double buckets = (double)(nwin - 1) * nb + nbt;
  return (double)n * nwin * 7.0 + buckets * 18.0 + (double)(nwin - 1) * c * 2.0 * 12600.0;
}
double model_cost_fixed(uint64_t n, uint32_t c, uint32_t sgn) {
  uint32_t nwin, nb, nbt;
  layout(c, sgn, nwin, nb, nbt);
  // 18 products per bucket in level 1, plus the level-2/3 combines and the bucket metadata
  // passes, measured at about a third more per bucket
  return (double)n * nwin * 7.0 + (double)std::max(nb, nbt) * 24.0;
}

// Run length that keeps buckets of mean load `mean` whole but for their Poisson tail: the
// smallest power of two (32 to 4096) at or above mean + 2 sqrt(mean).  Measured on GB300 with
// fixed-base tables: mean 26 (2^20 points, c = 20) 64 beats 32 and 128; mean 104 (2^22) 128
// beats 64 (merges) and 256 (longer runs unbalance the warps) by 1%; means 38 and 151 (2^24,
// 2^26 at c = 23) tie from 64 and 256 up.
uint32_t whole_bucket_run(double mean) {
  uint32_t s = 32;
  while (s < mean + 2.0 * std::sqrt(mean) && s < 4096) s <<= 1;
  return s;
}

// Longest run of entries one accumulate thread sums: whole buckets of `nwin_sharing` windows
// but for the tail, and short enough that the n x nwin entries make at least ~2^17 runs: with
// few, heavily loaded buckets (a fixed-base table of small width) whole-bucket runs would leave
// most of the GPU idle.  A pass of at most 2^21 entries does not fill the GPU, and its time is
// the longest run plus the merge of its split buckets: runs of about 2 sqrt(mean), at least 8,
// balance the two.  Measured on GB300 (one MSM on width-16 tables, mean bucket load 8: 2^14
// points): runs of 8 0.72 ms, 4 0.71 ms, 16 0.82 ms; at load 2 (2^12 points) runs of 2 to 32
// are within 4% of each other, and at load 32 (2^16 points) 16 is best (1.06 ms, 8: 1.08 ms).
uint32_t seg_len_for(uint64_t n, uint32_t nb, uint32_t nwin_sharing, uint32_t nwin) {
  const double mean = (double)n * nwin_sharing / std::max<uint32_t>(nb, 1);
  const uint32_t s = whole_bucket_run(mean);
  const uint64_t entries = n * (uint64_t)nwin;
  uint32_t cap = 16;
  while (cap < 4096 && ((uint64_t)cap << 18) <= entries) cap <<= 1;  // entries / cap >= 2^17
  uint32_t r = std::min(s, cap);
  if (entries <= (1ull << 21)) {
    uint32_t t = 8;
    while (t < 2.0 * std::sqrt(mean) && t < 4096) t <<= 1;
    r = std::min(r, t);
  }
  return r;
}

Cfg heuristic_cfg(uint64_t n) {
  Cfg cfg;
  double best = 1e300;
  for (uint32_t c = 6; c <= 20; c++) {
    const double v = model_cost(n, c, 1);
    if (v < best) {
      best = v;
      cfg.c = c;
    }
  }
  uint32_t nwin, nb, nbt;
  layout(cfg.c, 1, nwin, nb, nbt);
  cfg.seg_len = seg_len_for(n, nb, 1, nwin);
  cfg.red_log2 = 0;
  return cfg;
}

// ---------------------------------------------------------------------------------------------
// pass plan
// ---------------------------------------------------------------------------------------------
struct JobSpec {
  uint64_t n, base_off, scalar_off;
  Cfg cfg;
  uint64_t fb_stride = 0;  // fixed-base jobs: index step between the windows' tables
  uint64_t tab_base = 0;   // first record of the job's table set
};

struct Ctx;
void set_tables(const Ctx *cx, JobSpec &s);

struct Plan {
  std::vector<JobDesc> jobs;
  std::vector<WinDesc> wins;
  uint64_t n_points = 0, max_entries = 0;
  uint32_t n_buckets = 0, n_segs = 0, n_grps = 0, max_tasks = 0;
  uint32_t seg_len = 1024, red_log2 = 5, grp_log2 = 9;
  // staged sort: histogram chunks of MSM_POINTS_PER_CHUNK points, each with room for the
  // largest window count of the pass, and the key ranges of the scatter
  uint64_t n_chunks = 0;
  uint32_t stage_cap = 0, bin_shift = 0, n_bins = 0;
  bool ranks = false;  // entries carry their rank in the bucket (no slot atomics in the scatter)
  std::string key;
};

// Run length of a pass of several MSMs: whole buckets at the largest mean bucket load among them
// (as seg_len_for does for one MSM), capped so the whole pass makes at least 2^19 runs.  Each MSM's
// own choice is capped by its own entries and is too short in a shared pass.  Measured on GB300,
// the uneven 64-MSM mix (1.1e8 entries, 10% of each MSM's scalars one repeated value) over a
// 2^24-base context: runs of 64 (the largest MSM's own choice) 35.8 ms, 256 34.4 ms, 512 36.0 ms,
// 1024 42.2 ms; over a 2^20-base context 34.8, 33.8, 36.2 and 41.9 ms.
uint32_t pass_seg_len(const std::vector<JobSpec> &specs) {
  double mean = 0;
  uint64_t entries = 0;
  for (const JobSpec &sp : specs) {
    if (sp.n == 0) continue;
    uint32_t nwin, nb, nbt;
    layout(sp.cfg.c, sp.cfg.signed_digits, nwin, nb, nbt);
    const double load = sp.cfg.fixed ? (double)sp.n * nwin / std::max(nb, nbt)
                                     : (double)sp.n / std::max<uint32_t>(nb, 1);
    mean = std::max(mean, load);
    entries += sp.n * entries_per_point(sp.cfg.c, sp.cfg.signed_digits);
  }
  const uint32_t seg = whole_bucket_run(mean);
  uint32_t cap = 16;
  while (cap < 4096 && ((uint64_t)cap << 19) <= entries) cap <<= 1;
  return std::min(seg, cap);
}

int build_plan(const std::vector<JobSpec> &specs, Plan &pl) {
  pl = Plan();
  if (specs.empty()) return fail(ERR_ARG, "empty pass");
  pl.seg_len = specs[0].cfg.seg_len;
  pl.red_log2 = specs[0].cfg.red_log2;
  if (pl.red_log2 == 0) {  // automatic: from the pass's bucket count
    uint64_t total = 0;
    for (const JobSpec &s : specs) {
      if (s.n == 0) continue;
      uint32_t nwin, nb, nbt;
      layout(s.cfg.c, s.cfg.signed_digits, nwin, nb, nbt);
      total += s.cfg.fixed ? std::max(nb, nbt) : (uint64_t)(nwin - 1) * nb + nbt;
    }
    pl.red_log2 = red_log2_for(total);
  }
  // Level-2 groups of 2^grp_log2 level-1 runs.  A pass whose reduction is one window (one MSM on
  // fixed-base tables) takes groups of 128 to 512 runs, about 128 groups: level 3 then combines
  // enough groups to use a block (a window of at most 16 groups is combined serially by one
  // quad) and few enough to keep its tree shallow.  Measured on GB300 (ms per MSM, groups of
  // 512 / 256 / 128 runs): 2^12 and 2^16 points (4096 runs) 0.973 / 0.993 / 0.850 and 1.427 /
  // 1.448 / 1.300; 2^20 (32 K runs) 6.290 / 6.219 / 6.307; 2^24 (76 K runs) 71.58 / 71.79 / 72.10.
  // Passes of many windows (windowed MSMs, batches) keep groups of 512: the uneven 64-MSM mix
  // (64 windows of 2048 runs) took 34.44 ms with them and 34.99 ms with groups of 128, whose
  // 1024 level-2 blocks run in several waves.
  {
    uint32_t n_windows = 0;
    uint64_t max_nb = 0;
    for (const JobSpec &s : specs) {
      if (s.n == 0) continue;
      uint32_t nwin, nb, nbt;
      layout(s.cfg.c, s.cfg.signed_digits, nwin, nb, nbt);
      n_windows += s.cfg.fixed ? 1 : nwin;
      max_nb = std::max<uint64_t>(max_nb, std::max(nb, nbt));
    }
    const uint64_t max_nseg = (max_nb + (1ull << pl.red_log2) - 1) >> pl.red_log2;
    pl.grp_log2 = n_windows == 1 ? 7 : 9;
    while (pl.grp_log2 < 9 && (max_nseg >> pl.grp_log2) > 128) pl.grp_log2++;
  }
  uint64_t buckets = 0, segs = 0, wins = 0, grps = 0;
  char tmp[160];
  for (size_t j = 0; j < specs.size(); j++) {
    const JobSpec &s = specs[j];
    JobDesc d{};
    d.point_begin = pl.n_points;
    d.n = s.n;
    d.base_off = s.base_off;
    d.scalar_off = s.scalar_off;
    d.c = s.cfg.c;
    d.signed_digits = s.cfg.signed_digits;
    d.result_slot = (uint32_t)j;
    d.bucket_begin = (uint32_t)buckets;
    d.win_begin = (uint32_t)wins;
    if (s.n == 0) {
      d.nwin = 0;
      d.nb = d.nb_top = 0;
    } else {
      layout(d.c, d.signed_digits, d.nwin, d.nb, d.nb_top);
      d.fixed = s.cfg.fixed ? 1 : 0;
      d.fb_stride = s.fb_stride;
      d.tab_base = s.tab_base;
      d.nred = d.fixed ? 1 : d.nwin;
      const uint32_t L = 1u << pl.red_log2;
      for (uint32_t w = 0; w < d.nred; w++) {
        WinDesc wd{};
        wd.job = (uint32_t)j;
        wd.w = w;
        wd.bucket_begin = (uint32_t)(buckets + (uint64_t)w * d.nb);
        wd.nb = d.fixed ? std::max(d.nb, d.nb_top) : (w + 1 == d.nwin) ? d.nb_top : d.nb;
        wd.seg_begin = (uint32_t)segs;
        wd.nseg = (wd.nb + L - 1) / L;
        wd.grp_begin = (uint32_t)grps;
        wd.ngrp = (wd.nseg + (1u << pl.grp_log2) - 1) >> pl.grp_log2;
        segs += wd.nseg;
        grps += wd.ngrp;
        pl.wins.push_back(wd);
      }
      buckets += d.fixed ? (uint64_t)std::max(d.nb, d.nb_top)
                         : (uint64_t)(d.nwin - 1) * d.nb + d.nb_top;
      wins += d.nred;
      pl.max_entries += s.n * entries_per_point(d.c, d.signed_digits);
    }
    pl.n_points += s.n;
    pl.jobs.push_back(d);
    snprintf(tmp, sizeof(tmp), "%llu/%llu/%llu/%u/%u/%u;", (unsigned long long)s.n,
             (unsigned long long)s.base_off, (unsigned long long)s.scalar_off, d.c, d.signed_digits,
             d.fixed);
    pl.key += tmp;
  }
  if (buckets >= (1ull << 32) || pl.max_entries >= (1ull << 32) - 1 || segs >= (1ull << 31))
    return fail(ERR_BUDGET, "pass too large: %llu buckets, %llu entries",
                (unsigned long long)buckets, (unsigned long long)pl.max_entries);
  pl.n_buckets = (uint32_t)buckets;
  uint32_t max_epp = 0;  // entries per point
  for (const JobDesc &d : pl.jobs)
    if (d.nwin) max_epp = std::max(max_epp, entries_per_point(d.c, d.signed_digits));
  pl.n_chunks = (pl.n_points + MSM_POINTS_PER_CHUNK - 1) / MSM_POINTS_PER_CHUNK;
  pl.stage_cap = MSM_POINTS_PER_CHUNK * max_epp;
  // MSM_SORT_RANGES=<n> overrides the number of key ranges of the staged sort (tests, tuning)
  const char *sr = getenv("MSM_SORT_RANGES");
  // ranks from the histogram's atomics save the scatter's slot atomics, but the histogram's
  // atomics then return a value.  Measured on GB300 (count + scatter): the uneven 64-MSM mix
  // (up to 1.0e8 entries, 2^21 buckets) 2.03 ms with ranks, 2.67 ms without; 2^24 points on
  // tables of width 23 (2.0e8 entries, 4.9M buckets) 5.65 against 4.86 with ranges of 2^20 keys,
  // and the cursors 3.45 with ranges of 2^19 keys; 2^26 points (8.1e8) 16.5 against 14.0
  pl.ranks = pl.max_entries < (1ull << 27);
  pl.bin_shift =
      msm_bin_shift(pl.n_buckets, pl.max_entries, sr ? (uint32_t)atoi(sr) : 0u, !pl.ranks);
  pl.n_bins = pl.n_buckets ? ((pl.n_buckets - 1) >> pl.bin_shift) + 1 : 0;
  if (pl.n_bins > MSM_MAX_BINS) return fail(ERR_STATE, "too many key ranges: %u", pl.n_bins);
  snprintf(tmp, sizeof(tmp), "|r%u", pl.bin_shift);
  pl.key += tmp;
  pl.n_segs = (uint32_t)segs;
  pl.n_grps = (uint32_t)grps;
  const uint64_t mt = buckets + pl.max_entries / pl.seg_len + 1;
  if (mt >= (1ull << 31)) return fail(ERR_BUDGET, "too many tasks");
  pl.max_tasks = (uint32_t)mt;
  snprintf(tmp, sizeof(tmp), "|%u|%u|g%u", pl.seg_len, pl.red_log2, pl.grp_log2);
  pl.key += tmp;
  return 0;
}

// device bytes a pass needs besides the resident bases
uint64_t plan_bytes(const Plan &pl, bool with_scalars) {
  uint64_t b = 0;
  b += (uint64_t)pl.n_buckets * 4 * 5;                   // count, offset, fill, taskoff, heavy
  b += pl.max_entries * 4;                                // vals
  b += pl.n_chunks * ((uint64_t)pl.stage_cap * (pl.ranks ? 12 : 8) + (pl.n_bins + 1) * 4);
  b += (uint64_t)pl.max_tasks * (sizeof(Task) + 4 + MSM_BUCKET_BYTES);
  b += (uint64_t)(pl.n_segs + pl.n_grps) * 2 * MSM_BUCKET_BYTES;
  b += (uint64_t)pl.wins.size() * MSM_BUCKET_BYTES;
  b += pl.jobs.size() * (sizeof(JobDesc) + MSM_PROJ_BYTES) + pl.wins.size() * sizeof(WinDesc);
  if (with_scalars) b += pl.n_points * 32;
  return b + (1 << 20);
}

// ---------------------------------------------------------------------------------------------
// workspace: the buffers of one in-flight pass
// ---------------------------------------------------------------------------------------------
struct Workspace {
  DevBuf count, offset, fill, taskoff, scan_tmp, vals, tasks, partials, heavy, counters, seg_out,
      grp_out, win_sum, results, jobs, wins, order, len_hist, stage, stage_rank, blk_off;
  DevBuf scalars[2];
  HostPinned res_host;
  cudaEvent_t ev[MSM_NUM_STAGES + 1] = {};
  uint64_t generation = 0;  // bumps when any buffer moves (graphs must be re-captured)
  uint32_t acc_blocks_per_sm = 0;  // k_accumulate blocks per SM for this workspace's passes (0: 4)
  struct GraphEntry {
    cudaGraphExec_t exec;
    uint32_t kernels;  // kernel launches in one replay
  };
  std::unordered_map<std::string, GraphEntry> graphs;

  ~Workspace() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second.exec);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  }
  int ensure(const Plan &pl) {
    bool moved = false;
    CK(count.ensure((size_t)pl.n_buckets * 4, &moved));
    CK(offset.ensure((size_t)pl.n_buckets * 4, &moved));
    CK(fill.ensure((size_t)pl.n_buckets * 4, &moved));
    CK(taskoff.ensure((size_t)pl.n_buckets * 4, &moved));
    CK(heavy.ensure((size_t)pl.n_buckets * 4, &moved));
    CK(scan_tmp.ensure(msm_scan_tmp_words(pl.n_buckets) * 4, &moved));
    CK(vals.ensure((size_t)pl.max_entries * 4, &moved));
    CK(stage.ensure((size_t)pl.n_chunks * pl.stage_cap * 8, &moved));
    if (pl.ranks) CK(stage_rank.ensure((size_t)pl.n_chunks * pl.stage_cap * 4, &moved));
    CK(blk_off.ensure((size_t)pl.n_chunks * (pl.n_bins + 1) * 4, &moved));
    CK(tasks.ensure((size_t)pl.max_tasks * sizeof(Task), &moved));
    CK(partials.ensure((size_t)pl.max_tasks * MSM_BUCKET_BYTES, &moved));
    CK(order.ensure((size_t)pl.max_tasks * 4, &moved));
    CK(len_hist.ensure((size_t)(pl.seg_len + 1) * 4, &moved));
    CK(counters.ensure(CNT_WORDS * 4, &moved));
    CK(seg_out.ensure((size_t)pl.n_segs * 2 * MSM_BUCKET_BYTES, &moved));
    CK(grp_out.ensure((size_t)pl.n_grps * 2 * MSM_BUCKET_BYTES, &moved));
    CK(win_sum.ensure(pl.wins.size() * MSM_BUCKET_BYTES, &moved));
    CK(results.ensure(pl.jobs.size() * MSM_PROJ_BYTES, &moved));
    CK(jobs.ensure(pl.jobs.size() * sizeof(JobDesc), &moved));
    CK(wins.ensure(pl.wins.size() * sizeof(WinDesc), &moved));
    CK(res_host.ensure(pl.jobs.size() * MSM_PROJ_BYTES));
    if (!ev[0])
      for (auto &e : ev) CK(cudaEventCreate(&e));
    if (moved) {
      generation++;
      for (auto &kv : graphs) cudaGraphExecDestroy(kv.second.exec);
      graphs.clear();
    }
    return 0;
  }
};

// ---------------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------------
struct Ctx {
  int device = 0;
  int num_sms = 0;
  uint64_t npoints = 0;
  uint32_t fb_c = 0, fb_w = 1;  // fixed-base tables: window width and windows (fb_c 0: none)
  // second table set of width 16 after the main one (fb2_c 0: none), for the context's small
  // MSMs: records [npoints * fb_w, npoints * (fb_w + fb2_w))
  uint32_t fb2_c = 0, fb2_w = 0;
  DevBuf bases, flags, special_idx, special_cls, class_pts;
  uint32_t n_special = 0, n_classes = 0;
  cudaStream_t stream = nullptr, copy_stream = nullptr;
  cudaEvent_t copied[2] = {}, freed[2] = {};
  static constexpr int kCopyChunks = 4;
  cudaEvent_t chunk_ev[2][kCopyChunks] = {};
  // the device reads pageable host memory coherently (Grace: ATS over NVLink-C2C), so host
  // scalars are uploaded by the histogram kernel itself instead of a separate copy
  bool host_pull = false;
  Workspace ws;
  std::mutex mu;
  bool timing = false;
  double last_ms[MSM_NUM_STAGES] = {0};
  uint64_t last_stats[5] = {0};  // tasks, heavy buckets, sorted entries, buckets, kernels
  std::map<uint32_t, Cfg> tuned;  // by log2 size class
  // forms tuned for MSMs that share a pass with others (msm_tune_uneven), by log2 size class;
  // a shared pass overlaps the serial tails of its MSMs, so the best form can differ from the
  // best for one MSM alone
  std::map<uint32_t, Cfg> tuned_batch;
  // guards tuned and tuned_batch: a server's worker reads them while a tuner may write them
  std::mutex tune_mu;
  ~Ctx() {
    if (stream) cudaStreamDestroy(stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    for (int i = 0; i < 2; i++) {
      if (copied[i]) cudaEventDestroy(copied[i]);
      if (freed[i]) cudaEventDestroy(freed[i]);
      for (auto &e : chunk_ev[i])
        if (e) cudaEventDestroy(e);
    }
  }
};

// Where a job's entries point: the plain bases (windowed), the main tables or the width-16 set.
void set_tables(const Ctx *cx, JobSpec &s) {
  s.fb_stride = s.cfg.fixed ? cx->npoints : 0;
  s.tab_base = s.cfg.fixed == 2 ? cx->npoints * cx->fb_w : 0;
}

PassBuffers make_pass_buffers(Ctx *cx, Workspace &ws, const Plan &pl, const void *d_scalars) {
  PassBuffers pb{};
  pb.acc_blocks_per_sm = ws.acc_blocks_per_sm;
  pb.bases = cx->bases.as<uint4>();
  pb.flags = cx->flags.as<uint8_t>();
  pb.special_idx = cx->special_idx.as<uint32_t>();
  pb.special_cls = cx->special_cls.as<uint8_t>();
  pb.class_pts = cx->class_pts.as<uint4>();
  pb.n_special = cx->n_special;
  pb.n_classes = cx->n_classes;
  pb.n_bases = cx->npoints * (cx->fb_w + cx->fb2_w);
  pb.scalars = (const uint4 *)d_scalars;
  pb.jobs = ws.jobs.as<JobDesc>();
  pb.wins = ws.wins.as<WinDesc>();
  pb.n_jobs = (uint32_t)pl.jobs.size();
  pb.n_wins = (uint32_t)pl.wins.size();
  pb.n_points = pl.n_points;
  pb.n_buckets = pl.n_buckets;
  pb.n_segs = pl.n_segs;
  pb.n_grps = pl.n_grps;
  pb.seg_len = pl.seg_len;
  pb.red_len_log2 = pl.red_log2;
  pb.grp_len_log2 = pl.grp_log2;
  pb.max_entries = pl.max_entries;
  pb.max_tasks = pl.max_tasks;
  pb.count = ws.count.as<uint32_t>();
  pb.offset = ws.offset.as<uint32_t>();
  pb.fill = ws.fill.as<uint32_t>();
  pb.taskoff = ws.taskoff.as<uint32_t>();
  pb.scan_tmp = ws.scan_tmp.as<uint32_t>();
  pb.vals = ws.vals.as<uint32_t>();
  pb.stage = pl.n_chunks ? ws.stage.as<uint2>() : nullptr;
  pb.blk_off = ws.blk_off.as<uint32_t>();
  pb.stage_rank = pl.ranks && pb.stage ? ws.stage_rank.as<uint32_t>() : nullptr;
  pb.stage_cap = pl.stage_cap;
  pb.bin_shift = pl.bin_shift;
  pb.n_bins = pl.n_bins;
  pb.tasks = ws.tasks.as<Task>();
  pb.partials = ws.partials.as<uint4>();
  pb.heavy = ws.heavy.as<uint32_t>();
  pb.order = ws.order.as<uint32_t>();
  pb.len_hist = ws.len_hist.as<uint32_t>();
  pb.counters = ws.counters.as<uint32_t>();
  pb.seg_out = ws.seg_out.as<uint4>();
  pb.grp_out = ws.grp_out.as<uint4>();
  pb.win_sum = ws.win_sum.as<uint4>();
  pb.results = ws.results.as<uint64_t>();
  return pb;
}

// Enqueue one pass on `st`: upload the plan, run the pipeline (directly or from a captured
// graph), copy the results to ws.res_host + res_offset jobs.  Does not synchronize.
int enqueue_pass(Ctx *cx, Workspace &ws, const Plan &pl, const void *d_scalars, cudaStream_t st,
                 bool use_graph, bool timing, size_t res_offset,
                 const cudaEvent_t *chunk_ready = nullptr, int nchunks = 0,
                 const void *host_src = nullptr) {
  if (ws.ensure(pl)) return g_err;
  CK(cudaMemcpyAsync(ws.jobs.p, pl.jobs.data(), pl.jobs.size() * sizeof(JobDesc),
                     cudaMemcpyHostToDevice, st));
  if (!pl.wins.empty())
    CK(cudaMemcpyAsync(ws.wins.p, pl.wins.data(), pl.wins.size() * sizeof(WinDesc),
                       cudaMemcpyHostToDevice, st));
  PassBuffers pb = make_pass_buffers(cx, ws, pl, d_scalars);
  pb.host_scalars = (const uint4 *)host_src;
  char *res_dst = (char *)ws.res_host.p;
  if (res_offset * MSM_PROJ_BYTES + pl.jobs.size() * MSM_PROJ_BYTES > ws.res_host.bytes)
    return fail(ERR_STATE, "result staging too small");
  res_dst += res_offset * MSM_PROJ_BYTES;
  if (use_graph && !timing && !chunk_ready && !host_src) {
    char tmp[64];
    snprintf(tmp, sizeof(tmp), "#%p#%p", d_scalars, (void *)res_dst);
    const std::string key = pl.key + tmp;
    auto it = ws.graphs.find(key);
    if (it == ws.graphs.end()) {
      cudaGraph_t g;
      uint32_t nk = 0;
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = msm_launch_pass(pb, cx->num_sms, st, nullptr, nullptr, 0, &nk);
      cudaError_t e2 = cudaMemcpyAsync(res_dst, ws.results.p, pl.jobs.size() * MSM_PROJ_BYTES,
                                       cudaMemcpyDeviceToHost, st);
      cudaError_t e3 = cudaStreamEndCapture(st, &g);
      if (e != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
        return fail(ERR_CUDA, "graph capture failed: %s / %s / %s", cudaGetErrorString(e),
                    cudaGetErrorString(e2), cudaGetErrorString(e3));
      cudaGraphExec_t ex;
      CK(cudaGraphInstantiate(&ex, g, 0));
      cudaGraphDestroy(g);
      it = ws.graphs.emplace(key, Workspace::GraphEntry{ex, nk}).first;
    }
    CK(cudaGraphLaunch(it->second.exec, st));
    cx->last_stats[4] = it->second.kernels;
    return 0;
  }
  uint32_t nk = 0;
  CK(msm_launch_pass(pb, cx->num_sms, st, timing ? ws.ev : nullptr, chunk_ready, nchunks, &nk));
  cx->last_stats[4] = nk;
  CK(cudaMemcpyAsync(res_dst, ws.results.p, pl.jobs.size() * MSM_PROJ_BYTES,
                     cudaMemcpyDeviceToHost, st));
  return 0;
}

int check_pass_errors(Workspace &ws, cudaStream_t st, uint64_t *stats_out) {
  uint32_t cnt[CNT_WORDS];
  CK(cudaMemcpyAsync(cnt, ws.counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (stats_out) {
    stats_out[0] = cnt[CNT_TASKS];
    stats_out[1] = cnt[CNT_HEAVY];
    stats_out[2] = cnt[CNT_ENTRIES];
  }
  if (cnt[CNT_ERROR]) {
    // the codes msm_pipeline.cu's kernels record (they skip the access that would be out of bounds)
    static const char *const what[] = {
        "", "sorted entries exceed the plan", "tasks exceed the plan", "scatter position out of range",
        "task slot out of range", "base index out of range", "stage chunk overflow",
        "staged bucket key out of range"};
    const uint32_t code = cnt[CNT_ERROR];
    return fail(ERR_STATE, "device bounds check %u fired (%s; info %u)", code,
                code < sizeof(what) / sizeof(what[0]) ? what[code] : "unknown", cnt[CNT_ERROR_INFO]);
  }
  return 0;
}

Cfg resolve_cfg(Ctx *cx, uint64_t n, const msm_options_t *opt, bool shared_pass = false) {
  Cfg cfg = heuristic_cfg(n);
  const uint32_t cls = log2_ceil(std::max<uint64_t>(n, 1));
  bool tuned = false;
  {
    std::lock_guard<std::mutex> lk(cx->tune_mu);
    const std::map<uint32_t, Cfg> &tmap =
        shared_pass && cx->tuned_batch.count(cls) ? cx->tuned_batch : cx->tuned;
    auto it = tmap.find(cls);
    tuned = it != tmap.end();
    if (tuned) cfg = it->second;
  }
  const bool forced_c = opt && opt->window_bits > 0;
  if (opt) {
    if (forced_c) {
      cfg.c = (uint32_t)std::min(std::max(opt->window_bits, 4), 22);
      uint32_t nwin, nb, nbt;
      layout(cfg.c, 1, nwin, nb, nbt);
      cfg.seg_len = seg_len_for(n, nb, 1, nwin);
    }
    if (opt->signed_digits == 1) cfg.signed_digits = 1;
    if (opt->signed_digits == 2) cfg.signed_digits = 0;
  }
  if (!cfg.signed_digits && cfg.c > 21) cfg.c = 21;
  // the table sets that exist: 1 main (width fb_c), 2 the width-16 set (fb2_c)
  auto table_c = [&](uint32_t which) { return which == 1 ? cx->fb_c : which == 2 ? cx->fb2_c : 0u; };
  const uint32_t tuned_fixed = tuned && table_c(cfg.fixed) ? cfg.fixed : 0u;
  cfg.fixed = 0;
  // fixed-base tables: every window shares one bucket array and there is no serial window
  // combine; chosen when asked (the cheaper set by the cost model), by the tuner's measurement
  // for this size class, or else when the cost model says so
  const int fb = opt ? opt->fixed_base : 0;
  uint32_t use = 0;
  if ((cx->fb_c || cx->fb2_c) && fb != 2) {
    double best = 1e300;
    uint32_t cheapest = 0;
    for (uint32_t which = 1; which <= 2; which++) {
      if (!table_c(which)) continue;
      const double v = model_cost_fixed(n, table_c(which), 1);
      if (v < best) {
        best = v;
        cheapest = which;
      }
    }
    if (fb == 1)
      use = cheapest;
    else if (!forced_c)
      use = tuned ? tuned_fixed
                  : (best < model_cost(n, cfg.c, cfg.signed_digits) ? cheapest : 0u);
  }
  if (use) {
    uint32_t nwin, nb, nbt;
    layout(table_c(use), 1, nwin, nb, nbt);
    cfg.fixed = use;
    cfg.c = table_c(use);
    cfg.signed_digits = 1;
    if (tuned_fixed != use) {
      cfg.seg_len = seg_len_for(n, std::max(nb, nbt), nwin, nwin);
      cfg.red_log2 = 0;
    }
  }
  if (opt) {
    if (opt->seg_len > 0) cfg.seg_len = (uint32_t)std::min(opt->seg_len, 4096);
    if (opt->red_len_log2 > 0) cfg.red_log2 = (uint32_t)std::min(opt->red_len_log2, 12);
  }
  return cfg;
}

void record_timings(Ctx *cx, Workspace &ws) {
  for (int k = 0; k < MSM_NUM_STAGES; k++) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, ws.ev[k], ws.ev[k + 1]) != cudaSuccess) ms = -1;
    cx->last_ms[k] = ms;
  }
}

// Host scalars the histogram kernel may read directly: the device reads pageable memory and the
// buffer is 16-byte aligned (the kernel loads uint4).
bool host_pullable(const Ctx *cx, const void *h) {
  return cx->host_pull && h && ((uintptr_t)h & 15u) == 0;
}

// Run a list of MSMs whose scalars are in host memory (d_scalars == nullptr) or already on the
// device.  mode 1: one pass per MSM with the next MSM's scalars copied during the current pass;
// mode 2: all MSMs in one pass with one shared sort.
int run_msms(Ctx *cx, g1_projective_t *out, const std::vector<uint64_t> &sizes,
             const std::vector<uint64_t> &offs, const biginteger256_t *h_scalars,
             const void *d_scalars, const msm_options_t *opt) {
  const size_t m = sizes.size();
  if (m == 0) return 0;
  for (size_t j = 0; j < m; j++)
    if (offs[j] > cx->npoints || sizes[j] > cx->npoints - offs[j])
      return fail(ERR_ARG, "MSM %zu: bases [%llu, %llu) outside the %llu resident bases", j,
                  (unsigned long long)offs[j], (unsigned long long)(offs[j] + sizes[j]),
                  (unsigned long long)cx->npoints);
  const int mode = (opt && opt->mode == 2) ? 2 : 1;
  const bool use_graph = !(opt && opt->use_graph == 2) && !cx->timing;
  Workspace &ws = cx->ws;
  std::vector<uint64_t> first(m + 1, 0);
  for (size_t j = 0; j < m; j++) first[j + 1] = first[j] + sizes[j];

  if (mode == 2) {
    std::vector<JobSpec> specs(m);
    uint64_t maxn = 0;
    for (size_t j = 0; j < m; j++) maxn = std::max(maxn, sizes[j]);
    for (size_t j = 0; j < m; j++) {
      specs[j] = {sizes[j], offs[j], first[j], resolve_cfg(cx, sizes[j], opt, m > 1)};
      specs[j].cfg.seg_len = resolve_cfg(cx, maxn, opt, m > 1).seg_len;
      specs[j].cfg.red_log2 = resolve_cfg(cx, maxn, opt, m > 1).red_log2;
      set_tables(cx, specs[j]);
    }
    if (m > 1 && !(opt && opt->seg_len > 0)) {
      const uint32_t seg = pass_seg_len(specs);
      for (JobSpec &sp : specs) sp.cfg.seg_len = seg;
    }
    Plan pl;
    if (build_plan(specs, pl)) return g_err;
    const void *src = d_scalars, *pull = nullptr;
    if (!src) {
      CK(ws.scalars[0].ensure(first[m] * 32));
      if (host_pullable(cx, h_scalars)) {
        pull = h_scalars;
      } else if (first[m]) {
        CK(cudaMemcpyAsync(ws.scalars[0].p, h_scalars, first[m] * 32, cudaMemcpyHostToDevice,
                           cx->stream));
      }
      src = ws.scalars[0].p;
    }
    if (enqueue_pass(cx, ws, pl, src, cx->stream, use_graph, cx->timing, 0, nullptr, 0, pull))
      return g_err;
    if (check_pass_errors(ws, cx->stream, cx->last_stats)) return g_err;
    if (cx->timing) record_timings(cx, ws);
    cx->last_stats[3] = pl.n_buckets;
    memcpy(out, ws.res_host.p, m * MSM_PROJ_BYTES);
    return 0;
  }

  // mode 1: one pass per MSM; results land in ws.res_host at slot j
  Plan probe;
  {
    std::vector<JobSpec> one(1);
    uint64_t maxn = 0;
    for (size_t j = 0; j < m; j++) maxn = std::max(maxn, sizes[j]);
    one[0] = {maxn, 0, 0, resolve_cfg(cx, maxn, opt)};
    set_tables(cx, one[0]);
    if (build_plan(one, probe)) return g_err;
    if (ws.ensure(probe)) return g_err;
  }
  CK(ws.res_host.ensure(m * MSM_PROJ_BYTES));
  uint64_t maxn = 0;
  for (size_t j = 0; j < m; j++) maxn = std::max(maxn, sizes[j]);
  if (!d_scalars)
    for (int s = 0; s < 2; s++) CK(ws.scalars[s].ensure(std::max<uint64_t>(maxn, 1) * 32));
  for (size_t j = 0; j < m; j++) {
    std::vector<JobSpec> one(1);
    one[0] = {sizes[j], offs[j], d_scalars ? first[j] : 0, resolve_cfg(cx, sizes[j], opt)};
    set_tables(cx, one[0]);
    Plan pl;
    if (build_plan(one, pl)) return g_err;
    const void *src = d_scalars, *pull = nullptr;
    const cudaEvent_t *chunks = nullptr;
    if (!src && j == 0 && host_pullable(cx, h_scalars + first[j])) {
      // the first MSM's histogram kernel reads its scalars from host memory and leaves the
      // device copy; later MSMs' scalars are copied while the previous pass computes
      src = ws.scalars[(int)(j & 1)].p;
      pull = h_scalars + first[j];
    } else if (!src) {
      // the copy goes up in chunks on the copy stream; each chunk's histogram starts when it lands
      const int slot = (int)(j & 1);
      const int nch = Ctx::kCopyChunks;
      CK(cudaStreamWaitEvent(cx->copy_stream, cx->freed[slot], 0));
      const uint64_t per = msm_upload_chunk_points(sizes[j], nch);
      for (int c = 0; c < nch; c++) {
        const uint64_t a = std::min<uint64_t>((uint64_t)c * per, sizes[j]);
        const uint64_t b = std::min<uint64_t>(a + per, sizes[j]);
        if (b > a)
          CK(cudaMemcpyAsync((char *)ws.scalars[slot].p + a * 32, h_scalars + first[j] + a,
                             (b - a) * 32, cudaMemcpyHostToDevice, cx->copy_stream));
        CK(cudaEventRecord(cx->chunk_ev[slot][c], cx->copy_stream));
      }
      // every kernel after the chunked histogram is ordered after the last chunk's event
      src = ws.scalars[slot].p;
      chunks = cx->chunk_ev[slot];
    }
    if (enqueue_pass(cx, ws, pl, src, cx->stream, use_graph, cx->timing, j, chunks,
                     chunks ? Ctx::kCopyChunks : 0, pull))
      return g_err;
    if (!d_scalars) CK(cudaEventRecord(cx->freed[(int)(j & 1)], cx->stream));
    if (cx->timing) {
      if (check_pass_errors(ws, cx->stream, cx->last_stats)) return g_err;
      record_timings(cx, ws);
      cx->last_stats[3] = pl.n_buckets;
    }
  }
  if (check_pass_errors(ws, cx->stream, cx->timing ? nullptr : cx->last_stats)) return g_err;
  memcpy(out, ws.res_host.p, m * MSM_PROJ_BYTES);
  return 0;
}

// ---------------------------------------------------------------------------------------------
// init: resident bases
// ---------------------------------------------------------------------------------------------
// Tuned configurations persisted by msm_tune (one line per size class:
// "log2n c signed seg_len red_log2 ms fixed"); the last line for a size class wins.
void load_tune_cache(Ctx *cx) {
  const char *path = getenv("MSM_TUNE_CACHE");
  if (!path) return;
  FILE *f = fopen(path, "r");
  if (!f) return;
  unsigned lg, c, sg, seg, red, fx;
  double ms;
  char line[256];
  while (fgets(line, sizeof(line), f)) {
    fx = 0;  // a seventh field (1: the fixed-base form) is optional
    // lines starting with "b" hold forms tuned for MSMs sharing a pass (msm_tune_uneven)
    const bool shared = line[0] == 'b';
    if (sscanf(line + (shared ? 1 : 0), "%u %u %u %u %u %lf %u", &lg, &c, &sg, &seg, &red, &ms, &fx) < 6)
      continue;
    if (lg > 40 || c < 4 || c > 24 || seg == 0 || seg > 4096 || red > 12) continue;
    Cfg cf;
    cf.c = c;
    cf.signed_digits = sg ? 1 : 0;
    cf.seg_len = seg;
    cf.red_log2 = red;
    cf.fixed = fx <= 2 ? fx : 0;
    (shared ? cx->tuned_batch : cx->tuned)[lg] = cf;
  }
  fclose(f);
}

int init_device(Ctx *cx) {
  const char *dev = getenv("MSM_DEVICE");
  cx->device = dev ? atoi(dev) : 0;
  CK(cudaSetDevice(cx->device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, cx->device));
  cx->num_sms = prop.multiProcessorCount;
  // kernels read pageable host memory through the host's page tables (address translation
  // services over a coherent link, as on Grace); HMM systems report pageable access without
  // host page tables and keep the copy path
  int pageable = 0, host_tables = 0;
  CK(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, cx->device));
  CK(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                            cx->device));
  const char *hp = getenv("MSM_HOST_PULL");
  cx->host_pull = pageable != 0 && host_tables != 0 && !(hp && strcmp(hp, "0") == 0);
  CK(cudaStreamCreateWithFlags(&cx->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&cx->copy_stream, cudaStreamNonBlocking));
  for (int i = 0; i < 2; i++) {
    CK(cudaEventCreateWithFlags(&cx->copied[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&cx->freed[i], cudaEventDisableTiming));
    CK(cudaEventRecord(cx->freed[i], cx->stream));
    for (auto &e : cx->chunk_ev[i]) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  return 0;
}

// Width of the fixed-base tables for n resident bases (0: none).  MSM_FIXED_BASE=0 turns them
// off, MSM_FIXED_BASE=<c> forces window width c; by default they are built for n >= 2^20 when
// n * W * 144 bytes fit in MSM_FIXED_BASE_MAX_GB (default 160) and leave 16 GiB of HBM free.
uint32_t choose_fixed_base(uint64_t n) {
  const char *e = getenv("MSM_FIXED_BASE");
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
  double budget = 160.0 * (1ull << 30);
  if (const char *g = getenv("MSM_FIXED_BASE_MAX_GB")) budget = atof(g) * (1ull << 30);
  budget = std::min(budget, (double)free_b - 16.0 * (1ull << 30));
  auto fits = [&](uint32_t c) {
    const uint32_t w = windows_of(c);
    return w <= 24 && (double)n * w * MSM_BASE_BYTES <= budget &&
           (double)n * w < 2147483647.0;
  };
  if (e) {
    if (!strcmp(e, "0") || !strcmp(e, "off")) return 0;
    const int c = atoi(e);
    if (c >= 11 && c <= 24 && windows_of(c) <= 24 &&
        (double)n * windows_of(c) < 2147483647.0)
      return (uint32_t)c;
    if (strcmp(e, "auto")) return 0;
  }
  // below 2^20 bases MSMs are latency-bound: the windowed form's serial combine (c (W - 1)
  // dependent doublings, ~1.2 ms) dominates, and tables of width 16 (16 windows, 2^15 shared
  // buckets, at most 2.4 GB) measured fastest or within 5% at 2^12..2^18 bases
  if (n < (1ull << 20)) return fits(16) ? 16u : 0u;
  uint32_t best = 0;
  double best_cost = 1e300;
  for (uint32_t c = 11; c <= 24; c++) {
    if (!fits(c)) continue;
    const double v = model_cost_fixed(n, c, 1);
    if (v < best_cost) {
      best_cost = v;
      best = c;
    }
  }
  return best;
}

// A second table set of width 16 for contexts of 2^20 bases or more whose main tables are
// wider: the context's small MSMs (slices of a few thousand to a few hundred thousand points)
// then skip the windowed form's serial window combine too.  Built when the automatic choice
// made the main set (MSM_FIXED_BASE unset or "auto") and both sets fit the table budget.
uint32_t choose_small_tables(uint64_t n, uint32_t fb_c, uint32_t fb_w) {
  const char *e = getenv("MSM_FIXED_BASE");
  if (e && strcmp(e, "auto")) return 0;
  if (!fb_c || fb_c == 16 || n < (1ull << 20)) return 0;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
  double budget = 160.0 * (1ull << 30);
  if (const char *g = getenv("MSM_FIXED_BASE_MAX_GB")) budget = atof(g) * (1ull << 30);
  budget = std::min(budget, (double)free_b - 16.0 * (1ull << 30));
  const double w = fb_w + windows_of(16);
  if ((double)n * w * MSM_BASE_BYTES > budget || (double)n * w >= 2147483647.0) return 0;
  return 16;
}

int load_bases(Ctx *cx, const g1_affine_t *points, uint64_t n) {
  cx->npoints = n;
  cx->fb_c = choose_fixed_base(n);
  cx->fb_w = cx->fb_c ? windows_of(cx->fb_c) : 1;
  cx->fb2_c = choose_small_tables(n, cx->fb_c, cx->fb_w);
  cx->fb2_w = cx->fb2_c ? windows_of(cx->fb2_c) : 0;
  CK(cx->bases.ensure(std::max<uint64_t>(n, 1) * (cx->fb_w + cx->fb2_w) * MSM_BASE_BYTES));
  CK(cx->flags.ensure(std::max<uint64_t>(n, 1)));
  CK(cx->special_idx.ensure(std::max<uint64_t>(n, 1) * 4));
  DevBuf cnt, staging;
  CK(cnt.ensure(4));
  CK(cudaMemsetAsync(cnt.p, 0, 4, cx->stream));
  const uint64_t chunk = std::min<uint64_t>(std::max<uint64_t>(n, 1), 1ull << 22);
  CK(staging.ensure(chunk * MSM_AFFINE_BYTES));
  for (uint64_t i0 = 0; i0 < n; i0 += chunk) {
    const uint64_t k = std::min(chunk, n - i0);
    CK(cudaMemcpyAsync(staging.p, points + i0, k * MSM_AFFINE_BYTES, cudaMemcpyHostToDevice,
                       cx->stream));
    CK(msm_launch_precompute(staging.p, k, cx->bases.as<uint4>() + i0 * 9,
                             cx->flags.as<uint8_t>() + i0, cx->special_idx.as<uint32_t>(),
                             cnt.as<uint32_t>(), (uint32_t)i0, cx->stream));
  }
  if (cx->fb_c) {
    DevBuf fb_fail;
    CK(fb_fail.ensure(4));
    CK(cudaMemsetAsync(fb_fail.p, 0, 4, cx->stream));
    const uint64_t fchunk = 1ull << 20;
    for (uint64_t i0 = 0; i0 < n; i0 += fchunk)
      CK(msm_launch_fixed_base(cx->bases.as<uint4>(), cx->flags.as<uint8_t>(), n, i0,
                               std::min(fchunk, n - i0), cx->fb_c, cx->fb_w,
                               fb_fail.as<uint32_t>(), cx->stream));
    uint32_t nfail = 0;
    CK(cudaMemcpyAsync(&nfail, fb_fail.p, 4, cudaMemcpyDeviceToHost, cx->stream));
    CK(cudaStreamSynchronize(cx->stream));
    if (nfail) {  // a base of 2-power order: keep the plain table only
      cx->fb_c = 0;
      cx->fb_w = 1;
      cx->fb2_c = 0;
      cx->fb2_w = 0;
    }
  }
  if (cx->fb2_c) {  // the width-16 set: window 0 is the plain table again
    uint4 *region = cx->bases.as<uint4>() + n * cx->fb_w * 9;
    CK(cudaMemcpyAsync(region, cx->bases.p, n * MSM_BASE_BYTES, cudaMemcpyDeviceToDevice,
                       cx->stream));
    DevBuf fb_fail;
    CK(fb_fail.ensure(4));
    CK(cudaMemsetAsync(fb_fail.p, 0, 4, cx->stream));
    const uint64_t fchunk = 1ull << 20;
    for (uint64_t i0 = 0; i0 < n; i0 += fchunk)
      CK(msm_launch_fixed_base(region, cx->flags.as<uint8_t>(), n, i0, std::min(fchunk, n - i0),
                               cx->fb2_c, cx->fb2_w, fb_fail.as<uint32_t>(), cx->stream));
    uint32_t nfail = 0;
    CK(cudaMemcpyAsync(&nfail, fb_fail.p, 4, cudaMemcpyDeviceToHost, cx->stream));
    CK(cudaStreamSynchronize(cx->stream));
    if (nfail) {
      cx->fb2_c = 0;
      cx->fb2_w = 0;
    }
  }
  uint32_t nspecial = 0;
  CK(cudaMemcpyAsync(&nspecial, cnt.p, 4, cudaMemcpyDeviceToHost, cx->stream));
  CK(cudaStreamSynchronize(cx->stream));
  // reject coordinates that are not reduced field elements
  {
    std::vector<uint8_t> fl(n);
    CK(cudaMemcpy(fl.data(), cx->flags.p, n, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < n; i++)
      if (fl[i] == BASE_BAD_INPUT)
        return fail(ERR_INPUT, "point %llu: coordinate not below the field modulus",
                    (unsigned long long)i);
  }
  cx->n_special = nspecial;
  cx->n_classes = 0;
  if (nspecial) {
    // group the special bases into classes of equal points (at most 5 exist on the curve:
    // three of order 2 with y = 0 and two of order 4 with Montgomery u = -1)
    std::vector<uint32_t> idx(nspecial);
    CK(cudaMemcpy(idx.data(), cx->special_idx.p, nspecial * 4, cudaMemcpyDeviceToHost));
    std::sort(idx.begin(), idx.end());
    CK(cudaMemcpy(cx->special_idx.p, idx.data(), nspecial * 4, cudaMemcpyHostToDevice));
    std::vector<uint8_t> cls(nspecial);
    std::vector<uint32_t> class_words;  // 24 u32 per class: x then y
    for (uint32_t s = 0; s < nspecial; s++) {
      const g1_affine_t &p = points[idx[s]];
      int found = -1;
      for (uint32_t c = 0; c < cx->n_classes; c++)
        if (!memcmp(&class_words[c * 24], p.x.data, 48) &&
            !memcmp(&class_words[c * 24 + 12], p.y.data, 48))
          found = (int)c;
      if (found < 0) {
        if (cx->n_classes == 8)
          return fail(ERR_INPUT, "more than 8 distinct points without a twisted-Edwards image");
        class_words.resize((cx->n_classes + 1) * 24);
        memcpy(&class_words[cx->n_classes * 24], p.x.data, 48);
        memcpy(&class_words[cx->n_classes * 24 + 12], p.y.data, 48);
        found = (int)cx->n_classes++;
      }
      cls[s] = (uint8_t)found;
    }
    CK(cx->special_cls.ensure(nspecial));
    CK(cudaMemcpy(cx->special_cls.p, cls.data(), nspecial, cudaMemcpyHostToDevice));
    CK(cx->class_pts.ensure(cx->n_classes * 96));
    CK(cudaMemcpy(cx->class_pts.p, class_words.data(), cx->n_classes * 96, cudaMemcpyHostToDevice));
    DevBuf ok;
    CK(ok.ensure(cx->n_classes * 4));
    CK(msm_launch_check_classes(cx->class_pts.as<uint4>(), cx->n_classes, ok.as<uint32_t>(),
                                cx->stream));
    std::vector<uint32_t> okh(cx->n_classes);
    CK(cudaMemcpyAsync(okh.data(), ok.p, cx->n_classes * 4, cudaMemcpyDeviceToHost, cx->stream));
    CK(cudaStreamSynchronize(cx->stream));
    for (uint32_t c = 0; c < cx->n_classes; c++)
      if (!okh[c])
        return fail(ERR_INPUT, "a point without a twisted-Edwards image is not a curve point of "
                               "order 2 or 4");
  } else {
    CK(cx->special_cls.ensure(1));
    CK(cx->class_pts.ensure(96));
  }
  return 0;
}

// ---------------------------------------------------------------------------------------------
// host generators (SplitMix64, counter-based; the same function as the oracle's and the GPU's)
// ---------------------------------------------------------------------------------------------
inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline uint64_t rand_u64(uint64_t seed, uint64_t stream, uint64_t index, uint64_t word) {
  const uint64_t s = splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull));
  const uint64_t h = splitmix64(s ^ splitmix64(index));
  return splitmix64(h + word);
}
inline bool lt_r(const uint64_t *v) {
  for (int k = 3; k >= 0; k--) {
    if (v[k] < R_WORDS[k]) return true;
    if (v[k] > R_WORDS[k]) return false;
  }
  return false;
}
void uniform_scalar(uint64_t seed, uint64_t i, uint64_t *out, uint64_t stream = 2) {
  for (uint64_t a = 0;; a++) {
    for (int j = 0; j < 4; j++) out[j] = rand_u64(seed, stream, i, 4 * a + j);
    out[3] &= (1ull << 61) - 1;
    if (lt_r(out)) return;
  }
}
void mixed_scalar(uint64_t seed, uint64_t msm, uint64_t i, uint64_t *out) {
  const uint64_t key = (msm << 32) | i;
  const uint64_t sel = rand_u64(seed, 3, key, 0) % 10;
  if (sel < 7) return uniform_scalar(seed, key, out);
  if (sel == 7) {
    out[0] = rand_u64(seed, 3, key, 1) & 0xffff;
    out[1] = out[2] = out[3] = 0;
    return;
  }
  if (sel == 8) {
    if ((rand_u64(seed, 3, key, 2) & 1) == 0) {
      out[0] = out[1] = out[2] = out[3] = 0;
    } else {
      for (int k = 0; k < 4; k++) out[k] = R_WORDS[k];
      out[0] -= 1;
    }
    return;
  }
  uniform_scalar(seed, (msm << 32) | 0xffffffffull, out);
}

// ---------------------------------------------------------------------------------------------
// server: continuous batching
// ---------------------------------------------------------------------------------------------
struct Request {
  int64_t id;
  uint64_t n, base_off;
  std::vector<biginteger256_t> scalars;
  uint8_t result[MSM_PROJ_BYTES];
  int status = 1;  // 1 pending/running, 0 done, <0 error
  std::chrono::steady_clock::time_point t_submit, t_done;
};

// Server passes of at most this many points run on their slot's high-priority stream.
constexpr uint64_t kServerSmallPass = 1ull << 19;

struct Slot {
  Workspace ws;
  cudaStream_t st = nullptr;     // passes of many points, at the lowest stream priority
  cudaStream_t st_hi = nullptr;  // passes of few points, at the highest
  cudaEvent_t done = nullptr;
  bool busy = false;
  uint64_t bytes = 0;
  std::vector<std::shared_ptr<Request>> reqs;
  DevBuf scal;
  Plan plan;
};

struct Server {
  Ctx *cx = nullptr;
  uint64_t budget = 0;
  int max_inflight = 2;
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cv, cv_done;
  std::deque<std::shared_ptr<Request>> pending;
  std::unordered_map<int64_t, std::shared_ptr<Request>> all;
  std::atomic<bool> stop{false};
  std::thread worker;
  int64_t next_id = 0;
  uint64_t bytes_in_use = 0;
  msm_server_stats_t stats{};

  uint64_t request_bytes(uint64_t n) {
    std::vector<JobSpec> one(1);
    one[0] = {n, 0, 0, resolve_cfg(cx, n, nullptr)};
    set_tables(cx, one[0]);
    Plan pl;
    if (build_plan(one, pl)) return ~0ull;
    return plan_bytes(pl, true);
  }

  void loop();
};

void Server::loop() {
  std::unique_lock<std::mutex> lk(mu);
  while (!stop) {
    // retire finished passes
    bool any_done = false;
    for (auto &sl : slots) {
      if (!sl->busy) continue;
      if (cudaEventQuery(sl->done) == cudaSuccess) {
        uint32_t cnt[CNT_WORDS];
        cudaMemcpy(cnt, sl->ws.counters.p, sizeof(cnt), cudaMemcpyDeviceToHost);
        const auto now = std::chrono::steady_clock::now();
        for (size_t j = 0; j < sl->reqs.size(); j++) {
          auto &r = sl->reqs[j];
          memcpy(r->result, (char *)sl->ws.res_host.p + j * MSM_PROJ_BYTES, MSM_PROJ_BYTES);
          r->status = cnt[CNT_ERROR] ? ERR_STATE : 0;
          r->t_done = now;
          stats.completed++;
        }
        sl->reqs.clear();
        bytes_in_use -= sl->bytes;
        sl->bytes = 0;
        sl->busy = false;
        any_done = true;
      }
    }
    if (any_done) cv_done.notify_all();
    // admit: every pending request that fits the budget joins one pass on a free slot
    Slot *free_slot = nullptr;
    for (auto &sl : slots)
      if (!sl->busy) {
        free_slot = sl.get();
        break;
      }
    if (free_slot && !pending.empty()) {
      std::vector<std::shared_ptr<Request>> batch;
      uint64_t bytes = 0, total_n = 0;
      while (!pending.empty()) {
        auto &r = pending.front();
        const uint64_t b = request_bytes(r->n);
        if (bytes_in_use + bytes + b > budget && !batch.empty()) break;
        if (bytes_in_use + bytes + b > budget && bytes_in_use > 0) break;
        bytes += b;
        total_n += r->n;
        batch.push_back(r);
        pending.pop_front();
      }
      if (!batch.empty()) {
        std::vector<JobSpec> specs(batch.size());
        uint64_t maxn = 0, first = 0;
        for (auto &r : batch) maxn = std::max(maxn, r->n);
        const bool shared = batch.size() > 1;
        const Cfg big = resolve_cfg(cx, maxn, nullptr, shared);
        for (size_t j = 0; j < batch.size(); j++) {
          specs[j] = {batch[j]->n, batch[j]->base_off, first,
                      resolve_cfg(cx, batch[j]->n, nullptr, shared)};
          specs[j].cfg.seg_len = big.seg_len;
          specs[j].cfg.red_log2 = big.red_log2;
          set_tables(cx, specs[j]);
          first += batch[j]->n;
        }
        if (specs.size() > 1) {
          const uint32_t seg = pass_seg_len(specs);
          for (JobSpec &sp : specs) sp.cfg.seg_len = seg;
        }
        Slot &sl = *free_slot;
        // a pass of few points goes ahead of a large one: its kernels take SM space first as the
        // large pass's blocks retire, and the large pass's k_accumulate leaves a quarter of
        // every SM free for them (slots' workspaces run it with 3 blocks per SM)
        cudaStream_t st = total_n <= kServerSmallPass ? sl.st_hi : sl.st;
        int rc = build_plan(specs, sl.plan);
        if (!rc && sl.scal.ensure(std::max<uint64_t>(first, 1) * 32) != cudaSuccess)
          rc = fail(ERR_CUDA, "server scalar buffer allocation failed");
        if (!rc) {
          uint64_t off = 0;
          for (auto &r : batch) {
            if (r->n)
              cudaMemcpyAsync((char *)sl.scal.p + off * 32, r->scalars.data(), r->n * 32,
                              cudaMemcpyHostToDevice, st);
            off += r->n;
          }
          rc = enqueue_pass(cx, sl.ws, sl.plan, sl.scal.p, st, false, false, 0);
        }
        if (!rc) rc = cudaEventRecord(sl.done, st) == cudaSuccess ? 0 : ERR_CUDA;
        if (rc) {
          for (auto &r : batch) {
            r->status = rc;
            r->t_done = std::chrono::steady_clock::now();
          }
          cv_done.notify_all();
        } else {
          sl.busy = true;
          sl.bytes = bytes;
          sl.reqs = batch;
          bytes_in_use += bytes;
          stats.passes++;
          stats.bytes_peak = std::max(stats.bytes_peak, bytes_in_use);
          uint64_t inflight = 0;
          for (auto &s2 : slots) inflight += s2->busy;
          stats.inflight_peak = std::max(stats.inflight_peak, inflight);
        }
        continue;
      }
    }
    bool busy = false;
    for (auto &sl : slots) busy |= sl->busy;
    if (busy) {
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(50));
      lk.lock();
    } else {
      cv.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

int msm_last_error(char *buf, size_t len) {
  if (buf && len) {
    strncpy(buf, g_msg, len - 1);
    buf[len - 1] = 0;
  }
  return g_err;
}

void *msm_init(const char *xclbin, ssize_t xclbin_len, const g1_affine_t *points, ssize_t npoints) {
  (void)xclbin;
  (void)xclbin_len;
  g_err = 0;
  g_msg[0] = 0;
  if (npoints < 0 || (npoints > 0 && !points)) {
    fail(ERR_ARG, "msm_init: bad point array");
    return nullptr;
  }
  if ((uint64_t)npoints >= (1ull << 31)) {
    fail(ERR_ARG, "msm_init: at most 2^31 - 1 points");
    return nullptr;
  }
  auto *cx = new Ctx();
  load_tune_cache(cx);
  if (init_device(cx) || load_bases(cx, points, (uint64_t)npoints)) {
    fprintf(stderr, "msm_init: %s\n", g_msg);
    delete cx;
    return nullptr;
  }
  return cx;
}

void msm_free(void *context) { delete (Ctx *)context; }

int msm_mult_ex(void *context, g1_projective_t *out, uint64_t batch_size,
                const biginteger256_t *scalars, const msm_options_t *opt) {
  g_err = 0;
  auto *cx = (Ctx *)context;
  if (!cx || (batch_size && (!out || !scalars))) return fail(ERR_ARG, "msm_mult: null argument");
  std::lock_guard<std::mutex> lk(cx->mu);
  if (cudaSetDevice(cx->device) != cudaSuccess) return fail(ERR_DEVICE, "cudaSetDevice failed");
  std::vector<uint64_t> sizes(batch_size, cx->npoints), offs(batch_size, 0);
  int rc = run_msms(cx, out, sizes, offs, scalars, nullptr, opt);
  if (rc && out) memset(out, 0, batch_size * sizeof(g1_projective_t));
  return rc;
}

void msm_mult(void *context, g1_projective_t *out, uint64_t batch_size,
              const biginteger256_t *scalars) {
  if (msm_mult_ex(context, out, batch_size, scalars, nullptr))
    fprintf(stderr, "msm_mult: %s\n", g_msg);
}

// The naive driver's names for the same two calls (host/naive_driver/naive_driver.cpp:109-138),
// which test_naive_harness binds.  There the "fpga" product is a CPU double-and-add loop and the
// "pippenger" product a CPU Pippenger; both are the full MSM, as here.
void *zprize_msm_fpga_init(const g1_affine_t *points, ssize_t npoints) {
  return msm_init(nullptr, 0, points, npoints);
}

void zprize_msm_fpga_mult(void *context, g1_projective_t *out, uint64_t batch_size,
                          const biginteger256_t *scalars) {
  msm_mult(context, out, batch_size, scalars);
}

void zprize_msm_pippenger_mult(void *context, g1_projective_t *out, uint64_t batch_size,
                               const biginteger256_t *scalars) {
  msm_mult(context, out, batch_size, scalars);
}

int msm_mult_uneven(void *context, g1_projective_t *out, uint64_t num_msms, const uint64_t *sizes,
                    const uint64_t *base_offsets, const biginteger256_t *scalars,
                    const msm_options_t *opt) {
  g_err = 0;
  auto *cx = (Ctx *)context;
  if (!cx || (num_msms && (!out || !sizes || !scalars)))
    return fail(ERR_ARG, "msm_mult_uneven: null argument");
  std::lock_guard<std::mutex> lk(cx->mu);
  if (cudaSetDevice(cx->device) != cudaSuccess) return fail(ERR_DEVICE, "cudaSetDevice failed");
  std::vector<uint64_t> sz(sizes, sizes + num_msms), of(num_msms, 0);
  if (base_offsets) of.assign(base_offsets, base_offsets + num_msms);
  int rc = run_msms(cx, out, sz, of, scalars, nullptr, opt);
  if (rc && out) memset(out, 0, num_msms * sizeof(g1_projective_t));
  return rc;
}

int msm_mult_device(void *context, g1_projective_t *out, uint64_t num_msms, const uint64_t *sizes,
                    const uint64_t *base_offsets, const void *d_scalars, const msm_options_t *opt) {
  g_err = 0;
  auto *cx = (Ctx *)context;
  if (!cx || (num_msms && (!out || !sizes || !d_scalars)))
    return fail(ERR_ARG, "msm_mult_device: null argument");
  std::lock_guard<std::mutex> lk(cx->mu);
  if (cudaSetDevice(cx->device) != cudaSuccess) return fail(ERR_DEVICE, "cudaSetDevice failed");
  std::vector<uint64_t> sz(sizes, sizes + num_msms), of(num_msms, 0);
  if (base_offsets) of.assign(base_offsets, base_offsets + num_msms);
  int rc = run_msms(cx, out, sz, of, nullptr, d_scalars, opt);
  if (rc && out) memset(out, 0, num_msms * sizeof(g1_projective_t));
  return rc;
}

int msm_get_config(void *context, uint64_t npoints, msm_options_t *out) {
  auto *cx = (Ctx *)context;
  if (!cx || !out) return fail(ERR_ARG, "msm_get_config: null argument");
  const Cfg c = resolve_cfg(cx, npoints, nullptr);
  out->window_bits = (int32_t)c.c;
  out->signed_digits = c.signed_digits ? 1 : 2;
  out->seg_len = (int32_t)c.seg_len;
  uint32_t red = c.red_log2;
  if (red == 0) {  // what a pass of this one MSM would use
    uint32_t nwin, nb, nbt;
    layout(c.c, c.signed_digits, nwin, nb, nbt);
    red = red_log2_for(c.fixed ? std::max(nb, nbt) : (uint64_t)(nwin - 1) * nb + nbt);
  }
  out->red_len_log2 = (int32_t)red;
  out->use_graph = 0;
  out->mode = 1;
  out->fixed_base = c.fixed ? 1 : 2;
  return 0;
}

int msm_context_info(void *context, uint64_t *info, int32_t max_info) {
  auto *cx = (Ctx *)context;
  if (!cx || !info) return fail(ERR_ARG, "msm_context_info: null argument");
  const uint64_t v[6] = {cx->npoints, (uint64_t)cx->bases.bytes, cx->fb_c, cx->fb_c ? cx->fb_w : 0,
                         cx->fb2_c, cx->fb2_c ? cx->fb2_w : 0};
  const int32_t k = std::min<int32_t>(max_info, 6);
  for (int32_t i = 0; i < k; i++) info[i] = v[i];
  return k;
}

int msm_set_timing(void *context, int32_t enable) {
  auto *cx = (Ctx *)context;
  if (!cx) return fail(ERR_ARG, "null context");
  std::lock_guard<std::mutex> lk(cx->mu);
  cx->timing = enable != 0;
  return 0;
}

int msm_last_timings(void *context, double *ms, int32_t max_stages) {
  auto *cx = (Ctx *)context;
  if (!cx || !ms) return fail(ERR_ARG, "null argument");
  const int n = std::min<int>(max_stages, MSM_NUM_STAGES);
  for (int k = 0; k < n; k++) ms[k] = cx->last_ms[k];
  return n;
}

int msm_last_pass_stats(void *context, uint64_t *stats, int32_t max_stats) {
  auto *cx = (Ctx *)context;
  if (!cx || !stats) return fail(ERR_ARG, "null argument");
  const int n = std::min<int>(max_stats, 5);
  for (int k = 0; k < n; k++) stats[k] = cx->last_stats[k];
  return n;
}

int msm_tune(void *context, uint64_t npoints, int32_t budget_ms, msm_options_t *best_out) {
  g_err = 0;
  auto *cx = (Ctx *)context;
  if (!cx || npoints == 0 || npoints > cx->npoints) return fail(ERR_ARG, "msm_tune: bad size");
  if (budget_ms <= 0) budget_ms = 20000;
  std::vector<biginteger256_t> sc(npoints);
  for (uint64_t i = 0; i < npoints; i++) uniform_scalar(0x7475e3ull, i, sc[i].data);
  const Cfg h = heuristic_cfg(npoints);
  std::vector<Cfg> cands;
  for (int dc = -2; dc <= 2; dc++) {
    const int c = (int)h.c + dc;
    if (c < 6 || c > 21) continue;
    for (uint32_t sg : {1u, 0u}) {
      if (!sg && dc != 0) continue;
      msm_options_t o{};
      o.window_bits = c;
      o.signed_digits = sg ? 1 : 2;
      Cfg cf = resolve_cfg(cx, npoints, &o);
      cands.push_back(cf);
      if (sg && dc == 0) {
        Cfg cf2 = cf;
        cf2.seg_len = std::max<uint32_t>(32, cf.seg_len / 4);
        cands.push_back(cf2);
      }
    }
  }
  for (uint32_t which = 1; which <= 2; which++) {  // each table set, at two run lengths
    const uint32_t tc = which == 1 ? cx->fb_c : cx->fb2_c;
    if (!tc) continue;
    uint32_t nwin, nb, nbt;
    layout(tc, 1, nwin, nb, nbt);
    Cfg cf;
    cf.fixed = which;
    cf.c = tc;
    cf.signed_digits = 1;
    cf.seg_len = seg_len_for(npoints, std::max(nb, nbt), nwin, nwin);
    cf.red_log2 = 0;
    cands.push_back(cf);
    Cfg cf2 = cf;
    cf2.seg_len = std::max<uint32_t>(16, cf.seg_len / 4);
    cands.push_back(cf2);
  }
  std::lock_guard<std::mutex> lk(cx->mu);
  if (cudaSetDevice(cx->device) != cudaSuccess) return fail(ERR_DEVICE, "cudaSetDevice failed");
  DevBuf dsc;
  CK(dsc.ensure(npoints * 32));
  CK(cudaMemcpy(dsc.p, sc.data(), npoints * 32, cudaMemcpyHostToDevice));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const auto t_start = std::chrono::steady_clock::now();
  double best_ms = 1e300;
  Cfg best = h;
  for (const Cfg &cf : cands) {
    std::vector<JobSpec> one(1);
    one[0] = {npoints, 0, 0, cf};
    set_tables(cx, one[0]);
    Plan pl;
    if (build_plan(one, pl)) continue;
    double t = 1e300;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, cx->stream);
      if (enqueue_pass(cx, cx->ws, pl, dsc.p, cx->stream, false, false, 0)) break;
      cudaEventRecord(e1, cx->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) break;
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) t = std::min(t, (double)ms);
    }
    if (t < best_ms) {
      best_ms = t;
      best = cf;
    }
    const double spent = std::chrono::duration<double, std::milli>(
                             std::chrono::steady_clock::now() - t_start).count();
    if (spent > budget_ms) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lk(cx->tune_mu);
    cx->tuned[log2_ceil(npoints)] = best;
  }
  if (const char *path = getenv("MSM_TUNE_CACHE")) {
    if (FILE *f = fopen(path, "a")) {
      fprintf(f, "%u %u %u %u %u %.4f %u\n", log2_ceil(npoints), best.c, best.signed_digits,
              best.seg_len, best.red_log2, best_ms, best.fixed);  // fixed: 0, 1 main, 2 width 16
      fclose(f);
    }
  }
  if (best_out) {
    best_out->window_bits = (int32_t)best.c;
    best_out->signed_digits = best.signed_digits ? 1 : 2;
    best_out->seg_len = (int32_t)best.seg_len;
    best_out->red_len_log2 = (int32_t)best.red_log2;
    best_out->use_graph = 0;
    best_out->mode = 1;
    best_out->fixed_base = best.fixed ? 1 : 2;
  }
  return 0;
}

int msm_tune_uneven(void *context, uint64_t num_msms, const uint64_t *sizes,
                    const uint64_t *base_offsets, const biginteger256_t *scalars, int32_t budget_ms,
                    msm_options_t *best_out, double *report) {
  g_err = 0;
  auto *cx = (Ctx *)context;
  if (!cx || num_msms == 0 || !sizes || !base_offsets || !scalars)
    return fail(ERR_ARG, "msm_tune_uneven: null argument");
  const size_t m = num_msms;
  std::vector<uint64_t> first(m + 1, 0);
  for (size_t j = 0; j < m; j++) {
    if (base_offsets[j] > cx->npoints || sizes[j] > cx->npoints - base_offsets[j])
      return fail(ERR_ARG, "msm_tune_uneven: MSM %zu outside the resident bases", j);
    first[j + 1] = first[j] + sizes[j];
  }
  if (budget_ms <= 0) budget_ms = 20000;
  std::lock_guard<std::mutex> lk(cx->mu);
  if (cudaSetDevice(cx->device) != cudaSuccess) return fail(ERR_DEVICE, "cudaSetDevice failed");
  DevBuf dsc;
  CK(dsc.ensure(std::max<uint64_t>(first[m], 1) * 32));
  if (first[m]) CK(cudaMemcpy(dsc.p, scalars, first[m] * 32, cudaMemcpyHostToDevice));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const auto t_start = std::chrono::steady_clock::now();
  auto spent_ms = [&] {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start)
        .count();
  };
  // one pass of the whole mix with the forms in `form` (by size class) and the pass-level run
  // length (0: the automatic rule) and level-1 reduction run (0: automatic); best of 2 timed runs
  auto time_pass = [&](const std::map<uint32_t, Cfg> &form, uint32_t seg, uint32_t red) -> double {
    std::vector<JobSpec> specs(m);
    for (size_t j = 0; j < m; j++) {
      specs[j] = {sizes[j], base_offsets[j], first[j], form.at(log2_ceil(std::max<uint64_t>(sizes[j], 1)))};
      specs[j].cfg.red_log2 = red;
      set_tables(cx, specs[j]);
    }
    const uint32_t s2 = seg ? seg : pass_seg_len(specs);
    for (JobSpec &sp : specs) sp.cfg.seg_len = s2;
    Plan pl;
    if (build_plan(specs, pl)) return 1e300;
    double t = 1e300;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, cx->stream);
      if (enqueue_pass(cx, cx->ws, pl, dsc.p, cx->stream, false, false, 0)) return 1e300;
      cudaEventRecord(e1, cx->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) return 1e300;
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) t = std::min(t, (double)ms);
    }
    uint32_t cnt[CNT_WORDS];
    if (cudaMemcpy(cnt, cx->ws.counters.p, sizeof(cnt), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cnt[CNT_ERROR])
      return 1e300;
    return t;
  };
  // size classes, largest total points first, and their starting forms: what a shared pass
  // would use untuned (the cost model's choice at the class's largest size)
  std::map<uint32_t, uint64_t> pts_of, max_of;
  for (size_t j = 0; j < m; j++) {
    const uint32_t cls = log2_ceil(std::max<uint64_t>(sizes[j], 1));
    pts_of[cls] += sizes[j];
    max_of[cls] = std::max(max_of[cls], sizes[j]);
  }
  std::map<uint32_t, Cfg> form;
  for (auto &kv : max_of) form[kv.first] = resolve_cfg(cx, kv.second, nullptr, false);
  std::vector<uint32_t> order;
  for (auto &kv : pts_of) order.push_back(kv.first);
  std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return pts_of[a] > pts_of[b]; });
  const double untuned = time_pass(form, 0, 0);
  double best = untuned;
  int measured = 1;
  // coordinate descent over the classes: windowed signed c = 10..16, windowed unsigned at the
  // best windowed width, and each table set of the context
  for (uint32_t cls : order) {
    if (spent_ms() > budget_ms) break;
    std::vector<Cfg> cands;
    for (uint32_t c = 10; c <= 16; c++) {
      Cfg cf;
      cf.c = c;
      cf.signed_digits = 1;
      cf.fixed = 0;
      cands.push_back(cf);
    }
    for (uint32_t which = 1; which <= 2; which++) {
      const uint32_t tc = which == 1 ? cx->fb_c : cx->fb2_c;
      if (!tc) continue;
      Cfg cf;
      cf.c = tc;
      cf.signed_digits = 1;
      cf.fixed = which;
      cands.push_back(cf);
    }
    uint32_t best_windowed_c = form[cls].fixed ? 0 : form[cls].c;
    double best_windowed = 1e300;
    for (size_t k = 0; k <= cands.size(); k++) {
      if (spent_ms() > budget_ms) break;
      Cfg cf;
      if (k < cands.size()) {
        cf = cands[k];
      } else {  // unsigned digits at the best windowed width
        if (!best_windowed_c) break;
        cf.c = std::min<uint32_t>(best_windowed_c, 16);
        cf.signed_digits = 0;
        cf.fixed = 0;
      }
      std::map<uint32_t, Cfg> trial = form;
      trial[cls] = cf;
      const double t = time_pass(trial, 0, 0);
      measured++;
      if (!cf.fixed && cf.signed_digits && t < best_windowed) {
        best_windowed = t;
        best_windowed_c = cf.c;
      }
      if (t < best) {
        best = t;
        form[cls] = cf;
      }
    }
  }
  // pass-level knobs: run length (how many threads share a heavy bucket) and level-1 reduction
  uint32_t best_seg = 0, best_red = 0;
  {
    std::vector<JobSpec> specs(m);
    for (size_t j = 0; j < m; j++) {
      specs[j] = {sizes[j], base_offsets[j], first[j], form.at(log2_ceil(std::max<uint64_t>(sizes[j], 1)))};
      set_tables(cx, specs[j]);
    }
    const uint32_t auto_seg = pass_seg_len(specs);
    for (uint32_t seg : {auto_seg / 4, auto_seg / 2, auto_seg * 2, auto_seg * 4}) {
      if (seg < 8 || seg > 4096 || spent_ms() > budget_ms) continue;
      const double t = time_pass(form, seg, 0);
      measured++;
      if (t < best) {
        best = t;
        best_seg = seg;
      }
    }
    for (uint32_t red = 2; red <= 6; red++) {
      if (spent_ms() > budget_ms) break;
      const double t = time_pass(form, best_seg, red);
      measured++;
      if (t < best) {
        best = t;
        best_red = red;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lk(cx->tune_mu);
    for (auto &kv : form) cx->tuned_batch[kv.first] = kv.second;
  }
  if (const char *path = getenv("MSM_TUNE_CACHE")) {
    if (FILE *f = fopen(path, "a")) {
      for (auto &kv : form)
        fprintf(f, "b %u %u %u %u %u %.4f %u\n", kv.first, kv.second.c, kv.second.signed_digits,
                kv.second.seg_len, kv.second.red_log2, best, kv.second.fixed);
      fclose(f);
    }
  }
  if (best_out) {
    *best_out = msm_options_t{};
    best_out->seg_len = (int32_t)best_seg;
    best_out->red_len_log2 = (int32_t)best_red;
    best_out->mode = 2;
  }
  if (report) {
    report[0] = untuned;
    report[1] = best;
    report[2] = measured;
  }
  return 0;
}

int msm_tuned_form(void *context, uint64_t npoints, int32_t shared_pass, msm_options_t *out) {
  auto *cx = (Ctx *)context;
  if (!cx || !out) return fail(ERR_ARG, "msm_tuned_form: null argument");
  const Cfg c = resolve_cfg(cx, npoints, nullptr, shared_pass != 0);
  *out = msm_options_t{};
  out->window_bits = (int32_t)c.c;
  out->signed_digits = c.signed_digits ? 1 : 2;
  out->seg_len = (int32_t)c.seg_len;
  out->red_len_log2 = (int32_t)c.red_log2;
  out->fixed_base = (int32_t)c.fixed;  // 0 plain records, 1 main tables, 2 width-16 tables
  out->mode = shared_pass ? 2 : 1;
  return 0;
}

void *msm_server_create(void *context, uint64_t hbm_budget_bytes, int32_t max_inflight) {
  g_err = 0;
  auto *cx = (Ctx *)context;
  if (!cx || max_inflight <= 0) {
    fail(ERR_ARG, "msm_server_create: bad argument");
    return nullptr;
  }
  auto *sv = new Server();
  sv->cx = cx;
  sv->budget = hbm_budget_bytes;
  sv->max_inflight = max_inflight;
  int prio_least = 0, prio_greatest = 0;
  if (cudaSetDevice(cx->device) != cudaSuccess ||
      cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest) != cudaSuccess) {
    fail(ERR_CUDA, "msm_server_create: stream priorities unavailable");
    delete sv;
    return nullptr;
  }
  for (int i = 0; i < max_inflight; i++) {
    auto sl = std::make_unique<Slot>();
    const bool ok =
        cudaStreamCreateWithPriority(&sl->st, cudaStreamNonBlocking, prio_least) == cudaSuccess &&
        cudaStreamCreateWithPriority(&sl->st_hi, cudaStreamNonBlocking, prio_greatest) == cudaSuccess &&
        cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming) == cudaSuccess;
    // with passes in flight side by side, k_accumulate leaves room on every SM for the others
    if (max_inflight > 1) sl->ws.acc_blocks_per_sm = 3;
    sv->slots.push_back(std::move(sl));
    if (!ok) {
      fail(ERR_CUDA, "msm_server_create: stream creation failed");
      msm_server_destroy(sv);
      return nullptr;
    }
  }
  sv->worker = std::thread([sv] {
    cudaSetDevice(sv->cx->device);
    sv->loop();
  });
  return sv;
}

int64_t msm_server_submit(void *server, const biginteger256_t *scalars, uint64_t n,
                          uint64_t base_offset) {
  auto *sv = (Server *)server;
  if (!sv || (n && !scalars)) return fail(ERR_ARG, "msm_server_submit: null argument");
  if (base_offset > sv->cx->npoints || n > sv->cx->npoints - base_offset)
    return fail(ERR_ARG, "msm_server_submit: bases outside the resident set");
  const uint64_t need = sv->request_bytes(n);
  if (need > sv->budget)
    return fail(ERR_BUDGET, "request of %llu points needs %llu bytes, over the %llu byte budget",
                (unsigned long long)n, (unsigned long long)need, (unsigned long long)sv->budget);
  auto r = std::make_shared<Request>();
  r->n = n;
  r->base_off = base_offset;
  r->scalars.assign(scalars, scalars + n);
  r->t_submit = std::chrono::steady_clock::now();
  std::lock_guard<std::mutex> lk(sv->mu);
  r->id = sv->next_id++;
  sv->all[r->id] = r;
  sv->pending.push_back(r);
  sv->stats.submitted++;
  sv->cv.notify_all();
  return r->id;
}

int msm_server_poll(void *server, int64_t id, g1_projective_t *out, int32_t wait_ms,
                    double *latency_ms) {
  auto *sv = (Server *)server;
  if (!sv) return fail(ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->all.find(id);
  if (it == sv->all.end()) return fail(ERR_ARG, "unknown request id %lld", (long long)id);
  auto r = it->second;
  if (r->status == 1 && wait_ms > 0)
    sv->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return r->status != 1; });
  if (r->status == 1) return 1;
  if (r->status < 0) return fail(r->status, "request %lld failed", (long long)id);
  if (out) memcpy(out, r->result, MSM_PROJ_BYTES);
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  sv->all.erase(it);
  return 0;
}

int msm_server_stats(void *server, msm_server_stats_t *st) {
  auto *sv = (Server *)server;
  if (!sv || !st) return fail(ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  *st = sv->stats;
  st->bytes_in_use = sv->bytes_in_use;
  return 0;
}

void msm_server_destroy(void *server) {
  auto *sv = (Server *)server;
  if (!sv) return;
  sv->stop = true;
  sv->cv.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  for (auto &sl : sv->slots) {
    for (cudaStream_t x : {sl->st, sl->st_hi})
      if (x) {
        cudaStreamSynchronize(x);
        cudaStreamDestroy(x);
      }
    if (sl->done) cudaEventDestroy(sl->done);
  }
  delete sv;
}

int msm_generate_bases(uint64_t seed, uint64_t first, uint64_t n, g1_affine_t *out) {
  g_err = 0;
  if (n && !out) return fail(ERR_ARG, "null output");
  const char *dev = getenv("MSM_DEVICE");
  CK(cudaSetDevice(dev ? atoi(dev) : 0));
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  DevBuf table, buf;
  int rc = 0;
  if (table.ensure(2048 * MSM_BASE_BYTES) != cudaSuccess) rc = fail(ERR_CUDA, "alloc failed");
  if (!rc && msm_build_gen_table(table.as<uint4>(), st) != cudaSuccess)
    rc = fail(ERR_CUDA, "table launch failed");
  const uint64_t chunk = std::min<uint64_t>(std::max<uint64_t>(n, 1), 1ull << 22);
  if (!rc && buf.ensure(chunk * MSM_AFFINE_BYTES) != cudaSuccess) rc = fail(ERR_CUDA, "alloc failed");
  for (uint64_t i0 = 0; !rc && i0 < n; i0 += chunk) {
    const uint64_t k = std::min(chunk, n - i0);
    if (msm_launch_gen_bases(seed, first + i0, k, buf.p, table.as<uint4>(), st) != cudaSuccess ||
        cudaMemcpyAsync(out + i0, buf.p, k * MSM_AFFINE_BYTES, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = fail(ERR_CUDA, "base generation failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return rc;
}

int msm_generate_scalars(uint64_t seed, uint64_t n, int32_t kind, uint64_t msm_index,
                         biginteger256_t *out) {
  if (n && !out) return fail(ERR_ARG, "null output");
  if (kind != 0 && kind != 1) return fail(ERR_ARG, "unknown scalar kind %d", kind);
  const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++) {
    th.emplace_back([=] {
      const uint64_t a = n * t / nt, b = n * (t + 1) / nt;
      for (uint64_t i = a; i < b; i++) {
        if (kind == 0) uniform_scalar(seed, i, out[i].data);
        else mixed_scalar(seed, msm_index, i, out[i].data);
      }
    });
  }
  for (auto &t : th) t.join();
  return 0;
}

int msm_measure_int_peaks(double *rates, int32_t n) {
  const char *dev = getenv("MSM_DEVICE");
  if (!rates || n <= 0) return fail(ERR_ARG, "null argument");
  CK(cudaSetDevice(dev ? atoi(dev) : 0));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, dev ? atoi(dev) : 0));
  DevBuf sink;
  CK(sink.ensure(16));
  const int threads = 256, blocks = prop.multiProcessorCount * 8, iters = 8000;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  // about 200 ms of warm-up so the clocks settle before timing
  for (int k = 0; k < 40; k++) msm_launch_imad_peak(sink.as<uint32_t>(), blocks, threads, iters, 0, 0);
  CK(cudaDeviceSynchronize());
  const int modes = std::min<int>(n, 3);
  for (int mode = 0; mode < modes; mode++) {
    double best = 0;
    for (int rep = 0; rep < 5; rep++) {
      cudaEventRecord(e0);
      msm_launch_imad_peak(sink.as<uint32_t>(), blocks, threads, iters, mode, 0);
      cudaEventRecord(e1);
      CK(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::max(best, (double)blocks * threads * iters * 16.0 / (ms * 1e-3));
    }
    rates[mode] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return modes;
}

double msm_measure_imad_peak(int32_t iters) {
  (void)iters;
  double r[1] = {0};
  return msm_measure_int_peaks(r, 1) == 1 ? r[0] : -1.0;
}

double msm_measure_madd_rate(void *context, int32_t iters) {
  auto *cx = (Ctx *)context;
  if (!cx || cx->npoints == 0) return -1;
  std::lock_guard<std::mutex> lk(cx->mu);
  cudaSetDevice(cx->device);
  if (iters <= 0) iters = 2000;
  const int threads = 256, blocks = cx->num_sms * 2;
  DevBuf out;
  if (out.ensure((size_t)blocks * threads * MSM_BUCKET_BYTES) != cudaSuccess) return -1;
  const uint32_t nb = (uint32_t)std::min<uint64_t>(cx->npoints, 1u << 16);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0, cx->stream);
    msm_launch_madd_bench(cx->bases.as<uint4>(), nb, out.as<uint4>(), blocks, threads, iters,
                          cx->stream);
    cudaEventRecord(e1, cx->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) return -1;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) best = std::max(best, (double)blocks * threads * iters / (ms * 1e-3));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

int msm_device_info(char *buf, size_t len) {
  const char *dev = getenv("MSM_DEVICE");
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, dev ? atoi(dev) : 0));
  int clk = 0;
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev ? atoi(dev) : 0);
  if (buf && len)
    snprintf(buf, len, "%s; sm_%d%d; %d SMs; %d MHz max SM clock; %.1f GiB", prop.name,
             prop.major, prop.minor, prop.multiProcessorCount, clk / 1000,
             prop.totalGlobalMem / 1073741824.0);
  return 0;
}

int msm_field_selftest(int32_t op, const uint32_t *a, const uint32_t *b, uint32_t *out, uint64_t n) {
  g_err = 0;
  if (n && (!a || !b || !out)) return fail(ERR_ARG, "null argument");
  const char *dev = getenv("MSM_DEVICE");
  CK(cudaSetDevice(dev ? atoi(dev) : 0));
  DevBuf da, db, dout;
  const size_t bytes = std::max<uint64_t>(n, 1) * 48;
  CK(da.ensure(bytes));
  CK(db.ensure(bytes));
  CK(dout.ensure(bytes));
  CK(cudaMemcpy(da.p, a, n * 48, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(db.p, b, n * 48, cudaMemcpyHostToDevice));
  CK(msm_launch_field_test(op, da.as<uint32_t>(), db.as<uint32_t>(), dout.as<uint32_t>(), n, 0));
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(out, dout.p, n * 48, cudaMemcpyDeviceToHost));
  return 0;
}

}  // extern "C"

// =============================================================================================
// msm_mult_noalloc: one MSM whose scratch lives in a fixed, file-scope device array.
//
// Some callers cannot allocate device memory at call time.  Examples: a plugin that runs inside
// another runtime's memory pool, a request loop that must not stall, and a host callback that
// may not call CUDA allocation functions.  cudaMalloc and cudaFree synchronise the device, and
// an allocation can fail halfway through a request.  This entry point uses only memory that
// exists before the call: the context's resident bases (allocated once by msm_init), the
// caller's scalars and output, and the array below for every intermediate buffer.
//
// The array takes MSM_NOALLOC_SCRATCH_BYTES (24 MiB) on every GPU that loads the library, until
// the process exits.  Every call shares it and it keeps the last call's contents.  The pipeline
// clears its own counters at the start of each call, so nothing leaks from one call into the
// next.  Calls that overlap on the GPU (different streams, or other threads) race on the array;
// callers must order them, for example by issuing them on one stream.
// =============================================================================================
#define MSM_NOALLOC_MAX_POINTS (1u << 16)
#define MSM_NOALLOC_SCRATCH_BYTES (24u << 20)
#define MSM_NOALLOC_WINDOW_BITS 12u
#define MSM_NOALLOC_SEG_LEN 256u
#define MSM_NOALLOC_RED_LOG2 3u

static __device__ __align__(256) uint8_t g_noalloc_scratch[MSM_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[256] = {};  // device address of g_noalloc_scratch, per device ordinal

// window descriptors of the single MSM, written on the device so no host staging is needed
__global__ void k_noalloc_plan(JobDesc jd, uint32_t red_log2, JobDesc *jobs, WinDesc *wins) {
  const uint32_t w = threadIdx.x;
  if (w == 0) jobs[0] = jd;
  if (w >= jd.nwin) return;
  const uint32_t L = 1u << red_log2;
  const uint32_t nseg_low = (jd.nb + L - 1) / L;
  const uint32_t ngrp_low = (nseg_low + 511) / 512;
  WinDesc wd;
  wd.job = 0;
  wd.w = w;
  wd.bucket_begin = jd.bucket_begin + w * jd.nb;
  wd.nb = (w + 1 == jd.nwin) ? jd.nb_top : jd.nb;
  wd.seg_begin = w * nseg_low;
  wd.nseg = (wd.nb + L - 1) / L;
  wd.grp_begin = w * ngrp_low;
  wd.ngrp = (wd.nseg + 511) / 512;
  wins[w] = wd;
}

size_t carve(size_t &off, size_t bytes) {
  const size_t at = off;
  off += (bytes + 255) & ~(size_t)255;
  return at;
}

}  // namespace

extern "C" int msm_mult_noalloc(void *context, g1_projective_t *d_out, uint64_t n,
                                uint64_t base_offset, const biginteger256_t *d_scalars,
                                void *stream) {
  g_err = 0;
  auto *cx = (Ctx *)context;
  if (!cx || !d_out || (n && !d_scalars)) return fail(ERR_ARG, "msm_mult_noalloc: null argument");
  if (n > MSM_NOALLOC_MAX_POINTS)
    return fail(ERR_BUDGET, "msm_mult_noalloc: %llu points is over the maximum of %u",
                (unsigned long long)n, MSM_NOALLOC_MAX_POINTS);
  if (base_offset > cx->npoints || n > cx->npoints - base_offset)
    return fail(ERR_ARG, "msm_mult_noalloc: bases outside the resident set");
  CK(cudaSetDevice(cx->device));
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (cx->device < 0 || cx->device >= 256) return fail(ERR_DEVICE, "device ordinal out of range");
    if (!g_noalloc_ptr[cx->device]) {
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return fail(ERR_CUDA, "msm_mult_noalloc: cudaGetSymbolAddress failed: %s",
                    cudaGetErrorString(e));
      g_noalloc_ptr[cx->device] = p;
    }
    scratch = g_noalloc_ptr[cx->device];
  }
  // fixed layout: c = 12 signed windows (22 windows, 2048 buckets each, 2 in the top window)
  JobDesc jd{};
  jd.n = n;
  jd.base_off = base_offset;
  jd.c = MSM_NOALLOC_WINDOW_BITS;
  jd.signed_digits = 1;
  uint32_t nbk = 0, nsegs = 0, ngrps = 0;
  const uint32_t L = 1u << MSM_NOALLOC_RED_LOG2;
  if (n) {
    layout(jd.c, 1, jd.nwin, jd.nb, jd.nb_top);
    jd.nred = jd.nwin;
    nbk = (jd.nwin - 1) * jd.nb + jd.nb_top;
    const uint32_t nseg_low = (jd.nb + L - 1) / L, nseg_top = (jd.nb_top + L - 1) / L;
    nsegs = (jd.nwin - 1) * nseg_low + nseg_top;
    ngrps = (jd.nwin - 1) * ((nseg_low + 511) / 512) + (nseg_top + 511) / 512;
  }
  const uint64_t entries = n * entries_per_point(jd.c, 1);
  const uint32_t tasks = (uint32_t)(nbk + entries / MSM_NOALLOC_SEG_LEN + 1);
  size_t off = 0;
  const size_t o_jobs = carve(off, sizeof(JobDesc));
  const size_t o_wins = carve(off, 64 * sizeof(WinDesc));
  const size_t o_count = carve(off, (size_t)nbk * 4), o_offset = carve(off, (size_t)nbk * 4);
  const size_t o_fill = carve(off, (size_t)nbk * 4), o_taskoff = carve(off, (size_t)nbk * 4);
  const size_t o_heavy = carve(off, (size_t)nbk * 4);
  const size_t o_scan = carve(off, msm_scan_tmp_words(nbk) * 4);
  const size_t o_cnt = carve(off, CNT_WORDS * 4);
  const size_t o_vals = carve(off, entries * 4);
  const size_t o_tasks = carve(off, (size_t)tasks * sizeof(Task));
  const size_t o_part = carve(off, (size_t)tasks * MSM_BUCKET_BYTES);
  const size_t o_order = carve(off, (size_t)tasks * 4);
  const size_t o_lenh = carve(off, (size_t)(MSM_NOALLOC_SEG_LEN + 1) * 4);
  const size_t o_seg = carve(off, (size_t)nsegs * 2 * MSM_BUCKET_BYTES);
  const size_t o_grp = carve(off, (size_t)ngrps * 2 * MSM_BUCKET_BYTES);
  const size_t o_win = carve(off, (size_t)jd.nwin * MSM_BUCKET_BYTES);
  if (off > MSM_NOALLOC_SCRATCH_BYTES)
    return fail(ERR_BUDGET, "msm_mult_noalloc: scratch layout needs %zu bytes", off);
  uint8_t *s = (uint8_t *)scratch;
  PassBuffers pb{};
  pb.bases = cx->bases.as<uint4>();
  pb.flags = cx->flags.as<uint8_t>();
  pb.special_idx = cx->special_idx.as<uint32_t>();
  pb.special_cls = cx->special_cls.as<uint8_t>();
  pb.class_pts = cx->class_pts.as<uint4>();
  pb.n_special = cx->n_special;
  pb.n_classes = cx->n_classes;
  pb.n_bases = cx->npoints * (cx->fb_w + cx->fb2_w);
  pb.scalars = (const uint4 *)d_scalars;
  pb.jobs = (const JobDesc *)(s + o_jobs);
  pb.wins = (const WinDesc *)(s + o_wins);
  pb.n_jobs = 1;
  pb.n_wins = jd.nwin;
  pb.n_points = n;
  pb.n_buckets = nbk;
  pb.n_segs = nsegs;
  pb.n_grps = ngrps;
  pb.seg_len = MSM_NOALLOC_SEG_LEN;
  pb.red_len_log2 = MSM_NOALLOC_RED_LOG2;
  pb.grp_len_log2 = 9;
  pb.max_entries = entries;
  pb.max_tasks = tasks;
  pb.count = (uint32_t *)(s + o_count);
  pb.offset = (uint32_t *)(s + o_offset);
  pb.fill = (uint32_t *)(s + o_fill);
  pb.taskoff = (uint32_t *)(s + o_taskoff);
  pb.heavy = (uint32_t *)(s + o_heavy);
  pb.scan_tmp = (uint32_t *)(s + o_scan);
  pb.counters = (uint32_t *)(s + o_cnt);
  pb.vals = (uint32_t *)(s + o_vals);
  pb.tasks = (Task *)(s + o_tasks);
  pb.partials = (uint4 *)(s + o_part);
  pb.order = (uint32_t *)(s + o_order);
  pb.len_hist = (uint32_t *)(s + o_lenh);
  pb.seg_out = (uint4 *)(s + o_seg);
  pb.grp_out = (uint4 *)(s + o_grp);
  pb.win_sum = (uint4 *)(s + o_win);
  pb.results = (uint64_t *)d_out;
  cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_plan<<<1, 64, 0, st>>>(jd, MSM_NOALLOC_RED_LOG2, (JobDesc *)(s + o_jobs),
                                   (WinDesc *)(s + o_wins));
  CK(cudaGetLastError());
  CK(msm_launch_pass(pb, cx->num_sms, st, nullptr));
  return 0;
}
