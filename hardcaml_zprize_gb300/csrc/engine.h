// Internal interfaces between the host driver and the device pipeline (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#define MSM_BASE_BYTES 144      // precomputed twisted-Edwards base: 3 x 48 B
#define MSM_BUCKET_BYTES 192    // extended twisted-Edwards point: 4 x 48 B
#define MSM_AFFINE_BYTES 104    // g1_affine_t
#define MSM_PROJ_BYTES 144      // g1_projective_t
#define MSM_SCALAR_BITS 253

// base flags written by the precompute kernel
enum : uint8_t {
  BASE_OK = 0,
  BASE_INFINITY = 1,     // contributes nothing
  BASE_SPECIAL = 2,      // on the curve but without a twisted-Edwards image: Weierstrass path
  BASE_BAD_INPUT = 3,    // a coordinate >= q: rejected by msm_init
};

// One MSM inside a pipeline pass.
struct JobDesc {
  uint64_t point_begin;   // first index of this MSM in the pass's flattened point space
  uint64_t n;             // number of (scalar, base) pairs
  uint64_t base_off;      // first base of the MSM's slice of the resident base set
  uint64_t scalar_off;    // first scalar in the pass's scalar buffer
  uint32_t c;             // window width in bits
  uint32_t nwin;          // number of windows
  uint32_t nb;            // buckets per window below the top one
  uint32_t nb_top;        // buckets in the top window (signed: capped at the largest top digit
                          // of a scalar below r; a larger digit is split into two entries)
  uint32_t bucket_begin;  // first global bucket id
  uint32_t win_begin;     // first global window id
  uint32_t signed_digits; // 1: signed c-bit digits, 0: unsigned
  uint32_t result_slot;   // index into the pass's result array
  uint32_t fixed;         // 1: fixed-base tables, every window shares one bucket array
  uint32_t nred;          // windows of the bucket reduction (1 for fixed-base jobs)
  uint64_t fb_stride;     // base-table index step from one window's table to the next
  uint64_t tab_base;      // first record of the job's table set in the resident base array
};

// One (MSM, window) pair for the bucket reduction.
struct WinDesc {
  uint32_t job;
  uint32_t w;
  uint32_t bucket_begin;  // global id of this window's bucket index 0 (digit magnitude 1)
  uint32_t nb;            // buckets in this window
  uint32_t seg_begin;     // first level-1 reduction segment
  uint32_t nseg;          // level-1 segments in this window
  uint32_t grp_begin;     // first level-2 group (2^grp_len_log2 segments each)
  uint32_t ngrp;          // level-2 groups in this window
};

struct Task {             // a run of sorted entries that one thread accumulates
  uint32_t start;         // first entry in the sorted value array
  uint32_t len;           // number of entries (<= seg_len)
  uint32_t bucket;        // global bucket id
  uint32_t pad;
};

enum : int {
  CNT_TASKS = 0,          // number of tasks built
  CNT_HEAVY = 1,          // buckets split over more than one task
  CNT_TASK_CURSOR = 2,    // persistent accumulate work counter
  CNT_HEAVY_CURSOR = 3,
  CNT_ERROR = 4,          // nonzero: a device-side bounds check fired (code)
  CNT_ERROR_INFO = 5,
  CNT_ENTRIES = 6,        // sorted entries of the pass (nonzero digits)
  CNT_WORDS = 8,
};

#define MSM_POINTS_PER_CHUNK 256  // points per histogram block (one chunk of the stage)
#define MSM_MAX_BINS 32           // key ranges of the staged sort

// Everything a pass needs on the device; sized by the host (msm_plan_pass).
struct PassBuffers {
  const uint4 *bases;           // resident bases, 9 x uint4 each
  const uint8_t *flags;         // resident base flags
  const uint32_t *special_idx;  // resident list of BASE_SPECIAL base indices
  const uint8_t *special_cls;   // class id of each special base
  const uint4 *class_pts;       // affine Weierstrass class points: x(3 uint4), y(3 uint4)
  uint32_t n_special;
  uint32_t n_classes;
  uint64_t n_bases;             // resident bases (bounds of every base index)
  uint32_t acc_blocks_per_sm;   // resident k_accumulate blocks per SM (0: 4, the whole SM)

  const uint4 *scalars;         // 2 x uint4 per scalar
  const uint4 *host_scalars;    // or null: k_count first copies each scalar from this host buffer
                                // (same indexing) into `scalars`, reading over the C2C link
  const JobDesc *jobs;
  const WinDesc *wins;
  uint32_t n_jobs;
  uint32_t n_wins;
  uint64_t n_points;            // sum of job sizes
  uint32_t n_buckets;           // global bucket count
  uint32_t n_segs;              // level-1 reduction segments
  uint32_t seg_len;             // max entries per accumulate task
  uint32_t red_len_log2;        // level-1 reduction segment length = 1 << red_len_log2
  uint32_t grp_len_log2;        // level-2 group = 1 << grp_len_log2 level-1 segments
  uint32_t n_grps;              // level-2 groups
  uint64_t max_entries;         // capacity of vals
  uint32_t max_tasks;           // capacity of tasks / partials

  // staged sort (or stage == null: the scatter re-reads the scalars once per key range).
  // k_count writes the entries of its 256 points, (key, base index | sign << 31), into the
  // block's chunk of `stage`, grouped by key range (key >> bin_shift); blk_off holds each
  // chunk's n_bins + 1 range starts.  The scatter then reads one key range per launch and
  // places each entry at offset + rank (stage_rank set) or at a slot-cursor atomic (null).
  uint2 *stage;                 // [n_chunks * stage_cap]
  uint32_t *stage_rank;         // or null: [n_chunks * stage_cap] each staged entry's rank in its
                                // bucket, taken from the bucket count when the entry is staged
  uint32_t *blk_off;            // [n_chunks * (n_bins + 1)]
  uint32_t stage_cap;           // entries per chunk: 256 x the pass's most entries per point
  uint32_t bin_shift;           // key range of a bucket key
  uint32_t n_bins;              // key ranges (<= MSM_MAX_BINS)

  uint32_t *count;              // [n_buckets]
  uint32_t *offset;             // [n_buckets]
  uint32_t *fill;               // [n_buckets] slot cursors (the scan seeds them with offset)
  uint32_t *taskoff;            // [n_buckets]
  uint32_t *scan_tmp;           // block partials for the scans
  uint32_t *vals;               // [max_entries]
  Task *tasks;                  // [max_tasks]
  uint4 *partials;              // [max_tasks] x 12 uint4
  uint32_t *heavy;              // [n_buckets]
  uint32_t *order;              // [max_tasks] task ids, longest first
  uint32_t *len_hist;           // [seg_len + 1] task-length histogram, then start cursors
  uint32_t *counters;           // [CNT_WORDS]
  uint4 *seg_out;               // [n_segs] x 2 x 12 uint4
  uint4 *grp_out;               // [n_grps] x 2 x 12 uint4
  uint4 *win_sum;               // [n_wins] x 12 uint4
  uint64_t *results;            // [n_jobs] x 18 u64 (g1_projective_t)
};

// launch the whole pipeline of one pass on `stream` (graph-capturable: fixed launch shapes)
// `stage_events` (10 events, or null) are recorded around the stages for per-kernel timing
// `chunk_ready` (nchunks events, or null): the scalars arrive in nchunks equal point ranges and
// the histogram of range c waits for event c (copy/compute overlap for host-resident scalars)
// `n_kernels` (or null) receives the number of kernels launched
cudaError_t msm_launch_pass(const PassBuffers &pb, int num_sms, cudaStream_t stream,
                            cudaEvent_t *stage_events, const cudaEvent_t *chunk_ready = nullptr,
                            int nchunks = 0, uint32_t *n_kernels = nullptr);
#define MSM_NUM_STAGES 10
size_t msm_scan_tmp_words(uint32_t n_buckets);
uint32_t msm_scatter_passes(uint64_t max_entries);
uint32_t msm_bin_shift(uint32_t n_buckets, uint64_t max_entries, uint32_t ranges, bool cursors);
uint64_t msm_upload_chunk_points(uint64_t n_points, int nchunks);

// resident-base preparation
cudaError_t msm_launch_precompute(const void *d_affine, size_t n, uint4 *d_bases, uint8_t *d_flags,
                                  uint32_t *d_special_idx, uint32_t *d_special_count,
                                  uint32_t index_offset, cudaStream_t stream);
cudaError_t msm_launch_check_classes(const uint4 *d_class_pts, uint32_t n, uint32_t *d_ok,
                                     cudaStream_t stream);
// fixed-base tables: bases[(w * n + i)] = 2^(c w) * P_i for w in [1, nwin), from window 0;
// sets *d_fail when a base's doubling chain leaves the affine curve (a point of 2-power order)
cudaError_t msm_launch_fixed_base(uint4 *d_bases, const uint8_t *d_flags, uint64_t n, uint64_t first,
                                  uint64_t count, uint32_t c, uint32_t nwin, uint32_t *d_fail,
                                  cudaStream_t stream);
// bases k_i * G with k_i from the seeded generator, written as g1_affine_t
cudaError_t msm_launch_gen_bases(uint64_t seed, uint64_t first, size_t n, void *d_affine,
                                 const uint4 *d_table, cudaStream_t stream);
cudaError_t msm_build_gen_table(uint4 *d_table, cudaStream_t stream);
// self-test hooks
cudaError_t msm_launch_field_test(int op, const uint32_t *a, const uint32_t *b, uint32_t *out,
                                  size_t n, cudaStream_t stream);
cudaError_t msm_launch_imad_peak(uint32_t *sink, int blocks, int threads, int iters, int mode,
                                 cudaStream_t stream);
cudaError_t msm_launch_madd_bench(const uint4 *bases, uint32_t nbases, uint4 *out, int blocks,
                                  int threads, int iters, cudaStream_t stream);
