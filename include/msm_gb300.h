/* GB300 multi-scalar multiplication engine for BLS12-377 G1 -- C ABI of libdriver.so.
 *
 * The first two entry points are a drop-in for the host driver of fyquah/hardcaml_zprize's MSM
 * track: same symbol names, same argument meaning, same struct layout, so the reference's Rust
 * harness (zprize/msm_pippenger/test_fpga_harness/src/lib.rs:18-33, linked with
 * `cargo:rustc-link-lib=dylib=driver`, build.rs:19) binds them unchanged.
 *
 * Data layout (zprize/msm_pippenger/host/msm_compute/include/bls12_377_g1/rust_types.h:8-83):
 *   - base-field elements are six little-endian u64 limbs in arkworks Montgomery form
 *     (value * 2^384 mod q), fully reduced;
 *   - scalars are four little-endian u64 limbs, the raw integer the harness transmutes out of
 *     ark_bls12_377::Fr (tests/msm.rs:30-32); bits 253..255 are ignored, as the reference's
 *     253-bit scalar path does (driver.cpp:15, bls12_377_g1.h:17);
 *   - results are arkworks 0.3 Jacobian projective points: (x*R, y*R, R) for a finite point,
 *     (R, R, 0) for the point at infinity (the reference writes (x*R, y*R, R) too,
 *     bls12_377_g1.h:427-439, 667-690).
 */
#ifndef MSM_GB300_H
#define MSM_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <sys/types.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  uint64_t data[4];
} biginteger256_t; /* 32 B, rust_types.h:8-63 */

typedef struct {
  uint64_t data[6];
} biginteger384_t; /* 48 B, rust_types.h:65-71 */

typedef struct {
  biginteger384_t x;
  biginteger384_t y;
  bool infinity;
} g1_affine_t; /* 104 B with padding, rust_types.h:73-77 (arkworks GroupAffine) */

typedef struct {
  biginteger384_t x;
  biginteger384_t y;
  biginteger384_t z;
} g1_projective_t; /* 144 B, rust_types.h:79-83 (arkworks GroupProjective, Jacobian) */

/* ---------------------------------------------------------------------------------------------
 * Drop-in entry points
 * ------------------------------------------------------------------------------------------- */

/* Load the bases once and keep them resident on the GPU in precomputed twisted-Edwards form.
 * When HBM allows it also keeps fixed-base tables 2^(c w) P_i for every window w (width from a
 * cost model for 2^20 bases or more, 16 below; large contexts add a second set of width 16 for
 * their small MSMs). Environment: MSM_FIXED_BASE=0 off, =<c> force width c (one set);
 * MSM_FIXED_BASE_MAX_GB caps the tables.
 * Replaces `extern "C" Driver *msm_init(const char *xclbin, ssize_t xclbin_len,
 * g1_affine_t *rust_points, ssize_t npoints)` (zprize/msm_pippenger/host/driver/driver.cpp:603-617).
 * `xclbin` names an FPGA bitstream in the reference; here it is accepted and ignored (it may be
 * NULL). `points` is borrowed for the call. Returns NULL on failure (msm_last_error() says why);
 * the reference exits the process instead (driver.cpp:248-251). */
void *msm_init(const char *xclbin, ssize_t xclbin_len, const g1_affine_t *points, ssize_t npoints);

/* Run `batch_size` MSMs over all resident bases: out[b] = sum_i scalars[b*npoints + i] * P_i.
 * Replaces `extern "C" void msm_mult(Driver *driver, g1_projective_t *out, uint64_t num_batches,
 * biginteger256_t *ptr_scalars)` (driver.cpp:619-636). `out` holds batch_size results (caller
 * allocated, as lib.rs:70 does). On failure every output is zeroed and msm_last_error() is set. */
void msm_mult(void *context, g1_projective_t *out, uint64_t batch_size,
              const biginteger256_t *scalars);

/* The naive driver's names for the same two calls (zprize/msm_pippenger/host/naive_driver/
 * naive_driver.cpp:109-138, bound by test_naive_harness/src/lib.rs:16-37):
 * `zprize_msm_fpga_init(points, npoints)` is msm_init without the bitstream arguments, and
 * `zprize_msm_fpga_mult` / `zprize_msm_pippenger_mult(ctx, out, batch_size, scalars)` are
 * msm_mult.  In the reference they run a CPU double-and-add and a CPU Pippenger; both compute
 * the same MSMs. */
void *zprize_msm_fpga_init(const g1_affine_t *points, ssize_t npoints);
void zprize_msm_fpga_mult(void *context, g1_projective_t *out, uint64_t batch_size,
                          const biginteger256_t *scalars);
void zprize_msm_pippenger_mult(void *context, g1_projective_t *out, uint64_t batch_size,
                               const biginteger256_t *scalars);

/* ---------------------------------------------------------------------------------------------
 * Additions (no counterpart in the reference unless stated)
 * ------------------------------------------------------------------------------------------- */

/* Tuning knobs; 0 (or a negative value) means "choose automatically". */
typedef struct {
  int32_t window_bits;   /* c, 6..22 */
  int32_t signed_digits; /* 1 signed c-bit digits, 2 unsigned digits, 0 auto (signed) */
  int32_t seg_len;       /* max entries one thread accumulates before a bucket is split */
  int32_t red_len_log2;  /* log2 of buckets per level-1 reduction segment */
  int32_t use_graph;     /* 1 replay the pass from a captured CUDA graph, 2 never, 0 auto */
  int32_t mode;          /* msm_mult: 1 one pass per MSM (default), 2 all MSMs in one pass */
  int32_t fixed_base;    /* 1 use the context's fixed-base tables, 2 never, 0 auto (cost model) */
} msm_options_t;

/* Error code of the last failed call on this thread (0 if none) and its message. */
int msm_last_error(char *buf, size_t len);

/* Release a context (the reference never frees its Driver). */
void msm_free(void *context);

/* msm_mult with explicit options; returns 0 or a negative error code. */
int msm_mult_ex(void *context, g1_projective_t *out, uint64_t batch_size,
                const biginteger256_t *scalars, const msm_options_t *opt);

/* Many MSMs of uneven sizes in one pass with one shared sort. MSM j uses sizes[j] bases starting
 * at base_offsets[j] and the next sizes[j] scalars of the concatenated `scalars` array.
 * opt->mode == 1 runs them one pass per MSM instead (the plain form). */
int msm_mult_uneven(void *context, g1_projective_t *out, uint64_t num_msms, const uint64_t *sizes,
                    const uint64_t *base_offsets, const biginteger256_t *scalars,
                    const msm_options_t *opt);

/* As msm_mult_uneven, with the scalars already in device memory (`d_scalars`, 32 B each);
 * results are written to host memory. */
int msm_mult_device(void *context, g1_projective_t *out, uint64_t num_msms, const uint64_t *sizes,
                    const uint64_t *base_offsets, const void *d_scalars, const msm_options_t *opt);

/* The configuration the engine would use for one MSM of `npoints` (after tuning, if any). */
int msm_get_config(void *context, uint64_t npoints, msm_options_t *out);

/* Measure candidate configurations for MSMs of `npoints` on the device and keep the fastest for
 * that size class (persisted to the file named by MSM_TUNE_CACHE, if set). `budget_ms` bounds
 * the time spent (0: default). Returns 0 and fills `best` (may be NULL). */
int msm_tune(void *context, uint64_t npoints, int32_t budget_ms, msm_options_t *best);

/* What a context keeps resident: number of bases, bytes of the base records (the 144 B plain
 * records, or every fixed-base table record), main table width and windows (0 and 0 without
 * tables), second table set width and windows (0 and 0 when absent). Returns the number of
 * values written (at most 6). */
int msm_context_info(void *context, uint64_t *info, int32_t max_info);

/* Tune the one-pass form of a batch of uneven MSMs on that batch itself (same arguments as
 * msm_mult_uneven, host scalars). Per size class (log2 of the MSM size) it measures whole passes
 * of the batch with signed windows of width 10..16, unsigned windows at the best width and each
 * fixed-base table set of the context, by coordinate descent from the largest classes down; then
 * the pass's run length (entries one thread accumulates before a bucket is split over more
 * threads: the threads-per-bucket knob) and level-1 reduction run. The class forms are kept for
 * later passes that several MSMs share (msm_mult_uneven with mode 2, server passes) and appended
 * to MSM_TUNE_CACHE as "b ..." lines; the pass-level knobs come back in `best` (mode 2) for the
 * caller to pass with the same mix. `report` (may be NULL) receives the untuned and tuned pass
 * times in ms and the number of passes measured. `budget_ms` bounds the time (0: 20 s).
 * The reference fixes its window layout in RTL (hardcaml/src/config.ml:5-21,
 * config_utils.ml:7-49); this has no counterpart there. */
int msm_tune_uneven(void *context, uint64_t num_msms, const uint64_t *sizes,
                    const uint64_t *base_offsets, const biginteger256_t *scalars, int32_t budget_ms,
                    msm_options_t *best, double *report);
/* The form the engine uses for an MSM of `npoints`, alone (shared_pass 0) or in a pass with
 * others (1): window_bits, signed_digits, and in fixed_base the bases it reads (here 0: the plain
 * records, windowed; 1: the main fixed-base table set; 2: the second, width-16 set). */
int msm_tuned_form(void *context, uint64_t npoints, int32_t shared_pass, msm_options_t *out);

/* Per-stage device times (ms, CUDA events on the pipeline stream) of the last pass when timing
 * is enabled with msm_set_timing(ctx, 1). Stage order: count, scan, scatter, tasks, accumulate,
 * merge, reduce1, reduce2, reduce3, final. Returns the number of stages written. */
int msm_set_timing(void *context, int32_t enable);
int msm_last_timings(void *context, double *ms, int32_t max_stages);
/* Counters of the last pass: tasks, heavy buckets, sorted entries, buckets, kernel launches. */
int msm_last_pass_stats(void *context, uint64_t *stats, int32_t max_stats);

/* One MSM that allocates no device memory; it has no counterpart in the reference.
 * For callers that cannot call cudaMalloc at call time: a plugin running inside another
 * runtime's memory pool, a request loop that must not stall, a host callback that may not
 * allocate (cudaMalloc/cudaFree synchronise the device and can fail mid-request).
 * Inputs and output are the caller's device memory: `d_scalars` (n x 32 B) and `d_out`
 * (one g1_projective_t); the bases are the context's resident slice [base_offset,
 * base_offset + n).  Intermediate buffers live in one file-scope device array of 24 MiB that
 * every GPU loading the library holds until the process exits; n may be at most 65536 (larger n
 * is rejected with an error).  The first call on a device looks up that array's address, so
 * make the first call before any stream capture.  The call only enqueues work on `stream`
 * (NULL: the legacy default stream); synchronise it before reading `d_out`.  All calls share
 * the array: calls that overlap on the GPU race, so order them (for example on one stream).
 * The array's address is looked up once per device and kept for the life of the process, so do
 * not keep using the library on a device after cudaDeviceReset.  The return code covers the
 * arguments and the launches only: when a device bounds check stops the MSM, `d_out` receives
 * 144 zero bytes, which no result can be (the zero point is written as (R, R, 0)). */
int msm_mult_noalloc(void *context, g1_projective_t *d_out, uint64_t n, uint64_t base_offset,
                     const biginteger256_t *d_scalars, void *stream);

/* ---- serving: continuous batching of MSM requests against the resident bases ---- */
typedef struct {
  uint64_t submitted, completed, passes, inflight_peak;
  uint64_t bytes_in_use, bytes_peak;
} msm_server_stats_t;

/* `hbm_budget_bytes` bounds the device memory of scalar/sort/bucket buffers of passes in
 * flight; `max_inflight` bounds concurrent passes (each slot has a stream at the lowest and one
 * at the highest priority: a pass of at most 2^19 points takes the high one, and with more than
 * one slot every pass's accumulation leaves a quarter of each SM free, so small requests do not
 * wait for a large pass to finish). */
void *msm_server_create(void *context, uint64_t hbm_budget_bytes, int32_t max_inflight);
/* Copy the request's scalars and queue it; returns its id (>= 0) or a negative error. */
int64_t msm_server_submit(void *server, const biginteger256_t *scalars, uint64_t n,
                          uint64_t base_offset);
/* 0 done (result in *out, latency from submit to completion in *latency_ms if not NULL),
 * 1 still pending after waiting up to wait_ms, negative on error. */
int msm_server_poll(void *server, int64_t id, g1_projective_t *out, int32_t wait_ms,
                    double *latency_ms);
int msm_server_stats(void *server, msm_server_stats_t *stats);
void msm_server_destroy(void *server);

/* ---- data formats either side of the path ----
 * The harness's test-data files (TEST_LOAD_DATA_FROM / TEST_WRITE_DATA_TO,
 * test_fpga_harness/src/util.rs:126-172) hold ark-serialize canonical field elements; the ABI
 * above carries arkworks' Montgomery form.  In place on n elements, all host cores:
 *   Fq (6 x u64): x <-> x * 2^384 mod q;  Fr (4 x u64): v <-> v * 2^256 mod r (the raw integer
 *   the harness transmutes out of Fr, tests/msm.rs:30-32).
 * Return 0, or -3 when an input is not below the modulus. */
int msm_fq_to_montgomery(uint64_t *v, uint64_t n);
int msm_fq_from_montgomery(uint64_t *v, uint64_t n);
int msm_fr_to_montgomery(uint64_t *v, uint64_t n);
int msm_fr_from_montgomery(uint64_t *v, uint64_t n);

/* ---- utilities for tests and benchmarks ---- */
/* Bases k_i * G, k_i a seeded counter-based 64-bit draw (SplitMix64), computed on the GPU. */
int msm_generate_bases(uint64_t seed, uint64_t first, uint64_t n, g1_affine_t *out);
/* Scalars on the host: kind 0 uniform in [0, r); kind 1 the uneven-batch mix (70% uniform,
 * 10% 16-bit, 10% 0 or r-1, 10% one repeated value), drawn for MSM `msm_index`. */
int msm_generate_scalars(uint64_t seed, uint64_t n, int32_t kind, uint64_t msm_index,
                         biginteger256_t *out);
/* Measured peak rate of the GPU's IMAD pipe on independent mad.lo/mad.hi pairs (32-bit
 * multiply-adds per second, all SMs, after a warm-up). `iters` is ignored. */
double msm_measure_imad_peak(int32_t iters);
/* The same for up to three instruction mixes: rates[0] mad.lo/mad.hi pairs, rates[1] mad.lo
 * only, rates[2] mad.hi only.  Returns the number of rates written. */
int msm_measure_int_peaks(double *rates, int32_t n);
/* Device name, SM count and clock as text. */
int msm_device_info(char *buf, size_t len);
/* Field self-test: op 0 mul (Montgomery), 1 add, 2 sub, 3 inverse (Fermat), 4 canonicalise,
 * 5 negate, 6 inverse (binary extended Euclid);
 * operands are 12 little-endian u32 limbs each. */
int msm_field_selftest(int32_t op, const uint32_t *a, const uint32_t *b, uint32_t *out, uint64_t n);
/* Throughput of the mixed twisted-Edwards addition on cached bases (adds per second). */
double msm_measure_madd_rate(void *context, int32_t iters);

#ifdef __cplusplus
}
#endif

#endif /* MSM_GB300_H */
