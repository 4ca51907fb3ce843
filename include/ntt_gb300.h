/* GB300 NTT over the Goldilocks field (p = 2^64 - 2^32 + 1) -- C ABI of libdriver.so.
 *
 * The transform is the one of fyquah/hardcaml_zprize's NTT track: X[k] = sum_j x[j] w^(j k) with
 * w the 2^log_n-th root of unity of the reference's table (zprize/ntt/host/gf.h:65-99), natural
 * order in and out, as its host model computes it (zprize/ntt/host/reference.cpp:94-139).  The
 * reference drives an FPGA through the C++ class NttFpgaDriver (zprize/ntt/host/driver.h:62-227):
 * its constructor and load_xclbin become ntt_init, simple_evaluate becomes ntt_evaluate, and
 * input_vector_size keeps its name; the FPGA-only pieces (memory layouts, user buffers of the
 * PCIe transfers, the debug "reverse" core) have no counterpart, since the GPU takes the vector
 * in natural order.  Elements are little-endian u64; inputs at or above p are taken modulo p.
 */
#ifndef NTT_GB300_H
#define NTT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NTT_ERR_ARG -1
#define NTT_ERR_CUDA -2

/* A context for transforms of 2^log_n points (log_n <= 24) on the GPU named by MSM_DEVICE
 * (default 0): twiddle tables and input, output and intermediate buffers, allocated once.
 * Replaces NttFpgaDriver(NttFpgaDriverArg::create_ntt_2_24(...)) + load_xclbin
 * (driver.h:158-170; host/driver.cpp).  Returns NULL on failure (ntt_last_error says why). */
void *ntt_init(uint32_t log_n);

/* A context for the inverse transform of 2^log_n points: x[j] = (1/n) sum_k X[k] w^(-j k), so
 * that it undoes ntt_evaluate of an ntt_init context of the same size.  Every other entry point
 * takes it unchanged.  The FPGA computes one direction only; the reference's software model
 * holds both (libs/hardcaml_ntt/src/reference_model.ml:6-55, forward_dit with the other root
 * table) and its round-trip test scales by 1/n (libs/hardcaml_ntt/test/test_ntt_roundtrip.ml:7-23). */
void *ntt_init_inverse(uint32_t log_n);

/* Number of elements of one transform (NttFpgaDriver::input_vector_size, driver.h:160). */
uint64_t ntt_input_vector_size(void *context);

/* out = NTT(in), host memory, synchronous; len must equal the transform size.  Replaces
 * NttFpgaDriver::simple_evaluate(output, input, data_length) (driver.h:207-209).  Returns 0 or a
 * negative error code. */
int ntt_evaluate(void *context, uint64_t *out, const uint64_t *in, uint64_t len);

/* `count` transforms back to back: out[i n ..] = NTT(in[i n ..]).  Two device vector pairs and
 * three streams overlap the upload of vector i + 1 and the download of vector i - 1 with the
 * transform of vector i, as the reference driver overlaps its user buffers
 * (enqueue_evaluation_async / wait_for_result, driver.h:185-199; bench_throughput.cpp).  The
 * second vector pair is allocated on the first call.  Synchronous. */
int ntt_evaluate_batch(void *context, uint64_t *out, const uint64_t *in, uint64_t count);

/* The same transform between device buffers, enqueued on `stream` (NULL: the context's own
 * stream); out must not alias in for transforms of at most 2^12 points.  No counterpart in the
 * reference (its buffers are the driver's). */
int ntt_evaluate_device(void *context, uint64_t *d_out, const uint64_t *d_in, void *stream);

/* Device times (ms, CUDA events) of the last ntt_evaluate: host-to-device copy, pass A, pass B,
 * device-to-host copy.  Returns the number of values written. */
int ntt_last_timings(void *context, double *ms, int32_t max_stages);

/* Self-test hook: out[i] = a[i] op b[i] for op 0 (add), 1 (sub), 2 (mul) modulo p, inputs
 * below p, on the GPU named by MSM_DEVICE. */
int ntt_field_selftest(int32_t op, const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n);

/* Error code of the last failed call on this thread (0 if none) and its message. */
int ntt_last_error(char *buf, size_t len);

/* Release a context. */
void ntt_free(void *context);

#ifdef __cplusplus
}

#include <stdexcept>
#include <string>

/* The reference host programs' calls, on the GPU (zprize/ntt/host/bench_latency.cpp,
 * test_random.cpp call simple_evaluate and input_vector_size). */
class NttGb300Driver {
 public:
  explicit NttGb300Driver(uint32_t log_n) : ctx_(ntt_init(log_n)) {
    if (!ctx_) throw std::runtime_error(error());
  }
  ~NttGb300Driver() { ntt_free(ctx_); }
  NttGb300Driver(const NttGb300Driver &) = delete;
  NttGb300Driver &operator=(const NttGb300Driver &) = delete;
  uint64_t input_vector_size() const { return ntt_input_vector_size(ctx_); }
  void simple_evaluate(uint64_t *output, const uint64_t *input, uint64_t data_length) {
    if (ntt_evaluate(ctx_, output, input, data_length) != 0) throw std::runtime_error(error());
  }
  /* count vectors of input_vector_size() elements, transfers overlapping the transforms */
  void evaluate_batch(uint64_t *output, const uint64_t *input, uint64_t count) {
    if (ntt_evaluate_batch(ctx_, output, input, count) != 0) throw std::runtime_error(error());
  }

 private:
  static std::string error() {
    char buf[512];
    ntt_last_error(buf, sizeof buf);
    return buf;
  }
  void *ctx_;
};
#endif

#endif /* NTT_GB300_H */
