// gbns_api.cu -- the extern "C" entry points of libgbns.so (declared in include/gbns.h).
// Argument checks happen here on the host; every entry point returns 0 or a negative
// error code and leaves a thread-local message for gbns_last_error().
#include <cstdio>
#include <cstring>
#include "gbns_device.cuh"
#include "gbns_launch.h"

namespace {
thread_local char g_err[512] = {0};

int fail(int code, const char *fmt, const char *detail = nullptr) {
  std::snprintf(g_err, sizeof(g_err), fmt, detail ? detail : "");
  return code;
}

int check(cudaError_t e, const char *where) {
  if (e == cudaSuccess) return 0;
  std::snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(e));
  return -2;
}

int check_batch(const gbns_batch *b) {
  if (!b) return fail(-1, "batch is NULL%s");
  if (b->num_runs <= 0) return fail(-1, "batch has no runs%s");
  if (!b->runs || !b->state || !b->ncoef) return fail(-1, "batch descriptors missing%s");
  if (b->nmax <= 0 || b->nmax > 4096) return fail(-1, "nmax must be in [1, 4096]%s");
  if (b->ncoef_n < b->nmax) return fail(-1, "the ncoef table must cover every live-point count (ncoef_n >= nmax)%s");
  if (b->chains_per_item <= 0 || b->chains_per_item > 128 || (b->chains_per_item & 31))
    return fail(-1, "chains_per_item must be a multiple of 32 in [32, 128]%s");
  return 0;
}
}  // namespace

namespace gbns {
void record_error(const char *msg) { std::snprintf(g_err, sizeof(g_err), "%s", msg); }
}  // namespace gbns

extern "C" {

int gbns_version(void) { return GBNS_VERSION; }

int gbns_abi_sizes(long long *out, int n) {
  const long long sz[6] = {(long long)sizeof(gbns_term_cond), (long long)sizeof(gbns_evcalc),
                           (long long)sizeof(gbns_run_desc),  (long long)sizeof(gbns_run_state),
                           (long long)sizeof(gbns_batch),     (long long)sizeof(gbns_results_bufs)};
  if (!out || n < 6) return fail(-1, "gbns_abi_sizes: need room for 6 sizes%s");
  for (int i = 0; i < 6; ++i) out[i] = sz[i];
  return 0;
}

const char *gbns_last_error(void) { return g_err; }

int gbns_threefry2x32(const uint32_t *key_dev, const uint32_t *counts_dev, uint32_t *out_dev, long long n,
                      void *stream) {
  if (!key_dev || !counts_dev || !out_dev || n < 0) return fail(-1, "gbns_threefry2x32: bad arguments%s");
  return check(gbns::launch_rng(0, key_dev, counts_dev, out_dev, n, (cudaStream_t)stream), "gbns_threefry2x32");
}

int gbns_threefry_split(const uint32_t *key_dev, uint32_t *out_dev, long long n, void *stream) {
  if (!key_dev || !out_dev || n < 0 || n > 0xFFFFFFFFll) return fail(-1, "gbns_threefry_split: bad arguments%s");
  return check(gbns::launch_rng(1, key_dev, nullptr, out_dev, n, (cudaStream_t)stream), "gbns_threefry_split");
}

int gbns_random_bits64(const uint32_t *key_dev, uint64_t *out_dev, long long n, void *stream) {
  if (!key_dev || !out_dev || n < 0 || n > 0xFFFFFFFFll) return fail(-1, "gbns_random_bits64: bad arguments%s");
  return check(gbns::launch_rng(2, key_dev, nullptr, out_dev, n, (cudaStream_t)stream), "gbns_random_bits64");
}

int gbns_uniform(const uint32_t *key_dev, float *out_dev, long long n, void *stream) {
  if (!key_dev || !out_dev || n < 0 || n > 0xFFFFFFFFll) return fail(-1, "gbns_uniform: bad arguments%s");
  return check(gbns::launch_rng(3, key_dev, nullptr, out_dev, n, (cudaStream_t)stream), "gbns_uniform");
}

int gbns_normal(const uint32_t *key_dev, float *out_dev, long long n, void *stream) {
  if (!key_dev || !out_dev || n < 0 || n > 0xFFFFFFFFll) return fail(-1, "gbns_normal: bad arguments%s");
  return check(gbns::launch_rng(4, key_dev, nullptr, out_dev, n, (cudaStream_t)stream), "gbns_normal");
}

int gbns_forward(const gbns_batch *batch, int run, const float *U_dev, float *logL_dev, long long B, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  if (run < 0 || run >= batch->num_runs || !U_dev || !logL_dev || B < 0)
    return fail(-1, "gbns_forward: bad arguments%s");
  return check(gbns::launch_forward(*batch, run, U_dev, logL_dev, B, (cudaStream_t)stream), "gbns_forward");
}

int gbns_batch_init(const gbns_batch *batch, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  // total live points = live_off + n of the last run (runs are packed in order)
  gbns_run_desc last;
  cudaError_t ce = cudaMemcpyAsync(&last, batch->runs + (batch->num_runs - 1), sizeof(last), cudaMemcpyDeviceToHost,
                                   (cudaStream_t)stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize((cudaStream_t)stream);
  if ((e = check(ce, "gbns_batch_init: reading the run table"))) return e;
  return check(gbns::launch_init(*batch, last.live_off + last.n, (cudaStream_t)stream), "gbns_batch_init");
}

int gbns_batch_iterate(const gbns_batch *batch, int num_iterations, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  if (num_iterations < 0) return fail(-1, "gbns_batch_iterate: negative iteration count%s");
  for (int it = 0; it < num_iterations; ++it) {
    if ((e = check(gbns::launch_slice_shells(*batch, nullptr, nullptr, (cudaStream_t)stream), "slice shell"))) return e;
    if ((e = check(gbns::launch_merge(*batch, (cudaStream_t)stream), "merge"))) return e;
  }
  return 0;
}

int gbns_batch_shell(const gbns_batch *batch, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  return check(gbns::launch_slice_shells(*batch, nullptr, nullptr, (cudaStream_t)stream), "gbns_batch_shell");
}

int gbns_batch_merge(const gbns_batch *batch, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  return check(gbns::launch_merge(*batch, (cudaStream_t)stream), "gbns_batch_merge");
}

int gbns_record_event(void *event, void *stream) {
  if (!event) return fail(-1, "gbns_record_event: event is NULL%s");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing((cudaStream_t)stream, &cs);
  if (e != cudaSuccess) return check(e, "gbns_record_event");
  if (cs == cudaStreamCaptureStatusActive)
    return check(cudaEventRecordWithFlags((cudaEvent_t)event, (cudaStream_t)stream, cudaEventRecordExternal),
                 "gbns_record_event");
  return check(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream), "gbns_record_event");
}

int gbns_batch_finalize(const gbns_batch *batch, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  return check(gbns::launch_finalize(*batch, (cudaStream_t)stream), "gbns_batch_finalize");
}

int gbns_batch_results(const gbns_batch *batch, const gbns_results_bufs *res, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  if (!res || !res->samples_indices || !res->num_live_points || !res->log_L_samples || !res->log_dp_mean ||
      !res->log_X_mean || !res->nevals_sorted || !res->scalars || !res->scratch_ll || !res->scratch_i)
    return fail(-1, "gbns_batch_results: missing result buffers%s");
  return check(gbns::launch_results(*batch, *res, (cudaStream_t)stream), "gbns_batch_results");
}

int gbns_slice_shell(const gbns_batch *batch, const float *Lstar_dev, const uint32_t *keys_dev, void *stream) {
  int e = check_batch(batch);
  if (e) return e;
  if (!Lstar_dev || !keys_dev) return fail(-1, "gbns_slice_shell: Lstar and keys are required%s");
  return check(gbns::launch_slice_shells(*batch, Lstar_dev, keys_dev, (cudaStream_t)stream), "gbns_slice_shell");
}

int gbns_count_crossed_edges(const int *sender_dev, const float *log_L_dev, long long N, int *samples_indices_dev,
                             int *num_live_points_dev, long long *scratch_ll_dev, int *scratch_i_dev, void *stream) {
  if (N < 0 || N >= 0x7FFFFFFFll || (N > 0 && (!sender_dev || !log_L_dev)) || !samples_indices_dev ||
      !num_live_points_dev || !scratch_ll_dev || !scratch_i_dev)
    return fail(-1, "gbns_count_crossed_edges: bad arguments%s");
  return check(gbns::launch_count_crossed_edges(sender_dev, log_L_dev, N, samples_indices_dev, num_live_points_dev,
                                                scratch_ll_dev, scratch_i_dev, (cudaStream_t)stream),
               "gbns_count_crossed_edges");
}

int gbns_evidence_stats(const float *log_L_dev, const int *num_live_dev, long long N, const double *ncoef_dev, int nmax,
                        gbns_evcalc *final_dev, double *log_X_mean_dev, double *log_dZ_mean_dev, double *log_Z_mean_dev,
                        void *stream) {
  if (N < 0 || !ncoef_dev || nmax <= 0 || !final_dev || (N > 0 && (!log_L_dev || !num_live_dev)))
    return fail(-1, "gbns_evidence_stats: bad arguments%s");
  return check(gbns::launch_evidence_stats(log_L_dev, num_live_dev, N, ncoef_dev, nmax, final_dev, log_X_mean_dev,
                                           log_dZ_mean_dev, log_Z_mean_dev, (cudaStream_t)stream),
               "gbns_evidence_stats");
}

int gbns_sample_evidence(const uint32_t *key_dev, const int *num_live_dev, const double *log_L_dev, long long M,
                         int S, double *log_Z_dev, void *stream) {
  if (M < 0 || M > 4294967295ll || S < 0 || !key_dev || (S > 0 && !log_Z_dev) ||
      (M > 0 && (!num_live_dev || !log_L_dev)))
    return fail(-1, "gbns_sample_evidence: bad arguments%s");
  return check(gbns::launch_sample_evidence(key_dev, num_live_dev, log_L_dev, M, S, log_Z_dev, (cudaStream_t)stream),
               "gbns_sample_evidence");
}

int gbns_prior_transform(const gbns_prior_table *prior, const float *U32_dev, const double *U64_dev, long long M,
                         const double *log_L_dev, double *X_dev, double *log_density_dev, void *stream) {
  if (!prior || M < 0 || prior->D <= 0 || (M > 0 && ((U32_dev == nullptr) == (U64_dev == nullptr))) ||
      !prior->kind || !prior->a || !prior->b || !prior->log_norm)
    return fail(-1, "gbns_prior_transform: bad arguments%s");
  if (prior->A && (!prior->row_start || !prior->c || prior->D > 3600))
    return fail(-1, "gbns_prior_transform: an affine map needs row_start and c, and D <= 3600%s");
  return check(gbns::launch_prior_transform(*prior, U32_dev, U64_dev, M, log_L_dev, X_dev, log_density_dev,
                                            (cudaStream_t)stream),
               "gbns_prior_transform");
}

}  // extern "C"
