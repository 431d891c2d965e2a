// gbns_launch.h -- host-side launchers shared between the translation units of libgbns.so.
#pragma once
#include <cuda_runtime.h>
#include "../../include/gbns.h"

namespace gbns {

// Lock-step chain flags of the linear-Gaussian sampler (gbns_lg_bufs.flags).
enum : int {
  LG_START = 1,
  LG_NEED_DIR = 2,
  LG_PENDING = 4,
  LG_FAILED = 8,
  LG_DONE = 16,
  LG_WAIT_REFLECT = 32,  // gradient_guided: reflect the direction at the accepted point first
  LG_HAVE_GRAD = 64      // the gradient launch has written the chain's gradient at its point
};

cudaError_t launch_slice_shells(const gbns_batch &b, const float *Lstar, const uint32_t *keys, cudaStream_t stream);
cudaError_t launch_slice_warp(const gbns_batch &b, const float *Lstar, const uint32_t *keys, cudaStream_t stream);
cudaError_t launch_init(const gbns_batch &b, long long total_points, cudaStream_t stream);
cudaError_t launch_merge(const gbns_batch &b, cudaStream_t stream);
cudaError_t launch_finalize(const gbns_batch &b, cudaStream_t stream);
cudaError_t launch_forward(const gbns_batch &b, int run, const float *U, float *logL, long long B, cudaStream_t stream);
cudaError_t launch_results(const gbns_batch &b, const gbns_results_bufs &res, cudaStream_t stream);
cudaError_t launch_count_crossed_edges(const int *sender, const float *L, long long N, int *samples_indices,
                                       int *num_live, long long *scratch_ll, int *scratch_i, cudaStream_t stream);
cudaError_t launch_evidence_stats(const float *L, const int *num_live, long long N, const double *ncoef, int nmax,
                                  gbns_evcalc *final_out, double *lX, double *ldZ, double *lZ, cudaStream_t stream);
cudaError_t launch_lg_resid_cc(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t stream);
cudaError_t launch_lg_step_kernel(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t stream);
cudaError_t launch_lg_chain_step(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t stream);
cudaError_t launch_lg_steps_tc(const gbns_batch &b, const gbns_lg_bufs &lg, int steps, cudaStream_t stream);
cudaError_t lg_tc_prepare(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t stream);
cudaError_t launch_lg_shell_fused(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t stream);
cudaError_t lg_fused_max_clusters(const gbns_lg_bufs &lg, int *out);
cudaError_t launch_adjoint_reduce(const double *log_w, long long M, int N, double log_sigma, const double *ss,
                                  const double *ry, double *out, cudaStream_t stream);
cudaError_t launch_adjoint_tc(const double *U, const double *log_w, long long M, int P, const float *Phi,
                              const float *y, int N, double log_tau, double log_sigma, double *out, double *ss,
                              double *ry, float *w_scratch, float *phi_scratch, int *status, cudaStream_t stream);
cudaError_t launch_sample_evidence(const uint32_t *key, const int *num_live, const double *log_L, long long M, int S,
                                   double *out, cudaStream_t stream);
cudaError_t launch_prior_transform(const gbns_prior_table &t, const float *U32, const double *U64, long long M,
                                   const double *log_L, double *X, double *out, cudaStream_t stream);
// Sets the thread-local message returned by gbns_last_error().
void record_error(const char *msg);
cudaError_t launch_rng(int mode, const uint32_t *key, const uint32_t *counts, void *out, long long n,
                       cudaStream_t stream);

}  // namespace gbns
