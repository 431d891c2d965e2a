/*
 * gbns.h -- C ABI of libgbns.so, the GB300 (sm_103a) nested-sampling inner loop.
 *
 * All pointers named *_dev are device pointers; the caller owns every buffer (the packed
 * per-run offsets and sizes are the caller's layout, e.g. jaxns_gb300/engine.py NSBatch;
 * gbns_abi_sizes reports the struct sizes).  The library never allocates device memory inside a run, never
 * synchronises inside gbns_batch_iterate, and reports errors through the return code
 * (0 = OK, negative = argument/launch error; message from gbns_last_error()).
 * Per-run device status words (gbns_run_state.status) carry budget/overflow errors.
 *
 * Reference interfaces replaced (paths inside the jaxns v2.6.9 source tree, src/jaxns/):
 *   gbns_batch_init       <- create_init_state            nested_samplers/common/initialisation.py:20-84
 *                            + create_init_termination_register                   :87-108
 *   gbns_batch_iterate    <- _main_ns_thread loop body    nested_samplers/sharded/sharded_static.py:487-555
 *                            (_collect_shell :210-324, get_samples :88-129,
 *                             UniDimSliceSampler.get_sample samplers/uni_slice_sampler.py:343-441,
 *                             determine_termination nested_samplers/common/termination.py:13-147)
 *   gbns_batch_finalize   <- final live-point append      sharded_static.py:833-838
 *   gbns_batch_results    <- ShardedStaticNestedSampler._to_results  sharded_static.py:652-773
 *                            (count_crossed_edges internals/tree_structure.py:33-108,
 *                             compute_evidence_stats internals/shrinkage_statistics.py:131-157)
 *   gbns_forward          <- Model.forward (vmapped)      framework/model.py:167-176
 *   gbns_threefry_split   <- jax.random.split under jax_threefry_partitionable
 *                            (set by internals/mixed_precision.py:11)
 *   gbns_random_bits64 / gbns_uniform / gbns_normal <- jax.random.bits/uniform/normal (test hooks)
 *   gbns_count_crossed_edges <- count_crossed_edges       internals/tree_structure.py:33-108
 *   gbns_evidence_stats   <- compute_evidence_stats       internals/shrinkage_statistics.py:131-157
 *   gbns_sample_evidence  <- sample_evidence              utils.py:433-484
 *   gbns_lg_shell_begin / gbns_lg_steps / gbns_lg_prepare_tc
 *                         <- _collect_shell + UniDimSliceSampler for a linear-Gaussian model
 *                            (the user likelihood N(y; Phi w, sigma^2 I), which a jaxns user
 *                            writes in JAX; no reference kernel), chains in lock step with the
 *                            Phi w contraction batched over all pending proposals
 *   gbns_evidence_adjoint / gbns_evidence_adjoint_tc
 *                         <- jax.grad of EvidenceMaximisation's reweighted log-evidence
 *                            experimental/evidence_maximisation.py:151-160 (weights :213)
 */
#ifndef GBNS_H
#define GBNS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBNS_VERSION 1

/* Rows of the shrinkage-coefficient table (gbns_batch.ncoef, gbns_evidence_stats): row n holds
 * the n-only terms of _update_evidence_calc_op (internals/shrinkage_statistics.py:55-73) for
 * n live points,
 *   doubles 0-4   FP64 log T = -log1p(1/n), log t = -log(n+1), log T2 = -log1p(2/n),
 *                 log t2 = log 2 - log(n+1) - log(n+2), log tT = -log1p(1/n) - log(n+2);
 *   bytes 64-103  the same five as fp32 pairs (hi, lo), hi = fl32(v), lo = fl32(v - hi)
 *                 (lo = 0 where hi is infinite);
 * the rest of the row is unused.  The table must be 16-byte aligned. */
#define GBNS_NCOEF_STRIDE 16

/* likelihood families (a fused CUDA likelihood cannot be an arbitrary Python callable) */
enum gbns_family {
    GBNS_LIK_MVN = 0,      /* log N(x; mu, L L^T), L lower Cholesky (params: mu, Linv, c0) */
    GBNS_LIK_SHELLS = 1,   /* logaddexp of two Gaussian shells (params: c1, c2, R, w)       */
    GBNS_LIK_LINGAUSS = 2  /* log N(y; Phi w, sigma^2 I) (params: Phi, y, sigma)            */
};

/* prior quantile per U dimension */
enum gbns_prior { GBNS_PRIOR_UNIFORM = 0, GBNS_PRIOR_NORMAL = 1 };

/* per-run status bits (gbns_run_state.status) */
enum gbns_status {
    GBNS_OK = 0,
    GBNS_ERR_INIT_BUDGET = 1,    /* init rejection sampling ran out of its evaluation budget */
    GBNS_ERR_SHRINK_BUDGET = 2,  /* a slice shrink loop ran out of its evaluation budget      */
    GBNS_ERR_STORE_FULL = 4,     /* iteration budget / store capacity exhausted               */
    GBNS_ERR_BAD_PARAM = 8,
    GBNS_ERR_WAIT_TIMEOUT = 16   /* a tensor-core kernel gave up waiting on its copies / MMAs  */
};

/* TerminationCondition (nested_samplers/common/types.py:26-60); has_* flags mark the
 * fields that are not None.  max_samples is the already-clamped limit. */
typedef struct {
    int has_ess, has_evidence_uncert, has_dlogZ, has_max_samples, has_max_nlik;
    int has_log_L_contour, has_efficiency, has_rtol, has_atol, has_peak_XL;
    double ess, evidence_uncert, dlogZ, max_samples, max_nlik;
    double log_L_contour, efficiency_threshold, rtol, atol, peak_XL_frac;
} gbns_term_cond;

/* EvidenceCalculation (nested_samplers/common/types.py:12-23), log space, FP64 */
typedef struct {
    double log_L, log_X_mean, log_X2_mean, log_Z_mean, log_ZX_mean, log_Z2_mean, log_dZ_mean, log_dZ2_mean;
} gbns_evcalc;

/* static description of one run */
typedef struct {
    int D;            /* U dimensions */
    int n;            /* live points */
    int s;            /* shell size (discards per iteration) */
    int S;            /* num_slices */
    int K;            /* phantoms saved per chain (num_phantom_save) */
    int family;       /* gbns_family */
    int midpoint;     /* midpoint_shrink */
    int uniform_phase;/* 1: run the UniformSampler phase first (init_efficiency_threshold > 0) */
    int N;            /* rows of Phi (linear-Gaussian family) */
    int ucols;      /* 32-bit words of U storage per point: D (fp32 U), or 2 D for the
                       linear-Gaussian family, whose U is FP64 (the Normal prior's tails need
                       it; stored as D doubles in the same float buffers) */
    double init_efficiency_threshold;
    double log_L_offset;   /* FP64 constant part of log L; device values are log L - log_L_offset */
    long long cap;         /* store capacity (max_samples, rounded) */
    long long live_off;    /* index of the run's first live point */
    long long store_off;   /* index of the run's first store slot */
    long long shell_off;   /* index of the run's first shell output */
    long long param_off;   /* index of the run's first float parameter */
    long long prior_off;   /* index of the run's first prior-table entry */
    long long ustore_off;  /* float offset of the run's U store, or -1 when U is not stored */
    long long liveU_off;   /* float offset of the run's live U block ([n, D]) */
    long long newU_off;    /* float offset of the run's shell-output U block ([s, D]) */
    long long phU_off;     /* float offset of the run's phantom U block ([s, K, D]) */
    long long phL_off;     /* index of the run's first phantom log L ([s, K]) */
    gbns_term_cond tc;
} gbns_run_desc;

/* TerminationRegister (types.py:127-138) + NestedSamplerState scalars (types.py:141-145) */
typedef struct {
    gbns_evcalc ev;
    gbns_evcalc ev_rem;
    double log_L_contour;
    double efficiency;
    double relative_spread;
    double absolute_spread;
    double peak_log_XL;
    long long num_likelihood_evaluations;
    long long num_samples;      /* NestedSamplerState.num_samples */
    long long next_sample_idx;  /* NestedSamplerState.next_sample_idx */
    long long iterations;
    uint32_t key[2];            /* NestedSamplerState.key */
    int plateau;
    int no_seed_points;
    int phase;                  /* 0: uniform phase, 1: slice phase, 2: finished */
    int done;                   /* termination decided for the current phase */
    int termination_reason;
    int parity;                 /* which live buffer is current */
    int status;                 /* gbns_status bits */
    int pad1;
} gbns_run_state;

/* Log-likelihoods are held on the device in fp32 relative to the run's FP64 log_L_offset
 * (e.g. the Gaussian normalisation), so the resolution near a likelihood peak is that of
 * -0.5 z^2 rather than of the absolute value; the shift is monotone, so every comparison,
 * tie and sort order is that of the absolute values.  FP64 code adds the offset back.
 * device buffers of a batch of runs (all *_dev, caller-allocated) */
typedef struct {
    int num_runs;
    int nmax;                       /* largest n over runs (<= 4096) */
    int ncoef_n;                    /* largest count covered by the ncoef table */
    const gbns_run_desc *runs;      /* [R] */
    gbns_run_state *state;          /* [R] */
    float *live_U[2];               /* [sum n*D] */
    float *live_L[2];               /* [sum n] */
    float *live_Lc[2];              /* [sum n] */
    int *live_E[2];                 /* [sum n] likelihood evaluations */
    int *live_S[2];                 /* [sum n] sender node */
    float *new_U;                   /* [sum s*D] */
    float *new_L;                   /* [sum s] */
    int *new_E;                     /* [sum s] */
    float *ph_U;                    /* [sum s*K*D] */
    float *ph_L;                    /* [sum s*K] */
    float *store_L;                 /* [sum cap] */
    int *store_S;                   /* [sum cap] */
    int *store_E;                   /* [sum cap] */
    uint8_t *store_P;               /* [sum cap] phantom flag */
    float *store_U;                 /* [sum cap*D] or NULL */
    const float *fparams;           /* family parameters */
    const int *prior_kind;          /* [sum D] */
    const float *prior_a;           /* [sum D] */
    const float *prior_b;           /* [sum D] */
    const double *ncoef;            /* [(ncoef_n+1) * GBNS_NCOEF_STRIDE] shrinkage coefficients per count
                                       (layout at GBNS_NCOEF_STRIDE) */
    const int *items;               /* [num_items * 4] (run, chain_begin, chain_count, 0) */
    int num_items;
    int bucket_begin[8];            /* work-item ranges per dimension bucket */
    int bucket_end[8];
    int chains_per_item;
    int max_evals_per_slice;        /* shrink-loop evaluation budget per slice */
    int gradient_guided;            /* UniDimSliceSampler(gradient_guided=True): after each accepted point
                                       the direction is reflected about the U-space gradient of log L
                                       (every family; the linear-Gaussian family on its lock step) */
    int gradient_slice;             /* UniDimSliceSampler(gradient_slice=True): every slice runs along the
                                       normalised U-space gradient at its seed point, t in [0, right]
                                       (one extra evaluation per slice; every family, the linear-Gaussian
                                       family on its lock step) */
} gbns_batch;

/* Lock-step chain state of the linear-Gaussian family (device, caller-allocated).  Its
 * likelihood is one dense contraction over all proposals of a step, so the slice sampler
 * runs as alternating launches: gbns_lg_step (slice logic + next proposal per chain) and a
 * batched residual kernel (|y - Phi w|^2 for every pending proposal).  Per-chain arrays are
 * indexed like the shell outputs ([sum s] and [sum s * D]). */
typedef struct {
    int *j, *in_slice, *total, *flags;      /* [sum s] */
    float *left, *right, *t, *alpha, *logL0; /* [sum s] slice interval, point, shrink factor */
    uint32_t *ck, *after_key, *slices_key, *dir_key; /* [sum s * 2] */
    float *u0, *u0_lo, *dir;                /* [sum s * D]: seed point as an fp32 pair u0 + u0_lo (U space
                                               to ~1e-14 near 0 and 1), direction */
    float *W;                               /* [sum s * D]: proposal w (CUDA-core residual path) */
    double *ss;                             /* [sum s] residual sums of the pending proposals */
    int *chains_left;                       /* [R] chains of the current shell not yet finished */
    const int *items;                       /* [num_items * 4]: (run, first chain, chain count, first data row) */
    int num_items;
    int pmax;                               /* largest D (= P) over the runs, <= 64 */
    long long total_chains;                 /* sum of s over the runs */
    /* Tensor-core (tcgen05) residual path, used when use_tc != 0 (after gbns_lg_prepare_tc
     * has filled Phi_hi / Phi_lo).  Proposals and Phi are held as TF32 hi + lo parts, rows
     * padded to 64 floats (256 B, zero beyond P); the contraction is hi*hi + hi*lo + lo*hi
     * (3xTF32).  Work units: (run, 128-chain tile, range of 128-row tiles), walked by a
     * persistent kernel of num_ctas_tc CTAs. */
    int use_tc;
    int num_items_tc;
    const int *items_tc;                    /* [num_items_tc * 4]: (run, first chain (multiple of 128),
                                               first 128-row tile, number of row tiles) */
    float *W_hi, *W_lo;                     /* [total_chains * 64], row = global chain index */
    float *Phi_hi, *Phi_lo;                 /* [total_rows * 64] */
    const long long *row_base;              /* [R] first row of each run in Phi_hi / Phi_lo */
    long long total_rows;                   /* sum of N over the runs */
    int num_ctas_tc;                        /* cap on the persistent grid; 0 = one CTA per SM (two when
                                               every P <= 32) */
    int num_tiles;                          /* 128-chain tiles over all runs */
    const int *chain_run;                   /* [total_chains] run of each chain */
    const int *tile_base;                   /* [R] first 128-chain tile of each run */
    int *tile_pending;                      /* [num_tiles] set by the chain step when a chain of the tile
                                               has a pending proposal; cleared by the residual launch */
    int *tc_done;                           /* [1] CTA completion counter of the residual launch (zeroed) */
    /* Fused shell (gbns_lg_shell_fused / gbns_lg_iterate): one thread-block cluster of
     * cluster_size CTAs per (run, 128-chain tile); CTA rank q holds data rows
     * [q * rows_per_cta, (q + 1) * rows_per_cta) of the run's Phi (TF32 hi / lo) in shared
     * memory for the whole shell and owns chains q * (128 / cluster_size) ... of the tile. */
    const int *items_fused;                 /* [num_items_fused * 2]: (run, first chain of the tile) */
    int num_items_fused;
    int cluster_size;                       /* 4, 8 or 16 */
    int rows_per_cta;                       /* 128, 256 or 512; rows_per_cta * ceil(pmax / 32) <= 512 */
    int pad_fused;
    long long max_steps;                    /* lock-step budget of one shell (sets GBNS_ERR_SHRINK_BUDGET) */
    /* The slice sampler's gradient options (gbns_batch.gradient_guided / gradient_slice) on the
     * lock step: a chain that needs the U-space gradient at its point sits out one step while
     * a gradient launch computes Phi^T (y - Phi w) / sigma^2 times dw/du for every listed chain.
     * Not used by the fused shell. */
    float *grad;                            /* [sum s * D] the gradient of each listed chain */
    long long *grad_list;                   /* [sum s] chains that asked for a gradient this step */
    int *grad_count;                        /* [1] entries of grad_list (zeroed before each chain step) */
} gbns_lg_bufs;

/* results buffers (device) */
typedef struct {
    int *samples_indices;           /* [sum cap] */
    int *num_live_points;           /* [sum cap] */
    double *log_L_samples;          /* [sum cap] sorted, absolute (offset added in FP64) */
    double *log_dp_mean;            /* [sum cap] */
    double *log_X_mean;             /* [sum cap] */
    int *nevals_sorted;             /* [sum cap] */
    float *U_sorted;                /* [sum cap*D] or NULL */
    double *scalars;                /* [R * 8]: log_Z_mean, log_Z_uncert, ESS, H_mean,
                                       total_num_samples, total_phantom, total_nevals, log_efficiency */
    long long *scratch_ll;          /* [2 * (sum cap + R)] sort scratch */
    int *scratch_i;                 /* [sum cap + R] degree scratch */
} gbns_results_bufs;

int gbns_version(void);
const char *gbns_last_error(void);
/* sizeof of gbns_term_cond, gbns_evcalc, gbns_run_desc, gbns_run_state, gbns_batch,
 * gbns_results_bufs (binding self-check; no reference counterpart) */
int gbns_abi_sizes(long long *out, int n);

/* RNG test hooks (device pointers): key is [2] uint32 */
int gbns_threefry2x32(const uint32_t *key_dev, const uint32_t *counts_dev, uint32_t *out_dev, long long n,
                      void *stream);
int gbns_threefry_split(const uint32_t *key_dev, uint32_t *out_dev, long long n, void *stream);
int gbns_random_bits64(const uint32_t *key_dev, uint64_t *out_dev, long long n, void *stream);
int gbns_uniform(const uint32_t *key_dev, float *out_dev, long long n, void *stream);
int gbns_normal(const uint32_t *key_dev, float *out_dev, long long n, void *stream);

/* Model.forward over B points of one run's model: U [B, ucols] words -> log L [B]
 * (fp32 U [B, D], or FP64 U [B, D] for the linear-Gaussian family) */
int gbns_forward(const gbns_batch *batch, int run, const float *U_dev, float *logL_dev, long long B,
                 void *stream);

/* NS batch: init, K iterations (graph-capturable), finalize, results */
int gbns_batch_init(const gbns_batch *batch, void *stream);
int gbns_batch_iterate(const gbns_batch *batch, int num_iterations, void *stream);
int gbns_batch_finalize(const gbns_batch *batch, void *stream);
/* the two halves of one iteration (gbns_batch_iterate = shell + merge), so a caller can
 * time the slice sampler separately:
 *   gbns_batch_shell <- get_samples / UniDimSliceSampler.get_sample for every active run
 *                       (sharded_static.py:88-129, uni_slice_sampler.py:343-441)
 *   gbns_batch_merge <- the rest of _collect_shell + the while-loop condition
 *                       (sharded_static.py:240-323, :480-485, :833-838) */
int gbns_batch_shell(const gbns_batch *batch, void *stream);
/* record a CUDA event on a stream; inside stream capture it becomes an event-record node of
 * the graph, so kernel time can be read back after each replay (timing plumbing; no
 * reference counterpart) */
int gbns_record_event(void *event, void *stream);
int gbns_batch_merge(const gbns_batch *batch, void *stream);
int gbns_batch_results(const gbns_batch *batch, const gbns_results_bufs *res, void *stream);

/* One shell of the slice sampler for every run (test hook: no merge, no register);
 * Lstar_dev holds each run's contour relative to its log_L_offset */
int gbns_slice_shell(const gbns_batch *batch, const float *Lstar_dev, const uint32_t *keys_dev, void *stream);

/* Standalone tree count and evidence statistics for one sample set (device pointers) */
int gbns_count_crossed_edges(const int *sender_dev, const float *log_L_dev, long long N, int *samples_indices_dev,
                             int *num_live_points_dev, long long *scratch_ll_dev, int *scratch_i_dev, void *stream);
/* count_crossed_edges with no device allocation and no caller scratch, for callers that
 * cannot call cudaMalloc (a host runtime that owns all device memory, such as an XLA FFI
 * custom call; a real-time pipeline that cannot take cudaMalloc's implicit synchronisation;
 * a deployment that forbids allocation after start-up).  No counterpart in the reference.
 * Scratch is a file-scope device array (5 MiB per device, held until exit) shared by every
 * call: N <= 262143, the first call on a device sets up its address (make it before any
 * stream capture), and calls that overlap on the GPU race.  The address is looked up once per
 * device index and kept for the life of the process: it belongs to the device's primary
 * context (the CUDA runtime's), so the entry point is not for callers that run it under a
 * context of their own, and it must not be called again after cudaDeviceReset (the module's
 * device memory, and with it the cached address, is gone). */
int gbns_count_crossed_edges_static(const int *sender_dev, const float *log_L_dev, long long N,
                                    int *samples_indices_dev, int *num_live_points_dev, void *stream);
/* Linear-Gaussian family: start a shell for every active run (seed points, keys), then
 * advance every chain num_steps likelihood evaluations (graph-capturable).  When every
 * run's chains_left is 0, gbns_batch_merge completes the iteration.
 *   <- get_samples / UniDimSliceSampler.get_sample (sharded_static.py:88-129,
 *      uni_slice_sampler.py:343-441) for a likelihood evaluated in batches */
int gbns_lg_shell_begin(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream);
int gbns_lg_steps(const gbns_batch *batch, const gbns_lg_bufs *lg, int num_steps, void *stream);
/* The two halves of one gbns_lg_steps step: the chain step (consume the pending residuals,
 * propose the next point) and the residual contraction of all pending proposals. */
int gbns_lg_chain_step(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream);
int gbns_lg_residual(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream);
/* One whole linear-Gaussian shell in one launch: every chain of every active run from its seed
 * to its last slice (the work of gbns_lg_shell_begin + gbns_lg_steps until chains_left is 0),
 * with thread-block clusters that keep their share of Phi in shared memory, run the 3xTF32
 * tcgen05 contraction of each step's proposals and sum the residuals across the cluster in
 * distributed shared memory (no grid-wide synchronisation, no host round trip).  Needs
 * gbns_lg_prepare_tc and the fused fields of lg.  Graph-capturable.
 *   <- get_samples / UniDimSliceSampler.get_sample (sharded_static.py:88-129,
 *      uni_slice_sampler.py:343-441) for a likelihood evaluated in batches
 * gbns_lg_iterate: num_iterations x (fused shell + gbns_batch_merge)
 *   <- the _main_ns_thread loop body (sharded_static.py:487-555) */
int gbns_lg_shell_fused(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream);
int gbns_lg_iterate(const gbns_batch *batch, const gbns_lg_bufs *lg, int num_iterations, void *stream);
/* How many clusters of lg's fused configuration the current device holds at once (0: the
 * configuration cannot launch here; choose a smaller cluster).  No reference counterpart. */
int gbns_lg_fused_max_clusters(const gbns_batch *batch, const gbns_lg_bufs *lg, int *max_clusters);
/* Split each run's Phi (fparams) into the TF32 hi/lo row-padded copies lg->Phi_hi / Phi_lo
 * read by the tensor-core residual path.  Call once per batch, before the first step (and
 * after new parameters). */
int gbns_lg_prepare_tc(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream);

/* Reweighted fixed-dead-point evidence of the linear-Gaussian model and its gradient
 * (experimental/evidence_maximisation.py:151-160, weights :213):
 *   log Z(theta) = logsumexp_i(log L_theta(U_i) + log_w_i),  w_i = tau * ndtri(U_i),
 *   out[0] = log Z(theta), out[1] = d/d log tau, out[2] = d/d log sigma  (FP64 reductions).
 * Per-point residuals are recomputed from U [M, P] (FP64), never stored.  ss_scratch,
 * ry_scratch: [M]. */
int gbns_evidence_adjoint(const double *U_dev, const double *log_w_dev, long long M, int P, const float *Phi_dev,
                          const float *y_dev, int N, double log_tau, double log_sigma, double *out_dev,
                          double *ss_scratch_dev, double *ry_scratch_dev, void *stream);
/* The same on the tcgen05 tensor cores (3xTF32 contraction).  Extra scratch, with
 * ld = 32 for P <= 32 and 64 otherwise: w_scratch [2 * M * ld] floats, phi_scratch
 * [2 * N * ld] floats; status_dev: one int, GBNS_ERR_WAIT_TIMEOUT is or-ed in if a wait of
 * the kernel timed out (the outputs are then invalid).  M < 2^31. */
int gbns_evidence_adjoint_tc(const double *U_dev, const double *log_w_dev, long long M, int P, const float *Phi_dev,
                             const float *y_dev, int N, double log_tau, double log_sigma, double *out_dev,
                             double *ss_scratch_dev, double *ry_scratch_dev, float *w_scratch_dev,
                             float *phi_scratch_dev, int *status_dev, void *stream);
/* sample_evidence (utils.py:433-484): S replicas of log Z with the shrinkage T_i ~ Beta(n_i, 1)
 * drawn from the jax key (key_dev: 2 words); num_live, log_L: the sorted samples' live-point
 * counts and log-likelihoods (FP64), M < 2^32; log_Z_dev: [S]. */
int gbns_sample_evidence(const uint32_t *key_dev, const int *num_live_dev, const double *log_L_dev, long long M,
                         int S, double *log_Z_dev, void *stream);
/* The prior of a model, one entry per U dimension (device pointers), for gbns_prior_transform. */
typedef struct {
    int D;
    const int *kind;        /* [D] gbns_prior */
    const double *a, *b;    /* [D] Uniform: low, high - low; Normal: loc, scale */
    const double *log_norm; /* [D] the density's constant: -log b (Uniform), -log b - log(2 pi) / 2 (Normal) */
    const double *A;        /* [D, D] row-major lower-triangular map X = A q + c over the
                               MultivariateNormalTriL blocks (q their standard normals), or NULL: X = q */
    const int *row_start;   /* [D] first column of row d's nonzeros in A (with A) */
    const double *c;        /* [D] (with A) */
    double log_det;         /* added to every log density: -sum log L_ii over the blocks */
} gbns_prior_table;

/* Model.transform and Model.log_prob_prior (framework/model.py:155-187) of M sample rows, as
 * _to_results applies them to the sorted samples (sharded_static.py:744-745): U is fp32
 * (U32_dev) or FP64 (U64_dev, the linear-Gaussian family), exactly one of them given, [M, D]
 * row-major; X_dev [M, D] FP64 or NULL; log_density_dev [M] FP64 or NULL receives
 * log_L_dev[i] + log p(X_i) (log_L_dev NULL: the prior density alone).  D <= 3600 with A. */
int gbns_prior_transform(const gbns_prior_table *prior, const float *U32_dev, const double *U64_dev, long long M,
                         const double *log_L_dev, double *X_dev, double *log_density_dev, void *stream);
/* compute_evidence_stats over one sorted sample set: ncoef_dev is a coefficient table of nmax + 1
 * rows (GBNS_NCOEF_STRIDE) */
int gbns_evidence_stats(const float *log_L_dev, const int *num_live_dev, long long N, const double *ncoef_dev,
                        int nmax, gbns_evcalc *final_dev, double *log_X_mean_dev, double *log_dZ_mean_dev,
                        double *log_Z_mean_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif
