// gbns_results.cu -- sample-tree live-point counting, FP64 evidence statistics and the
// NestedSamplerResults scalars (ShardedStaticNestedSampler._to_results,
// nested_samplers/sharded/sharded_static.py:652-773), plus the RNG test hooks.
//
// count_crossed_edges (internals/tree_structure.py:33-108) needs a stable argsort of the
// N+1 node log-likelihoods.  Dead points are appended in non-decreasing order except for
// phantoms and rejection-sampler caps, so the CTA first tests sortedness and only runs the
// LSD radix sort (4 x 8-bit digits, stable by construction) when it is needed.
#include "gbns_device.cuh"
#include "gbns_launch.h"

namespace gbns {

__device__ __forceinline__ unsigned long long node_key(const float *L, long long i) {
  // node 0 is the root at -inf; node i+1 is sample i
  const float v = i == 0 ? -INFINITY : L[i - 1];
  return ((unsigned long long)ordered_key(v) << 32) | (unsigned long long)(unsigned)i;
}

struct RadixSmem {
  int wcount[32][257];
  int base[256];
  int tile_count[256];
  int hist[4][256];
  int flag;
  long long carry;
};

// LSD radix sort (4 x 8-bit digits of the upper 32 bits, stable by construction) of the
// M keys in a, with tmp as the ping-pong buffer; sm.hist holds the digit histograms.  The
// result is in a (an even number of passes).  blockDim.x must be 1024.
__device__ void cta_radix_keys(long long M, unsigned long long *a, unsigned long long *tmp, RadixSmem &sm);

// Whether the N+1 node keys are already in order (the usual case: dead points arrive sorted),
// and, when deg is given (zeroed by the caller), the out-degrees of the sender tree counted in
// the same pass over the store: out_degree.at[max(sender, 0)].add(1) (tree_structure.py:82-84);
// like jax's scatter, an update outside [0, N] is dropped, so a bad sender never writes past
// the scratch.  Four strided elements per thread per pass, their loads in flight together.
__device__ int cta_nodes_in_order(const float *L, const int *sender, long long N, int *deg, RadixSmem &sm) {
  const long long M = N + 1;
  const int tid = threadIdx.x;
  if (tid == 0) sm.flag = 1;
  __syncthreads();
  int sorted = 1;
  for (long long i0 = tid; i0 < M; i0 += 4ll * blockDim.x) {
    int sd[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long i = i0 + (long long)j * blockDim.x;
      sd[j] = deg && i < N ? max(sender[i], 0) : -1;
      if (i >= 1 && i < M && (node_key(L, i - 1) >> 32) > (node_key(L, i) >> 32)) sorted = 0;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (sd[j] >= 0 && (long long)sd[j] <= N) atomicAdd(&deg[sd[j]], 1);
  }
  if (!sorted) sm.flag = 0;
  __syncthreads();
  return sm.flag;
}

// Stable ascending sort of the N+1 node keys (by their upper 32 bits) of a store that is out
// of order: the keys in a (perm in the low 32 bits).  a, tmp: [N+1] scratch.  blockDim.x must
// be 1024.
__device__ const unsigned long long *cta_sort_node_keys(const float *L, long long N, unsigned long long *a,
                                                        unsigned long long *tmp, RadixSmem &sm) {
  const long long M = N + 1;
  const int tid = threadIdx.x;
  for (int q = tid; q < 4 * 256; q += blockDim.x) (&sm.hist[0][0])[q] = 0;
  __syncthreads();
  for (long long i = tid; i < M; i += blockDim.x) {
    const unsigned long long k = node_key(L, i);
    a[i] = k;
    const uint32_t key = (uint32_t)(k >> 32);
#pragma unroll
    for (int d = 0; d < 4; ++d) atomicAdd(&sm.hist[d][(key >> (8 * d)) & 255], 1);
  }
  __syncthreads();
  cta_radix_keys(M, a, tmp, sm);
  return a;
}

__device__ void cta_radix_keys(long long M, unsigned long long *a, unsigned long long *tmp, RadixSmem &sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  unsigned long long *src = a, *dst = tmp;
  for (int d = 0; d < 4; ++d) {
    // exclusive prefix of the digit histogram
    if (tid == 0) {
      int acc = 0;
      for (int q = 0; q < 256; ++q) {
        sm.base[q] = acc;
        acc += sm.hist[d][q];
      }
    }
    for (int q = tid; q < 32 * 257; q += blockDim.x) (&sm.wcount[0][0])[q] = 0;
    __syncthreads();
    for (long long t0 = 0; t0 < M; t0 += blockDim.x) {
      const long long i = t0 + tid;
      const bool valid = i < M;
      const unsigned long long k = valid ? src[i] : 0ull;
      const int dig = valid ? (int)(((uint32_t)(k >> 32) >> (8 * d)) & 255) : 256;
      const unsigned peers = __match_any_sync(0xffffffffu, dig);
      const int rank = __popc(peers & ((1u << lane) - 1u));
      if (valid && rank == 0) sm.wcount[warp][dig] = __popc(peers);
      __syncthreads();
      if (tid < 256) {
        int run = 0;
        for (int w = 0; w < 32; ++w) {
          const int c = sm.wcount[w][tid];
          sm.wcount[w][tid] = run;
          run += c;
        }
        sm.tile_count[tid] = run;
      }
      __syncthreads();
      if (valid) dst[sm.base[dig] + sm.wcount[warp][dig] + rank] = k;
      __syncthreads();
      if (tid < 256) {
        sm.base[tid] += sm.tile_count[tid];
        for (int w = 0; w < 32; ++w) sm.wcount[w][tid] = 0;
      }
      __syncthreads();
    }
    unsigned long long *t = src;
    src = dst;
    dst = t;
  }
}

// count_crossed_edges on one sample set (static variant).  perm: sorted node keys, or nullptr
// for nodes already in order.  deg: [N+1] scratch.  Outputs [N]; visit(pos, k) is called once
// for every sorted position pos < N with its sample index k (the caller's gather).
struct NoVisit {
  __device__ void operator()(long long, int) const {}
};

template <typename Visit>
__device__ void cta_count_edges(const int *sender, long long N, const unsigned long long *perm, int *deg,
                                int *samples_indices, int *num_live, RadixSmem &sm, bool deg_ready, Visit visit) {
  constexpr int K = 4;  // elements per thread per pass: their loads are in flight together
  const long long M = N + 1;
  const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, w = tid >> 5, nw = T >> 5;
  if (!deg_ready) {
    for (long long i = tid; i < M; i += T) deg[i] = 0;
    __syncthreads();
  }
  // out_degree.at[max(sender, 0)].add(1) (tree_structure.py:82-84); like jax's scatter, an
  // update outside [0, N] is dropped, so a bad sender never writes past the scratch
  for (long long i0 = tid; i0 < (deg_ready ? 0 : N); i0 += (long long)K * T) {
    int sd[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long i = i0 + (long long)j * T;
      sd[j] = i < N ? max(sender[i], 0) : -1;
    }
#pragma unroll
    for (int j = 0; j < K; ++j)
      if (sd[j] >= 0 && (long long)sd[j] <= N) atomicAdd(&deg[sd[j]], 1);
  }
  if (tid == 0) sm.carry = 1;
  __syncthreads();
  __shared__ long long wsum[32];
  // crossed-edge scan over the sorted positions, K consecutive positions per thread
  for (long long base = 0; base < M; base += (long long)K * T) {
    const long long i0 = base + (long long)tid * K;
    int node[K], v[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long i = i0 + j;
      node[j] = i < M ? (perm ? (int)(perm[i] & 0xffffffffu) : (int)i) : 0;
    }
#pragma unroll
    for (int j = 0; j < K; ++j) v[j] = i0 + j < M ? deg[node[j]] - 1 : 0;
    // the caller's gather has no part in the scan: its loads go out before the barriers
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long i = i0 + j;
      if (i >= 1 && i < M) {
        samples_indices[i - 1] = node[j] - 1;
        visit(i - 1, node[j] - 1);
      }
    }
    int loc[K];
    int run = 0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      run += v[j];
      loc[j] = run;
    }
    const long long tsum = run;
    const long long incl = warp_incl_scan(tsum);
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
      long long x = lane < nw ? wsum[lane] : 0;
      x = warp_incl_scan(x);
      wsum[lane] = x;
    }
    __syncthreads();
    const long long excl = sm.carry + (incl - tsum) + (w > 0 ? wsum[w - 1] : 0);
#pragma unroll
    for (int j = 0; j < K; ++j)
      if (i0 + j < N) num_live[i0 + j] = (int)(excl + loc[j]);
    __syncthreads();
    if (tid == T - 1) sm.carry = excl + loc[K - 1];  // positions past M add nothing
    __syncthreads();
  }
}

// count_crossed_edges (internals/tree_structure.py:33-108) of one sample set on one CTA:
// stable sort of the N+1 nodes, out-degrees, crossed-edge scan (gbns_count_crossed_edges).
__global__ void __launch_bounds__(1024) k_count_edges(const int *sender, const float *L, long long N,
                                                      int *samples_indices, int *num_live,
                                                      unsigned long long *scratch, int *deg) {
  __shared__ RadixSmem sm;
  const unsigned long long *perm =
      cta_nodes_in_order(L, nullptr, N, nullptr, sm) ? nullptr : cta_sort_node_keys(L, N, scratch, scratch + (N + 1), sm);
  cta_count_edges(sender, N, perm, deg, samples_indices, num_live, sm, false, NoVisit{});
}

// ---- count_crossed_edges of one large sample set over many CTAs ---------------------------
//
// A: node keys, sortedness, out-degrees (grid-wide; flag and degrees zeroed before);
// B: one CTA radix-sorts the keys in place only when A found them out of order;
// C: per chunk of the sorted order, the sum of (out-degree - 1);
// D: one CTA turns the chunk sums into exclusive prefixes;
// E: per chunk, the crossed-edge scan from its prefix and the outputs.
// Every step is integer arithmetic, so the result is the single-CTA kernel's, bit for bit.
constexpr int CE_CHUNK = 4096;  // sorted positions per CTA in C and E

__global__ void __launch_bounds__(256) k_ce_keys(const int *sender, const float *L, long long N, unsigned long long *a,
                                                 unsigned long long *flag, int *deg) {
  const long long M = N + 1;
  int unsorted = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = node_key(L, i);
    a[i] = k;
    if (i > 0 && (node_key(L, i - 1) >> 32) > (k >> 32)) unsorted = 1;
    if (i < N) {
      const int sd = max(sender[i], 0);
      if ((long long)sd <= N) atomicAdd(&deg[sd], 1);
    }
  }
  if (__any_sync(0xffffffffu, unsorted) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
}

__global__ void __launch_bounds__(1024) k_ce_sort(long long N, unsigned long long *a, unsigned long long *tmp,
                                                  const unsigned long long *flag) {
  __shared__ RadixSmem sm;
  // every thread reads the flag before the first barrier, and the sort writes tmp (which
  // holds the flag) only after it
  if (*flag == 0ull) return;  // already in order (the usual case: dead points arrive sorted)
  const long long M = N + 1;
  for (int q = threadIdx.x; q < 4 * 256; q += blockDim.x) (&sm.hist[0][0])[q] = 0;
  __syncthreads();
  for (long long i = threadIdx.x; i < M; i += blockDim.x) {
    const uint32_t key = (uint32_t)(a[i] >> 32);
#pragma unroll
    for (int d = 0; d < 4; ++d) atomicAdd(&sm.hist[d][(key >> (8 * d)) & 255], 1);
  }
  __syncthreads();
  cta_radix_keys(M, a, tmp, sm);
}

__global__ void __launch_bounds__(256) k_ce_chunk_sums(long long N, const unsigned long long *perm, const int *deg,
                                                       long long *bsum) {
  __shared__ long long red[32];
  const long long M = N + 1, i0 = (long long)blockIdx.x * CE_CHUNK;
  long long v = 0;
  for (long long i = i0 + threadIdx.x; i < min(M, i0 + CE_CHUNK); i += blockDim.x)
    v += (long long)deg[(int)(perm[i] & 0xffffffffu)] - 1;
  v = cta_sum_ll(v, red);
  if (threadIdx.x == 0) bsum[blockIdx.x] = v;
}

__global__ void __launch_bounds__(1024) k_ce_chunk_scan(long long *bsum, int nchunks) {
  __shared__ long long wsum[32];
  __shared__ long long carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 1;  // crossed edges before the first node: the root's one edge
  __syncthreads();
  for (int c0 = 0; c0 < nchunks; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    const long long x = c < nchunks ? bsum[c] : 0;
    long long v = warp_incl_scan(x);
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    if (w == 0) {
      long long y = wsum[lane];
      y = warp_incl_scan(y);
      wsum[lane] = y;
    }
    __syncthreads();
    const long long incl = carry + v + (w > 0 ? wsum[w - 1] : 0);
    if (c < nchunks) bsum[c] = incl - x;  // exclusive prefix, including the initial 1
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024) k_ce_chunk_out(long long N, const unsigned long long *perm, const int *deg,
                                                       const long long *bsum, int *samples_indices, int *num_live) {
  __shared__ long long wsum[32];
  __shared__ long long carry;
  const long long M = N + 1, i0 = (long long)blockIdx.x * CE_CHUNK, i1 = min(M, i0 + CE_CHUNK);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = bsum[blockIdx.x];
  __syncthreads();
  for (long long t0 = i0; t0 < i1; t0 += blockDim.x) {
    const long long i = t0 + threadIdx.x;
    const int node = i < i1 ? (int)(perm[i] & 0xffffffffu) : 0;
    long long v = i < i1 ? (long long)deg[node] - 1 : 0;
    v = warp_incl_scan(v);
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    if (w == 0) {
      long long y = wsum[lane];
      y = warp_incl_scan(y);
      wsum[lane] = y;
    }
    __syncthreads();
    const long long crossed = carry + v + (w > 0 ? wsum[w - 1] : 0);
    if (i < N && i < i1) num_live[i] = (int)crossed;
    if (i >= 1 && i < i1) samples_indices[i - 1] = node - 1;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = crossed;
    __syncthreads();
  }
}

// Evidence scans over sample sets: threads per CTA and consecutive samples per thread.
constexpr int RESULTS_K = 4;
constexpr int RESULTS_EV_THREADS = 512;

// compute_evidence_stats (internals/shrinkage_statistics.py:131-157) of one sample set on one
// CTA: the final register and the per-sample log X, log dZ and log Z, FP64 (gbns_evidence_stats).
template <bool OUT_LZ>
__global__ void __launch_bounds__(RESULTS_EV_THREADS)
    k_evidence_stats(const float *L, const int *nl, long long N, const double *ncoef, int nmax, gbns_evcalc *fin,
                     double *lX, double *ldZ, double *lZ) {
  __shared__ EvScanSmem esm;
  gbns_evcalc e;
  e.log_L = -INFINITY; e.log_X_mean = 0.0; e.log_X2_mean = 0.0; e.log_Z_mean = -INFINITY;
  e.log_ZX_mean = -INFINITY; e.log_Z2_mean = -INFINITY; e.log_dZ_mean = -INFINITY; e.log_dZ2_mean = -INFINITY;
  EvAcc acc = evacc_from(e);
  evidence_scan_cta<OUT_LZ, RESULTS_K>(acc, L, N, 0, 0, nl, ncoef, nmax, lX, ldZ, lZ, 0.0, nullptr, esm);
  if (threadIdx.x == 0) *fin = evacc_to(acc, N > 0 ? (double)L[N - 1] : -INFINITY);
}

// ------------------------------------------------------------ results ----

// _to_results (sharded_static.py:652-773) for every run of a batch, one CTA per run, in two
// launches.  k_results_tree: tree count of the run's store and the gather in sorted order
// (1024 threads: the radix sort and the crossed-edge scan are latency-bound passes).
// k_results_ev: FP64 evidence per sample, log Z mean and uncertainty with the phantom
// correction, ESS, H, efficiency (512 threads of RESULTS_K consecutive samples each: the
// evidence scan is instruction-bound and runs its prefixes per thread; 256 x 8 and 1024 x 1
// were slower, 256 x 8 by 1.3x: too few warps to hide the per-thread chains).

__global__ void __launch_bounds__(1024) k_results_tree(gbns_batch b, gbns_results_bufs res, int deg_smem_cap) {
  extern __shared__ int sdeg[];  // the out-degrees of a run of up to deg_smem_cap - 1 samples
  __shared__ RadixSmem sm;
  __shared__ long long lred[32];
  const int r = blockIdx.x;
  const gbns_run_desc &rd = b.runs[r];
  const gbns_run_state &st = b.state[r];
  const long long N = st.num_samples < rd.cap ? st.num_samples : rd.cap;
  const long long so = rd.store_off;
  const int D = rd.ucols;  // 32-bit words of U per sample
  unsigned long long *scratch = (unsigned long long *)res.scratch_ll + 2 * (so + r);
  int *deg_g = res.scratch_i + (so + r);
  int *deg = N + 1 <= deg_smem_cap ? sdeg : deg_g;  // shared-memory atomics and reads when they fit
  int *si = res.samples_indices + so;
  int *nl = res.num_live_points + so;
  // out-degrees counted in the pass that checks the order
  for (long long i = threadIdx.x; i < N + 1; i += blockDim.x) deg[i] = 0;
  __syncthreads();
  const unsigned long long *perm = cta_nodes_in_order(b.store_L + so, b.store_S + so, N, deg, sm)
                                       ? nullptr
                                       : cta_sort_node_keys(b.store_L + so, N, scratch, scratch + (N + 1), sm);
  // the gather in sorted order rides on the crossed-edge scan's pass over the sorted positions
  double *Ls = res.log_L_samples + so;
  const double off = rd.log_L_offset;
  int *Es = res.nevals_sorted + so;
  const float *Lst = b.store_L + so;
  const int *Est = b.store_E + so;
  const uint8_t *Pst = b.store_P + so;
  long long ev_sum = 0, ph_sum = 0;
  cta_count_edges(b.store_S + so, N, perm, deg, si, nl, sm, true, [&](long long pos, int k) {
    Ls[pos] = (double)Lst[k] + off;
    const int e = Est[k];
    Es[pos] = e;
    ev_sum += e;
    ph_sum += Pst[pos];
  });
  __syncthreads();
  if (res.U_sorted && rd.ustore_off >= 0 && b.store_U) {
    float *Us = res.U_sorted + rd.ustore_off;
    const float *Ust = b.store_U + rd.ustore_off;
    for (long long q = threadIdx.x; q < N * D; q += blockDim.x) {
      const long long i = q / D, j = q % D;
      Us[q] = Ust[(long long)si[i] * D + j];
    }
  }
  const long long total_evals = cta_sum_ll(ev_sum, lred);
  const long long total_phantom = cta_sum_ll(ph_sum, lred);
  if (threadIdx.x == 0) {
    double *sc = res.scalars + 8 * (size_t)r;
    sc[4] = (double)N;
    sc[5] = (double)total_phantom;
    sc[6] = (double)total_evals;
    deg_g[0] = perm != nullptr;  // the degree scratch is spent: its first word tells the evidence pass to gather
  }
}

template <int K>
__global__ void __launch_bounds__(RESULTS_EV_THREADS) k_results_ev(gbns_batch b, gbns_results_bufs res) {
  __shared__ double s_lz[4];
  __shared__ double s_h[2];
  __shared__ double dred[32];
  __shared__ EvScanSmem esm;
  const int r = blockIdx.x;
  const gbns_run_desc &rd = b.runs[r];
  const gbns_run_state &st = b.state[r];
  const long long N = st.num_samples < rd.cap ? st.num_samples : rd.cap;
  const long long so = rd.store_off;
  const int *si = res.samples_indices + so;
  const int *nl = res.num_live_points + so;
  const bool gathered = res.scratch_i[so + r] != 0;
  const double off = rd.log_L_offset;
  double *lX = res.log_X_mean + so, *ldp = res.log_dp_mean + so;
  {
    gbns_evcalc e;
    e.log_L = -INFINITY; e.log_X_mean = 0.0; e.log_X2_mean = 0.0; e.log_Z_mean = -INFINITY;
    e.log_ZX_mean = -INFINITY; e.log_Z2_mean = -INFINITY; e.log_dZ_mean = -INFINITY; e.log_dZ2_mean = -INFINITY;
    EvAcc acc = evacc_from(e);
    evidence_scan_cta<false, K>(acc, b.store_L + so, N, 0, 0, nl, b.ncoef, b.ncoef_n, lX, ldp, nullptr, off,
                                gathered ? si : nullptr, esm, s_h);
    if (threadIdx.x == 0) {
      const gbns_evcalc f = evacc_to(acc, 0.0);
      s_lz[0] = f.log_Z_mean;
      s_lz[1] = f.log_Z2_mean;
      s_lz[2] = f.log_dZ2_mean;
    }
  }
  __syncthreads();
  // normalise_log_space(log_dZ_mean) and H (sharded_static.py:726-737): the normaliser
  // logsumexp(log_dZ_mean) is log sum dZ = log Z, which the scan has just accumulated, and the
  // scan has formed the dZ-weighted mean of L that H takes
  const double lZ = s_lz[0], lZ2 = s_lz[1], ldZ2 = s_lz[2];
  const double norm = lZ;
  const double mu = 2.0 * lZ - 0.5 * lZ2;
  for (long long i0 = threadIdx.x; i0 < N; i0 += 4ll * blockDim.x) {
    double v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long i = i0 + (long long)j * blockDim.x;
      v[j] = i < N ? ldp[i] : 0.0;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long i = i0 + (long long)j * blockDim.x;
      if (i < N) ldp[i] = (norm > -INFINITY) ? v[j] - norm : -INFINITY;
    }
  }
  const double h1 = (s_h[0] - s_h[1]) + off;
  const double H_inst = -(h1 - mu);
  // the stable form E[-log X] only where the direct one is not finite (every thread takes the
  // same branch)
  double h2 = 0.0;
  if (!isfinite(H_inst)) {
    __syncthreads();  // the normalised log dp of every sample is written
    for (long long i = threadIdx.x; i < N; i += blockDim.x) h2 += ldp[i] > -INFINITY ? exp(ldp[i]) * -lX[i] : 0.0;
    h2 = cta_sum_d(h2, dred);
  }
  if (threadIdx.x == 0) {
    double *sc = res.scalars + 8 * (size_t)r;
    const double total_phantom = sc[5], total_evals = sc[6];
    double var = lZ2 - 2.0 * lZ;
    var = (var != var) ? var : fmax(var, 2.220446049250313e-16);
    const double pf = total_phantom / (double)N;
    const double k = pf / (1.0 - pf);
    sc[0] = mu;
    sc[1] = sqrt(var) * sqrt(1.0 + k);
    sc[2] = exp(2.0 * lZ - ldZ2) / (1.0 + k);
    sc[3] = isfinite(H_inst) ? H_inst : -h2;
    sc[7] = log((double)N) - log(total_evals);
  }
}

// ---------------------------------------------------------- RNG hooks ----

// jax.random under jax_threefry_partitionable (set by internals/mixed_precision.py:11), for the
// parity tests: mode 0 raw threefry2x32 words, 1 split, 2 64-bit words, 3 uniform, 4 normal.
__global__ void k_rng(int mode, const uint32_t *key, const uint32_t *counts, void *out, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Key k = {key[0], key[1]};
  if (mode == 0) {  // raw threefry2x32 of (counts[2i], counts[2i+1])
    uint32_t a, c;
    threefry2x32(k.k0, k.k1, counts[2 * i], counts[2 * i + 1], a, c);
    ((uint32_t *)out)[2 * i] = a;
    ((uint32_t *)out)[2 * i + 1] = c;
  } else if (mode == 1) {  // split
    const Key s = fold(k, (uint32_t)i);
    ((uint32_t *)out)[2 * i] = s.k0;
    ((uint32_t *)out)[2 * i + 1] = s.k1;
  } else if (mode == 2) {
    ((uint64_t *)out)[i] = bits64(k, (uint32_t)i);
  } else if (mode == 3) {
    ((float *)out)[i] = uniform01(bits64(k, (uint32_t)i));
  } else {
    ((float *)out)[i] = normal_from_bits(bits64(k, (uint32_t)i));
  }
}

// sample_evidence (utils.py:433-484): S replicas of log Z with the shrinkage drawn.
// Replica s (one CTA): u_i = uniform(split(split(key, S)[s], M)[i]), log T_i = log(u_i) / n_i,
// log X_i = sum_{j<i} log T_j (FP64 block scan), and log Z = logsumexp_i(log X_i +
// log(1 - T_i) + log L_i) -- the sequential LogSpace accumulation of the reference written
// as a prefix sum and one log-sum-exp.
__global__ void __launch_bounds__(1024) k_sample_evidence(const uint32_t *key, const int *__restrict__ num_live,
                                                          const double *__restrict__ log_L, long long M,
                                                          double *__restrict__ out) {
  __shared__ double wsum[32];
  __shared__ double red_m[32], red_s[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const Key ks = fold(Key{key[0], key[1]}, (uint32_t)blockIdx.x);
  double carry = 0.0;                  // log X at the start of the chunk
  double m = -INFINITY, acc = 0.0;     // this thread's running log-sum-exp: m + log(acc)
  for (long long base = 0; base < M; base += blockDim.x) {
    const long long i = base + tid;
    double lt = 0.0;
    if (i < M) lt = log(uniform01_d(bits64(fold(ks, (uint32_t)i), 0u))) / (double)num_live[i];
    // inclusive scan of lt over the block
    double v = lt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane == 31) wsum[warp] = v;
    __syncthreads();
    if (warp == 0) {
      double w = lane < nw ? wsum[lane] : 0.0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      if (lane < nw) wsum[lane] = w;
    }
    __syncthreads();
    const double before = (warp > 0 ? wsum[warp - 1] : 0.0) + (v - lt);  // exclusive prefix in the chunk
    const double total = wsum[nw - 1];
    if (i < M) {
      // X_i (1 - T_i) L_i; T_i = 1 only if u_i rounds to 1, which the 52-bit uniform cannot
      const double term = (carry + before) + log1p(-exp(lt)) + log_L[i];
      if (term > m) {
        acc = acc * exp(m - term) + 1.0;
        m = term;
      } else if (term > -INFINITY) {
        acc += exp(term - m);
      }
    }
    carry += total;
    __syncthreads();
  }
  // combine the threads' (m, acc)
  double gm = m;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) gm = fmax(gm, __shfl_xor_sync(0xffffffffu, gm, o));
  if (lane == 0) red_m[warp] = gm;
  __syncthreads();
  gm = -INFINITY;
  for (int q = 0; q < nw; ++q) gm = fmax(gm, red_m[q]);
  double a = (m > -INFINITY) ? acc * exp(m - gm) : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) red_s[warp] = a;
  __syncthreads();
  if (tid == 0) {
    double sum = 0.0;
    for (int q = 0; q < nw; ++q) sum += red_s[q];
    out[blockIdx.x] = (gm > -INFINITY) ? gm + log(sum) : -INFINITY;
  }
}

// ------------------------------------------------------- prior transform ----

// Model.transform and Model.log_prob_prior (framework/model.py:155-187) over the sorted samples
// of _to_results (sharded_static.py:744-745), FP64: one warp per sample row, dimensions strided
// over the lanes (coalesced row reads).  Uniform q = a + b u, Normal q = a + b Phi^-1(u) (AS 241
// PPND16); with an affine map, X_d = c_d + sum_{k = row_start_d}^{d} A_dk q_k over q staged in
// shared memory (the MultivariateNormalTriL blocks), else X = q.  The density is each
// dimension's constant plus -z^2 / 2 (Normal) or 0 / -inf (Uniform, inside / outside), summed
// per lane in dimension order and then over the warp by the xor butterfly, plus log_det and,
// when given, log L (the log posterior density).
template <typename UT>
__global__ void __launch_bounds__(256) k_prior_transform(gbns_prior_table t, const UT *U, long long M,
                                                         const double *log_L, double *X, double *out) {
  extern __shared__ double qs_all[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int D = t.D;
  double *qs = qs_all + (size_t)warp * D;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long row = (long long)blockIdx.x * (blockDim.x >> 5) + warp; row < M; row += nwarps) {
    const UT *u_row = U + row * D;
    double *x_row = X ? X + row * D : nullptr;
    double lp = 0.0;
    for (int d = lane; d < D; d += 32) {
      const double u = (double)u_row[d];
      const double a = t.a[d], b = t.b[d];
      double q, ld;
      if (t.kind[d] == GBNS_PRIOR_NORMAL) {
        const double z = gbns_fm_ndtri64(u);
        q = fma(b, z, a);
        ld = fma(-0.5 * z, z, t.log_norm[d]);
      } else {
        q = fma(b, u, a);
        ld = (q >= a && q <= a + b) ? t.log_norm[d] : -INFINITY;
      }
      lp += ld;
      if (t.A) qs[d] = q;
      else if (x_row) x_row[d] = q;
    }
    if (t.A) {
      __syncwarp();
      if (x_row) {
        for (int d = lane; d < D; d += 32) {
          const double *a_row = t.A + (size_t)d * D;
          double acc = t.c[d];
          const int k0 = t.row_start[d] > 0 ? t.row_start[d] : 0;  // k stays in [0, d]
          for (int k = k0; k <= d; ++k) acc = fma(a_row[k], qs[k], acc);
          x_row[d] = acc;
        }
      }
      __syncwarp();
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) lp += __shfl_xor_sync(0xffffffffu, lp, m);
    if (lane == 0 && out) out[row] = (log_L ? log_L[row] : 0.0) + (lp + t.log_det);
  }
}

cudaError_t launch_prior_transform(const gbns_prior_table &t, const float *U32, const double *U64, long long M,
                                   const double *log_L, double *X, double *out, cudaStream_t stream) {
  if (M <= 0) return cudaSuccess;
  const size_t smem = t.A ? (size_t)8 * t.D * sizeof(double) : 0;
  int dev = 0, sms = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  const long long want = (M + 7) / 8;
  const unsigned grid = (unsigned)(want < (long long)sms * 8 ? want : (long long)sms * 8);
  if (U32) {
    if (smem > 48 * 1024 &&
        (e = cudaFuncSetAttribute(k_prior_transform<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem)) != cudaSuccess)
      return e;
    k_prior_transform<float><<<grid, 256, smem, stream>>>(t, U32, M, log_L, X, out);
  } else {
    if (smem > 48 * 1024 &&
        (e = cudaFuncSetAttribute(k_prior_transform<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem)) != cudaSuccess)
      return e;
    k_prior_transform<double><<<grid, 256, smem, stream>>>(t, U64, M, log_L, X, out);
  }
  return cudaGetLastError();
}

cudaError_t launch_sample_evidence(const uint32_t *key, const int *num_live, const double *log_L, long long M, int S,
                                   double *out, cudaStream_t stream) {
  if (S > 0) k_sample_evidence<<<S, 1024, 0, stream>>>(key, num_live, log_L, M, out);
  return cudaGetLastError();
}

cudaError_t launch_rng(int mode, const uint32_t *key, const uint32_t *counts, void *out, long long n,
                       cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_rng<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(mode, key, counts, out, n);
  return cudaGetLastError();
}

cudaError_t launch_results(const gbns_batch &b, const gbns_results_bufs &res, cudaStream_t stream) {
  // out-degrees in dynamic shared memory beside the kernel's static shared memory
  int dev = 0, optin = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
  cudaFuncAttributes fa;
  if ((e = cudaFuncGetAttributes(&fa, k_results_tree)) != cudaSuccess) return e;
  const int dyn = ((optin - (int)fa.sharedSizeBytes - 1024) / 16) * 16;
  if ((e = cudaFuncSetAttribute(k_results_tree, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn)) != cudaSuccess)
    return e;
  k_results_tree<<<b.num_runs, 1024, dyn, stream>>>(b, res, dyn / (int)sizeof(int));
  k_results_ev<RESULTS_K><<<b.num_runs, RESULTS_EV_THREADS, 0, stream>>>(b, res);
  return cudaGetLastError();
}

// Up to CE_MULTI_MIN samples one CTA does everything; beyond, the work is spread over the grid
// (scratch: 2 (N + 1) 64-bit words and N + 1 counters either way).
constexpr long long CE_MULTI_MIN = 65536;

cudaError_t launch_count_crossed_edges(const int *sender, const float *L, long long N, int *samples_indices,
                                       int *num_live, long long *scratch_ll, int *scratch_i, cudaStream_t stream) {
  unsigned long long *a = (unsigned long long *)scratch_ll, *tmp = a + (N + 1);
  if (N <= CE_MULTI_MIN) {
    k_count_edges<<<1, 1024, 0, stream>>>(sender, L, N, samples_indices, num_live, a, scratch_i);
    return cudaGetLastError();
  }
  // tmp[0] is A's out-of-order flag, then the sort's ping-pong buffer, then the chunk sums
  cudaError_t e = cudaMemsetAsync(tmp, 0, sizeof(unsigned long long), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch_i, 0, sizeof(int) * (size_t)(N + 1), stream);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  k_ce_keys<<<sms * 8, 256, 0, stream>>>(sender, L, N, a, tmp, scratch_i);
  k_ce_sort<<<1, 1024, 0, stream>>>(N, a, tmp, tmp);
  const long long nchunks = (N + 1 + CE_CHUNK - 1) / CE_CHUNK;
  long long *bsum = (long long *)tmp;
  k_ce_chunk_sums<<<(unsigned)nchunks, 256, 0, stream>>>(N, a, scratch_i, bsum);
  k_ce_chunk_scan<<<1, 1024, 0, stream>>>(bsum, (int)nchunks);
  k_ce_chunk_out<<<(unsigned)nchunks, 1024, 0, stream>>>(N, a, scratch_i, bsum, samples_indices, num_live);
  return cudaGetLastError();
}

cudaError_t launch_evidence_stats(const float *L, const int *num_live, long long N, const double *ncoef, int nmax,
                                  gbns_evcalc *final_out, double *lX, double *ldZ, double *lZ, cudaStream_t stream) {
  if (lZ) k_evidence_stats<true><<<1, RESULTS_EV_THREADS, 0, stream>>>(L, num_live, N, ncoef, nmax, final_out, lX, ldZ, lZ);
  else k_evidence_stats<false><<<1, RESULTS_EV_THREADS, 0, stream>>>(L, num_live, N, ncoef, nmax, final_out, lX, ldZ, lZ);
  return cudaGetLastError();
}

}  // namespace gbns
