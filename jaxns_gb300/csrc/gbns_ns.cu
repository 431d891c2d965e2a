// gbns_ns.cu -- initial live points, the per-iteration shell merge (store append, stable
// sort, FP64 evidence register, termination) and the final live-point append.
//
// One CTA per run for the bookkeeping kernels: a run's live set (n <= 4096) is sorted in
// shared memory with a bitonic network on (ordered key, index) pairs, which is exactly the
// stable argsort of jnp.argsort (sharded_static.py:274).
#include "gbns_device.cuh"
#include "gbns_launch.h"

namespace gbns {

// ------------------------------------------------------ generic likelihood ----

// Model.forward for any family with runtime D (parameters read from global memory),
// relative to the run's log_L_offset: MVN -0.5 |Linv (x - mu)|^2, shells
// logaddexp(-0.5 z1^2, -0.5 z2^2), linear Gaussian -0.5 |y - Phi w|^2 / sigma^2.
__device__ float loglik_generic(const gbns_batch &b, const gbns_run_desc &rd, const float *U) {
  const int D = rd.D;
  const float *fp = b.fparams + rd.param_off;
  float x[64];
  for (int j = 0; j < D; ++j)
    x[j] = prior_quantile(b.prior_kind[rd.prior_off + j], b.prior_a[rd.prior_off + j], b.prior_b[rd.prior_off + j], U[j]);
  float v;
  if (rd.family == GBNS_LIK_MVN) {
    for (int j = 0; j < D; ++j) x[j] -= fp[j];
    float s = 0.f;
    for (int i = 0; i < D; ++i) {
      float acc = 0.f;
      for (int j = 0; j <= i; ++j) acc = fmaf(fp[D + i * D + j], x[j], acc);
      s = fmaf(acc, acc, s);
    }
    v = -0.5f * s;
  } else if (rd.family == GBNS_LIK_SHELLS) {
    float r1 = 0.f, r2 = 0.f;
    for (int j = 0; j < D; ++j) {
      const float e1 = x[j] - fp[j], e2 = x[j] - fp[D + j];
      r1 = fmaf(e1, e1, r1);
      r2 = fmaf(e2, e2, r2);
    }
    const float R = fp[2 * D], w = fp[2 * D + 1];
    const float iw = 1.0f / w;  // the shell width's reciprocal, as the sampler kernel forms it
    const float z1 = (sqrtf(r1) - R) * iw, z2 = (sqrtf(r2) - R) * iw;
    const float s1 = -0.5f * z1 * z1, s2 = -0.5f * z2 * z2;
    const float m = fmaxf(s1, s2), dd = s1 - s2;
    v = (dd != dd) ? s1 + s2 : m + gbns_fm_log1p(gbns_fm_exp(-fabsf(dd)));
  } else {
    const int N = rd.N;
    const float *Phi = fp, *y = fp + (size_t)N * D;
    const float sigma = fp[(size_t)N * D + N];
    float ss = 0.f;
    for (int a = 0; a < N; ++a) {
      float r = y[a];
      for (int j = 0; j < D; ++j) r = fmaf(-Phi[(size_t)a * D + j], x[j], r);
      ss = fmaf(r, r, ss);
    }
    v = -0.5f * ss / (sigma * sigma);
  }
  return (v != v) ? -INFINITY : v;
}

// Linear-Gaussian log L (relative to the run's offset) of an FP64 U: -|y - Phi w|^2 / (2 sigma^2).
__device__ float loglik_lg_d(const gbns_batch &b, const gbns_run_desc &rd, const double *U) {
  const int D = rd.D, N = rd.N;
  const float *fp = b.fparams + rd.param_off;
  float x[64];
  for (int j = 0; j < D; ++j)
    x[j] = prior_quantile_d(b.prior_kind[rd.prior_off + j], b.prior_a[rd.prior_off + j],
                            b.prior_b[rd.prior_off + j], U[j]);
  const float *Phi = fp, *y = fp + (size_t)N * D;
  const float sigma = fp[(size_t)N * D + N];
  float ss = 0.f;
  for (int a = 0; a < N; ++a) {
    float r = y[a];
    for (int j = 0; j < D; ++j) r = fmaf(-Phi[(size_t)a * D + j], x[j], r);
    ss = fmaf(r, r, ss);
  }
  const float v = -0.5f * ss / (sigma * sigma);
  return (v != v) ? -INFINITY : v;
}

// U: [B, ucols] 32-bit words (FP64 U for the linear-Gaussian family).
__global__ void k_forward(gbns_batch b, int run, const float *__restrict__ U, float *__restrict__ out, long long B) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= B) return;
  const gbns_run_desc &rd = b.runs[run];
  const float v = rd.family == GBNS_LIK_LINGAUSS ? loglik_lg_d(b, rd, (const double *)U + i * rd.D)
                                                 : loglik_generic(b, rd, U + i * rd.D);
  out[i] = (float)((double)v + rd.log_L_offset);
}

// ------------------------------------------------------------ termination ----

// determine_termination for one TerminationCondition (nested_samplers/common/termination.py:13-147)
__device__ bool determine_termination(const gbns_term_cond &tc, const gbns_run_state &st, int &reason) {
  bool done = false;
  int rs = 0;
#define SETBIT(c, bit) do { if (c) { done = true; rs += (1 << (bit)); } } while (0)
  if (tc.has_max_samples) SETBIT((double)st.num_samples >= tc.max_samples, 0);
  if (tc.has_evidence_uncert) {
    double v = st.ev_rem.log_Z2_mean - 2.0 * st.ev_rem.log_Z_mean;
    v = (v != v) ? v : fmax(v, 2.220446049250313e-16);
    SETBIT(v <= tc.evidence_uncert * tc.evidence_uncert, 1);
  }
  if (tc.has_dlogZ) {
    const double m1 = 2.0 * st.ev_rem.log_Z_mean - 0.5 * st.ev_rem.log_Z2_mean;
    const double m0 = 2.0 * st.ev.log_Z_mean - 0.5 * st.ev.log_Z2_mean;
    SETBIT((m1 - m0) < tc.dlogZ, 2);
  }
  if (tc.has_ess) SETBIT(exp(2.0 * st.ev_rem.log_Z_mean - st.ev_rem.log_dZ2_mean) >= tc.ess, 3);
  if (tc.has_max_nlik) SETBIT((double)st.num_likelihood_evaluations >= tc.max_nlik, 4);
  if (tc.has_log_L_contour) SETBIT(st.log_L_contour >= tc.log_L_contour, 5);
  if (tc.has_efficiency) SETBIT(st.efficiency < tc.efficiency_threshold, 6);
  SETBIT(st.plateau != 0, 7);
  if (tc.has_rtol) SETBIT(st.relative_spread < tc.rtol, 8);
  if (tc.has_atol) SETBIT(st.absolute_spread < tc.atol, 9);
  SETBIT(st.no_seed_points != 0, 10);
  if (tc.has_peak_XL) SETBIT(st.ev.log_X_mean + st.ev.log_L < st.peak_log_XL + log(tc.peak_XL_frac), 11);
#undef SETBIT
  reason = rs;
  return done;
}

// Term condition of phase `phase` with max_samples clamped as _main_ns_thread does
// (sharded_static.py:460-470).
__device__ gbns_term_cond phase_term_cond(const gbns_run_desc &rd, int phase) {
  gbns_term_cond tc;
  if (phase == 0) {
    tc = gbns_term_cond{};
    tc.has_efficiency = 1;
    tc.efficiency_threshold = rd.init_efficiency_threshold;
    tc.has_dlogZ = 1;
    tc.dlogZ = 0.0;
    tc.has_max_samples = 1;
    tc.max_samples = fmin((double)rd.cap, (double)(rd.cap - rd.s));
  } else {
    tc = rd.tc;
    if (tc.has_max_samples) tc.max_samples = fmin(tc.max_samples, (double)(rd.cap - (long long)rd.s * (1 + rd.K)));
  }
  return tc;
}

// ------------------------------------------------------- CTA primitives ----

__device__ __forceinline__ unsigned long long sort_key(float L, int i) {
  return ((unsigned long long)ordered_key(L) << 32) | (unsigned)i;
}

// Bitonic sort of NP (power of two) 64-bit keys in shared memory, ascending.
__device__ void cta_bitonic(unsigned long long *k, int NP) {
  for (int size = 2; size <= NP; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      const int lg = __ffs(stride) - 1;  // stride is a power of two
      for (int t = threadIdx.x; t < NP / 2; t += blockDim.x) {
        const int lo = ((t >> lg) << (lg + 1)) + (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = ((lo & size) == 0);
        const unsigned long long a = k[lo], c = k[hi];
        if ((a > c) == up) {
          k[lo] = c;
          k[hi] = a;
        }
      }
    }
  }
  __syncthreads();
}

// Append cnt entries of a run to its store at next_sample_idx, with the start clamped like
// lax.dynamic_update_slice (internals/maps.py:15-25, sharded_static.py:40-85).
__device__ void store_append(const gbns_batch &b, const gbns_run_desc &rd, long long nsi, long long cnt,
                             const float *L, const int *S, int S_const, const int *E, const float *U, int phantom) {
  if (cnt <= 0) return;
  long long start = nsi;
  if (start > rd.cap - cnt) start = rd.cap - cnt;
  if (start < 0) start = 0;
  const int W = rd.ucols;
  for (long long i = threadIdx.x; i < cnt; i += blockDim.x) {
    const long long o = rd.store_off + start + i;
    b.store_L[o] = L[i];
    b.store_S[o] = S ? S[i] : S_const;
    b.store_E[o] = E ? E[i] : 0;
    b.store_P[o] = (uint8_t)phantom;
  }
  if (rd.ustore_off >= 0 && b.store_U) {
    float *dst = b.store_U + rd.ustore_off + (start * W);
    for (long long q = threadIdx.x; q < cnt * W; q += blockDim.x) dst[q] = U[q];
  }
}

// ------------------------------------------------------------------ init ----

// create_init_state (nested_samplers/common/initialisation.py:20-84): n uniform samples
// strictly above -inf (_single_uniform_sample, common/uniform_sample.py:12-60).
__global__ void k_init_points(gbns_batch b, long long total) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= total) return;
  int lo = 0, hi = b.num_runs;  // live points are packed: run r owns [live_off, live_off + n)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (b.runs[mid].live_off <= g) lo = mid; else hi = mid;
  }
  const int r = lo;
  const gbns_run_desc &rd = b.runs[r];
  const int i = (int)(g - rd.live_off);
  const int D = rd.D;
  const bool lg = rd.family == GBNS_LIK_LINGAUSS;
  const Key K0 = {b.state[r].key[0], b.state[r].key[1]};
  const Key sample_key = fold(K0, 1u);
  const Key ki = fold(sample_key, (uint32_t)i);
  Key k = fold(ki, 0u), sk = fold(ki, 1u);
  float U[64];
  double Ud[64];
  float logL;
  int ne = 0;
  for (;;) {
    const Key uk = fold(sk, 1u);  // Model.sample_U: uniform(split(key)[1], (D,))
    if (lg) {
      for (int j = 0; j < D; ++j) Ud[j] = uniform01_d(bits64(uk, (uint32_t)j));
      logL = loglik_lg_d(b, rd, Ud);
    } else {
      for (int j = 0; j < D; ++j) U[j] = uniform01(bits64(uk, (uint32_t)j));
      logL = loglik_generic(b, rd, U);
    }
    ++ne;
    if (!(logL <= -INFINITY)) break;
    if (ne >= 1000000) { atomicOr(&b.state[r].status, (int)GBNS_ERR_INIT_BUDGET); break; }
    const Key nk = fold(k, 0u);
    sk = fold(k, 1u);
    k = nk;
  }
  const long long o = rd.live_off + i;
  if (lg) {
    double *dst = (double *)(b.live_U[1] + rd.liveU_off) + (long long)i * D;
    for (int j = 0; j < D; ++j) dst[j] = Ud[j];
  } else {
    for (int j = 0; j < D; ++j) b.live_U[1][rd.liveU_off + (long long)i * D + j] = U[j];
  }
  b.live_L[1][o] = logL;
  b.live_Lc[1][o] = -INFINITY;
  b.live_E[1][o] = ne;
  b.live_S[1][o] = 0;
}

// After k_init_points: sort buffer 1 into buffer 0, set up the register and run the
// termination checks that precede the first iteration of each phase.
__global__ void k_init_finish(gbns_batch b) {
  extern __shared__ unsigned long long sk[];
  const int r = blockIdx.x;
  const gbns_run_desc &rd = b.runs[r];
  gbns_run_state &st = b.state[r];
  const int n = rd.n, W = rd.ucols;
  int NP = 1;
  while (NP < n) NP <<= 1;
  const float *iL = b.live_L[1] + rd.live_off;
  for (int i = threadIdx.x; i < NP; i += blockDim.x) sk[i] = i < n ? sort_key(iL[i], i) : ~0ull;
  cta_bitonic(sk, NP);
  const long long o = rd.live_off;
  for (long long q = threadIdx.x; q < (long long)n * W; q += blockDim.x) {
    const int i = (int)(q / W), j = (int)(q % W);
    const int src = (int)(sk[i] & 0xffffffffu);
    b.live_U[0][rd.liveU_off + (long long)i * W + j] = b.live_U[1][rd.liveU_off + (long long)src * W + j];
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int src = (int)(sk[i] & 0xffffffffu);
    b.live_L[0][o + i] = iL[src];
    b.live_Lc[0][o + i] = -INFINITY;
    b.live_E[0][o + i] = b.live_E[1][o + src];
    b.live_S[0][o + i] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const Key K0 = {st.key[0], st.key[1]};
    const Key nk = fold(K0, 0u);
    st.key[0] = nk.k0;
    st.key[1] = nk.k1;
    // create_init_termination_register (initialisation.py:87-108)
    gbns_evcalc e;
    e.log_L = -INFINITY; e.log_X_mean = 0.0; e.log_X2_mean = 0.0; e.log_Z_mean = -INFINITY;
    e.log_ZX_mean = -INFINITY; e.log_Z2_mean = -INFINITY; e.log_dZ_mean = -INFINITY; e.log_dZ2_mean = -INFINITY;
    st.ev = e;
    st.ev_rem = e;
    st.log_L_contour = -INFINITY;
    st.efficiency = 0.0;
    st.relative_spread = INFINITY;
    st.absolute_spread = INFINITY;
    st.peak_log_XL = -INFINITY;
    st.num_likelihood_evaluations = 0;
    st.num_samples = 0;
    st.next_sample_idx = 0;
    st.iterations = 0;
    st.plateau = 0;
    st.parity = 0;
    st.termination_reason = 0;
    const float *L = b.live_L[0] + o;
    st.no_seed_points = L[rd.s - 1] >= L[n - 1];
    int reason = 0;
    int phase = rd.uniform_phase ? 0 : 1;
    bool done = determine_termination(phase_term_cond(rd, phase), st, reason);
    if (phase == 0) {
      // The uniform phase stops before its first iteration whenever its efficiency test
      // fires on the initial register (efficiency 0 < threshold); that is always the case
      // for init_efficiency_threshold > 0.  A phase that would need iterations is reported.
      if (!done) atomicOr(&st.status, (int)GBNS_ERR_BAD_PARAM);
      phase = 1;
      st.no_seed_points = L[rd.s - 1] >= L[n - 1];
      done = determine_termination(phase_term_cond(rd, 1), st, reason);
    }
    st.phase = 1;
    st.done = done ? 1 : 0;
    st.termination_reason = reason;
  }
}

// ----------------------------------------------------------------- merge ----

// Consecutive elements per thread in the merge's evidence scans (chunks of 128 x 2; 4 per
// thread raised the merge to 160 registers and the default bench fell 0.4 %).
constexpr int MERGE_SCAN_K = 2;

// _collect_shell (sharded_static.py:210-324) after the chains have run, plus the loop
// condition of _main_ns_thread (:480-485) and the final live-point append (:833-838).
__global__ void __launch_bounds__(128) k_merge(gbns_batch b) {
  extern __shared__ unsigned long long sk[];
  __shared__ long long lred[32];
  __shared__ int ired[32];
  __shared__ int s_done;
  const int r = blockIdx.x;
  const gbns_run_desc &rd = b.runs[r];
  gbns_run_state &st = b.state[r];
  if (st.done || st.phase != 1) return;
  const int n = rd.n, s = rd.s, W = rd.ucols, K = rd.K;
  const int par = st.parity, npar = par ^ 1;
  const long long o = rd.live_off;
  const float *L = b.live_L[par] + o;
  const float *U = b.live_U[par] + rd.liveU_off;
  const float *Lc = b.live_Lc[par] + o;
  const int *E = b.live_E[par] + o;
  const int *Sd = b.live_S[par] + o;
  float *oL = b.live_L[npar] + o;
  float *oU = b.live_U[npar] + rd.liveU_off;
  float *oLc = b.live_Lc[npar] + o;
  int *oE = b.live_E[npar] + o;
  int *oS = b.live_S[npar] + o;
  const long long so = rd.shell_off;
  const float *nL = b.new_L + so;
  const float *nU = b.new_U + rd.newU_off;
  const int *nE = b.new_E + so;
  const float Lstar = L[s - 1];

  // discard the shell into the store
  long long nsi = st.next_sample_idx;
  store_append(b, rd, nsi, s, L, Sd, 0, E, U, 0);
  nsi = (nsi + s) % rd.cap;
  const int sender_idx = (int)(nsi - 1);

  // replace [0, s) with the new samples and stable-argsort the live set
  int NP = 1;
  while (NP < n) NP <<= 1;
  for (int i = threadIdx.x; i < NP; i += blockDim.x)
    sk[i] = i < n ? sort_key(i < s ? nL[i] : L[i], i) : ~0ull;
  cta_bitonic(sk, NP);
  // row i = q / W as a multiply-high: exact for q < 2^25 and W <= 128 (n W <= 4096 x 128)
  const uint32_t wmagic = W > 1 ? (uint32_t)(((1ull << 32) + (uint64_t)W - 1ull) / (uint64_t)W) : 0u;
  for (int q = threadIdx.x; q < n * W; q += blockDim.x) {
    const int i = W > 1 ? (int)__umulhi((uint32_t)q, wmagic) : q, j = q - i * W;
    const int src = (int)(sk[i] & 0xffffffffu);
    oU[(long long)i * W + j] = src < s ? nU[(long long)src * W + j] : U[(long long)src * W + j];
  }
  long long eloc = 0, enew = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int src = (int)(sk[i] & 0xffffffffu);
    const bool fresh = src < s;
    oL[i] = fresh ? nL[src] : L[src];
    oLc[i] = fresh ? Lstar : Lc[src];
    const int e = fresh ? nE[src] : E[src];
    oE[i] = e;
    oS[i] = fresh ? sender_idx : Sd[src];
    eloc += e;
  }
  for (int i = threadIdx.x; i < s; i += blockDim.x) enew += nE[i];
  __syncthreads();

  // phantoms (add_phantom_samples_to_state, sharded_static.py:181-207)
  if (K > 0) {
    store_append(b, rd, nsi, (long long)s * K, b.ph_L + rd.phL_off, nullptr, sender_idx, nullptr,
                 b.ph_U + rd.phU_off, 1);
    nsi = (nsi + (long long)s * K) % rd.cap;
  }

  const long long sumLive = cta_sum(eloc, lred);
  const long long sumNew = cta_sum(enew, lred);
  int flat = 1;
  const float L0 = oL[0];
  for (int i = threadIdx.x; i < n; i += blockDim.x) flat &= (oL[i] == L0);
  flat = cta_and(flat, ired);

  // evidence register (sharded_static.py:284-299): the discarded shell with n live points,
  // then the remaining live points with n, n-1, ..., 1 (CTA-wide FP64 scans)
  __shared__ EvScanSmem esm;
  const double off = rd.log_L_offset;
  EvAcc acc = evacc_from_shifted(st.ev, off);
  evidence_scan_cta<false, MERGE_SCAN_K>(acc, L, s, n, 0, nullptr, b.ncoef, b.ncoef_n, nullptr, nullptr, nullptr, off, nullptr,
                                         esm);
  const EvAcc acc_shell = acc;
  evidence_scan_cta<false, MERGE_SCAN_K>(acc, oL, n, 0, n, nullptr, b.ncoef, b.ncoef_n, nullptr, nullptr, nullptr, off, nullptr,
                                         esm);
  if (threadIdx.x == 0) {
    const gbns_evcalc ev = evacc_to(acc_shell, (double)L[s - 1] + off);
    const gbns_evcalc evr = evacc_to(acc, (double)oL[n - 1] + off);
    st.ev = ev;
    st.ev_rem = evr;
    st.num_samples += (long long)s * (1 + K);
    st.next_sample_idx = nsi;
    st.num_likelihood_evaluations += sumNew;
    st.log_L_contour = (double)Lstar + off;
    st.efficiency = (double)n / (double)sumLive;
    st.plateau = flat;
    const double Lmin = (double)oL[0] + off, Lmax = (double)oL[n - 1] + off;
    st.absolute_spread = fabs(Lmax - Lmin);
    st.relative_spread = 2.0 * st.absolute_spread / fabs(Lmin + Lmax);
    st.no_seed_points = oL[s - 1] >= oL[n - 1];
    const double pk = ev.log_X_mean + ev.log_L;
    st.peak_log_XL = (pk != pk || st.peak_log_XL != st.peak_log_XL) ? NAN : fmax(st.peak_log_XL, pk);
    // keys: split before the shell (:491), inside _collect_shell (:248), after (:510)
    const Key K0 = {st.key[0], st.key[1]};
    const Key k3 = fold(fold(fold(K0, 0u), 0u), 0u);
    st.key[0] = k3.k0;
    st.key[1] = k3.k1;
    st.parity = npar;
    st.iterations += 1;
    int reason = 0;
    bool done = determine_termination(phase_term_cond(rd, 1), st, reason);
    if (!done && nsi + (long long)s * (1 + K) > rd.cap && !rd.tc.has_max_samples) {
      // without a sample limit the next shell would overwrite the store
      atomicOr(&st.status, (int)GBNS_ERR_STORE_FULL);
      done = true;
    }
    st.termination_reason = reason;
    s_done = done ? 1 : 0;
  }
  __syncthreads();
  if (s_done) {
    // consume the live points (sharded_static.py:833-838)
    store_append(b, rd, st.next_sample_idx, n, oL, oS, 0, oE, oU, 0);
    __syncthreads();
    if (threadIdx.x == 0) {
      st.next_sample_idx = (st.next_sample_idx + n) % rd.cap;
      st.num_samples += n;
      st.done = 1;
      st.phase = 2;
    }
  }
}

// Runs whose termination fired before their first iteration still own their live set.
__global__ void k_finalize(gbns_batch b) {
  const int r = blockIdx.x;
  const gbns_run_desc &rd = b.runs[r];
  gbns_run_state &st = b.state[r];
  if (st.phase == 2 || !st.done) return;
  const int par = st.parity;
  const long long o = rd.live_off;
  store_append(b, rd, st.next_sample_idx, rd.n, b.live_L[par] + o, b.live_S[par] + o, 0, b.live_E[par] + o,
               b.live_U[par] + rd.liveU_off, 0);
  __syncthreads();
  if (threadIdx.x == 0) {
    st.next_sample_idx = (st.next_sample_idx + rd.n) % rd.cap;
    st.num_samples += rd.n;
    st.phase = 2;
  }
}

// ------------------------------------------------------------- launchers ----

static int max_n(const gbns_batch &b) { return b.nmax; }

cudaError_t launch_init(const gbns_batch &b, long long total_points, cudaStream_t stream) {
  const int T = 128;
  const long long blocks = (total_points + T - 1) / T;
  if (blocks > 0) k_init_points<<<(unsigned)blocks, T, 0, stream>>>(b, total_points);
  int NP = 1;
  while (NP < max_n(b)) NP <<= 1;
  k_init_finish<<<b.num_runs, 1024, NP * sizeof(unsigned long long), stream>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_merge(const gbns_batch &b, cudaStream_t stream) {
  int NP = 1;
  while (NP < max_n(b)) NP <<= 1;
  // 128 threads: a run's live set is at most a few thousand points, so narrow CTAs let several
  // runs' sorts and scans share an SM (against 256 threads: +0.5 % on the Gaussian-shells bench
  // with 1000 live points, +4.2 % on the 240-live-point correlated-Gaussian benchmark)
  k_merge<<<b.num_runs, 128, NP * sizeof(unsigned long long), stream>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const gbns_batch &b, cudaStream_t stream) {
  k_finalize<<<b.num_runs, 256, 0, stream>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_forward(const gbns_batch &b, int run, const float *U, float *logL, long long B, cudaStream_t stream) {
  if (B <= 0) return cudaSuccess;
  k_forward<<<(unsigned)((B + 127) / 128), 128, 0, stream>>>(b, run, U, logL, B);
  return cudaGetLastError();
}

}  // namespace gbns
