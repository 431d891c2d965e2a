// gbns_slice.cu -- the fused uni-dimensional slice sampler for one shell of every run.
//
// One thread owns one Markov chain (UniDimSliceSampler.get_sample,
// samplers/uni_slice_sampler.py:343-441, via BaseAbstractMarkovSampler._get_sample,
// samplers/bases.py:63-75).  The chain's slice loop and the shrink while-loop of
// _new_proposal (uni_slice_sampler.py:114-273) are flattened into one loop in which every
// iteration makes exactly one likelihood evaluation, so the threads of a warp stay in step
// whatever their shrink counts.  The U->X prior quantile and the likelihood are evaluated
// in registers; the run's parameters (mu, Linv, prior tables) sit in shared memory and
// are read as broadcasts because every thread of a CTA works on chains of the same run.
#include "gbns_device.cuh"
#include "gbns_launch.h"

namespace gbns {

template <int DMAX, int FAM>
struct RunSmem {
  float a[DMAX], b[DMAX];
  int kind[DMAX];
  float p0[DMAX];                       // MVN: mu      SHELLS: c1
  float p1[FAM == GBNS_LIK_MVN ? DMAX * DMAX : DMAX];  // MVN: Linv   SHELLS: c2
  float c0, R, w, norm;
  float iw;                             // SHELLS: 1 / w (correctly rounded)
  int m;                                // live points above the contour
  int all_uniform;                      // every prior of the run is Uniform
  float4 ab[DMAX];                      // (a, b, p0, SHELLS: c2 / MVN: prior kind's bits): one 16-byte load per dimension
};

// Per-warp scratch of the direction pass (dynamic shared memory, one per warp of the CTA, so
// a CTA reserves only what its warps use)
template <int DMAX>
struct DirWarp {
  uint4 key[32];            // (direction key, lane) of each lane that needs a direction
  float buf[32][DMAX + 1];  // the normals, one row per lane
};

// jax.grad of Model.forward w.r.t. U at u (analytic): d log L / dx through the prior quantile
// (Uniform: dx/du = b; Normal: dx/du = b sqrt(2 pi) exp(z^2 / 2)).  MVN: -Linv^T Linv (x - mu);
// shells: sum_k softmax_k (-z_k / w) (x - c_k) / r_k.
template <int DMAX, int FAM>
__device__ __forceinline__ void grad_u(const RunSmem<DMAX, FAM> &P, int D, const float *u, float *g) {
  float x[DMAX], dxdu[DMAX];
#pragma unroll
  for (int j = 0; j < DMAX; ++j)
    if (j < D) prior_quantile_slope(P.kind[j], P.a[j], P.b[j], u[j], x[j], dxdu[j]);
  if (FAM == GBNS_LIK_MVN) {
    float e[DMAX], z[DMAX];
#pragma unroll
    for (int j = 0; j < DMAX; ++j) e[j] = j < D ? x[j] - P.p0[j] : 0.0f;
#pragma unroll
    for (int i = 0; i < DMAX; ++i) {
      float acc = 0.0f;
#pragma unroll
      for (int j = 0; j <= i; ++j) acc = fmaf(P.p1[i * DMAX + j], e[j], acc);
      z[i] = acc;
    }
#pragma unroll
    for (int q = 0; q < DMAX; ++q) {
      float acc = 0.0f;
#pragma unroll
      for (int i = q; i < DMAX; ++i) acc = fmaf(P.p1[i * DMAX + q], z[i], acc);
      if (q < D) g[q] = -acc * dxdu[q];
    }
  } else {
    float r1 = 0.f, r2 = 0.f;
#pragma unroll
    for (int j = 0; j < DMAX; ++j) {
      if (j < D) {
        const float e1 = x[j] - P.p0[j], e2 = x[j] - P.p1[j];
        r1 = fmaf(e1, e1, r1);
        r2 = fmaf(e2, e2, r2);
      }
    }
    r1 = sqrtf(r1);
    r2 = sqrtf(r2);
    const float z1 = (r1 - P.R) / P.w, z2 = (r2 - P.R) / P.w;
    const float s1 = -0.5f * z1 * z1, s2 = -0.5f * z2 * z2, mx = fmaxf(s1, s2);
    const float q1 = gbns_fm_exp(s1 - mx), q2 = gbns_fm_exp(s2 - mx), tot = q1 + q2;
    const float f1 = (q1 / tot) * (-z1 / P.w) / r1, f2 = (q2 / tot) * (-z2 / P.w) / r2;
#pragma unroll
    for (int j = 0; j < DMAX; ++j)
      if (j < D) g[j] = (f1 * (x[j] - P.p0[j]) + f2 * (x[j] - P.p1[j])) * dxdu[j];
  }
}

// log L(u0 + t d) - offset.  When every prior of the run is Uniform (the correlated-Gaussian and
// shells workloads), the prior quantile is fmaf(b, u, a) in every dimension, and the dimension's
// a, b and centre(s) come from one 16-byte shared-memory load with no test of the prior kind: the
// same arithmetic in the same order, and 1.51x the shells sampler's throughput of the per-dimension
// kind test with four scalar loads.  Correlated Gaussians with other priors take the kind from the
// same load and select the quantile without a branch per dimension (gh168 workload: 1.037x).
template <int DMAX, int FAM>
__device__ __forceinline__ float loglik(const RunSmem<DMAX, FAM> &P, int D, const float *u0, const float *d, float t) {
  float v;
  if (FAM == GBNS_LIK_MVN) {
    float x[DMAX];
    if (P.all_uniform) {
      // every quantile is the Uniform one (the same fmaf), with no per-dimension kind test
#pragma unroll
      for (int j = 0; j < DMAX; ++j)
        if (j < D) {
          const float4 q = P.ab[j];
          x[j] = fmaf(q.y, fmaf(t, d[j], u0[j]), q.x) - q.z;
        }
    } else {
      // prior_quantile without a branch per dimension: the Normal quantile of every dimension,
      // selected where the prior is Normal (a run mixing the two kinds pays for the Uniform
      // dimensions' unused quantiles)
#pragma unroll
      for (int j = 0; j < DMAX; ++j)
        if (j < D) {
          const float4 q = P.ab[j];
          const float u = fmaf(t, d[j], u0[j]);
          const float z = gbns_fm_ndtri(u);
          x[j] = fmaf(q.y, __float_as_int(q.w) == GBNS_PRIOR_UNIFORM ? u : z, q.x) - q.z;
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < DMAX; ++i) {
      if (i < D) {
        float acc = 0.0f;
#pragma unroll
        for (int j = 0; j <= i; ++j) acc = fmaf(P.p1[i * DMAX + j], x[j], acc);
        s = fmaf(acc, acc, s);
      }
    }
    v = -0.5f * s;
  } else {
    float r1 = 0.0f, r2 = 0.0f;
    if (P.all_uniform) {
#pragma unroll
      for (int j = 0; j < DMAX; ++j) {
        if (j < D) {
          const float4 q = P.ab[j];
          const float x = fmaf(q.y, fmaf(t, d[j], u0[j]), q.x);
          const float e1 = x - q.z, e2 = x - q.w;
          r1 = fmaf(e1, e1, r1);
          r2 = fmaf(e2, e2, r2);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < DMAX; ++j) {
        if (j < D) {
          const float x = prior_quantile(P.kind[j], P.a[j], P.b[j], fmaf(t, d[j], u0[j]));
          const float e1 = x - P.p0[j], e2 = x - P.p1[j];
          r1 = fmaf(e1, e1, r1);
          r2 = fmaf(e2, e2, r2);
        }
      }
    }
    const float z1 = (sqrtf(r1) - P.R) * P.iw, z2 = (sqrtf(r2) - P.R) * P.iw;
    const float s1 = -0.5f * z1 * z1, s2 = -0.5f * z2 * z2;
    const float m = fmaxf(s1, s2), dd = s1 - s2;
    v = (dd != dd) ? s1 + s2 : m + gbns_fm_log1p(gbns_fm_exp(-fabsf(dd)));
  }
  return (v != v) ? -INFINITY : v;  // NaN -> -inf (framework/ops.py:323-325)
}

// linspace(0.5, 1, S)[j] as jnp.linspace evaluates it
__device__ __forceinline__ float slice_alpha(int j, int S) {
  if (S == 1) return 0.5f;
  if (j == S - 1) return 1.0f;
  const float step = (float)j / (float)(S - 1);
  return 0.5f * (1.0f - step) + step;
}

// Minimum resident 128-thread CTAs per SM (8 caps registers at 64): the sampler is latency-
// bound, and at DMAX <= 8 the cap costs a few tens of bytes of spills per thread (correlated
// Gaussians at D <= 8: 7 is 0.8 % faster than 8 and 6 is 18 % slower).  Gaussian
// shells at DMAX 16 run fastest at 7 (72 registers, 32 B of spills): 3.8 % faster than at 6
// (80 registers) once the direction scratch is sized per warp, so that shared memory no longer
// limits the resident CTAs.  The other instantiations keep the occupancy they reach without a
// cap (3 or 4 CTAs).
template <int DMAX, int FAM>
constexpr int slice_min_blocks() {
  return DMAX <= 8 ? (FAM == GBNS_LIK_MVN ? 7 : 8) : ((DMAX == 16 && FAM == GBNS_LIK_SHELLS) ? 7 : (DMAX >= 64 ? 3 : 4));
}

// GRAD: the gradient instantiation, for UniDimSliceSampler's two gradient options (runtime
// flags of the batch): gradient_guided (the direction of slice j + 1 is the reflection of slice
// j's direction about the U-space gradient at the accepted point) and gradient_slice (each
// slice runs along the normalised gradient at its seed point, t in [0, right]); it keeps its
// gradient arrays in registers at 2 CTAs per SM instead of spilling them.
template <int DMAX, int FAM, bool GRAD>
__global__ void __launch_bounds__(128, GRAD ? 2 : slice_min_blocks<DMAX, FAM>()) k_slice_shell(gbns_batch b, int item_begin,
                                                                                 const float *__restrict__ Lstar_in,
                                                      const uint32_t *__restrict__ keys_in) {
  __shared__ RunSmem<DMAX, FAM> P;
  const int *it = b.items + 4 * (size_t)(item_begin + blockIdx.x);
  const int r = it[0], c_begin = it[1], c_count = it[2];
  const gbns_run_desc &rd = b.runs[r];
  gbns_run_state &st = b.state[r];
  if (!keys_in && (st.done || st.phase != 1)) return;
  const int D = rd.D, n = rd.n, S = rd.S, K = rd.K;
  const int par = st.parity;
  const float *__restrict__ liveL = b.live_L[par] + rd.live_off;
  const float *__restrict__ liveU = b.live_U[par] + rd.liveU_off;

  // --- stage the run's parameters
  const float *fp = b.fparams + rd.param_off;
  for (int j = threadIdx.x; j < DMAX; j += blockDim.x) {
    const bool ok = j < D;
    P.a[j] = ok ? b.prior_a[rd.prior_off + j] : 0.0f;
    P.b[j] = ok ? b.prior_b[rd.prior_off + j] : 0.0f;
    P.kind[j] = ok ? b.prior_kind[rd.prior_off + j] : 0;
    P.p0[j] = ok ? fp[j] : 0.0f;
    if (FAM == GBNS_LIK_SHELLS) P.p1[j] = ok ? fp[D + j] : 0.0f;
    P.ab[j] = make_float4(P.a[j], P.b[j], P.p0[j],
                          FAM == GBNS_LIK_SHELLS ? (ok ? fp[D + j] : 0.0f) : __int_as_float(P.kind[j]));
  }
  if (FAM == GBNS_LIK_MVN) {
    for (int q = threadIdx.x; q < DMAX * DMAX; q += blockDim.x) {
      const int i = q / DMAX, j = q % DMAX;
      P.p1[q] = (i < D && j <= i) ? fp[D + i * D + j] : 0.0f;
    }
  }
  const float Lstar = Lstar_in ? Lstar_in[r] : liveL[rd.s - 1];
  __shared__ int s_next;
  if (threadIdx.x == 0) {
    s_next = 0;
    int uni = 1;
    for (int j = 0; j < D; ++j) uni &= b.prior_kind[rd.prior_off + j] == GBNS_PRIOR_UNIFORM;
    P.all_uniform = uni;
    if (FAM == GBNS_LIK_MVN) {
      P.c0 = fp[D + D * D];
    } else {
      P.R = fp[2 * D];
      P.w = fp[2 * D + 1];
      P.iw = 1.0f / P.w;
      P.norm = fp[2 * D + 2];
    }
    // m = #live points with log L > L* (the live set is sorted ascending)
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (liveL[mid] > Lstar) hi = mid; else lo = mid + 1;
    }
    P.m = n - lo;
  }
  __syncthreads();

  // Chain pool: the CTA owns chains [c_begin, c_begin + c_count) of run r (at most a few per
  // lane); a lane takes the next chain from the pool when its chain finishes, so the lanes of a
  // warp stay busy until the pool is drained.  Every lane stays in the loop until its whole
  // warp is done, so new directions can be generated warp-cooperatively.  A chain's arithmetic
  // does not depend on the lane that runs it.
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  extern __shared__ __align__(16) unsigned char slice_dyn[];
  DirWarp<DMAX> &W = reinterpret_cast<DirWarp<DMAX> *>(slice_dyn)[wid];
  const uint32_t dmagic = ((1u << 20) + (uint32_t)D - 1u) / (uint32_t)D;  // p / D = p * dmagic >> 20 for p < 2^14

  // --- keys: _collect_shell split (sharded_static.py:248) then split(sample_key, s)[c]
  Key sample_key;
  if (keys_in) {
    sample_key.k0 = keys_in[2 * r];
    sample_key.k1 = keys_in[2 * r + 1];
  } else {
    const Key k0 = {st.key[0], st.key[1]};
    sample_key = fold(fold(k0, 0u), 1u);
  }
  const int m = P.m;
  const int budget = b.max_evals_per_slice;

  int c = -1;          // current chain, -1 when the pool is drained
  int j = S;           // slice index of the current chain (S: no chain)
  bool start = true, need_dir = false, failed = false;
  float left = 0.f, right = 0.f, t = 0.f, alpha = 0.5f, logL0 = 0.f;
  Key ck = {0u, 0u}, after_key = {0u, 0u}, slices_key = {0u, 0u}, dir_key = {0u, 0u};
  int total = 0, in_slice = 0;
  float u0[DMAX], d[DMAX];
#pragma unroll
  for (int q = 0; q < DMAX; ++q) {
    u0[q] = 0.0f;
    d[q] = 0.0f;
  }

  // next chain of the pool: keys, seed point (resample_indicies over the mask log L > L*,
  // internals/random.py:34-84), first direction key (get_sample_from_seed)
  auto grab = [&]() {
    const int q = atomicAdd(&s_next, 1);
    if (q >= c_count) {
      c = -1;
      j = S;
      return;
    }
    c = c_begin + q;
    const Key kc = fold(sample_key, (uint32_t)c);
    const Key chain_key = fold(kc, 0u), seed_key = fold(kc, 1u);
    int idx = 0;
    if (m > 0) {
      const uint64_t M52 = bits64(seed_key, 0u) >> 12;
      const uint64_t qq = (1ull << 52) - M52;  // (1 - U) * 2^52
      const uint64_t lo = (uint64_t)m * qq, hi = __umul64hi((uint64_t)m, qq);
      uint64_t kk = (hi << 12) | (lo >> 52);
      if (lo & ((1ull << 52) - 1)) kk += 1;  // ceil(m (1 - U))
      idx = (n - m) + (int)kk - 1;
    }
#pragma unroll
    for (int q2 = 0; q2 < DMAX; ++q2)
      if (q2 < D) u0[q2] = liveU[(size_t)idx * D + q2];
    logL0 = liveL[idx];
    slices_key = fold(chain_key, 1u);
    dir_key = fold(chain_key, 0u);
    need_dir = true;
    j = 0;
    start = true;
    total = 0;
    in_slice = 0;
    failed = false;
  };
  grab();

  // --- flattened slice / shrink loop.  Slice starts (new direction, slice keys, chord bounds)
  // run on every kStartCadence-th loop trip only: a lane whose slice ended waits for that trip,
  // so the divergent start work of the warp's lanes is done together, once per kStartCadence
  // trips.  A chain's draws and arithmetic do not depend on when its lane runs them.  Shells
  // bench: 1.21x the throughput of starting at every trip (every second trip: 1.14x).
  constexpr int kStartCadence = 3;
  int phase = 0;  // loop trips modulo kStartCadence, the same in every lane of the warp
  for (;;) {
    const bool cadence = phase == 0;
    phase = phase + 1 == kStartCadence ? 0 : phase + 1;
    // ---- new directions: the D normals of every lane that needs one, flattened over
    // (lane, dimension) pairs across the warp; lanes publish their keys in rank order
    const unsigned dmask = __ballot_sync(0xffffffffu, need_dir && cadence);
    if (dmask) {
      if (D == 1) {
        if (need_dir) d[0] = 1.0f;
      } else {
        if (need_dir)
          W.key[__popc(dmask & ((1u << lane) - 1u))] = make_uint4(dir_key.k0, dir_key.k1, (uint32_t)lane, 0u);
        __syncwarp();
        const int cnt = __popc(dmask) * D;
        for (int p = lane; p < cnt; p += 32) {
          const int g = (int)(((uint32_t)p * dmagic) >> 20);
          const uint4 e = W.key[g];
          const uint32_t jj = (uint32_t)(p - g * D);
          W.buf[e.z][jj] = normal_from_bits(bits64(Key{e.x, e.y}, jj));
        }
        __syncwarp();
        if (need_dir) {
          float ss = 0.0f;
#pragma unroll
          for (int q = 0; q < DMAX; ++q)
            if (q < D) {
              d[q] = W.buf[lane][q];
              ss = fmaf(d[q], d[q], ss);
            }
          const float inv = 1.0f / sqrtf(ss);
#pragma unroll
          for (int q = 0; q < DMAX; ++q)
            if (q < D) d[q] = d[q] * inv;
        }
        __syncwarp();
      }
      need_dir = false;
    }
    const bool active = j < S;
    if (!__any_sync(0xffffffffu, active)) break;
    if (!active || (start && !cadence)) continue;

    // ---- one proposal: the first pick of slice j, or one shrink step (_new_proposal)
    Key B;
    if (start) B = fold(slices_key, (uint32_t)j);
    else B = ck;
    ck = fold(B, 0u);                              // run_key / next carry key
    const Key tk = fold(B, start ? 2u : 1u);       // t_key
    if (start) {
      after_key = fold(B, 3u);
      alpha = slice_alpha(j, S);
      bool climb = false;
      if (GRAD && b.gradient_slice) {
        // gradient_slice (uni_slice_sampler.py:202-214): slice along the normalised U-space
        // gradient at the seed point unless it vanishes or is not finite; one evaluation
        float g[DMAX];
        grad_u<DMAX, FAM>(P, D, u0, g);
        ++total;
        float gg = 0.0f;
#pragma unroll
        for (int q = 0; q < DMAX; ++q)
          if (q < D) gg = fmaf(g[q], g[q], gg);
        const float gn = sqrtf(gg);
        if (gn != 0.0f && isfinite(gn)) {
          climb = true;
#pragma unroll
          for (int q = 0; q < DMAX; ++q)
            if (q < D) d[q] = g[q] / gn;
        }
      }
      // _slice_bounds (uni_slice_sampler.py:41-64), with one reciprocal per direction component
      float t1r = INFINITY, t1l = -INFINITY, t0r = INFINITY, t0l = -INFINITY;
#pragma unroll
      for (int q = 0; q < DMAX; ++q) {
        if (q < D) {
          const float rc = 1.0f / d[q];
          const float t1 = (1.0f - u0[q]) * rc;
          const float t0 = -u0[q] * rc;
          t1r = fminf(t1r, t1 >= 0.f ? t1 : INFINITY);
          t1l = fmaxf(t1l, t1 <= 0.f ? t1 : -INFINITY);
          t0r = fminf(t0r, t0 >= 0.f ? t0 : INFINITY);
          t0l = fmaxf(t0l, t0 <= 0.f ? t0 : -INFINITY);
        }
      }
      right = fminf(t0r, t1r);
      left = climb ? 0.0f : fmaxf(t0l, t1l);  // climbing: only t >= 0 (uni_slice_sampler.py:214)
      in_slice = 0;
    } else {
      // _shrink_interval (uni_slice_sampler.py:92-111)
      if (t < 0.f) left = t;
      if (t > 0.f) right = t;
      if (rd.midpoint) {
        if (t < 0.f) left = alpha * left;
        if (t > 0.f) right = alpha * right;
      }
    }
    const float u = uniform01(bits64(tk, 0u));
    // _pick_point_in_interval (uni_slice_sampler.py:67-89)
    t = fmaf(u, right - left, left);
    const float logL = loglik<DMAX, FAM>(P, D, u0, d, t);
    ++total;
    ++in_slice;
    const bool accept = (logL > Lstar) || ((logL0 == Lstar) && (logL == Lstar));
    if (accept || in_slice >= budget) {
      if (!accept) failed = true;
#pragma unroll
      for (int q = 0; q < DMAX; ++q)
        if (q < D) u0[q] = fmaf(t, d[q], u0[q]);
      logL0 = logL;
      const int p = j - (S - 1 - K);
      if (K > 0 && p >= 0 && j < S - 1) {
        float *phU = b.ph_U + rd.phU_off + ((size_t)c * K + p) * D;
        for (int q = 0; q < D; ++q) phU[q] = u0[q];
        b.ph_L[rd.phL_off + (size_t)c * K + p] = logL;
      }
      ++j;
      start = true;
      if (GRAD && b.gradient_guided) {
        // Householder reflection at the accepted point (uni_slice_sampler.py:255-269); a
        // random direction from split(after_key)[0] when the gradient vanishes or is not
        // finite.  The gradient counts as one likelihood evaluation, also after the last slice.
        ++total;
        if (j < S) {
          float g[DMAX];
          grad_u<DMAX, FAM>(P, D, u0, g);
          float gg = 0.0f;
#pragma unroll
          for (int q = 0; q < DMAX; ++q)
            if (q < D) gg = fmaf(g[q], g[q], gg);
          const float gn = sqrtf(gg);
          if (!(gn >= 1e-10f) || isinf(gn)) {
            need_dir = true;
            dir_key = fold(after_key, 0u);
          } else {
            float dot = 0.0f;
#pragma unroll
            for (int q = 0; q < DMAX; ++q)
              if (q < D) dot = fmaf(d[q], g[q] / gn, dot);
            float dd = 0.0f;
#pragma unroll
            for (int q = 0; q < DMAX; ++q)
              if (q < D) {
                d[q] = fmaf(-2.0f * dot, g[q] / gn, d[q]);
                dd = fmaf(d[q], d[q], dd);
              }
            const float dn = sqrtf(dd);
#pragma unroll
            for (int q = 0; q < DMAX; ++q)
              if (q < D) d[q] = d[q] / dn;
          }
        }
      } else if (j < S) {
        need_dir = true;
        dir_key = after_key;
      }
      if (j >= S) {
        // chain finished: outputs, then the next chain of the pool
        const size_t out = (size_t)rd.shell_off + c;
        float *nu = b.new_U + rd.newU_off + (size_t)c * D;
        for (int q = 0; q < D; ++q) nu[q] = u0[q];
        b.new_L[out] = logL0;
        b.new_E[out] = total;
        if (failed) atomicOr(&st.status, (int)GBNS_ERR_SHRINK_BUDGET);
        grab();
      }
    } else {
      start = false;
    }
  }
}

using SliceKernel = void (*)(gbns_batch, int, const float *, const uint32_t *);

static size_t dir_warp_bytes(int dmax) {
  switch (dmax) {
    case 8: return sizeof(DirWarp<8>);
    case 16: return sizeof(DirWarp<16>);
    case 32: return sizeof(DirWarp<32>);
    default: return sizeof(DirWarp<64>);
  }
}

// One launch with the direction scratch of each warp in dynamic shared memory; kernels that
// need more than the default 48 KB get the opt-in first.
static cudaError_t launch_slice_kernel(SliceKernel k, int dmax, int nblk, int threads, const gbns_batch &b, int ib,
                                       const float *Lstar, const uint32_t *keys, cudaStream_t stream) {
  const size_t smem = (size_t)((threads + 31) / 32) * dir_warp_bytes(dmax);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k<<<nblk, threads, smem, stream>>>(b, ib, Lstar, keys);
  return cudaGetLastError();
}

template <int DMAX>
static cudaError_t launch_bucket(const gbns_batch &b, int fam, int ib, int ie, const float *Lstar, const uint32_t *keys,
                                 cudaStream_t stream) {
  const int nblk = ie - ib;
  if (nblk <= 0) return cudaSuccess;
  const int threads = b.chains_per_item;
  constexpr int DM = DMAX <= 16 ? DMAX : 16;
  if (fam == GBNS_LIK_MVN) {
    if (DMAX <= 16) {
      if (b.gradient_guided || b.gradient_slice)
        return launch_slice_kernel(k_slice_shell<DM, GBNS_LIK_MVN, true>, DM, nblk, threads, b, ib, Lstar, keys, stream);
      return launch_slice_kernel(k_slice_shell<DM, GBNS_LIK_MVN, false>, DM, nblk, threads, b, ib, Lstar, keys, stream);
    }
  } else {
    if (b.gradient_guided || b.gradient_slice)
      return launch_slice_kernel(k_slice_shell<DMAX, GBNS_LIK_SHELLS, true>, DMAX, nblk, threads, b, ib, Lstar, keys,
                                 stream);
    return launch_slice_kernel(k_slice_shell<DMAX, GBNS_LIK_SHELLS, false>, DMAX, nblk, threads, b, ib, Lstar, keys,
                               stream);
  }
  return cudaGetLastError();
}

// Buckets are (family, DMAX) pairs: bucket = fam * 4 + {0: D<=8, 1: D<=16, 2: D<=32, 3: D<=64}.
// The correlated-Gaussian buckets with D > 16 run the warp-cooperative kernel
// (gbns_slice_warp.cu); everything else runs one thread per chain here.
cudaError_t launch_slice_shells(const gbns_batch &b, const float *Lstar, const uint32_t *keys, cudaStream_t stream) {
  cudaError_t e;
  if ((e = launch_bucket<8>(b, 0, b.bucket_begin[0], b.bucket_end[0], Lstar, keys, stream))) return e;
  if ((e = launch_bucket<16>(b, 0, b.bucket_begin[1], b.bucket_end[1], Lstar, keys, stream))) return e;
  if ((e = launch_slice_warp(b, Lstar, keys, stream))) return e;
  if ((e = launch_bucket<8>(b, 1, b.bucket_begin[4], b.bucket_end[4], Lstar, keys, stream))) return e;
  if ((e = launch_bucket<16>(b, 1, b.bucket_begin[5], b.bucket_end[5], Lstar, keys, stream))) return e;
  if ((e = launch_bucket<32>(b, 1, b.bucket_begin[6], b.bucket_end[6], Lstar, keys, stream))) return e;
  if ((e = launch_bucket<64>(b, 1, b.bucket_begin[7], b.bucket_end[7], Lstar, keys, stream))) return e;
  return cudaSuccess;
}

}  // namespace gbns
