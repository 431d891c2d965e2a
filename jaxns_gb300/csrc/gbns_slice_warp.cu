// gbns_slice_warp.cu -- warp-cooperative uni-dimensional slice sampler for the correlated
// Gaussian family at 16 < D <= 64.
//
// Each lane owns one Markov chain's scalar state (keys, interval, counters) exactly as in
// gbns_slice.cu, but the O(D) and O(D^2) work is shared by the warp:
//   * likelihoods: the 32 proposals of a step form Delta[D x 32]; the warp computes
//     Z = Linv * Delta as a register-tiled GEMM (each lane: 4 chains x 8 rows), Linv^T in
//     shared memory (read as float4 broadcasts), then sum_i z_i^2 per chain;
//   * chord bounds, the accepted-point update and the D normal variates of each new
//     direction run lane-parallel over dimensions (two dimensions per lane).
// Every chain consumes the reference's RNG stream (uni_slice_sampler.py:114-273,
// :343-441) in the reference's order; only the work assignment differs.
// Warps refill finished lanes from the CTA's chain pool, so a CTA (one work item of up to
// a few thousand chains of one run) keeps all lanes busy until the pool is drained.
#include "gbns_device.cuh"
#include "gbns_launch.h"

namespace gbns {

constexpr int WARPS_PER_CTA_64 = 8;
constexpr int WARPS_PER_CTA_32 = 16;

// Row stride 33 for U0/DIR: a lane walking its own column and the warp walking one chain's
// column (two dimensions per lane) are both bank-conflict free.  DEL keeps stride 32 so the
// GEMM can read it as 16-byte vectors.
template <int DMAX>
struct WarpVecs {
  float DEL[DMAX][32];  // x - mu of the current proposals (column = lane)
  float U0[DMAX][33];   // seed point of each lane's chain
  float DIR[DMAX][33];  // current direction
};

template <int DMAX>
__device__ __forceinline__ float slice_alpha_w(int j, int S) {
  if (S == 1) return 0.5f;
  if (j == S - 1) return 1.0f;
  const float step = (float)j / (float)(S - 1);
  return 0.5f * (1.0f - step) + step;
}

// GRAD: the gradient-guided variant.  After each accepted point the chain's direction is
// reflected about the U-space gradient of log L there (uni_slice_sampler.py:255-269), computed
// warp-cooperatively: e = x - mu, z = Linv e, g = -Linv^T z (lanes over dimensions, the
// vectors staged in two columns of the proposal scratch), times the prior quantile's slope.
template <int DMAX, bool GRAD>
__global__ void __launch_bounds__(32 * (DMAX == 64 ? WARPS_PER_CTA_64 : WARPS_PER_CTA_32))
    k_slice_mvn_warp(gbns_batch b, int item_begin, const float *__restrict__ Lstar_in,
                     const uint32_t *__restrict__ keys_in) {
  extern __shared__ __align__(16) float smem[];
  float *LinvT = smem;                       // [DMAX][DMAX], LinvT[k * DMAX + row] = Linv[row][k]
  float *pa = LinvT + DMAX * DMAX;           // prior low / loc
  float *pb = pa + DMAX;                     // prior scale
  float *pmu = pb + DMAX;                    // mean
  int *pkind = (int *)(pmu + DMAX);
  __shared__ float s_Lstar;
  __shared__ int s_m, s_next, s_all_uniform;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpVecs<DMAX> &V = ((WarpVecs<DMAX> *)(pkind + DMAX))[warp];

  const int *it = b.items + 4 * (size_t)(item_begin + blockIdx.x);
  const int r = it[0], c_begin = it[1], c_count = it[2];
  const gbns_run_desc &rd = b.runs[r];
  gbns_run_state &st = b.state[r];
  if (!keys_in && (st.done || st.phase != 1)) return;
  const int D = rd.D, n = rd.n, S = rd.S, K = rd.K;
  const int par = st.parity;
  const float *__restrict__ liveL = b.live_L[par] + rd.live_off;
  const float *__restrict__ liveU = b.live_U[par] + rd.liveU_off;
  const float *fp = b.fparams + rd.param_off;

  for (int q = threadIdx.x; q < DMAX * DMAX; q += blockDim.x) {
    const int k = q / DMAX, row = q % DMAX;
    LinvT[q] = (row < D && k <= row) ? fp[D + row * D + k] : 0.0f;
  }
  int nonuni = 0;
  for (int j = threadIdx.x; j < DMAX; j += blockDim.x) {
    const bool ok = j < D;
    pa[j] = ok ? b.prior_a[rd.prior_off + j] : 0.0f;
    pb[j] = ok ? b.prior_b[rd.prior_off + j] : 0.0f;
    pmu[j] = ok ? fp[j] : 0.0f;
    pkind[j] = ok ? b.prior_kind[rd.prior_off + j] : 0;
    nonuni |= (ok && pkind[j] != GBNS_PRIOR_UNIFORM);
  }
  // rows k >= D of every warp's Delta stay zero
  for (int q = lane; q < DMAX * 32; q += 32) (&V.DEL[0][0])[q] = 0.0f;
  if (threadIdx.x == 0) {
    s_next = 0;
    s_all_uniform = 1;
    const float Ls = Lstar_in ? Lstar_in[r] : liveL[rd.s - 1];
    s_Lstar = Ls;
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (liveL[mid] > Ls) hi = mid; else lo = mid + 1;
    }
    s_m = n - lo;
  }
  __syncthreads();
  if (nonuni) atomicAnd(&s_all_uniform, 0);
  __syncthreads();
  const bool all_uniform = s_all_uniform != 0;
  const float Lstar = s_Lstar;
  const int m = s_m;

  Key sample_key;
  if (keys_in) {
    sample_key.k0 = keys_in[2 * r];
    sample_key.k1 = keys_in[2 * r + 1];
  } else {
    const Key k0 = {st.key[0], st.key[1]};
    sample_key = fold(fold(k0, 0u), 1u);
  }
  const int budget = b.max_evals_per_slice;
  const int cg = lane >> 2, rg = lane & 3;
  const int j0 = lane, j1 = lane + 32;

  // ---- per-lane chain state
  int c = -1, j = 0, total = 0, in_slice = 0;
  bool start = true, need_dir = false, failed = false;
  float left = 0.f, right = 0.f, t = 0.f, alpha = 0.5f, logL0 = 0.f;
  Key slices_key = {0u, 0u}, ck = {0u, 0u}, after_key = {0u, 0u}, dir_key = {0u, 0u};

  auto grab = [&]() {
    int q = -1;
    if (true) {
      const int g = atomicAdd(&s_next, 1);
      q = g < c_count ? g : -1;
    }
    if (q < 0) {
      c = -1;
      return;
    }
    c = c_begin + q;
    const Key kc = fold(sample_key, (uint32_t)c);
    const Key chain_key = fold(kc, 0u), seed_key = fold(kc, 1u);
    int idx = 0;
    if (m > 0) {
      const uint64_t M52 = bits64(seed_key, 0u) >> 12;
      const uint64_t qq = (1ull << 52) - M52;
      const uint64_t lo = (uint64_t)m * qq, hi = __umul64hi((uint64_t)m, qq);
      uint64_t kk = (hi << 12) | (lo >> 52);
      if (lo & ((1ull << 52) - 1)) kk += 1;
      idx = (n - m) + (int)kk - 1;
    }
    for (int d = 0; d < D; ++d) V.U0[d][lane] = liveU[(size_t)idx * D + d];
    logL0 = liveL[idx];
    dir_key = fold(chain_key, 0u);
    slices_key = fold(chain_key, 1u);
    need_dir = true;
    j = 0;
    start = true;
    total = 0;
    in_slice = 0;
    failed = false;
  };
  grab();

  // U-space gradient of log L at column q of U0, lanes over dimensions (j0, j1): e = x - mu,
  // z = Linv e, g = -Linv^T z, times the prior quantile's slope; columns 0 and 1 of the
  // proposal scratch hold e and z (the proposals of this step are written after it)
  auto grad_col = [&](int q, float &g0, float &g1) {
    float e0 = 0.f, e1 = 0.f, s0 = 0.f, s1 = 0.f;
    if (j0 < D) {
      float x;
      prior_quantile_slope(pkind[j0], pa[j0], pb[j0], V.U0[j0][q], x, s0);
      e0 = x - pmu[j0];
    }
    if (DMAX > 32 && j1 < D) {
      float x;
      prior_quantile_slope(pkind[j1], pa[j1], pb[j1], V.U0[j1][q], x, s1);
      e1 = x - pmu[j1];
    }
    __syncwarp();
    V.DEL[j0][0] = e0;
    if (DMAX > 32) V.DEL[j1][0] = e1;
    __syncwarp();
    float z0 = 0.f, z1 = 0.f;
    for (int k = 0; k < D; ++k) {
      const float ek = V.DEL[k][0];
      z0 = fmaf(LinvT[k * DMAX + j0], ek, z0);
      if (DMAX > 32) z1 = fmaf(LinvT[k * DMAX + j1], ek, z1);
    }
    V.DEL[j0][1] = z0;
    if (DMAX > 32) V.DEL[j1][1] = z1;
    __syncwarp();
    g0 = 0.f;
    g1 = 0.f;
    for (int i = 0; i < D; ++i) {
      const float zi = V.DEL[i][1];
      g0 = fmaf(LinvT[j0 * DMAX + i], zi, g0);
      if (DMAX > 32) g1 = fmaf(LinvT[j1 * DMAX + i], zi, g1);
    }
    g0 = -g0 * s0;
    g1 = -g1 * s1;
    __syncwarp();
  };

  for (;;) {
    // ---- new directions (initial or after an accepted slice), lane-parallel over dims
    unsigned dm = __ballot_sync(0xffffffffu, need_dir);
    while (dm) {
      const int q = __ffs(dm) - 1;
      dm &= dm - 1;
      const Key dk = {__shfl_sync(0xffffffffu, dir_key.k0, q), __shfl_sync(0xffffffffu, dir_key.k1, q)};
      if (D == 1) {
        if (lane == 0) V.DIR[0][q] = 1.0f;
      } else {
        const float v0 = (j0 < D) ? normal_from_bits(bits64(dk, (uint32_t)j0)) : 0.0f;
        const float v1 = (DMAX > 32 && j1 < D) ? normal_from_bits(bits64(dk, (uint32_t)j1)) : 0.0f;
        const float ss = warp_sum(fmaf(v1, v1, v0 * v0));
        const float inv = 1.0f / sqrtf(ss);
        if (j0 < D) V.DIR[j0][q] = v0 * inv;
        if (DMAX > 32 && j1 < D) V.DIR[j1][q] = v1 * inv;
      }
    }
    need_dir = false;
    const bool active = c >= 0;
    if (!__any_sync(0xffffffffu, active)) break;
    __syncwarp();

    // ---- chord bounds for lanes starting a slice (_slice_bounds, uni_slice_sampler.py:41-64)
    unsigned sm_ = __ballot_sync(0xffffffffu, active && start);
    while (sm_) {
      const int q = __ffs(sm_) - 1;
      sm_ &= sm_ - 1;
      bool climb = false;
      if (GRAD && b.gradient_slice) {
        // gradient_slice (uni_slice_sampler.py:202-214): slice along the normalised gradient at
        // the seed point unless it vanishes or is not finite (one evaluation, counted below)
        float g0, g1;
        grad_col(q, g0, g1);
        const float gn = sqrtf(warp_sum(fmaf(g0, g0, g1 * g1)));
        if (gn != 0.0f && isfinite(gn)) {
          climb = true;
          if (j0 < D) V.DIR[j0][q] = g0 / gn;
          if (DMAX > 32 && j1 < D) V.DIR[j1][q] = g1 / gn;
        }
        __syncwarp();
      }
      float t1r = INFINITY, t1l = -INFINITY, t0r = INFINITY, t0l = -INFINITY;
#pragma unroll
      for (int h = 0; h < (DMAX > 32 ? 2 : 1); ++h) {
        const int dd = h ? j1 : j0;
        if (dd < D) {
          const float u = V.U0[dd][q], di = 1.0f / V.DIR[dd][q];
          const float t1 = (1.0f - u) * di, t0 = -u * di;
          t1r = fminf(t1r, t1 >= 0.f ? t1 : INFINITY);
          t1l = fmaxf(t1l, t1 <= 0.f ? t1 : -INFINITY);
          t0r = fminf(t0r, t0 >= 0.f ? t0 : INFINITY);
          t0l = fmaxf(t0l, t0 <= 0.f ? t0 : -INFINITY);
        }
      }
      float rgt = fminf(t0r, t1r), lft = fmaxf(t0l, t1l);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        rgt = fminf(rgt, __shfl_xor_sync(0xffffffffu, rgt, o));
        lft = fmaxf(lft, __shfl_xor_sync(0xffffffffu, lft, o));
      }
      if (lane == q) {
        right = rgt;
        left = climb ? 0.0f : lft;  // climbing: only t >= 0 (uni_slice_sampler.py:214)
        if (GRAD && b.gradient_slice) ++total;
      }
    }

    // ---- this lane's proposal (_new_proposal: first pick or one shrink step)
    if (active) {
      float u;
      if (start) {
        const Key kj = fold(slices_key, (uint32_t)j);
        ck = fold(kj, 0u);
        const Key t_key = fold(kj, 2u);
        after_key = fold(kj, 3u);
        alpha = slice_alpha_w<DMAX>(j, S);
        u = uniform01(bits64(t_key, 0u));
        in_slice = 0;
      } else {
        const Key nk = fold(ck, 0u), tk = fold(ck, 1u);
        if (t < 0.f) left = t;
        if (t > 0.f) right = t;
        if (rd.midpoint) {
          if (t < 0.f) left = alpha * left;
          if (t > 0.f) right = alpha * right;
        }
        u = uniform01(bits64(tk, 0u));
        ck = nk;
      }
      t = fmaf(u, right - left, left);
      // x - mu of the proposal into this lane's column of Delta
      if (all_uniform) {
        for (int d = 0; d < D; ++d)
          V.DEL[d][lane] = fmaf(pb[d], fmaf(t, V.DIR[d][lane], V.U0[d][lane]), pa[d]) - pmu[d];
      } else {
        for (int d = 0; d < D; ++d)
          V.DEL[d][lane] =
              prior_quantile(pkind[d], pa[d], pb[d], fmaf(t, V.DIR[d][lane], V.U0[d][lane])) - pmu[d];
      }
    } else {
      for (int d = 0; d < D; ++d) V.DEL[d][lane] = 0.0f;
    }
    __syncwarp();

    // ---- Z = Linv * Delta, register tile of 4 chains x 8 rows per lane
    float s4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int p = 0; p < DMAX / 32; ++p) {
      const int row0 = 32 * p + 8 * rg;
      const int kend = min(D, 32 * p + 32);
      if (32 * p < D) {
        float acc[4][8];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc)
#pragma unroll
          for (int rr = 0; rr < 8; ++rr) acc[cc][rr] = 0.f;
#pragma unroll 4
        for (int k = 0; k < kend; ++k) {
          const float4 dv = *reinterpret_cast<const float4 *>(&V.DEL[k][4 * cg]);
          const float4 la = *reinterpret_cast<const float4 *>(&LinvT[k * DMAX + row0]);
          const float4 lb = *reinterpret_cast<const float4 *>(&LinvT[k * DMAX + row0 + 4]);
          const float dvv[4] = {dv.x, dv.y, dv.z, dv.w};
          const float lv[8] = {la.x, la.y, la.z, la.w, lb.x, lb.y, lb.z, lb.w};
#pragma unroll
          for (int cc = 0; cc < 4; ++cc)
#pragma unroll
            for (int rr = 0; rr < 8; ++rr) acc[cc][rr] = fmaf(lv[rr], dvv[cc], acc[cc][rr]);
        }
#pragma unroll
        for (int cc = 0; cc < 4; ++cc)
#pragma unroll
          for (int rr = 0; rr < 8; ++rr) s4[cc] = fmaf(acc[cc][rr], acc[cc][rr], s4[cc]);
      }
    }
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      s4[cc] += __shfl_xor_sync(0xffffffffu, s4[cc], 1);
      s4[cc] += __shfl_xor_sync(0xffffffffu, s4[cc], 2);
    }
    const float s_mine = rg == 0 ? s4[0] : (rg == 1 ? s4[1] : (rg == 2 ? s4[2] : s4[3]));
    float logL = -0.5f * s_mine;  // relative to the run's log_L_offset (= c0)
    if (logL != logL) logL = -INFINITY;  // NaN -> -inf (framework/ops.py:323-325)

    // ---- accept / shrink decision
    bool accept = false, advance = false;
    if (active) {
      ++total;
      ++in_slice;
      accept = (logL > Lstar) || ((logL0 == Lstar) && (logL == Lstar));
      advance = accept || in_slice >= budget;
      if (advance && !accept) failed = true;
    }
    // accepted point: U0 += t * DIR (lane-parallel over dims)
    unsigned am = __ballot_sync(0xffffffffu, advance);
    __syncwarp();
    {
      unsigned mm = am;
      while (mm) {
        const int q = __ffs(mm) - 1;
        mm &= mm - 1;
        const float tq = __shfl_sync(0xffffffffu, t, q);
        if (j0 < D) V.U0[j0][q] = fmaf(tq, V.DIR[j0][q], V.U0[j0][q]);
        if (DMAX > 32 && j1 < D) V.U0[j1][q] = fmaf(tq, V.DIR[j1][q], V.U0[j1][q]);
      }
    }
    __syncwarp();
    bool grad_fallback = false;
    if (GRAD && b.gradient_guided) {
      // reflect each advancing chain's direction about the gradient at its accepted point
      unsigned mm = am;
      while (mm) {
        const int q = __ffs(mm) - 1;
        mm &= mm - 1;
        float g0, g1;
        grad_col(q, g0, g1);
        const float gn = sqrtf(warp_sum(fmaf(g0, g0, g1 * g1)));
        if (!(gn >= 1e-10f) || isinf(gn)) {
          if (lane == q) grad_fallback = true;
        } else {
          const float d0 = j0 < D ? V.DIR[j0][q] : 0.f, d1 = (DMAX > 32 && j1 < D) ? V.DIR[j1][q] : 0.f;
          const float dot = warp_sum(fmaf(d0, g0 / gn, d1 * (g1 / gn)));
          const float r0 = fmaf(-2.0f * dot, g0 / gn, d0), r1 = fmaf(-2.0f * dot, g1 / gn, d1);
          const float rn = sqrtf(warp_sum(fmaf(r0, r0, r1 * r1)));
          if (j0 < D) V.DIR[j0][q] = r0 / rn;
          if (DMAX > 32 && j1 < D) V.DIR[j1][q] = r1 / rn;
        }
        __syncwarp();
      }
    }
    if (advance) {
      logL0 = logL;
      const int p = j - (S - 1 - K);
      if (K > 0 && p >= 0 && j < S - 1) {
        float *phU = b.ph_U + rd.phU_off + ((size_t)c * K + p) * D;
        for (int d = 0; d < D; ++d) phU[d] = V.U0[d][lane];
        b.ph_L[rd.phL_off + (size_t)c * K + p] = logL;
      }
      ++j;
      start = true;
      if (GRAD && b.gradient_guided) ++total;  // the gradient counts as one likelihood evaluation
      if (j < S) {
        if (!(GRAD && b.gradient_guided)) {
          need_dir = true;
          dir_key = after_key;
        } else if (grad_fallback) {
          need_dir = true;
          dir_key = fold(after_key, 0u);  // split(after_key)[0]
        }
      } else {
        // chain finished: outputs, then the next chain of the pool
        const size_t out = (size_t)rd.shell_off + c;
        float *nu = b.new_U + rd.newU_off + (size_t)c * D;
        for (int d = 0; d < D; ++d) nu[d] = V.U0[d][lane];
        b.new_L[out] = logL0;
        b.new_E[out] = total;
        if (failed) atomicOr(&st.status, (int)GBNS_ERR_SHRINK_BUDGET);
        grab();
      }
    } else if (active) {
      start = false;
    }
    __syncwarp();
  }
}

template <int DMAX>
static size_t warp_smem_bytes(int warps) {
  return sizeof(float) * (DMAX * DMAX + 3 * DMAX) + sizeof(int) * DMAX + sizeof(WarpVecs<DMAX>) * warps;
}

template <int DMAX>
static cudaError_t launch_warp_bucket(const gbns_batch &b, int ib, int ie, const float *Lstar, const uint32_t *keys,
                                      cudaStream_t stream) {
  const int nblk = ie - ib;
  if (nblk <= 0) return cudaSuccess;
  const int warps = DMAX == 64 ? WARPS_PER_CTA_64 : WARPS_PER_CTA_32;
  const size_t sm = warp_smem_bytes<DMAX>(warps);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_slice_mvn_warp<DMAX, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sm);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_slice_mvn_warp<DMAX, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (b.gradient_guided || b.gradient_slice)
    k_slice_mvn_warp<DMAX, true><<<nblk, 32 * warps, sm, stream>>>(b, ib, Lstar, keys);
  else k_slice_mvn_warp<DMAX, false><<<nblk, 32 * warps, sm, stream>>>(b, ib, Lstar, keys);
  return cudaGetLastError();
}

// MVN buckets 2 (16 < D <= 32) and 3 (32 < D <= 64) run here.
cudaError_t launch_slice_warp(const gbns_batch &b, const float *Lstar, const uint32_t *keys, cudaStream_t stream) {
  cudaError_t e;
  if ((e = launch_warp_bucket<32>(b, b.bucket_begin[2], b.bucket_end[2], Lstar, keys, stream))) return e;
  if ((e = launch_warp_bucket<64>(b, b.bucket_begin[3], b.bucket_end[3], Lstar, keys, stream))) return e;
  return cudaSuccess;
}

}  // namespace gbns
