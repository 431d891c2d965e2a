// gbns_phiw.cu -- the linear-Gaussian (Phi w) family: lock-step slice sampling with a
// batched residual contraction, and the reweighted-evidence adjoint.
//
// log L(w) = -N/2 log(2 pi sigma^2) - |y - Phi w|^2 / (2 sigma^2), w = tau * ndtri(U) (the
// Normal(0, tau^2) prior quantile).  One likelihood is an N x P contraction, so the chains of
// a shell advance together: gbns_lg_step runs each chain's slice logic up to its next
// proposal (same RNG stream and decisions as uni_slice_sampler.py:114-273, :343-441), and the
// residual kernel evaluates |y - Phi w|^2 for all proposals of the step at once.
//
// U is FP64 in this family (as in the reference, which runs in f64): with a Normal prior
// the posterior can sit where u is within 1e-8 of 0 or 1, which fp32 cannot resolve.  FP64 U
// is kept in the float U buffers as pairs of 32-bit words (gbns_run_desc.ucols = 2 D), so the
// generic merge / store / results kernels move it unchanged.  Inside the lock-step kernels a
// chain's point is an fp32 pair u = a + b (|b| <= ulp(a) / 2): FP64 runs at a small fraction
// of the fp32 rate on this GPU, and the pair keeps what the tails need -- 1 - u = (1 - a) - b
// is exact to fp32 relative precision, and a proposal adds its step t d into the low part.
// FP64 is touched only when a chain loads its seed and stores its result.
#include <cstdio>
#include "gbns_device.cuh"
#include "gbns_launch.h"
#include "gbns_lg.cuh"

namespace gbns {

// A chain's first state of the shell: seed point (resample_indicies over log L > L*),
// direction and slice keys (get_sample_from_seed, uni_slice_sampler.py:403-423).
__global__ void k_lg_init(gbns_batch b, gbns_lg_bufs lg, long long total_chains) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= total_chains) return;
  const int r = run_of_chain(b, g);
  const gbns_run_desc &rd = b.runs[r];
  const gbns_run_state &st = b.state[r];
  if (rd.family != GBNS_LIK_LINGAUSS || st.done || st.phase != 1) return;
  const int c = (int)(g - rd.shell_off);
  if (c >= rd.s) return;
  const int n = rd.n, P = rd.D;
  const float *liveL = b.live_L[st.parity] + rd.live_off;
  const double *liveU = (const double *)(b.live_U[st.parity] + rd.liveU_off);
  const float Lstar = liveL[rd.s - 1];
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (liveL[mid] > Lstar) hi = mid; else lo = mid + 1;
  }
  const int m = n - lo;
  const Key k0 = {st.key[0], st.key[1]};
  const Key sample_key = fold(fold(k0, 0u), 1u);
  const Key kc = fold(sample_key, (uint32_t)c);
  const Key chain_key = fold(kc, 0u), seed_key = fold(kc, 1u);
  int idx = 0;
  if (m > 0) {
    const uint64_t M52 = bits64(seed_key, 0u) >> 12;
    const uint64_t q = (1ull << 52) - M52;
    const uint64_t lo64 = (uint64_t)m * q, hi64 = __umul64hi((uint64_t)m, q);
    uint64_t kk = (hi64 << 12) | (lo64 >> 52);
    if (lo64 & ((1ull << 52) - 1)) kk += 1;
    idx = (n - m) + (int)kk - 1;
  }
  const size_t co = (rd.newU_off >> 1) + (size_t)c * P;
  for (int p = 0; p < P; ++p) pair_from_double(liveU[(size_t)idx * P + p], lg.u0[co + p], lg.u0_lo[co + p]);
  lg.logL0[g] = liveL[idx];
  const Key dk = fold(chain_key, 0u), sk = fold(chain_key, 1u);
  lg.dir_key[2 * g] = dk.k0;
  lg.dir_key[2 * g + 1] = dk.k1;
  lg.slices_key[2 * g] = sk.k0;
  lg.slices_key[2 * g + 1] = sk.k1;
  lg.flags[g] = LG_START | LG_NEED_DIR;
  lg.j[g] = 0;
  lg.total[g] = 0;
  lg.in_slice[g] = 0;
  lg.ss[g] = 0.0;
  if (c == 0) lg.chains_left[r] = rd.s;
}


// One likelihood evaluation per chain: consume the pending result, then prepare the next
// proposal w or finish the chain.  One warp per chain, lanes over the dimensions
// (p = lane, lane + 32), so every per-dimension read and write is a coalesced row access.
__global__ void __launch_bounds__(256) k_lg_step(gbns_batch b, gbns_lg_bufs lg, long long total_chains) {
  pdl_launch_dependents();
  pdl_wait_prior_grid();  // the residuals of the previous step
  const long long g = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= total_chains) return;
  const int r = lg.chain_run ? lg.chain_run[g] : run_of_chain(b, g);
  const gbns_run_desc &rd = b.runs[r];
  gbns_run_state &st = b.state[r];
  if (rd.family != GBNS_LIK_LINGAUSS || st.done || st.phase != 1) return;
  const int c = (int)(g - rd.shell_off);
  if (c >= rd.s) return;
  int flags = lg.flags[g];
  if (flags & LG_DONE) return;
  const int P = rd.D, S = rd.S, K = rd.K, N = rd.N;
  const int pa_ = lane, pb_ = lane + 32;
  const bool ha = pa_ < P, hb = pb_ < P;
  const float *fp = b.fparams + rd.param_off;
  const float sigma = fp[(size_t)N * P + N];
  const float inv2s2 = 0.5f / (sigma * sigma);
  const float Lstar = b.live_L[st.parity][rd.live_off + rd.s - 1];
  const long long du = rd.newU_off >> 1;  // chain vectors: D floats per chain
  float *u0 = lg.u0 + du + (size_t)c * P, *u0l = lg.u0_lo + du + (size_t)c * P;
  float *d = lg.dir + du + (size_t)c * P;
  float ua = ha ? u0[pa_] : 0.0f, ub = hb ? u0[pb_] : 0.0f;      // seed point: (ua, la), (ub, lb)
  float la = ha ? u0l[pa_] : 0.0f, lb = hb ? u0l[pb_] : 0.0f;
  float da = ha ? d[pa_] : 0.0f, db = hb ? d[pb_] : 0.0f;
  int j = lg.j[g], total = lg.total[g], in_slice = lg.in_slice[g];
  float left = lg.left[g], right = lg.right[g], t = lg.t[g], alpha = lg.alpha[g], logL0 = lg.logL0[g];
  Key ck = {lg.ck[2 * g], lg.ck[2 * g + 1]};
  Key after_key = {lg.after_key[2 * g], lg.after_key[2 * g + 1]};
  Key dir_key = {lg.dir_key[2 * g], lg.dir_key[2 * g + 1]};
  const Key slices_key = {lg.slices_key[2 * g], lg.slices_key[2 * g + 1]};
  bool u_changed = false, d_changed = false;

  if (flags & LG_PENDING) {
    const double ss = lg.ss[g];
    float logL = (float)(-ss * (double)inv2s2);  // relative to the run's log_L_offset
    if (logL != logL) logL = -INFINITY;
    ++total;
    ++in_slice;
    const bool accept = (logL > Lstar) || ((logL0 == Lstar) && (logL == Lstar));
    if (accept || in_slice >= b.max_evals_per_slice) {
      if (!accept) flags |= LG_FAILED;
      pair_add(ua, fmaf(t, da, la), ua, la);
      pair_add(ub, fmaf(t, db, lb), ub, lb);
      u_changed = true;
      logL0 = logL;
      const int ph = j - (S - 1 - K);
      if (K > 0 && ph >= 0 && j < S - 1) {
        double *phU = (double *)(b.ph_U + rd.phU_off) + ((size_t)c * K + ph) * P;
        if (ha) phU[pa_] = (double)ua + (double)la;
        if (hb) phU[pb_] = (double)ub + (double)lb;
        if (lane == 0) b.ph_L[rd.phL_off + (size_t)c * K + ph] = logL;
      }
      ++j;
      flags |= LG_START;
      // gradient_guided (uni_slice_sampler.py:255-272): the gradient at the accepted point
      // counts as one evaluation, also after the last slice
      if (b.gradient_guided) ++total;
      if (j < S) {
        if (b.gradient_guided) {
          flags |= LG_WAIT_REFLECT;
        } else {
          flags |= LG_NEED_DIR;
          dir_key = after_key;
        }
      } else {
        flags |= LG_DONE;
      }
    } else {
      flags &= ~LG_START;
    }
    flags &= ~LG_PENDING;
  }
  // Gradient options: a chain that needs the U-space gradient at its point (after an accepted
  // point with gradient_guided, at a slice start with gradient_slice) lists itself and sits out
  // this step; the gradient launch that follows fills lg.grad and sets LG_HAVE_GRAD.
  bool park = false;
  float ga = 0.0f, gb = 0.0f;
  if (!(flags & LG_DONE) && (b.gradient_guided || b.gradient_slice)) {
    const bool want = (flags & LG_WAIT_REFLECT) || ((flags & LG_START) && b.gradient_slice);
    if (want && !(flags & LG_HAVE_GRAD)) {
      park = true;
      if (lane == 0) lg.grad_list[atomicAdd(lg.grad_count, 1)] = g;
    } else if (flags & LG_HAVE_GRAD) {
      const float *gr = lg.grad + (rd.newU_off >> 1) + (size_t)c * P;
      ga = ha ? gr[pa_] : 0.0f;
      gb = hb ? gr[pb_] : 0.0f;
    }
  }
  if (flags & LG_DONE) {
    double *nu = (double *)(b.new_U + rd.newU_off) + (size_t)c * P;
    if (ha) nu[pa_] = (double)ua + (double)la;
    if (hb) nu[pb_] = (double)ub + (double)lb;
    if (lane == 0) {
      b.new_L[rd.shell_off + c] = logL0;
      b.new_E[rd.shell_off + c] = total;
      if (flags & LG_FAILED) atomicOr(&st.status, (int)GBNS_ERR_SHRINK_BUDGET);
      atomicSub(&lg.chains_left[r], 1);
    }
  } else if (!park) {
    if (flags & LG_WAIT_REFLECT) {
      // Householder reflection about the normalised gradient (uni_slice_sampler.py:255-269);
      // a random direction from split(after_key)[0] when the gradient vanishes or is not finite
      const float gn = sqrtf(warp_sum(fmaf(ga, ga, gb * gb)));
      if (!(gn >= 1e-10f) || isinf(gn)) {
        flags |= LG_NEED_DIR;
        dir_key = fold(after_key, 0u);
      } else {
        const float na = ga / gn, nb = gb / gn;
        const float dot = warp_sum(fmaf(da, na, db * nb));
        da = fmaf(-2.0f * dot, na, da);
        db = fmaf(-2.0f * dot, nb, db);
        const float dn = sqrtf(warp_sum(fmaf(da, da, db * db)));
        da = da / dn;
        db = db / dn;
        d_changed = true;
      }
      flags &= ~LG_WAIT_REFLECT;
    }
    if (flags & LG_NEED_DIR) {
      if (P == 1) {
        da = 1.0f;
      } else {
        const float va = ha ? normal_from_bits(bits64(dir_key, (uint32_t)pa_)) : 0.0f;
        const float vb = hb ? normal_from_bits(bits64(dir_key, (uint32_t)pb_)) : 0.0f;
        const float nrm = sqrtf(warp_sum(fmaf(va, va, vb * vb)));
        da = va / nrm;
        db = vb / nrm;
      }
      d_changed = true;
      flags &= ~LG_NEED_DIR;
    }
    const bool start = (flags & LG_START) != 0;
    const Key B = start ? fold(slices_key, (uint32_t)j) : ck;
    ck = fold(B, 0u);
    const Key tk = fold(B, start ? 2u : 1u);
    if (start) {
      after_key = fold(B, 3u);
      alpha = lg_alpha(j, S);
      bool climb = false;
      if (b.gradient_slice) {
        // gradient_slice (uni_slice_sampler.py:202-214): slice along the normalised U-space
        // gradient at the seed point (t >= 0) unless it vanishes or is not finite; one evaluation
        ++total;
        const float gn = sqrtf(warp_sum(fmaf(ga, ga, gb * gb)));
        if (gn != 0.0f && isfinite(gn)) {
          climb = true;
          da = ga / gn;
          db = gb / gn;
          d_changed = true;
        }
      }
      // chord of u0 + t d in the unit cube; 1 - u = (1 - a) - b keeps the tails exact
      float t1r = INFINITY, t1l = -INFINITY, t0r = INFINITY, t0l = -INFINITY;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const bool have = h ? hb : ha;
        if (have) {
          const float uu = h ? ub : ua, ll = h ? lb : la, dd = h ? db : da;
          const float t1 = ((1.0f - uu) - ll) / dd, t0 = -(uu + ll) / dd;
          t1r = fminf(t1r, t1 >= 0.f ? t1 : INFINITY);
          t1l = fmaxf(t1l, t1 <= 0.f ? t1 : -INFINITY);
          t0r = fminf(t0r, t0 >= 0.f ? t0 : INFINITY);
          t0l = fmaxf(t0l, t0 <= 0.f ? t0 : -INFINITY);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        t1r = fminf(t1r, __shfl_xor_sync(0xffffffffu, t1r, o));
        t1l = fmaxf(t1l, __shfl_xor_sync(0xffffffffu, t1l, o));
        t0r = fminf(t0r, __shfl_xor_sync(0xffffffffu, t0r, o));
        t0l = fmaxf(t0l, __shfl_xor_sync(0xffffffffu, t0l, o));
      }
      right = fminf(t0r, t1r);
      left = climb ? 0.0f : fmaxf(t0l, t1l);
      in_slice = 0;
    } else {
      if (t < 0.f) left = t;
      if (t > 0.f) right = t;
      if (rd.midpoint) {
        if (t < 0.f) left = alpha * left;
        if (t > 0.f) right = alpha * right;
      }
    }
    // _pick_point_in_interval (uni_slice_sampler.py:67-89): t = left + u (right - left)
    t = fmaf(uniform01(bits64(tk, 0u)), right - left, left);
    const int *kind = b.prior_kind + rd.prior_off;
    const float *pa = b.prior_a + rd.prior_off, *pb = b.prior_b + rd.prior_off;
    // proposal u0 + t d = a + (b + t d): the step goes into the low part
    const float wa = ha ? prior_quantile_pair(kind[pa_], pa[pa_], pb[pa_], ua, fmaf(t, da, la)) : 0.0f;
    const float wb = hb ? prior_quantile_pair(kind[pb_], pa[pb_], pb[pb_], ub, fmaf(t, db, lb)) : 0.0f;
    if (lg.use_tc) {
      float *wh = lg.W_hi + (size_t)g * 64, *wl = lg.W_lo + (size_t)g * 64;
      if (ha) tf32_split(wa, wh[pa_], wl[pa_]);
      if (hb) tf32_split(wb, wh[pb_], wl[pb_]);
    } else {
      float *W = lg.W + du + (size_t)c * P;
      if (ha) W[pa_] = wa;
      if (hb) W[pb_] = wb;
    }
    flags |= LG_PENDING;
    flags &= ~LG_HAVE_GRAD;
    if (lane == 0 && lg.tile_pending) lg.tile_pending[lg.tile_base[r] + (c >> 7)] = 1;
  }
  if (u_changed) {
    if (ha) {
      u0[pa_] = ua;
      u0l[pa_] = la;
    }
    if (hb) {
      u0[pb_] = ub;
      u0l[pb_] = lb;
    }
  }
  if (d_changed) {
    if (ha) d[pa_] = da;
    if (hb) d[pb_] = db;
  }
  if (lane == 0) {
    lg.ss[g] = 0.0;
    lg.flags[g] = flags;
    lg.j[g] = j;
    lg.total[g] = total;
    lg.in_slice[g] = in_slice;
    lg.left[g] = left;
    lg.right[g] = right;
    lg.t[g] = t;
    lg.alpha[g] = alpha;
    lg.logL0[g] = logL0;
    lg.ck[2 * g] = ck.k0;
    lg.ck[2 * g + 1] = ck.k1;
    lg.after_key[2 * g] = after_key.k0;
    lg.after_key[2 * g + 1] = after_key.k1;
    lg.dir_key[2 * g] = dir_key.k0;
    lg.dir_key[2 * g + 1] = dir_key.k1;
  }
}

// U-space gradient of log L at the point of every chain listed by the chain step (jax.grad of
// Model.forward through the prior quantile, as for the other families): d log L / dw =
// Phi^T (y - Phi w) / sigma^2, times dw/du (Uniform: b; Normal: b sqrt(2 pi) exp(z^2 / 2)).
// One CTA per listed chain, grid-stride over the list: threads over data rows form the
// residuals and their products with Phi, then a CTA reduction per dimension (fp32).
template <int PM>
__global__ void __launch_bounds__(256) k_lg_grad(gbns_batch b, gbns_lg_bufs lg) {
  __shared__ float w_s[PM], slope_s[PM];
  __shared__ float red[8][PM];
  const int count = *lg.grad_count;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int e = blockIdx.x; e < count; e += gridDim.x) {
    const long long g = lg.grad_list[e];
    const int r = lg.chain_run ? lg.chain_run[g] : run_of_chain(b, g);
    const gbns_run_desc &rd = b.runs[r];
    const int P = rd.D, N = rd.N;
    const int c = (int)(g - rd.shell_off);
    const size_t co = (rd.newU_off >> 1) + (size_t)c * P;
    const float *fp = b.fparams + rd.param_off;
    const float *Phi = fp, *y = fp + (size_t)N * P;
    const float sigma = fp[(size_t)N * P + N];
    if (tid < P) {
      const int kind = b.prior_kind[rd.prior_off + tid];
      const float pa = b.prior_a[rd.prior_off + tid], pb = b.prior_b[rd.prior_off + tid];
      const float ua = lg.u0[co + tid], la = lg.u0_lo[co + tid];
      w_s[tid] = prior_quantile_pair(kind, pa, pb, ua, la);
      if (kind == GBNS_PRIOR_UNIFORM) {
        slope_s[tid] = pb;
      } else {
        const float z = ndtri_pair(ua, la);
        slope_s[tid] = pb * 2.50662827463f * gbns_fm_exp(0.5f * z * z);
      }
    }
    __syncthreads();
    float acc[PM];
#pragma unroll
    for (int q = 0; q < PM; ++q) acc[q] = 0.0f;
    for (int i = tid; i < N; i += blockDim.x) {
      const float *row = Phi + (size_t)i * P;
      float pw = 0.0f;
#pragma unroll
      for (int q = 0; q < PM; ++q)
        if (q < P) pw = fmaf(row[q], w_s[q], pw);
      const float res = y[i] - pw;
#pragma unroll
      for (int q = 0; q < PM; ++q)
        if (q < P) acc[q] = fmaf(row[q], res, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < PM; ++q) {
      const float v = warp_sum(acc[q]);
      if (lane == 0) red[wid][q] = v;
    }
    __syncthreads();
    if (tid < P) {
      float sum = 0.0f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += red[w][tid];
      lg.grad[co + tid] = sum / (sigma * sigma) * slope_s[tid];
    }
    if (tid == 0) lg.flags[g] |= LG_HAVE_GRAD;
    __syncthreads();
  }
}

// |y - Phi w|^2 (and y . (y - Phi w)) for a 64-point x 64-row tile; FP64 atomics per point.
// Points are rows of W (the pending proposals), or for the adjoint rows of an FP64 U with
// w = tau * ndtri(u).
template <int PMAX>
__device__ __forceinline__ void resid_tile(const float *__restrict__ Wsrc, const double *__restrict__ Usrc, float tau,
                                           int npts, int P,
                                           const float *__restrict__ Phi, const float *__restrict__ y, int N,
                                           int row0, double *ss_out, double *ry_out) {
  __shared__ float Ws[64][PMAX + 1];
  __shared__ float Ps[64][PMAX + 1];
  __shared__ float ys[64];
  __shared__ float red_ss[16][65];
  __shared__ float red_ry[16][65];
  const int tid = threadIdx.x;
  for (int q = tid; q < 64 * PMAX; q += blockDim.x) {
    const int i = q / PMAX, k = q % PMAX;
    float w = 0.0f;
    if (i < npts && k < P) {
      w = Usrc ? tau * ndtri_from_double(Usrc[(size_t)i * P + k]) : Wsrc[(size_t)i * P + k];
    }
    Ws[i][k] = w;
    const int row = row0 + i;
    Ps[i][k] = (row < N && k < P) ? Phi[(size_t)row * P + k] : 0.0f;
  }
  if (tid < 64) ys[tid] = (row0 + tid < N) ? y[row0 + tid] : 0.0f;
  __syncthreads();
  const int tx = tid & 15, ty = tid >> 4;
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = 0.0f;
#pragma unroll 4
  for (int k = 0; k < P; ++k) {
    float wv[4], pv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) wv[c] = Ws[4 * tx + c][k];
#pragma unroll
    for (int a = 0; a < 4; ++a) pv[a] = Ps[4 * ty + a][k];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][c] = fmaf(pv[a], wv[c], acc[a][c]);
  }
  float pss[4] = {0.f, 0.f, 0.f, 0.f}, pry[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    if (row0 + 4 * ty + a < N) {
      const float yy = ys[4 * ty + a];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float rr = yy - acc[a][c];
        pss[c] = fmaf(rr, rr, pss[c]);
        pry[c] = fmaf(rr, yy, pry[c]);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    red_ss[ty][4 * tx + c] = pss[c];
    red_ry[ty][4 * tx + c] = pry[c];
  }
  __syncthreads();
  if (tid < 64 && tid < npts) {
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      s1 += (double)red_ss[q][tid];
      s2 += (double)red_ry[q][tid];
    }
    atomicAdd(&ss_out[tid], s1);
    if (ry_out) atomicAdd(&ry_out[tid], s2);
  }
}

template <int PMAX>
__global__ void __launch_bounds__(256) k_lg_resid(gbns_batch b, gbns_lg_bufs lg) {
  const int *it = lg.items + 4 * (size_t)blockIdx.x;
  const int r = it[0], c0 = it[1], nc = it[2], row0 = it[3];
  const gbns_run_desc &rd = b.runs[r];
  const gbns_run_state &st = b.state[r];
  if (st.done || st.phase != 1) return;
  const int t = threadIdx.x;
  const bool pending = t < nc && (lg.flags[rd.shell_off + c0 + t] & LG_PENDING) != 0;
  if (!__syncthreads_or(pending)) return;
  const int P = rd.D, N = rd.N;
  const float *fp = b.fparams + rd.param_off;
  resid_tile<PMAX>(lg.W + (rd.newU_off >> 1) + (size_t)c0 * P, nullptr, 0.0f, nc, P, fp, fp + (size_t)N * P, N, row0,
                   lg.ss + rd.shell_off + c0, nullptr);
}

template <int PMAX>
__global__ void __launch_bounds__(256) k_adj_resid(const double *U, long long M, int P, const float *Phi, const float *y,
                                                   int N, float tau, double *ss, double *ry) {
  const long long p0 = (long long)blockIdx.x * 64;
  const int row0 = blockIdx.y * 64;
  const int npts = (int)min(64ll, M - p0);
  resid_tile<PMAX>(nullptr, U + p0 * P, tau, npts, P, Phi, y, N, row0, ss + p0, ry + p0);
}

// log Z(theta) = logsumexp_i a_i, a_i = log L_theta(U_i) + log w_i, and its gradient
// sum_i softmax(a)_i dlogL_i/dtheta, all in FP64.
__global__ void __launch_bounds__(1024) k_adj_reduce(const double *log_w, long long M, int N, double log_sigma,
                                                     const double *ss, const double *ry, double *out) {
  __shared__ double red[32];
  const double s2 = exp(2.0 * log_sigma);
  const double c = -0.5 * (double)N * (log(2.0 * 3.141592653589793) + 2.0 * log_sigma);
  double mx = -INFINITY;
  for (long long i = threadIdx.x; i < M; i += blockDim.x) mx = fmax(mx, c - 0.5 * ss[i] / s2 + log_w[i]);
  // max over the CTA
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  mx = -INFINITY;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) mx = fmax(mx, red[q]);
  __syncthreads();
  double se = 0.0, gt = 0.0, gs = 0.0;
  if (mx > -INFINITY) {
    for (long long i = threadIdx.x; i < M; i += blockDim.x) {
      const double a = c - 0.5 * ss[i] / s2 + log_w[i];
      const double e = exp(a - mx);
      se += e;
      gt += e * ((ry[i] - ss[i]) / s2);   // r . (Phi w) / sigma^2
      gs += e * (ss[i] / s2 - (double)N);  // |r|^2 / sigma^2 - N
    }
  }
  se = cta_sum_d(se, red);
  gt = cta_sum_d(gt, red);
  gs = cta_sum_d(gs, red);
  if (threadIdx.x == 0) {
    out[0] = (mx > -INFINITY) ? mx + log(se) : -INFINITY;
    out[1] = gt / se;
    out[2] = gs / se;
  }
}

cudaError_t launch_lg_begin(const gbns_batch &b, const gbns_lg_bufs &lg, long long total_chains, cudaStream_t s) {
  if (total_chains <= 0) return cudaSuccess;
  k_lg_init<<<(unsigned)((total_chains + 127) / 128), 128, 0, s>>>(b, lg, total_chains);
  return cudaGetLastError();
}

cudaError_t launch_lg_step_kernel(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t s) {
  if (lg.total_chains <= 0) return cudaSuccess;
  // 8 chains (warps) per CTA; programmatic serialisation: may start while the previous
  // residual launch drains (the kernel waits for it before reading)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((lg.total_chains + 7) / 8));
  cfg.blockDim = dim3(256);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_lg_step, b, lg, (long long)lg.total_chains);
}

// One chain step; with the gradient options, the list of chains that ask for a gradient is
// reset before it and the gradient launch follows it.
cudaError_t launch_lg_chain_step(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t s) {
  const bool grads = b.gradient_guided || b.gradient_slice;
  cudaError_t e = cudaSuccess;
  if (grads && (e = cudaMemsetAsync(lg.grad_count, 0, sizeof(int), s)) != cudaSuccess) return e;
  if ((e = launch_lg_step_kernel(b, lg, s)) != cudaSuccess) return e;
  if (grads && lg.total_chains > 0) {
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const long long grid = lg.total_chains < 8LL * sms ? lg.total_chains : 8LL * sms;
    if (lg.pmax <= 32) k_lg_grad<32><<<(unsigned)grid, 256, 0, s>>>(b, lg);
    else k_lg_grad<64><<<(unsigned)grid, 256, 0, s>>>(b, lg);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t launch_lg_resid_cc(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t s) {
  if (lg.num_items > 0) {
    if (lg.pmax <= 32) k_lg_resid<32><<<lg.num_items, 256, 0, s>>>(b, lg);
    else k_lg_resid<64><<<lg.num_items, 256, 0, s>>>(b, lg);
  }
  return cudaGetLastError();
}

cudaError_t launch_lg_steps(const gbns_batch &b, const gbns_lg_bufs &lg, int steps, cudaStream_t s) {
  if (lg.use_tc) return launch_lg_steps_tc(b, lg, steps, s);
  for (int q = 0; q < steps; ++q) {
    cudaError_t e = launch_lg_chain_step(b, lg, s);
    if (e == cudaSuccess) e = launch_lg_resid_cc(b, lg, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t launch_adjoint(const double *U, const double *log_w, long long M, int P, const float *Phi, const float *y,
                           int N, double log_tau, double log_sigma, double *out, double *ss, double *ry,
                           cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(ss, 0, sizeof(double) * M, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ry, 0, sizeof(double) * M, s);
  if (e != cudaSuccess) return e;
  if (M > 0) {
    dim3 grid((unsigned)((M + 63) / 64), (unsigned)((N + 63) / 64));
    const float tau = (float)exp(log_tau);
    if (P <= 32) k_adj_resid<32><<<grid, 256, 0, s>>>(U, M, P, Phi, y, N, tau, ss, ry);
    else k_adj_resid<64><<<grid, 256, 0, s>>>(U, M, P, Phi, y, N, tau, ss, ry);
  }
  return launch_adjoint_reduce(log_w, M, N, log_sigma, ss, ry, out, s);
}

cudaError_t launch_adjoint_reduce(const double *log_w, long long M, int N, double log_sigma, const double *ss,
                                  const double *ry, double *out, cudaStream_t s) {
  k_adj_reduce<<<1, 1024, 0, s>>>(log_w, M, N, log_sigma, ss, ry, out);
  return cudaGetLastError();
}

}  // namespace gbns

namespace {
int lg_fail(int code, const char *msg) {
  gbns::record_error(msg);
  return code;
}
int lg_check(const gbns_batch *batch, const gbns_lg_bufs *lg) {
  if (!batch || !lg || batch->num_runs <= 0 || lg->total_chains < 0 || lg->pmax < 1 || lg->pmax > 64 || !lg->flags ||
      !lg->ss || !lg->W || !lg->u0 || !lg->dir || !lg->chains_left)
    return lg_fail(-1, "gbns_lg: bad arguments (1 <= pmax <= 64, chain buffers required)");
  if (lg->use_tc && (!lg->W_hi || !lg->W_lo || !lg->Phi_hi || !lg->Phi_lo || !lg->row_base || lg->total_rows < 1 ||
                     lg->num_items_tc < 0 || lg->num_ctas_tc < 0 || (lg->num_items_tc > 0 && !lg->items_tc) ||
                     !lg->tile_base || !lg->tile_pending || !lg->tc_done || lg->num_tiles < 0))
    return lg_fail(-1, "gbns_lg: use_tc needs W_hi, W_lo, Phi_hi, Phi_lo, row_base, items_tc and num_ctas_tc >= 0");
  if ((batch->gradient_guided || batch->gradient_slice) && (!lg->grad || !lg->grad_list || !lg->grad_count))
    return lg_fail(-1, "gbns_lg: the gradient options need grad, grad_list and grad_count");
  return 0;
}
}  // namespace

extern "C" {

int gbns_lg_shell_begin(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream) {
  int rc = lg_check(batch, lg);
  if (rc) return rc;
  cudaError_t e = gbns::launch_lg_begin(*batch, *lg, lg->total_chains, (cudaStream_t)stream);
  if (e != cudaSuccess) return lg_fail(-2, cudaGetErrorString(e));
  return 0;
}

// num_steps x (chain step + residual contraction); no host synchronisation.
int gbns_lg_steps(const gbns_batch *batch, const gbns_lg_bufs *lg, int num_steps, void *stream) {
  int rc = lg_check(batch, lg);
  if (rc) return rc;
  if (num_steps < 0) return lg_fail(-1, "gbns_lg_steps: negative step count");
  cudaError_t e = gbns::launch_lg_steps(*batch, *lg, num_steps, (cudaStream_t)stream);
  if (e != cudaSuccess) return lg_fail(-2, cudaGetErrorString(e));
  return 0;
}

// The two halves of one step, for callers that interleave their own work (e.g. timing events).
int gbns_lg_chain_step(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream) {
  int rc = lg_check(batch, lg);
  if (rc) return rc;
  cudaError_t e = gbns::launch_lg_chain_step(*batch, *lg, (cudaStream_t)stream);
  if (e != cudaSuccess) return lg_fail(-2, cudaGetErrorString(e));
  return 0;
}

int gbns_lg_residual(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream) {
  int rc = lg_check(batch, lg);
  if (rc) return rc;
  cudaError_t e = lg->use_tc ? gbns::launch_lg_steps_tc(*batch, *lg, -1, (cudaStream_t)stream)
                             : gbns::launch_lg_resid_cc(*batch, *lg, (cudaStream_t)stream);
  if (e != cudaSuccess) return lg_fail(-2, cudaGetErrorString(e));
  return 0;
}

int gbns_evidence_adjoint(const double *U_dev, const double *log_w_dev, long long M, int P, const float *Phi_dev,
                          const float *y_dev, int N, double log_tau, double log_sigma, double *out_dev,
                          double *ss_scratch_dev, double *ry_scratch_dev, void *stream) {
  if (M < 0 || P < 1 || P > 64 || N < 1 || !out_dev || (M > 0 && (!U_dev || !log_w_dev || !ss_scratch_dev ||
                                                                    !ry_scratch_dev)) || !Phi_dev || !y_dev)
    return lg_fail(-1, "gbns_evidence_adjoint: bad arguments (1 <= P <= 64)");
  cudaError_t e = gbns::launch_adjoint(U_dev, log_w_dev, M, P, Phi_dev, y_dev, N, log_tau, log_sigma, out_dev,
                                       ss_scratch_dev, ry_scratch_dev, (cudaStream_t)stream);
  if (e != cudaSuccess) return lg_fail(-2, cudaGetErrorString(e));
  return 0;
}

}  // extern "C"
