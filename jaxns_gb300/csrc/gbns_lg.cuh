// gbns_lg.cuh -- device helpers of the linear-Gaussian lock-step chains shared by the
// two-launch lock step (gbns_phiw.cu) and the fused shell kernel (gbns_phiw_tc.cu): the fp32
// pair representation of an FP64 U coordinate, the Normal prior quantile of a pair, the
// midpoint shrink factors, the run of a global chain index.
#pragma once
#include "gbns_device.cuh"

namespace gbns {

// fp32 pair <-> FP64
__device__ __forceinline__ void pair_from_double(double u, float &a, float &b) {
  a = (float)u;
  b = (float)(u - (double)a);
}

// a + b as an fp32 pair (TwoSum: exact for any magnitudes).
__device__ __forceinline__ void pair_add(float a, float s, float &hi, float &lo) {
  hi = a + s;
  const float bb = hi - a;
  lo = (a - (hi - bb)) + (s - bb);
}

// Standard-normal quantile of u = a + s (s may hold a whole proposal step), in fp32 with the
// offset from 1/2 and the tail mass formed exactly (AS 241 rational approximations,
// gbns_fmath.h): the pair is first renormalised to u = hi + lo (TwoSum), so hi lies in the
// same half of [0, 1] as u and 1 - hi is exact in the upper tail.
__device__ __forceinline__ float ndtri_pair(float a, float s) {
  float hi, lo;
  pair_add(a, s, hi, lo);
  const float q = (hi - 0.5f) + lo;  // u - 1/2
  if (fabsf(q) <= 0.425f) return gbns_fm_ndtri_center(q);
  if (q > 0.0f) return gbns_fm_ndtri_upper((1.0f - hi) - lo);
  return -gbns_fm_ndtri_upper(hi + lo);
}

__device__ __forceinline__ float prior_quantile_pair(int kind, float pa, float pb, float a, float s) {
  if (kind == GBNS_PRIOR_UNIFORM) return fmaf(pb, a, fmaf(pb, s, pa));
  return fmaf(pb, ndtri_pair(a, s), pa);
}

__device__ __forceinline__ int run_of_chain(const gbns_batch &b, long long g) {
  int lo = 0, hi = b.num_runs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (b.runs[mid].shell_off <= g) lo = mid; else hi = mid;
  }
  return lo;
}

// linspace(0.5, 1, S)[j] (the midpoint shrink factors, uni_slice_sampler.py:114-273).
__device__ __forceinline__ float lg_alpha(int j, int S) {
  if (S == 1) return 0.5f;
  if (j == S - 1) return 1.0f;
  const float step = (float)j / (float)(S - 1);
  return 0.5f * (1.0f - step) + step;
}

}  // namespace gbns
