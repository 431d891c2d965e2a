// gbns_device.cuh -- device building blocks shared by the sm_103a kernels:
// threefry-2x32 counter RNG in jax.random's partitionable layout, the uniform/normal
// transforms, prior quantiles, likelihood families, warp scans and the FP64 evidence
// accumulator.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/gbns.h"

#define GBNS_LN2 0.69314718055994530942
#define GBNS_INV_LN2 1.44269504088896340736
#define GBNS_SQRT2F 1.41421356237309505f
#define GBNS_LOG2PI 1.83787706640934548356

namespace gbns {

// ------------------------------------------------------------------ RNG ------

struct Key {
  uint32_t k0, k1;
};

// Threefry-2x32, 20 rounds (Salmon et al. SC'11), the cipher behind jax.random.
__host__ __device__ __forceinline__ void threefry2x32(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1,
                                                      uint32_t &o0, uint32_t &o1) {
  const uint32_t k2 = k0 ^ k1 ^ 0x1BD11BDAu;
  uint32_t x0 = c0 + k0, x1 = c1 + k1;
#define GBNS_R(r)                         \
  x0 += x1;                               \
  x1 = (x1 << (r)) | (x1 >> (32 - (r)));  \
  x1 ^= x0;
  GBNS_R(13) GBNS_R(15) GBNS_R(26) GBNS_R(6)
  x0 += k1; x1 += k2 + 1u;
  GBNS_R(17) GBNS_R(29) GBNS_R(16) GBNS_R(24)
  x0 += k2; x1 += k0 + 2u;
  GBNS_R(13) GBNS_R(15) GBNS_R(26) GBNS_R(6)
  x0 += k0; x1 += k1 + 3u;
  GBNS_R(17) GBNS_R(29) GBNS_R(16) GBNS_R(24)
  x0 += k1; x1 += k2 + 4u;
  GBNS_R(13) GBNS_R(15) GBNS_R(26) GBNS_R(6)
  x0 += k2; x1 += k0 + 5u;
#undef GBNS_R
  o0 = x0;
  o1 = x1;
}

// jax.random.split(key, n)[i] under jax_threefry_partitionable=True.
__host__ __device__ __forceinline__ Key fold(Key k, uint32_t i) {
  Key r;
  threefry2x32(k.k0, k.k1, 0u, i, r.k0, r.k1);
  return r;
}

// 64 random bits of element i (partitionable layout: hi word << 32 | lo word).
__device__ __forceinline__ uint64_t bits64(Key k, uint32_t i) {
  uint32_t a, b;
  threefry2x32(k.k0, k.k1, 0u, i, a, b);
  return ((uint64_t)a << 32) | (uint64_t)b;
}

// Round-to-nearest-even conversion of a 64-bit unsigned integer to fp32 using 32-bit
// operations only (a native 64-bit conversion runs on the FP64 pipe, which is scarce on
// GB300): normalise, keep the top 32 bits with a sticky bit for the rest, convert, rescale.
__device__ __forceinline__ float u64_to_float_rn(uint64_t x) {
  if (x == 0ull) return 0.0f;
  const int nz = __clzll(x);
  const uint64_t y = x << nz;
  const uint32_t top = (uint32_t)(y >> 32) | ((uint32_t)y != 0u ? 1u : 0u);
  const float f = __uint2float_rn(top);                       // exact scale 2^(32 - nz) follows
  return f * __int_as_float((127 + 32 - nz) << 23);           // 32 - nz in [-31, 32]
}

// jax.random.uniform(float64) in [0,1) from 64 bits: the top 52 bits M give M * 2^-52;
// rounded once to fp32.
__device__ __forceinline__ float uniform01(uint64_t b) {
  return u64_to_float_rn(b >> 12) * 2.220446049250313e-16f;  // 2^-52
}

// jax.random.normal(float64) = sqrt(2) * erfinv(u) with u = 2f - 1 + 2^-53, f = M * 2^-52
// (M = top 52 bits), i.e. u = (4M + 1 - 2^53) * 2^-53 exactly.  Evaluated as
// +-sqrt(2) * erfcinv(y) with y = 1 -+ u formed exactly from the integer M, so the tails keep
// full relative precision in fp32.
__device__ __forceinline__ float normal_from_bits(uint64_t b) {
  const uint64_t M = b >> 12;
  if (M >= (1ull << 51)) {
    const uint64_t q = (1ull << 54) - 4ull * M - 1ull;  // (1 - u) * 2^53
    return GBNS_SQRT2F * erfcinvf(u64_to_float_rn(q) * 1.1102230246251565e-16f);
  } else {
    const uint64_t q = 4ull * M + 1ull;  // (1 + u) * 2^53
    return -GBNS_SQRT2F * erfcinvf(u64_to_float_rn(q) * 1.1102230246251565e-16f);
  }
}

// ------------------------------------------------------------ log space ------

__device__ __forceinline__ double lae(double a, double b) {  // jnp.logaddexp
  const double amax = fmax(a, b);
  const double d = a - b;
  if (isnan(d)) return a + b;
  return amax + log1p(exp(-fabs(d)));
}

// ln(0.5) + logaddexp(a, b) for fp32 log-likelihoods, returned as FP64: the max is exact,
// the small correction term is evaluated in fp32.
__device__ __forceinline__ double log_midpoint(float a, float b) {
  const float m = fmaxf(a, b);
  const float d = a - b;
  if (isnan(d)) return (double)a + (double)b - GBNS_LN2;  // both -inf (or +inf)
  return (double)m + (double)(log1pf(__expf(-fabsf(d)))) - GBNS_LN2;
}

// float -> uint32 key with jnp.sort's total order: -0 == +0, NaN after +inf.
__device__ __forceinline__ uint32_t ordered_key(float x) {
  if (x != x) return 0xFFC00000u;
  if (x == 0.0f) x = 0.0f;
  uint32_t u = __float_as_uint(x);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ------------------------------------------------------------- warp scans ----

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ------------------------------------------------------- CTA reductions ----

template <typename T>
__device__ T cta_sum(T v, T *red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    T x = (l < (int)(blockDim.x >> 5)) ? red[l] : T(0);
    x = warp_sum(x);
    if (l == 0) red[0] = x;
  }
  __syncthreads();
  const T r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ long long cta_sum_ll(long long v, long long *red) { return cta_sum(v, red); }
__device__ __forceinline__ double cta_sum_d(double v, double *red) { return cta_sum(v, red); }

__device__ __forceinline__ float cta_max_f(float v, float *red) {
  v = warp_maxf(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  float r = -INFINITY;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r = fmaxf(r, red[q]);
  __syncthreads();
  return r;
}

__device__ __forceinline__ int cta_and(int v, int *red) {
  v = __all_sync(0xffffffffu, v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  int r = 1;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r &= red[q];
  __syncthreads();
  return r;
}

// ----------------------------------------------------- FP64 evidence scan ----
//
// The recurrence of _update_evidence_calc_op (internals/shrinkage_statistics.py:43-94),
// rewritten so that 32 elements are processed per warp step:
//   X_k  = X_{k-1} T_k,            X2_k = X2_{k-1} T2_k                 (FP64 log-space sums)
//   dZ_k = X_{k-1} t_k mid_k,      Z_k  = Z_{k-1} + dZ_k
//   A_k  = ZX_k / X_k = A_{k-1} + X2_{k-1} tT_k mid_k / X_k              (plain sum)
//   Z2_k = Z2_{k-1} + 2 X_{k-1} A_{k-1} t_k mid_k + X2_{k-1} t2_k mid_k^2
//   dZ2_k = dZ2_{k-1} + X2_{k-1} t2_k mid_k^2
// Sums are FP64 mantissas with an integer power-of-two exponent (rescaled exactly with
// ldexp); each term is exp2 of an FP64 log-value offset by the chunk maximum, evaluated in
// fp32 (the log-likelihoods are fp32).  Coefficients per n come from an FP64 table built
// on the host with the reference formulas.

struct ScaledSum {
  double q;
  int e;  // value = q * 2^e  (q == 0 means zero)
};

__device__ __forceinline__ ScaledSum ss_from_log(double lv) {
  ScaledSum s;
  if (!(lv > -1e300)) { s.q = 0.0; s.e = 0; return s; }
  const double y = lv * GBNS_INV_LN2;
  const int e = (int)floor(y) + 1;
  s.q = exp2(y - (double)e);
  s.e = e;
  return s;
}

__device__ __forceinline__ double ss_log(ScaledSum s) {
  if (!(s.q > 0.0)) return -INFINITY;
  return log(s.q) + (double)s.e * GBNS_LN2;
}

__device__ __forceinline__ void ss_add(ScaledSum &acc, double q, int e) {
  if (!(q > 0.0)) return;
  if (!(acc.q > 0.0)) { acc.q = q; acc.e = e; return; }
  if (e > acc.e) {
    acc.q = ldexp(acc.q, acc.e - e) + q;
    acc.e = e;
  } else {
    acc.q += ldexp(q, e - acc.e);
  }
}

struct EvAcc {
  double lX, lX2;
  ScaledSum Z, A, Z2, dZ2;
  double ldZ_last;
  float Lprev;
  bool lprev_valid;
};

__device__ __forceinline__ EvAcc evacc_from(const gbns_evcalc &e) {
  EvAcc a;
  a.lX = e.log_X_mean;
  a.lX2 = e.log_X2_mean;
  a.Z = ss_from_log(e.log_Z_mean);
  a.A = ss_from_log(e.log_ZX_mean - e.log_X_mean);
  a.Z2 = ss_from_log(e.log_Z2_mean);
  a.dZ2 = ss_from_log(e.log_dZ2_mean);
  a.ldZ_last = e.log_dZ_mean;
  a.Lprev = (float)e.log_L;
  return a;
}

// As evacc_from for a register whose log_L is absolute while the scanned values are
// relative to Loff.
__device__ __forceinline__ EvAcc evacc_from_shifted(const gbns_evcalc &e, double Loff) {
  EvAcc a = evacc_from(e);
  a.Lprev = (float)(e.log_L - Loff);
  return a;
}

__device__ __forceinline__ gbns_evcalc evacc_to(const EvAcc &a, double log_L_last) {
  gbns_evcalc e;
  e.log_L = log_L_last;
  e.log_X_mean = a.lX;
  e.log_X2_mean = a.lX2;
  e.log_Z_mean = ss_log(a.Z);
  e.log_ZX_mean = a.lX + ss_log(a.A);
  e.log_Z2_mean = ss_log(a.Z2);
  e.log_dZ_mean = a.ldZ_last;
  e.log_dZ2_mean = ss_log(a.dZ2);
  return e;
}

// The n-only coefficients of _update_evidence_calc_op (shrinkage_statistics.py:55-73) for a
// count beyond the host-built table.
__device__ __forceinline__ void ncoef_compute(double n, double *c) {
  const double lnn = log(n), lnn1 = log(n + 1.0), lnn2 = log(n + 2.0);
  c[0] = -lae(0.0, -lnn);
  c[1] = -lnn1;
  c[2] = -lae(0.0, GBNS_LN2 - lnn);
  c[3] = GBNS_LN2 - lnn1 - lnn2;
  c[4] = -lae(0.0, -lnn) - lnn2;
}

// Chunk-sum helper: every lane holds one FP64 log-term (or -inf); returns the warp sum as
// (q, e) on all lanes.
__device__ __forceinline__ void warp_logsum(double v, double &q, int &e) {
  const float vf = (float)(v * GBNS_INV_LN2);
  const float mx = warp_maxf(vf);
  if (!(mx > -1e30f)) { q = 0.0; e = 0; return; }
  e = (int)ceilf(mx) + 1;
  const float t = (v > -1e300) ? exp2f((float)(v * GBNS_INV_LN2 - (double)e)) : 0.0f;
  q = warp_sum((double)t);
}

// Inclusive warp scan of sum(exp(v)) as (q, e), value = q * 2^e: every lane keeps its own
// power-of-two exponent so prefixes far below the chunk maximum keep their precision.
__device__ __forceinline__ void warp_lse_incl_scan(double v, double &q, int &e) {
  const int lane = threadIdx.x & 31;
  if (v > -1e300) {
    const double y = v * GBNS_INV_LN2;
    e = (int)floor(y);
    q = (double)exp2f((float)(y - (double)e));
  } else {
    q = 0.0;
    e = 0;
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double q2 = __shfl_up_sync(0xffffffffu, q, o);
    const int e2 = __shfl_up_sync(0xffffffffu, e, o);
    if (lane >= o && q2 > 0.0) {
      if (!(q > 0.0)) {
        q = q2;
        e = e2;
      } else if (e2 > e) {
        q = ldexp(q, e - e2) + q2;
        e = e2;
      } else {
        q += ldexp(q2, e2 - e);
      }
    }
  }
}

// Process elements [0, M) of log-likelihoods L (fp32) with live-point counts given by
// nmode: nconst > 0 -> n_k = nconst; ndesc > 0 -> n_k = ndesc - k; else n_k = narr[k].
// Must be called by all 32 lanes of one warp.  Optional per-element outputs (FP64 logs).
// L values are relative to Loff (added back in FP64); Lidx, when given, gathers L[Lidx[k]].
__device__ inline void evidence_scan_warp(EvAcc &acc, const float *__restrict__ L, long long M, int nconst, int ndesc,
                                   const int *__restrict__ narr, const double *__restrict__ ncoef, int nmax,
                                   double *__restrict__ out_lX, double *__restrict__ out_ldZ,
                                   double *__restrict__ out_lZ, double Loff = 0.0,
                                   const int *__restrict__ Lidx = nullptr) {
  const int lane = threadIdx.x & 31;
  for (long long base = 0; base < M; base += 32) {
    const long long k = base + lane;
    const bool valid = k < M;
    const float Lk = valid ? L[Lidx ? Lidx[k] : k] : 0.0f;
    float Lm1 = __shfl_up_sync(0xffffffffu, Lk, 1);
    if (lane == 0) Lm1 = acc.Lprev;
    int nk = 1;
    if (valid) nk = nconst > 0 ? nconst : (ndesc > 0 ? (int)(ndesc - k) : narr[k]);
    nk = nk < 0 ? 0 : nk;
    double cf[5];
    if (nk <= nmax) {
      const double *c = ncoef + (size_t)nk * 8;
      cf[0] = c[0]; cf[1] = c[1]; cf[2] = c[2]; cf[3] = c[3]; cf[4] = c[4];
    } else {
      ncoef_compute((double)nk, cf);
    }
    const double lT = valid ? cf[0] : 0.0, lt = cf[1], lT2 = valid ? cf[2] : 0.0, lt2 = cf[3], ltT = cf[4];
    // exclusive prefix of log T and log T2
    const double sT = warp_incl_scan(lT), sT2 = warp_incl_scan(lT2);
    const double lX_prev = acc.lX + (sT - lT), lX2_prev = acc.lX2 + (sT2 - lT2);
    const double lX_cur = acc.lX + sT;
    const double lmid = valid ? log_midpoint(Lk, Lm1) + Loff : -INFINITY;
    const double v_dZ = valid ? (lX_prev + lt) + lmid : -INFINITY;
    const double v_c = valid ? ((lX2_prev + ltT) + lmid) - lX_cur : -INFINITY;
    const double v_t2 = valid ? (lX2_prev + lt2) + 2.0 * lmid : -INFINITY;
    // inclusive prefix of c in a chunk-local exponent
    const float vcf = (float)(v_c * GBNS_INV_LN2);
    const float mc = warp_maxf(vcf);
    double cincl = 0.0, cterm = 0.0;
    int ec = 0;
    if (mc > -1e30f) {
      ec = (int)ceilf(mc) + 1;
      cterm = (v_c > -1e300) ? (double)exp2f((float)(v_c * GBNS_INV_LN2 - (double)ec)) : 0.0;
      cincl = warp_incl_scan(cterm);
    }
    // log A_{k-1} = log(A0 + cexcl)
    double lA_prev;
    {
      const double cex = cincl - cterm;
      ScaledSum a = acc.A;
      if (cex > 0.0) ss_add(a, cex, ec);
      lA_prev = (a.q > 0.0) ? (double)logf((float)a.q) + (double)a.e * GBNS_LN2 : -INFINITY;
    }
    const double v_t1 = valid ? ((GBNS_LN2 + lX_prev + lt) + lmid) + lA_prev : -INFINITY;
    // per-element outputs
    if (valid) {
      if (out_lX) out_lX[k] = lX_cur;
      if (out_ldZ) out_ldZ[k] = v_dZ;
    }
    // chunk sums
    double q;
    int e;
    warp_logsum(v_dZ, q, e);
    if (out_lZ) {
      // running log Z per element (inclusive)
      double incl;
      int ee;
      warp_lse_incl_scan(v_dZ, incl, ee);
      ScaledSum z = acc.Z;
      if (incl > 0.0) ss_add(z, incl, ee);
      if (valid) out_lZ[k] = ss_log(z);
    }
    ss_add(acc.Z, q, e);
    double q1, q2;
    int e1, e2;
    warp_logsum(v_t1, q1, e1);
    warp_logsum(v_t2, q2, e2);
    ss_add(acc.Z2, q1, e1);
    ss_add(acc.Z2, q2, e2);
    ss_add(acc.dZ2, q2, e2);
    // carry
    const int last = (int)((M - base) < 32 ? (M - base - 1) : 31);
    const double cin_last = __shfl_sync(0xffffffffu, cincl, 31);
    if (cin_last > 0.0) ss_add(acc.A, cin_last, ec);
    acc.lX = __shfl_sync(0xffffffffu, lX_cur, last);
    acc.lX2 = acc.lX2 + __shfl_sync(0xffffffffu, sT2, last);
    acc.ldZ_last = __shfl_sync(0xffffffffu, v_dZ, last);
    acc.Lprev = __shfl_sync(0xffffffffu, Lk, last);
  }
}

// ------------------------------------------------------------- likelihood ----

// Programmatic dependent launch: let the next kernel in the stream start its prologue, and
// wait for the previous kernel's grid (and its memory) before reading what it wrote.  Both are
// no-ops for a kernel launched without the programmatic-serialisation attribute.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// x = hi + lo with hi and lo both TF32 (round to nearest, ties away): the operand split of
// the 3xTF32 tensor-core contraction (hi*hi + hi*lo + lo*hi).
__device__ __forceinline__ void tf32_split(float x, float &hi, float &lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(x - hi));
  lo = __uint_as_float(l);
}

// Standard-normal quantile of an FP64 u, evaluated in fp32 without losing the tails: the
// argument handed to the fp32 inverse is formed exactly in FP64 (2u - 1 near the centre,
// 2u or 2 - 2u in the tails), so u within 1e-12 of 0 or 1 still maps to its own quantile.
__device__ __forceinline__ float ndtri_from_double(double u) {
  const double z = 2.0 * u - 1.0;
  if (fabs(z) < 0.5) return GBNS_SQRT2F * erfinvf((float)z);
  return u < 0.5 ? -GBNS_SQRT2F * erfcinvf((float)(2.0 * u)) : GBNS_SQRT2F * erfcinvf((float)(2.0 - 2.0 * u));
}

// jax.random.uniform in FP64: the top 52 bits as the mantissa of [1, 2), minus 1.
__device__ __forceinline__ double uniform01_d(uint64_t bits) {
  return (double)(bits >> 12) * 2.220446049250313e-16;
}

// Per-run parameter views (fparams layout written by the host, see engine.py):
//  MVN:     [mu(D), Linv(D*D row-major, lower), c0]   c0 = -sum log L_ii - D/2 log 2pi
//  SHELLS:  [c1(D), c2(D), R, w, norm]                 norm = log sqrt(2 pi w^2)
//  LINGAUSS:[Phi(N*D row-major), y(N), sigma]
// Prior quantiles: Uniform a + b u (b = high - low), Normal a + b ndtri(u) (b = scale).
__device__ __forceinline__ float prior_quantile(int kind, float a, float b, float u) {
  if (kind == GBNS_PRIOR_UNIFORM) return fmaf(b, u, a);
  return fmaf(b, GBNS_SQRT2F * erfinvf(fmaf(2.0f, u, -1.0f)), a);
}

// Prior quantile x(u) and its slope dx/du (Uniform: b; Normal: b sqrt(2 pi) exp(z^2 / 2)),
// for U-space gradients of log L.
__device__ __forceinline__ void prior_quantile_slope(int kind, float a, float b, float u, float &x, float &dxdu) {
  if (kind == GBNS_PRIOR_UNIFORM) {
    x = fmaf(b, u, a);
    dxdu = b;
  } else {
    const float z = GBNS_SQRT2F * erfinvf(fmaf(2.0f, u, -1.0f));
    x = fmaf(b, z, a);
    dxdu = b * 2.5066282746310002f * __expf(0.5f * z * z);
  }
}

// The same of an FP64 u (the linear-Gaussian family's U space).
__device__ __forceinline__ float prior_quantile_d(int kind, float a, float b, double u) {
  if (kind == GBNS_PRIOR_UNIFORM) return (float)((double)a + (double)b * u);
  return fmaf(b, ndtri_from_double(u), a);
}

}  // namespace gbns
