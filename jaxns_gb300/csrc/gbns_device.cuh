// gbns_device.cuh -- device building blocks shared by the sm_103a kernels:
// threefry-2x32 counter RNG in jax.random's partitionable layout, the uniform/normal
// transforms, prior quantiles, likelihood families, warp scans and the FP64 evidence
// accumulator.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/gbns.h"
#include "gbns_fmath.h"

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

// Round-to-nearest-even conversion of a 64-bit unsigned integer to fp32 with 32-bit
// operations only (gbns_fmath.h).
__device__ __forceinline__ float u64_to_float_rn(uint64_t x) { return gbns_fm_u64_to_float(x); }

// jax.random.uniform(float64) in [0,1) from 64 bits: the top 52 bits M give M * 2^-52;
// rounded once to fp32.
__device__ __forceinline__ float uniform01(uint64_t b) {
  return u64_to_float_rn(b >> 12) * 2.220446049250313e-16f;  // 2^-52
}

// jax.random.normal(float64) = sqrt(2) erfinv(u), u = (4M + 1 - 2^53) 2^-53 (M = top 52
// bits): the standard normal quantile of p = (4M + 1) 2^-54 with |p - 1/2| and the tail mass
// formed exactly from the integer M (gbns_fmath.h), so the tails keep full relative precision.
__device__ __forceinline__ float normal_from_bits(uint64_t b) { return gbns_fm_normal_from_mantissa(b >> 12); }

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
// rewritten as prefix sums so that a whole CTA processes blockDim elements per step:
//   X_k  = X_{k-1} T_k,            X2_k = X2_{k-1} T2_k                 (FP64 log-space prefix sums)
//   dZ_k = X_{k-1} t_k mid_k,      Z_k  = Z_{k-1} + dZ_k
//   A_k  = ZX_k / X_k = A_{k-1} + X2_{k-1} tT_k mid_k / X_k              (an exclusive prefix sum)
//   Z2_k = Z2_{k-1} + 2 X_{k-1} A_{k-1} t_k mid_k + X2_{k-1} t2_k mid_k^2
//   dZ2_k = dZ2_{k-1} + X2_{k-1} t2_k mid_k^2
// Every term is held as a scaled sum q 2^e: an exact power of two from the FP64 log-value and
// an fp32-accurate mantissa, so no term loses relative precision however far it lies below
// the others; sums are FP64 mantissas rescaled exactly by powers of two.  Z, Z2 and dZ2 are
// accumulated per thread and reduced once at the end; log X, log X2 and A are CTA scans with
// carries between chunks.  Coefficients per n come from an FP64 table built on the host with
// the reference formulas.

struct ScaledSum {
  double q;
  int e;  // value = q * 2^e  (q == 0 means zero)
};

// 2^k for k <= 1023 (0 below the normal range: the terms it scales are negligible there)
__device__ __forceinline__ double pow2i(int k) {
  return k < -1022 ? 0.0 : __longlong_as_double((long long)(k + 1023) << 52);
}

__device__ __forceinline__ ScaledSum ss_zero() {
  ScaledSum s;
  s.q = 0.0;
  s.e = 0;
  return s;
}

// exp(lv) with an FP64-exact exponent (register initialisation)
__device__ __forceinline__ ScaledSum ss_from_log(double lv) {
  ScaledSum s;
  if (!(lv > -1e300)) { s.q = 0.0; s.e = 0; return s; }
  const double y = lv * GBNS_INV_LN2;
  const int e = (int)floor(y) + 1;
  s.q = exp2(y - (double)e);
  s.e = e;
  return s;
}

// exp(lv) as one term of a sum: exact power of two, mantissa in [1, 2) to fp32 precision
__device__ __forceinline__ ScaledSum ss_term(double lv) {
  ScaledSum s;
  if (!(lv > -1e300)) { s.q = 0.0; s.e = 0; return s; }
  const double y = lv * GBNS_INV_LN2;
  const double f = floor(y);
  s.q = (double)exp2f((float)(y - f));
  s.e = (int)f;
  return s;
}

__device__ __forceinline__ double ss_log(ScaledSum s) {
  if (!(s.q > 0.0)) return -INFINITY;
  return log(s.q) + (double)s.e * GBNS_LN2;
}

// a + b (commutative: the same bits either way round)
__device__ __forceinline__ ScaledSum ss_sum(ScaledSum a, ScaledSum b) {
  if (!(b.q > 0.0)) return a;
  if (!(a.q > 0.0)) return b;
  ScaledSum r;
  if (a.e >= b.e) {
    r.q = fma(b.q, pow2i(b.e - a.e), a.q);
    r.e = a.e;
  } else {
    r.q = fma(a.q, pow2i(a.e - b.e), b.q);
    r.e = b.e;
  }
  return r;
}

__device__ __forceinline__ ScaledSum shfl_up_ss(ScaledSum v, int o) {
  ScaledSum r;
  r.q = __shfl_up_sync(0xffffffffu, v.q, o);
  r.e = __shfl_up_sync(0xffffffffu, v.e, o);
  return r;
}

__device__ __forceinline__ ScaledSum shfl_xor_ss(ScaledSum v, int o) {
  ScaledSum r;
  r.q = __shfl_xor_sync(0xffffffffu, v.q, o);
  r.e = __shfl_xor_sync(0xffffffffu, v.e, o);
  return r;
}

struct EvScanSmem {
  double wa[32], wb[32];
  ScaledSum ws[32];
  ScaledSum red[3][32];
  double last_ldZ;
  float last_L;
};

// Inclusive CTA scan of two FP64 sums; every thread also gets the CTA totals.
__device__ __forceinline__ void cta_scan_d2(double &a, double &b, double &ta, double &tb, EvScanSmem &sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double a2 = __shfl_up_sync(0xffffffffu, a, o), b2 = __shfl_up_sync(0xffffffffu, b, o);
    if (lane >= o) {
      a += a2;
      b += b2;
    }
  }
  if (lane == 31) {
    sm.wa[w] = a;
    sm.wb[w] = b;
  }
  __syncthreads();
  if (w == 0) {
    double x = lane < nw ? sm.wa[lane] : 0.0, y = lane < nw ? sm.wb[lane] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double x2 = __shfl_up_sync(0xffffffffu, x, o), y2 = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) {
        x += x2;
        y += y2;
      }
    }
    if (lane < nw) {
      sm.wa[lane] = x;
      sm.wb[lane] = y;
    }
  }
  __syncthreads();
  if (w > 0) {
    a += sm.wa[w - 1];
    b += sm.wb[w - 1];
  }
  ta = sm.wa[nw - 1];
  tb = sm.wb[nw - 1];
  __syncthreads();
}

// CTA scan of scaled sums: inclusive and exclusive prefix of each thread's value, and the total.
__device__ __forceinline__ void cta_scan_ss(ScaledSum v, ScaledSum &incl, ScaledSum &excl, ScaledSum &tot,
                                            EvScanSmem &sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const ScaledSum u = shfl_up_ss(v, o);
    if (lane >= o) v = ss_sum(u, v);
  }
  ScaledSum wex = shfl_up_ss(v, 1);
  if (lane == 31) sm.ws[w] = v;
  __syncthreads();
  if (w == 0) {
    ScaledSum x = lane < nw ? sm.ws[lane] : ss_zero();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const ScaledSum u = shfl_up_ss(x, o);
      if (lane >= o) x = ss_sum(u, x);
    }
    if (lane < nw) sm.ws[lane] = x;
  }
  __syncthreads();
  const ScaledSum pw = w > 0 ? sm.ws[w - 1] : ss_zero();
  incl = ss_sum(pw, v);
  excl = lane == 0 ? pw : ss_sum(pw, wex);
  tot = sm.ws[nw - 1];
  __syncthreads();
}

struct EvAcc {
  double lX, lX2;
  ScaledSum Z, A, Z2, dZ2;
  double ldZ_last;
  float Lprev;
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

// Process elements [0, M) of log-likelihoods L (fp32) with live-point counts given by
// nmode: nconst > 0 -> n_k = nconst; ndesc > 0 -> n_k = ndesc - k; else n_k = narr[k].
// Called by every thread of the CTA (blockDim a multiple of 32).  Optional per-element
// outputs (FP64 logs): log X, log dZ and, with OUT_LZ, the running log Z.  L values are
// relative to Loff (added back in FP64); Lidx, when given, gathers L[Lidx[k]].
template <bool OUT_LZ>
__device__ void evidence_scan_cta(EvAcc &acc, const float *__restrict__ L, long long M, int nconst, int ndesc,
                                  const int *__restrict__ narr, const double *__restrict__ ncoef, int nmax,
                                  double *__restrict__ out_lX, double *__restrict__ out_ldZ,
                                  double *__restrict__ out_lZ, double Loff, const int *__restrict__ Lidx,
                                  EvScanSmem &sm) {
  const int tid = threadIdx.x, T = blockDim.x;
  ScaledSum pZ = ss_zero(), pZ2 = ss_zero(), pdZ2 = ss_zero();  // this thread's partial sums
  for (long long base = 0; base < M; base += T) {
    const long long k = base + tid;
    const bool valid = k < M;
    const float Lk = valid ? L[Lidx ? Lidx[k] : k] : 0.0f;
    const float Lm1 = !valid ? 0.0f : (k == 0 ? acc.Lprev : L[Lidx ? Lidx[k - 1] : k - 1]);
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
    double sT = lT, sT2 = lT2, totT, totT2;
    cta_scan_d2(sT, sT2, totT, totT2, sm);
    const double lX_prev = acc.lX + (sT - lT), lX2_prev = acc.lX2 + (sT2 - lT2);
    const double lX_cur = acc.lX + sT;
    const double lmid = valid ? log_midpoint(Lk, Lm1) + Loff : -INFINITY;
    const double v_dZ = valid ? (lX_prev + lt) + lmid : -INFINITY;
    const double v_c = valid ? ((lX2_prev + ltT) + lmid) - lX_cur : -INFINITY;
    const double v_t2 = valid ? (lX2_prev + lt2) + 2.0 * lmid : -INFINITY;
    // A_{k-1} = A_0 + the exclusive prefix of c
    ScaledSum cin, cex, ctot;
    cta_scan_ss(ss_term(v_c), cin, cex, ctot, sm);
    const ScaledSum Ap = ss_sum(acc.A, cex);
    const double lA_prev = (Ap.q > 0.0) ? (double)logf((float)Ap.q) + (double)Ap.e * GBNS_LN2 : -INFINITY;
    const double v_t1 = valid ? ((GBNS_LN2 + lX_prev + lt) + lmid) + lA_prev : -INFINITY;
    if (valid) {
      if (out_lX) out_lX[k] = lX_cur;
      if (out_ldZ) out_ldZ[k] = v_dZ;
    }
    const ScaledSum tdZ = ss_term(v_dZ), tt2 = ss_term(v_t2);
    if (OUT_LZ) {
      ScaledSum zin, zex, ztot;
      cta_scan_ss(tdZ, zin, zex, ztot, sm);
      if (valid && out_lZ) out_lZ[k] = ss_log(ss_sum(acc.Z, zin));
      acc.Z = ss_sum(acc.Z, ztot);
    } else {
      pZ = ss_sum(pZ, tdZ);
    }
    pZ2 = ss_sum(pZ2, ss_sum(ss_term(v_t1), tt2));
    pdZ2 = ss_sum(pdZ2, tt2);
    // carries into the next chunk (the same on every thread)
    const long long last = (M - base < T ? M - base : T) - 1;
    acc.lX += totT;
    acc.lX2 += totT2;
    acc.A = ss_sum(acc.A, ctot);
    if (tid == last) {
      sm.last_ldZ = v_dZ;
      sm.last_L = Lk;
    }
    __syncthreads();
    acc.ldZ_last = sm.last_ldZ;
    acc.Lprev = sm.last_L;
    __syncthreads();
  }
  // CTA reduction of the partial sums (butterfly in each warp, then across warps)
  const int lane = tid & 31, w = tid >> 5, nw = T >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pZ = ss_sum(pZ, shfl_xor_ss(pZ, o));
    pZ2 = ss_sum(pZ2, shfl_xor_ss(pZ2, o));
    pdZ2 = ss_sum(pdZ2, shfl_xor_ss(pdZ2, o));
  }
  if (lane == 0) {
    sm.red[0][w] = pZ;
    sm.red[1][w] = pZ2;
    sm.red[2][w] = pdZ2;
  }
  __syncthreads();
  ScaledSum rZ = ss_zero(), rZ2 = ss_zero(), rdZ2 = ss_zero();
  for (int q = 0; q < nw; ++q) {
    rZ = ss_sum(rZ, sm.red[0][q]);
    rZ2 = ss_sum(rZ2, sm.red[1][q]);
    rdZ2 = ss_sum(rdZ2, sm.red[2][q]);
  }
  __syncthreads();
  acc.Z = ss_sum(acc.Z, rZ);
  acc.Z2 = ss_sum(acc.Z2, rZ2);
  acc.dZ2 = ss_sum(acc.dZ2, rdZ2);
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
// offset from 1/2 and the tail mass are formed in FP64 and rounded once (gbns_fmath.h), so u
// within 1e-12 of 0 or 1 still maps to its own quantile.
__device__ __forceinline__ float ndtri_from_double(double u) { return gbns_fm_ndtri_d(u); }

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
  return fmaf(b, gbns_fm_ndtri(u), a);
}

// Prior quantile x(u) and its slope dx/du (Uniform: b; Normal: b sqrt(2 pi) exp(z^2 / 2)),
// for U-space gradients of log L.
__device__ __forceinline__ void prior_quantile_slope(int kind, float a, float b, float u, float &x, float &dxdu) {
  if (kind == GBNS_PRIOR_UNIFORM) {
    x = fmaf(b, u, a);
    dxdu = b;
  } else {
    const float z = gbns_fm_ndtri(u);
    x = fmaf(b, z, a);
    dxdu = b * 2.5066282746310002f * gbns_fm_exp(0.5f * z * z);
  }
}

// The same of an FP64 u (the linear-Gaussian family's U space).
__device__ __forceinline__ float prior_quantile_d(int kind, float a, float b, double u) {
  if (kind == GBNS_PRIOR_UNIFORM) return (float)((double)a + (double)b * u);
  return fmaf(b, ndtri_from_double(u), a);
}

}  // namespace gbns
