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
// Every term is held as a scaled sum q 2^e: an exact power of two from the log-value and an
// fp32-accurate mantissa, so no term loses relative precision however far it lies below the
// others.  Inside a chunk of blockDim elements the terms and their sums are fp32 pairs (FS,
// below); the accumulators carried from chunk to chunk are FP64 mantissas (ScaledSum), both
// rescaled exactly by powers of two.  Z, Z2 and dZ2 are accumulated per thread and reduced
// once at the end; log X and log X2 (FP64) and A are CTA scans with carries between chunks.
// Coefficients per n come from an FP64 table built on the host with the reference formulas.

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

struct EvScanSmem {
  double carry_lX, carry_lX2, fin_lX, fin_lX2;
  ScaledSum fin[4];  // A, Z, Z2, dZ2 after the scan
  double last_ldZ;
  float last_L;
};

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

// ---- fp32-pair scaled sums.  GB300 runs FP64 at about 1/64 of the FP32 rate, so inside a
// scan only the log-X prefix (which must stay within 1e-12 of the reference's FP64 values) is
// FP64; every exponential term and every sum of terms is an fp32 pair (h + l) 2^e: TwoSum
// additions (relative error a few units of 2^-48), exponents aligned by exact powers of two.
// The terms themselves carry fp32 mantissas (exp2f of a pair-accurate fraction), as the FP64
// scaled sums do.  Chunk totals are folded into the FP64 accumulators once per chunk.
struct FS {
  float h, l;
  int e;  // value = (h + l) 2^e, h == 0 means zero
};

__device__ __forceinline__ FS fs_zero() {
  FS s;
  s.h = 0.0f;
  s.l = 0.0f;
  s.e = 0;
  return s;
}

__device__ __forceinline__ void pair_sum2(float ah, float al, float bh, float bl, float &h, float &l) {
  const float s = ah + bh;
  const float bb = s - ah;
  const float err = (ah - (s - bb)) + (bh - bb);
  const float lo = (al + bl) + err;
  h = s + lo;
  l = lo - (h - s);
}

// an FP64 value as an fp32 pair
__device__ __forceinline__ void pair_of(double x, float &h, float &l) {
  h = __double2float_rn(x);
  l = (isinf(h) || isnan(h)) ? 0.0f : __double2float_rn(x - (double)h);
}

// h + l (an fp32 pair with |l| <= ulp(h) / 2, as pair_sum2 leaves it) as an FP64 value,
// built with integer operations only (GB300 issues FP64 at about 1/64 of the FP32 rate): h's
// significand widened to 53 bits plus l's significand aligned to it (bits below 2^-52 of h
// truncated), renormalised by at most one bit.  Zero, infinities and NaN pass through exactly;
// a subnormal h (not met by log-space values) takes the FP64 conversion.
__device__ __forceinline__ double pair_to_double(float h, float l) {
  const uint32_t hb = __float_as_uint(h);
  const uint32_t eh = (hb >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(hb >> 31) << 63;
  if (eh == 0xffu)
    return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull |
                                            ((unsigned long long)(hb & 0x7fffffu) << 29)));
  if (eh == 0u) return (hb & 0x7fffffffu) == 0u ? __longlong_as_double((long long)sign) : (double)h + (double)l;
  unsigned long long sig = (unsigned long long)((hb & 0x7fffffu) | 0x800000u) << 29;  // units of 2^(e - 52)
  int e = (int)eh - 127;
  const uint32_t lb = __float_as_uint(l);
  const uint32_t el = (lb >> 23) & 0xffu;
  if (el != 0u && el != 0xffu) {
    const unsigned long long ml = (lb & 0x7fffffu) | 0x800000u;
    const int sh = (int)el - 127 - e + 29;  // l = ml 2^(el - 150) in units of 2^(e - 52)
    const unsigned long long add = sh >= 0 ? (ml << (sh < 40 ? sh : 40)) : (sh > -40 ? (ml >> -sh) : 0ull);
    sig = ((lb ^ hb) >> 31) ? sig - add : sig + add;
    if (sig >= (1ull << 53)) {
      sig >>= 1;
      e += 1;
    } else if (sig < (1ull << 52)) {
      sig <<= 1;
      e -= 1;
    }
  }
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 1023) << 52) | (sig & 0xfffffffffffffull)));
}

// exp(vh + vl): an exact power of two times exp2f of the fraction (vh + vl) / ln 2 - e
__device__ __forceinline__ FS fs_term(float vh, float vl) {
  if (!(vh > -INFINITY) || !(vh < INFINITY)) return fs_zero();  // -inf, +inf or NaN: no term
  const float c_hi = 1.44269502162933349609375f, c_lo = 1.925963033500011079e-8f;  // 1/ln 2 as a pair
  const float p = vh * c_hi;
  const float pe = fmaf(vh, c_hi, -p) + fmaf(vh, c_lo, vl * c_hi);
  const float f = floorf(p);
  FS s;
  s.h = exp2f((p - f) + pe);
  s.l = 0.0f;
  s.e = (int)f;
  return s;
}

// a + b (commutative: the operand with the larger exponent is always the first)
__device__ __forceinline__ FS fs_sum(FS a, FS b) {
  if (!(b.h > 0.0f)) return a;
  if (!(a.h > 0.0f)) return b;
  if (a.e < b.e) {
    const FS t = a;
    a = b;
    b = t;
  }
  const int k = b.e - a.e;  // <= 0
  if (k < -100) return a;   // below 2^-100 of a: nothing left at pair precision
  const float sc = __int_as_float((k + 127) << 23);
  FS r;
  pair_sum2(a.h, a.l, b.h * sc, b.l * sc, r.h, r.l);
  r.e = a.e;
  return r;
}

// a * f for a finite f >= 0: f's exponent moves into e, its significand m in [1, 2) multiplies
// the pair (TwoProd by FMA); a subnormal or zero f gives zero
__device__ __forceinline__ FS fs_scale(FS a, float f) {
  const uint32_t fb = __float_as_uint(f);
  if (!(a.h > 0.0f) || !(f < INFINITY) || (fb >> 23) == 0u || (fb >> 31)) return fs_zero();
  const float m = __uint_as_float((fb & 0x7fffffu) | 0x3f800000u);
  FS r;
  r.h = a.h * m;
  r.l = fmaf(a.l, m, fmaf(a.h, m, -r.h));
  r.e = a.e + (int)(fb >> 23) - 127;
  return r;
}

// a * b (TwoProd of the heads by FMA, the cross terms added to the error, renormalised)
__device__ __forceinline__ FS fs_mul(FS a, FS b) {
  if (!(a.h > 0.0f) || !(b.h > 0.0f)) return fs_zero();
  const float p = a.h * b.h;
  const float lo = fmaf(a.h, b.h, -p) + fmaf(a.h, b.l, a.l * b.h);
  FS r;
  r.h = p + lo;
  r.l = lo - (r.h - p);
  r.e = a.e + b.e;
  return r;
}

__device__ __forceinline__ FS shfl_up_fs(FS v, int o) {
  FS r;
  r.h = __shfl_up_sync(0xffffffffu, v.h, o);
  r.l = __shfl_up_sync(0xffffffffu, v.l, o);
  r.e = __shfl_up_sync(0xffffffffu, v.e, o);
  return r;
}

__device__ __forceinline__ FS shfl_xor_fs(FS v, int o) {
  FS r;
  r.h = __shfl_xor_sync(0xffffffffu, v.h, o);
  r.l = __shfl_xor_sync(0xffffffffu, v.l, o);
  r.e = __shfl_xor_sync(0xffffffffu, v.e, o);
  return r;
}

// natural log of a (> 0) as an fp32 pair, to fp32 accuracy of the mantissa's log
__device__ __forceinline__ void fs_log_pair(FS a, float &lh, float &ll) {
  if (!(a.h > 0.0f)) {
    lh = -INFINITY;
    ll = 0.0f;
    return;
  }
  const float ln2_hi = 0.693147182464599609375f, ln2_lo = -1.904654323148236017e-9f;
  const float ef = (float)a.e;
  const float ph = ef * ln2_hi;
  const float pe = fmaf(ef, ln2_hi, -ph) + ef * ln2_lo;
  pair_sum2(ph, pe, logf(a.h) + a.l / a.h, 0.0f, lh, ll);
}

__device__ __forceinline__ FS fs_from_ss(ScaledSum s) {
  FS r;
  if (!(s.q > 0.0)) return fs_zero();
  pair_of(s.q, r.h, r.l);
  r.e = s.e;
  return r;
}

__device__ __forceinline__ ScaledSum ss_from_fs(FS f) {
  ScaledSum r;
  if (!(f.h > 0.0f)) return ss_zero();
  r.q = (double)f.h + (double)f.l;
  r.e = f.e;
  return r;
}

// log of a pair-scaled value as FP64 (an output)
__device__ __forceinline__ double fs_log_d(FS a) {
  if (!(a.h > 0.0f)) return -INFINITY;
  return (double)(logf(a.h) + a.l / a.h) + (double)a.e * GBNS_LN2;
}

struct EvScanFsSmem {
  FS ws[32];
  FS red[5][32];
};

// CTA scan of pair-scaled values: inclusive and exclusive prefix of each thread's value, and
// the total.
__device__ __forceinline__ void cta_scan_fs(FS v, FS &incl, FS &excl, FS &tot, EvScanFsSmem &sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const FS u = shfl_up_fs(v, o);
    if (lane >= o) v = fs_sum(u, v);
  }
  const FS wex = shfl_up_fs(v, 1);
  if (lane == 31) sm.ws[w] = v;
  __syncthreads();
  if (w == 0) {
    FS x = lane < nw ? sm.ws[lane] : fs_zero();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const FS u = shfl_up_fs(x, o);
      if (lane >= o) x = fs_sum(u, x);
    }
    if (lane < nw) sm.ws[lane] = x;
  }
  __syncthreads();
  const FS pw = w > 0 ? sm.ws[w - 1] : fs_zero();
  incl = fs_sum(pw, v);
  excl = lane == 0 ? pw : fs_sum(pw, wex);
  tot = sm.ws[nw - 1];
  __syncthreads();
}

struct EvScanPairSmem {
  float4 w[32];
};

// Inclusive CTA scan of two fp32 pairs (a = ah + al, b = bh + bl); every thread also gets
// the CTA totals.
__device__ __forceinline__ void cta_scan_p2(float &ah, float &al, float &bh, float &bl, float4 &tot,
                                            EvScanPairSmem &sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float uah = __shfl_up_sync(0xffffffffu, ah, o), ual = __shfl_up_sync(0xffffffffu, al, o);
    const float ubh = __shfl_up_sync(0xffffffffu, bh, o), ubl = __shfl_up_sync(0xffffffffu, bl, o);
    if (lane >= o) {
      pair_sum2(uah, ual, ah, al, ah, al);
      pair_sum2(ubh, ubl, bh, bl, bh, bl);
    }
  }
  if (lane == 31) sm.w[w] = make_float4(ah, al, bh, bl);
  __syncthreads();
  if (w == 0) {
    float4 x = lane < nw ? sm.w[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float uah = __shfl_up_sync(0xffffffffu, x.x, o), ual = __shfl_up_sync(0xffffffffu, x.y, o);
      const float ubh = __shfl_up_sync(0xffffffffu, x.z, o), ubl = __shfl_up_sync(0xffffffffu, x.w, o);
      if (lane >= o) {
        pair_sum2(uah, ual, x.x, x.y, x.x, x.y);
        pair_sum2(ubh, ubl, x.z, x.w, x.z, x.w);
      }
    }
    if (lane < nw) sm.w[lane] = x;
  }
  __syncthreads();
  if (w > 0) {
    const float4 p = sm.w[w - 1];
    pair_sum2(p.x, p.y, ah, al, ah, al);
    pair_sum2(p.z, p.w, bh, bl, bh, bl);
  }
  tot = sm.w[nw - 1];
  __syncthreads();
}

// The coefficient pairs of one live-point count n: (T, t, T2, t2, tT) as fp32 pairs, bytes
// 64-103 of the table row (computed in FP64 beyond the table)
__device__ __forceinline__ void ncoef_pairs(const double *__restrict__ ncoef, int nmax, int nk, float cp[10]) {
  if (nk <= nmax) {
    const float4 *c = (const float4 *)(ncoef + (size_t)nk * GBNS_NCOEF_STRIDE + 8);
    const float4 c0 = c[0], c1 = c[1];
    const float2 c2 = *(const float2 *)(c + 2);
    cp[0] = c0.x; cp[1] = c0.y; cp[2] = c0.z; cp[3] = c0.w;
    cp[4] = c1.x; cp[5] = c1.y; cp[6] = c1.z; cp[7] = c1.w;
    cp[8] = c2.x; cp[9] = c2.y;
  } else {
    double cf[5];
    ncoef_compute((double)nk, cf);
#pragma unroll
    for (int q = 0; q < 5; ++q) pair_of(cf[q], cp[2 * q], cp[2 * q + 1]);
  }
}

// Process elements [0, M) of log-likelihoods L (fp32) with live-point counts given by
// nmode: nconst > 0 -> n_k = nconst; ndesc > 0 -> n_k = ndesc - k; else n_k = narr[k].
// Called by every thread of the CTA (blockDim a multiple of 32), each holding the same acc.
// Optional per-element outputs (FP64 logs): log X, log dZ and, with OUT_LZ, the running log Z.
// L values are relative to Loff (added back in FP64); Lidx, when given, gathers L[Lidx[k]].
// A chunk is K consecutive elements per thread: each thread runs its elements' prefixes
// sequentially and the CTA scans only the threads' totals (log T and log T2 as fp32 pairs,
// the affine term c and, with OUT_LZ, dZ as pair-scaled sums).  Every thread carries pair
// copies of log X and log X2; thread 0 alone keeps the FP64 carries (in shared memory), which
// every thread reads back after each chunk and at the end.
// h_out (shared memory, OUT_LZ false only), when given, receives the dZ-weighted means of this
// scan's samples sum dZ max(L, 0) / sum dZ and sum dZ max(-L, 0) / sum dZ (L relative to
// Loff), for H.
template <bool OUT_LZ, int K = 1>
__device__ void evidence_scan_cta(EvAcc &acc, const float *__restrict__ L, long long M, int nconst, int ndesc,
                                  const int *__restrict__ narr, const double *__restrict__ ncoef, int nmax,
                                  double *__restrict__ out_lX, double *__restrict__ out_ldZ,
                                  double *__restrict__ out_lZ, double Loff, const int *__restrict__ Lidx,
                                  EvScanSmem &sm, double *h_out = nullptr) {
  __shared__ EvScanFsSmem fsm;
  __shared__ EvScanPairSmem psm;
  const int tid = threadIdx.x, T = blockDim.x;
  const long long CH = (long long)T * K;
  FS pZ = fs_zero(), pZ2 = fs_zero(), pdZ2 = fs_zero();  // this thread's partial sums
  FS pHP = fs_zero(), pHQ = fs_zero();  // sum dZ L+, dZ L- (h_out)
  float off_h, off_l;
  pair_of(Loff, off_h, off_l);
  const float ln2_h = 0.693147182464599609375f, ln2_l = -1.904654323148236017e-9f;
  float lxh, lxl, lx2h, lx2l;  // pair copies of the carried log X, log X2
  pair_of(acc.lX, lxh, lxl);
  pair_of(acc.lX2, lx2h, lx2l);
  FS A0 = fs_from_ss(acc.A), Z0 = fs_from_ss(acc.Z);
  if (tid == 0) {
    sm.carry_lX = acc.lX;
    sm.carry_lX2 = acc.lX2;
  }
  __syncthreads();
  for (long long base = 0; base < M; base += CH) {
    const long long k0 = base + (long long)tid * K;
    // (A) inputs, and this thread's running sums of log T and log T2 (pT[j]: through element j)
    float Lk[K];
    int nk[K];
    float pTh[K], pTl[K], pT2h[K], pT2l[K];
    float Lfirst_m1 = 0.0f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long k = k0 + j;
      const bool valid = k < M;
      Lk[j] = valid ? L[Lidx ? Lidx[k] : k] : 0.0f;
      if (j == 0) Lfirst_m1 = !valid ? 0.0f : (k == 0 ? acc.Lprev : L[Lidx ? Lidx[k - 1] : k - 1]);
      int n = 1;
      if (valid) n = nconst > 0 ? nconst : (ndesc > 0 ? (int)(ndesc - k) : narr[k]);
      nk[j] = n < 0 ? 0 : n;
    }
#pragma unroll
    for (int j = 0; j < K; ++j) {
      float cp[10];
      ncoef_pairs(ncoef, nmax, nk[j], cp);
      const bool valid = k0 + j < M;
      const float th = j == 0 ? 0.0f : pTh[j > 0 ? j - 1 : 0], tl = j == 0 ? 0.0f : pTl[j > 0 ? j - 1 : 0];
      const float t2h_ = j == 0 ? 0.0f : pT2h[j > 0 ? j - 1 : 0], t2l_ = j == 0 ? 0.0f : pT2l[j > 0 ? j - 1 : 0];
      pair_sum2(th, tl, valid ? cp[0] : 0.0f, valid ? cp[1] : 0.0f, pTh[j], pTl[j]);
      pair_sum2(t2h_, t2l_, valid ? cp[4] : 0.0f, valid ? cp[5] : 0.0f, pT2h[j], pT2l[j]);
    }
    // CTA prefix of the thread sums; base = the carried log X (log X2) plus the sums of the
    // elements before this thread's
    float ah = pTh[K - 1], al = pTl[K - 1], bh = pT2h[K - 1], bl = pT2l[K - 1];
    float4 tot;
    cta_scan_p2(ah, al, bh, bl, tot, psm);
    float bxh, bxl, bx2h, bx2l;
    pair_sum2(ah, al, -pTh[K - 1], -pTl[K - 1], bxh, bxl);
    pair_sum2(bh, bl, -pT2h[K - 1], -pT2l[K - 1], bx2h, bx2l);
    pair_sum2(lxh, lxl, bxh, bxl, bxh, bxl);
    pair_sum2(lx2h, lx2l, bx2h, bx2l, bx2h, bx2l);
    // (B) per element, independently: log X, the midpoint, dZ, the affine term c and t2
    float dzh[K], dzl[K], t2h[K], t2l[K], xch[K], xcl[K];
    FS cj[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long k = k0 + j;
      const bool valid = k < M;
      float cp[10];
      ncoef_pairs(ncoef, nmax, nk[j], cp);
      float xph = bxh, xpl = bxl, x2ph = bx2h, x2pl = bx2l;  // log X_{k-1}, log X2_{k-1}
      if (j > 0) {
        pair_sum2(bxh, bxl, pTh[j > 0 ? j - 1 : 0], pTl[j > 0 ? j - 1 : 0], xph, xpl);
        pair_sum2(bx2h, bx2l, pT2h[j > 0 ? j - 1 : 0], pT2l[j > 0 ? j - 1 : 0], x2ph, x2pl);
      }
      pair_sum2(bxh, bxl, pTh[j], pTl[j], xch[j], xcl[j]);  // log X_k
      // log((L_k + L_{k-1}) / 2) + Loff as a pair: max + log1p(exp(-|d|)) - ln 2 + Loff; -inf
      // outside the chunk
      const float Lcur = Lk[j], Lprev = j == 0 ? Lfirst_m1 : Lk[j > 0 ? j - 1 : 0];
      float mh = -INFINITY, ml = 0.0f;
      if (valid) {
        const float m = fmaxf(Lcur, Lprev), d = Lcur - Lprev;
        if (isnan(d)) {
          mh = Lcur + Lprev;  // both -inf (or +inf)
        } else {
          float th, tl;
          pair_sum2(m, 0.0f, log1pf(__expf(-fabsf(d))), 0.0f, th, tl);
          pair_sum2(th, tl, -ln2_h, -ln2_l, th, tl);
          pair_sum2(th, tl, off_h, off_l, mh, ml);
        }
      }
      // v_dZ = (lX_prev + lt) + lmid, v_c = ((lX2_prev + ltT) - lX_cur) + lmid,
      // v_t2 = (lX2_prev + lt2) + 2 lmid
      float vch = -INFINITY, vcl = 0.0f;
      dzh[j] = -INFINITY; dzl[j] = 0.0f; t2h[j] = -INFINITY; t2l[j] = 0.0f;
      if (valid && mh > -INFINITY) {
        float qh, ql;
        pair_sum2(xph, xpl, cp[2], cp[3], qh, ql);
        pair_sum2(qh, ql, mh, ml, dzh[j], dzl[j]);
        pair_sum2(x2ph, x2pl, cp[8], cp[9], qh, ql);
        pair_sum2(qh, ql, -xch[j], -xcl[j], qh, ql);
        pair_sum2(qh, ql, mh, ml, vch, vcl);
        pair_sum2(x2ph, x2pl, cp[6], cp[7], qh, ql);
        pair_sum2(qh, ql, 2.0f * mh, 2.0f * ml, t2h[j], t2l[j]);
      }
      cj[j] = fs_term(vch, vcl);
    }
    // this thread's exclusive sums of c (cex[j]: elements before j), then A_{k-1} = A_0 + the
    // CTA's exclusive prefix of c + cex[j]
    FS cex[K];
    cex[0] = fs_zero();
#pragma unroll
    for (int j = 1; j < K; ++j) cex[j] = fs_sum(cex[j - 1], cj[j - 1]);
    const FS crun = fs_sum(cex[K - 1], cj[K - 1]);
    FS cin, cthr, ctot;
    cta_scan_fs(crun, cin, cthr, ctot, fsm);
    const FS At = fs_sum(A0, cthr);
    // with OUT_LZ, the running Z needs the CTA's prefix of dZ as well
    FS tdZ[K];
#pragma unroll
    for (int j = 0; j < K; ++j) tdZ[j] = fs_term(dzh[j], dzl[j]);
    FS zthr = fs_zero(), ztot = fs_zero();
    if (OUT_LZ) {
      FS zrun = fs_zero();
#pragma unroll
      for (int j = 0; j < K; ++j) zrun = fs_sum(zrun, tdZ[j]);
      FS zin;
      cta_scan_fs(zrun, zin, zthr, ztot, fsm);
      zthr = fs_sum(Z0, zthr);
    }
    // (C) per element, independently: the outputs and the terms of this thread's sums, which
    // are added as a tree
    FS sZ[K], sZ2[K], sdZ2[K], sP[K], sQ[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long k = k0 + j;
      const bool valid = k < M;
      if (valid) {
        if (out_lX) out_lX[k] = pair_to_double(xch[j], xcl[j]);
        if (out_ldZ) out_ldZ[k] = pair_to_double(dzh[j], dzl[j]);
      }
      const FS tt2 = fs_term(t2h[j], t2l[j]);
      // 2 dZ_k A_{k-1}, a product of pair-scaled values (no log and exp round trip)
      FS t1 = fs_mul(tdZ[j], fs_sum(At, cex[j]));
      t1.e += 1;
      sZ[j] = tdZ[j];
      sZ2[j] = fs_sum(t1, tt2);
      sdZ2[j] = tt2;
      sP[j] = fs_zero();
      sQ[j] = fs_zero();
      if (h_out && valid) {
        const FS tl = fs_scale(tdZ[j], fabsf(Lk[j]));
        if (Lk[j] >= 0.0f) sP[j] = tl;
        else sQ[j] = tl;
      }
      // the chunk's last element carries its log dZ and L to the next call
      if (k == (M - base < CH ? M : base + CH) - 1) {
        sm.last_ldZ = pair_to_double(dzh[j], dzl[j]);
        sm.last_L = Lk[j];
      }
    }
    if (OUT_LZ) {
#pragma unroll
      for (int j = 0; j < K; ++j) {
        zthr = fs_sum(zthr, tdZ[j]);
        if (k0 + j < M && out_lZ) out_lZ[k0 + j] = fs_log_d(zthr);
      }
    }
#pragma unroll
    for (int w = 1; w < K; w <<= 1) {
#pragma unroll
      for (int j = 0; j + w < K; j += 2 * w) {
        sZ[j] = fs_sum(sZ[j], sZ[j + w]);
        sZ2[j] = fs_sum(sZ2[j], sZ2[j + w]);
        sdZ2[j] = fs_sum(sdZ2[j], sdZ2[j + w]);
        if (h_out) {
          sP[j] = fs_sum(sP[j], sP[j + w]);
          sQ[j] = fs_sum(sQ[j], sQ[j + w]);
        }
      }
    }
    if (!OUT_LZ) pZ = fs_sum(pZ, sZ[0]);
    pZ2 = fs_sum(pZ2, sZ2[0]);
    pdZ2 = fs_sum(pdZ2, sdZ2[0]);
    if (h_out) {
      pHP = fs_sum(pHP, sP[0]);
      pHQ = fs_sum(pHQ, sQ[0]);
    }
    // carries into the next chunk: FP64 in thread 0, re-read as pairs by every thread
    A0 = fs_sum(A0, ctot);
    if (OUT_LZ) Z0 = fs_sum(Z0, ztot);
    __syncthreads();  // every thread has read sm.carry_lX for this chunk
    if (tid == 0) {
      acc.lX += (double)tot.x + (double)tot.y;
      acc.lX2 += (double)tot.z + (double)tot.w;
      acc.A = ss_sum(acc.A, ss_from_fs(ctot));
      if (OUT_LZ) acc.Z = ss_sum(acc.Z, ss_from_fs(ztot));
      sm.carry_lX = acc.lX;
      sm.carry_lX2 = acc.lX2;
    }
    __syncthreads();
    acc.ldZ_last = sm.last_ldZ;
    acc.Lprev = sm.last_L;
    pair_of(sm.carry_lX, lxh, lxl);
    pair_of(sm.carry_lX2, lx2h, lx2l);
  }
  // CTA reduction of the partial sums (butterfly in each warp, then across warps in order)
  const int lane = tid & 31, w = tid >> 5, nw = T >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pZ = fs_sum(pZ, shfl_xor_fs(pZ, o));
    pZ2 = fs_sum(pZ2, shfl_xor_fs(pZ2, o));
    pdZ2 = fs_sum(pdZ2, shfl_xor_fs(pdZ2, o));
    if (h_out) {
      pHP = fs_sum(pHP, shfl_xor_fs(pHP, o));
      pHQ = fs_sum(pHQ, shfl_xor_fs(pHQ, o));
    }
  }
  if (lane == 0) {
    fsm.red[0][w] = pZ;
    fsm.red[1][w] = pZ2;
    fsm.red[2][w] = pdZ2;
    fsm.red[3][w] = pHP;
    fsm.red[4][w] = pHQ;
  }
  __syncthreads();
  if (tid == 0) {
    FS rZ = fs_zero(), rZ2 = fs_zero(), rdZ2 = fs_zero(), rP = fs_zero(), rQ = fs_zero();
    for (int q = 0; q < nw; ++q) {
      rZ = fs_sum(rZ, fsm.red[0][q]);
      rZ2 = fs_sum(rZ2, fsm.red[1][q]);
      rdZ2 = fs_sum(rdZ2, fsm.red[2][q]);
      if (h_out) {
        rP = fs_sum(rP, fsm.red[3][q]);
        rQ = fs_sum(rQ, fsm.red[4][q]);
      }
    }
    if (h_out) {
      // each sum over this scan's own sum of dZ (FP64 ratio of the two scaled sums)
      const ScaledSum z = ss_from_fs(rZ);
      const ScaledSum hs[2] = {ss_from_fs(rP), ss_from_fs(rQ)};
      for (int q = 0; q < 2; ++q)
        h_out[q] = (z.q > 0.0 && hs[q].q > 0.0) ? (hs[q].q / z.q) * pow2i(hs[q].e - z.e) : 0.0;
    }
    acc.Z = ss_sum(acc.Z, ss_from_fs(rZ));
    acc.Z2 = ss_sum(acc.Z2, ss_from_fs(rZ2));
    acc.dZ2 = ss_sum(acc.dZ2, ss_from_fs(rdZ2));
    sm.fin_lX = acc.lX;
    sm.fin_lX2 = acc.lX2;
    sm.fin[0] = acc.A;
    sm.fin[1] = acc.Z;
    sm.fin[2] = acc.Z2;
    sm.fin[3] = acc.dZ2;
  }
  __syncthreads();
  acc.lX = sm.fin_lX;
  acc.lX2 = sm.fin_lX2;
  acc.A = sm.fin[0];
  acc.Z = sm.fin[1];
  acc.Z2 = sm.fin[2];
  acc.dZ2 = sm.fin[3];
  __syncthreads();
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
