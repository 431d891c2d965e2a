/*
 * ns_oracle.c -- CPU restatement of jaxns (v2.6.9) static nested sampling, FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA path is checked
 * against; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * Nothing in the product path calls it.
 *
 * Every function restates one reference function, in the reference's operation order,
 * in double precision (the reference runs with jax_enable_x64, measures f64, counts i64).
 * Reference paths are relative to the jaxns source tree (src/jaxns/...).
 *
 * Parity pins:
 *   - threefry2x32_20 is checked against the Random123 known-answer vectors (tests).
 *   - count_crossed_edges / cumulative ops against the reference's own unit-test values.
 *   - the key-derivation layout (jax_threefry_partitionable=True) and XLA's f64 erfinv
 *     cannot be checked here (no JAX in this environment): "parity unpinned" for those;
 *     tests/golden/make_jax_golden.py records jax's outputs where jax is installed.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime under strict C modes as well */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <time.h>

#define ORC_PI 3.14159265358979323846
#define ORC_SQRT2 1.4142135623730951
#define ORC_LOG2 0.6931471805599453

/* ------------------------------------------------------------------ RNG ---- */

static inline uint32_t rotl32(uint32_t v, int r) { return (v << r) | (v >> (32 - r)); }

/* Threefry-2x32 with 20 rounds (Salmon et al., SC'11, "Parallel random numbers: as easy
 * as 1, 2, 3"); the block cipher behind jax.random's default PRNG. */
void orc_threefry2x32(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t out[2]) {
    static const int R[8] = {13, 15, 26, 6, 17, 29, 16, 24};
    uint32_t ks[3] = {k0, k1, k0 ^ k1 ^ 0x1BD11BDAu};
    uint32_t x0 = c0 + ks[0], x1 = c1 + ks[1];
    for (int blk = 0; blk < 5; ++blk) {
        const int *rot = &R[(blk & 1) * 4];
        for (int r = 0; r < 4; ++r) {
            x0 += x1;
            x1 = rotl32(x1, rot[r]);
            x1 ^= x0;
        }
        x0 += ks[(blk + 1) % 3];
        x1 += ks[(blk + 2) % 3] + (uint32_t)(blk + 1);
    }
    out[0] = x0;
    out[1] = x1;
}

typedef struct { uint32_t k0, k1; } okey;

/* jax.random.split(key, n)[i] under jax_threefry_partitionable=True: threefry of the
 * 64-bit iota index (hi word, lo word) under the parent key. */
static inline okey key_fold(okey k, uint64_t i) {
    uint32_t o[2];
    orc_threefry2x32(k.k0, k.k1, (uint32_t)(i >> 32), (uint32_t)i, o);
    okey r = {o[0], o[1]};
    return r;
}

/* 64 random bits for element i of a shape (partitionable layout: hi<<32 | lo). */
static inline uint64_t bits64(okey k, uint64_t i) {
    uint32_t o[2];
    orc_threefry2x32(k.k0, k.k1, (uint32_t)(i >> 32), (uint32_t)i, o);
    return ((uint64_t)o[0] << 32) | (uint64_t)o[1];
}

/* jax.random.uniform(key, shape, float64, minval, maxval), element i. */
static inline double uniform_f64(okey k, uint64_t i, double minval, double maxval) {
    uint64_t b = bits64(k, i);
    uint64_t fb = (b >> 12) | 0x3FF0000000000000ull;
    double f;
    memcpy(&f, &fb, 8);
    f -= 1.0;
    double v = f * (maxval - minval) + minval;
    return v > minval ? v : minval;
}

/* erfinv in f64: Winitzki initial guess, then three Halley steps on erf (|u|<=0.5)
 * or erfc (|u|>0.5, where 1-|u| is exact).  Accurate to ~1 ulp; XLA's own f64 erfinv is
 * a different polynomial, so the last bits of jax.random.normal are unpinned. */
double orc_erfinv(double u) {
    if (isnan(u)) return u;
    if (u >= 1.0) return INFINITY;
    if (u <= -1.0) return -INFINITY;
    if (u == 0.0) return u;
    double a = fabs(u);
    double w = log((1.0 - a) * (1.0 + a));
    double c = 2.0 / (ORC_PI * 0.147) + 0.5 * w;
    double x = sqrt(sqrt(c * c - w / 0.147) - c);
    const double k = 2.0 / sqrt(ORC_PI);
    for (int it = 0; it < 3; ++it) {
        double g = (a <= 0.5) ? (erf(x) - a) : ((1.0 - a) - erfc(x));
        double gp = k * exp(-x * x);
        x -= g / (gp + x * g);
    }
    return u < 0 ? -x : x;
}

/* jax.random.normal(key, shape, float64), element i: sqrt(2) * erfinv(uniform(lo, 1))
 * with lo = nextafter(-1, 0). */
static inline double normal_f64(okey k, uint64_t i) {
    double lo = nextafter(-1.0, 0.0);
    double u = uniform_f64(k, i, lo, 1.0);
    return ORC_SQRT2 * orc_erfinv(u);
}

/* ------------------------------------------------------------ log space ---- */

/* jnp.logaddexp (jax/_src/numpy/ufuncs.py): NaN delta -> x1 + x2. */
static inline double lae(double a, double b) {
    double amax = a > b ? a : b;
    double d = a - b;
    if (isnan(d)) return a + b;
    return amax + log1p(exp(-fabs(d)));
}

/* ---------------------------------------------------------------- model ---- */

enum { ORC_PRIOR_UNIFORM = 0, ORC_PRIOR_NORMAL = 1 };
enum { ORC_LIK_MVN = 0, ORC_LIK_SHELLS = 1, ORC_LIK_LINGAUSS = 2 };

typedef struct {
    int D;
    int family;
    const int *prior_kind;   /* [D] */
    const double *prior_a;   /* [D] uniform: low;  normal: loc   */
    const double *prior_b;   /* [D] uniform: high - low; normal: scale */
    const double *p;         /* family parameters */
    int N;                   /* rows of Phi for the linear-Gaussian family */
    const double *prior_A;   /* [D x D] lower triangular, or NULL: X = A q + c after the per-dimension
                                quantiles q (MultivariateNormalTriL blocks: the bijector loc + L z) */
    const double *prior_c;   /* [D] */
} orc_model;

/* U -> X: the prior quantile (tfp Uniform / Normal quantile as used by
 * framework/wrapped_tfp_distribution.py:77-84). */
static void prior_transform(const orc_model *m, const double *U, double *X) {
    for (int j = 0; j < m->D; ++j) {
        if (m->prior_kind[j] == ORC_PRIOR_UNIFORM)
            X[j] = m->prior_a[j] + m->prior_b[j] * U[j];
        else
            X[j] = m->prior_a[j] + m->prior_b[j] * (ORC_SQRT2 * orc_erfinv(2.0 * U[j] - 1.0));
    }
    if (m->prior_A) {
        /* tfp MultivariateNormalTriL: the bijector loc + L z after the base quantile
         * (framework/wrapped_tfp_distribution.py:77-84); rows from the last, so X[k], k <= i,
         * still hold the quantiles */
        int D = m->D;
        for (int i = D - 1; i >= 0; --i) {
            double acc = m->prior_c[i];
            for (int k = 0; k <= i; ++k) acc += m->prior_A[i * D + k] * X[k];
            X[i] = acc;
        }
    }
}

static double loglik_x(const orc_model *m, const double *X) {
    int D = m->D;
    double v;
    if (m->family == ORC_LIK_MVN) {
        /* p = [mu(D), L(DxD row-major lower Cholesky)]; MultivariateNormalTriL log_prob */
        const double *mu = m->p, *L = m->p + D;
        double z[128], s = 0.0, ld = 0.0;
        for (int i = 0; i < D; ++i) {
            double acc = X[i] - mu[i];
            for (int j = 0; j < i; ++j) acc -= L[i * D + j] * z[j];
            z[i] = acc / L[i * D + i];
            s += z[i] * z[i];
            ld += log(L[i * D + i]);
        }
        v = -0.5 * s - ld - 0.5 * D * log(2.0 * ORC_PI);
    } else if (m->family == ORC_LIK_SHELLS) {
        /* p = [c1(D), c2(D), R, w]: logaddexp of two Gaussian shells */
        const double *c1 = m->p, *c2 = m->p + D;
        double R = m->p[2 * D], w = m->p[2 * D + 1];
        double r1 = 0, r2 = 0;
        for (int j = 0; j < D; ++j) {
            r1 += (X[j] - c1[j]) * (X[j] - c1[j]);
            r2 += (X[j] - c2[j]) * (X[j] - c2[j]);
        }
        r1 = sqrt(r1);
        r2 = sqrt(r2);
        double norm = log(sqrt(2.0 * ORC_PI * w * w));
        double s1 = -0.5 * ((r1 - R) / w) * ((r1 - R) / w) - norm;
        double s2 = -0.5 * ((r2 - R) / w) * ((r2 - R) / w) - norm;
        v = lae(s1, s2);
    } else {
        /* p = [Phi(N x D row-major), y(N), sigma]: log N(y; Phi w, sigma^2 I) */
        int N = m->N;
        const double *Phi = m->p, *y = m->p + (size_t)N * D;
        double sigma = m->p[(size_t)N * D + N];
        double s = 0;
        for (int i = 0; i < N; ++i) {
            double r = y[i];
            for (int j = 0; j < D; ++j) r -= Phi[(size_t)i * D + j] * X[j];
            s += r * r;
        }
        v = -0.5 * N * log(2.0 * ORC_PI * sigma * sigma) - 0.5 * s / (sigma * sigma);
    }
    return v;
}

/* Model.forward (framework/model.py:167) -> compute_log_likelihood, NaN -> -inf
 * (framework/ops.py:323-325). */
double orc_forward(const orc_model *m, const double *U) {
    double X[128];
    prior_transform(m, U, X);
    double v = loglik_x(m, X);
    return isnan(v) ? -INFINITY : v;
}

void orc_forward_batch(const orc_model *m, const double *U, long B, double *out) {
    for (long b = 0; b < B; ++b) out[b] = orc_forward(m, U + b * m->D);
}

/* jax.grad of Model.forward w.r.t. U, analytically: d log L / dX through the prior quantile
 * (Uniform: dX/dU = high - low; Normal: dX/dU = scale sqrt(2 pi) exp(z^2 / 2), z the standard
 * normal quantile of U). */
void orc_grad_U(const orc_model *m, const double *U, double *g) {
    int D = m->D;
    double X[128], gx[128];
    prior_transform(m, U, X);
    if (m->family == ORC_LIK_MVN) {
        const double *mu = m->p, *L = m->p + D;
        double z[128];
        for (int i = 0; i < D; ++i) {              /* L z = X - mu */
            double acc = X[i] - mu[i];
            for (int j = 0; j < i; ++j) acc -= L[i * D + j] * z[j];
            z[i] = acc / L[i * D + i];
        }
        for (int i = D - 1; i >= 0; --i) {         /* L^T v = z, d log L / dX = -v */
            double acc = z[i];
            for (int j = i + 1; j < D; ++j) acc -= L[j * D + i] * gx[j];
            gx[i] = acc / L[i * D + i];
        }
        for (int i = 0; i < D; ++i) gx[i] = -gx[i];
    } else if (m->family == ORC_LIK_SHELLS) {
        const double *c1 = m->p, *c2 = m->p + D;
        double R = m->p[2 * D], w = m->p[2 * D + 1];
        double r1 = 0, r2 = 0;
        for (int j = 0; j < D; ++j) {
            r1 += (X[j] - c1[j]) * (X[j] - c1[j]);
            r2 += (X[j] - c2[j]) * (X[j] - c2[j]);
        }
        r1 = sqrt(r1);
        r2 = sqrt(r2);
        double z1 = (r1 - R) / w, z2 = (r2 - R) / w;
        double s1 = -0.5 * z1 * z1, s2 = -0.5 * z2 * z2, mx = s1 > s2 ? s1 : s2;
        double p1 = exp(s1 - mx), p2 = exp(s2 - mx), tot = p1 + p2;
        p1 /= tot;
        p2 /= tot;
        for (int j = 0; j < D; ++j)
            gx[j] = p1 * (-z1 / w) * (X[j] - c1[j]) / r1 + p2 * (-z2 / w) * (X[j] - c2[j]) / r2;
    } else {
        int N = m->N;
        const double *Phi = m->p, *y = m->p + (size_t)N * D;
        double sigma = m->p[(size_t)N * D + N];
        for (int j = 0; j < D; ++j) gx[j] = 0.0;
        for (int i = 0; i < N; ++i) {
            double r = y[i];
            for (int j = 0; j < D; ++j) r -= Phi[(size_t)i * D + j] * X[j];
            for (int j = 0; j < D; ++j) gx[j] += Phi[(size_t)i * D + j] * r / (sigma * sigma);
        }
    }
    if (m->prior_A) {
        /* d log L / dq = A^T d log L / dX */
        double gq[128];
        for (int k = 0; k < D; ++k) {
            double acc = 0.0;
            for (int i = k; i < D; ++i) acc += m->prior_A[i * D + k] * gx[i];
            gq[k] = acc;
        }
        for (int k = 0; k < D; ++k) gx[k] = gq[k];
    }
    for (int j = 0; j < D; ++j) {
        double dxdu;
        if (m->prior_kind[j] == ORC_PRIOR_UNIFORM) {
            dxdu = m->prior_b[j];
        } else {
            double z = ORC_SQRT2 * orc_erfinv(2.0 * U[j] - 1.0);
            dxdu = m->prior_b[j] * sqrt(2.0 * ORC_PI) * exp(0.5 * z * z);
        }
        g[j] = gx[j] * dxdu;
    }
}

/* Model.sample_U (framework/model.py:135-138): uniform(split(key)[1], (D,)) via
 * Ctx.next_rng_key (framework/context.py:107-109). */
static void sample_U(okey key, int D, double *U) {
    okey k = key_fold(key, 1);
    for (int j = 0; j < D; ++j) U[j] = uniform_f64(k, (uint64_t)j, 0.0, 1.0);
}

/* ------------------------------------------------------- slice sampler ---- */

/* _sample_direction (samplers/uni_slice_sampler.py:23-38) */
static void sample_direction(okey k, int D, double *d) {
    if (D == 1) { d[0] = 1.0; return; }
    double s = 0;
    for (int j = 0; j < D; ++j) { d[j] = normal_f64(k, (uint64_t)j); s += d[j] * d[j]; }
    double nrm = sqrt(s);
    for (int j = 0; j < D; ++j) d[j] /= nrm;
}

/* _slice_bounds (uni_slice_sampler.py:41-64) */
static void slice_bounds(const double *U0, const double *d, int D, double *left, double *right) {
    double t1r = INFINITY, t1l = -INFINITY, t0r = INFINITY, t0l = -INFINITY;
    for (int j = 0; j < D; ++j) {
        double t1 = (1.0 - U0[j]) / d[j];
        double t0 = -U0[j] / d[j];
        double a = (t1 >= 0) ? t1 : INFINITY;  if (a < t1r) t1r = a;
        double b = (t1 <= 0) ? t1 : -INFINITY; if (b > t1l) t1l = b;
        double c = (t0 >= 0) ? t0 : INFINITY;  if (c < t0r) t0r = c;
        double e = (t0 <= 0) ? t0 : -INFINITY; if (e > t0l) t0l = e;
    }
    *right = t0r < t1r ? t0r : t1r;
    *left = t0l > t1l ? t0l : t1l;
}

/* _pick_point_in_interval (uni_slice_sampler.py:67-89) */
static double pick_point(okey tkey, const double *U0, const double *d, int D, double left,
                         double right, double *U) {
    double u = uniform_f64(tkey, 0, 0.0, 1.0);
    double t = left + u * (right - left);
    for (int j = 0; j < D; ++j) U[j] = U0[j] + t * d[j];
    return t;
}

typedef struct {
    int num_slices;
    int num_phantom;
    int midpoint_shrink;
    int gradient_guided;
    int gradient_slice;
} orc_slice_cfg;

/* linspace(0.5, 1., S)[j] as jnp.linspace evaluates it. */
static double slice_alpha(int j, int S) {
    if (S == 1) return 0.5;
    if (j == S - 1) return 1.0;
    double step = (double)j / (double)(S - 1);
    return 0.5 * (1.0 - step) + 1.0 * step;
}

/* _new_proposal (uni_slice_sampler.py:114-273) with perfect=True, no gradient options.
 * U0/logL0 is the seed; on return U holds the accepted point, d the new direction. */
/* When set (orc_slice_shell_margin), every accept test of the calling thread lowers
 * *orc_margin_sink to |log L - L*|: how close the chain came to a tie with the contour. */
static _Thread_local double *orc_margin_sink = NULL;

static inline void note_margin(double logL, double Lstar) {
    if (orc_margin_sink) {
        double d = fabs(logL - Lstar);
        if (!(d >= *orc_margin_sink)) *orc_margin_sink = d;
    }
}

static double new_proposal(const orc_model *m, okey key, const double *U0, double logL0,
                           double *d, int midpoint, double alpha, double Lstar, double *U,
                           long *nevals, int gradient_guided, int gradient_slice) {
    int D = m->D;
    okey run_key = key_fold(key, 0);
    okey t_key = key_fold(key, 2);
    okey after_key = key_fold(key, 3);
    double left, right;
    long ne = 0;
    int climb = 0;
    if (gradient_slice) {
        /* climb the gradient (uni_slice_sampler.py:202-214): slice along the normalised U-space
         * gradient at the seed point, t >= 0, unless the gradient vanishes or is not finite */
        double g[128], gn = 0.0;
        orc_grad_U(m, U0, g);
        ne += 1;
        for (int j = 0; j < D; ++j) gn += g[j] * g[j];
        gn = sqrt(gn);
        if (!(gn == 0.0 || !isfinite(gn))) {
            for (int j = 0; j < D; ++j) d[j] = g[j] / gn;
            climb = 1;
        }
    }
    slice_bounds(U0, d, D, &left, &right);
    if (climb) left = 0.0;
    double t = pick_point(t_key, U0, d, D, left, right, U);
    double logL = orc_forward(m, U);
    ne += 1;
    okey ck = run_key;
    note_margin(logL, Lstar);
    while (!((logL > Lstar) || ((logL0 == Lstar) && (logL == Lstar)))) {
        okey nk = key_fold(ck, 0);
        okey tk = key_fold(ck, 1);
        /* _shrink_interval (uni_slice_sampler.py:92-111) */
        if (t < 0) left = t;
        if (t > 0) right = t;
        if (midpoint) {
            if (t < 0) left = alpha * left;
            if (t > 0) right = alpha * right;
        }
        t = pick_point(tk, U0, d, D, left, right, U);
        logL = orc_forward(m, U);
        note_margin(logL, Lstar);
        ne += 1;
        ck = nk;
    }
    if (gradient_guided) {
        /* Householder reflection of the direction at the accepted point
         * (uni_slice_sampler.py:255-269); a random direction from split(after_key)[0] when the
         * gradient vanishes or is not finite.  The gradient counts as one evaluation. */
        double g[128], gn = 0.0, dot = 0.0, dn = 0.0;
        orc_grad_U(m, U, g);
        ne += 1;
        for (int j = 0; j < D; ++j) gn += g[j] * g[j];
        gn = sqrt(gn);
        if (gn < 1e-10 || !isfinite(gn)) {
            sample_direction(key_fold(after_key, 0), D, d);
        } else {
            for (int j = 0; j < D; ++j) { g[j] /= gn; dot += d[j] * g[j]; }
            for (int j = 0; j < D; ++j) { d[j] -= 2.0 * dot * g[j]; dn += d[j] * d[j]; }
            dn = sqrt(dn);
            for (int j = 0; j < D; ++j) d[j] /= dn;
        }
    } else {
        sample_direction(after_key, D, d);
    }
    *nevals = ne;
    return logL;
}

/* cumulative_logsumexp + searchsorted for resample_indicies(replace=True, S=1)
 * (internals/random.py:34-84) over the mask log_L > Lstar. */
static long seed_index(okey seed_key, const double *live_logL, long n, double Lstar) {
    double acc = -INFINITY;
    double *cum = (double *)malloc(sizeof(double) * (size_t)n);
    for (long i = 0; i < n; ++i) {
        double w = (live_logL[i] > Lstar) ? 0.0 : -INFINITY;
        acc = lae(acc, w);
        cum[i] = acc;
    }
    double u = uniform_f64(seed_key, 0, 0.0, 1.0);
    double log_r = cum[n - 1] + log(1.0 - u);
    /* searchsorted side='left': first i with cum[i] >= log_r */
    long lo = 0, hi = n;
    while (lo < hi) {
        long mid = (lo + hi) / 2;
        if (cum[mid] < log_r) lo = mid + 1; else hi = mid;
    }
    free(cum);
    return lo < n ? lo : n - 1;
}

long orc_seed_index_export(uint32_t k0, uint32_t k1, const double *live_logL, long n, double Lstar) {
    okey k = {k0, k1};
    return seed_index(k, live_logL, n, Lstar);
}

/* UniDimSliceSampler.get_sample (bases.py:63-75 -> uni_slice_sampler.py:343-441).
 * phantom_U: [k, D], phantom_logL: [k]. */
void orc_slice_get_sample(const orc_model *m, const orc_slice_cfg *cfg, uint32_t k0, uint32_t k1,
                          double Lstar, const double *live_U, const double *live_logL, long n,
                          double *U_out, double *logL_out, long *nevals_out, double *phantom_U,
                          double *phantom_logL) {
    int D = m->D, S = cfg->num_slices, K = cfg->num_phantom;
    okey key = {k0, k1};
    okey sample_key = key_fold(key, 0);
    okey seed_key = key_fold(key, 1);
    long idx = seed_index(seed_key, live_logL, n, Lstar);
    double U0[128], U[128], d[128];
    memcpy(U0, live_U + idx * D, sizeof(double) * D);
    double logL0 = live_logL[idx];
    okey direction_key = key_fold(sample_key, 0);
    okey slices_key = key_fold(sample_key, 1);
    sample_direction(direction_key, D, d);
    long total = 0;
    for (int j = 0; j < S; ++j) {
        okey kj = key_fold(slices_key, (uint64_t)j);
        long ne;
        double logL = new_proposal(m, kj, U0, logL0, d, cfg->midpoint_shrink, slice_alpha(j, S), Lstar,
                                   U, &ne, cfg->gradient_guided, cfg->gradient_slice);
        total += ne;
        memcpy(U0, U, sizeof(double) * D);
        logL0 = logL;
        /* cumulative_samples[-(k+1):-1] are the phantoms */
        int p = j - (S - 1 - K);
        if (K > 0 && p >= 0 && j < S - 1) {
            memcpy(phantom_U + (size_t)p * D, U, sizeof(double) * D);
            phantom_logL[p] = logL;
        }
    }
    memcpy(U_out, U0, sizeof(double) * D);
    *logL_out = logL0;
    *nevals_out = total;
}

/* UniformSampler._get_sample (samplers/uniform_samplers.py:42-85), and with
 * max_evals <= 0 the uncapped init variant (_single_uniform_sample,
 * nested_samplers/common/uniform_sample.py:12-60, Lstar = -inf). */
void orc_uniform_get_sample(const orc_model *m, uint32_t k0, uint32_t k1, double Lstar, long max_evals,
                            double *U_out, double *logL_out, long *nevals_out) {
    int D = m->D;
    okey key = {k0, k1};
    okey k = key_fold(key, 0), sk = key_fold(key, 1);
    sample_U(sk, D, U_out);
    double logL = orc_forward(m, U_out);
    long ne = 1;
    for (;;) {
        int done;
        if (max_evals > 0)
            done = (logL > Lstar) || (logL == Lstar) || (ne >= max_evals);
        else
            done = !(logL <= Lstar);
        if (done) break;
        okey nk = key_fold(k, 0);
        sk = key_fold(k, 1);
        k = nk;
        sample_U(sk, D, U_out);
        logL = orc_forward(m, U_out);
        ne += 1;
    }
    *logL_out = logL;
    *nevals_out = ne;
}

/* --------------------------------------------------------------- sorting ---- */

/* jnp.argsort / lax.sort_key_val ordering: -0 == +0, NaN after +inf, stable. */
static inline int key_lt(double a, double b) {
    if (isnan(a)) return 0;
    if (isnan(b)) return 1;
    return a < b;
}

void orc_stable_argsort(const double *keys, long n, long *perm) {
    long *tmp = (long *)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
    for (long i = 0; i < n; ++i) perm[i] = i;
    for (long width = 1; width < n; width *= 2) {
        for (long lo = 0; lo < n; lo += 2 * width) {
            long mid = lo + width < n ? lo + width : n;
            long hi = lo + 2 * width < n ? lo + 2 * width : n;
            long a = lo, b = mid, o = lo;
            while (a < mid && b < hi) {
                if (key_lt(keys[perm[b]], keys[perm[a]])) tmp[o++] = perm[b++];
                else tmp[o++] = perm[a++];
            }
            while (a < mid) tmp[o++] = perm[a++];
            while (b < hi) tmp[o++] = perm[b++];
        }
        memcpy(perm, tmp, sizeof(long) * (size_t)n);
    }
    free(tmp);
}

/* ------------------------------------------------------------- evidence ---- */

typedef struct {
    double log_L, log_X_mean, log_X2_mean, log_Z_mean, log_ZX_mean, log_Z2_mean, log_dZ_mean,
        log_dZ2_mean;
} orc_evcalc;

/* create_init_evidence_calc (internals/shrinkage_statistics.py:112-128) */
void orc_evcalc_init(orc_evcalc *e) {
    e->log_L = -INFINITY;
    e->log_X_mean = 0.0;
    e->log_X2_mean = 0.0;
    e->log_Z_mean = -INFINITY;
    e->log_ZX_mean = -INFINITY;
    e->log_Z2_mean = -INFINITY;
    e->log_dZ_mean = -INFINITY;
    e->log_dZ2_mean = -INFINITY;
}

/* _update_evidence_calc_op (internals/shrinkage_statistics.py:43-94), LogSpace algebra
 * (internals/log_semiring.py: * -> +, + -> logaddexp, ** n -> n *). */
void orc_evcalc_update(orc_evcalc *c, double n, double log_L_next) {
    double midL = log(0.5) + lae(log_L_next, c->log_L);
    double lnn = log(n), lnn1 = log(n + 1.0), lnn2 = log(n + 2.0);
    double T = -lae(0.0, -lnn);
    double t = -lnn1;
    double T2 = -lae(0.0, ORC_LOG2 - lnn);
    double t2 = ORC_LOG2 - lnn1 - lnn2;
    double tT = -lae(0.0, -lnn) - lnn2;
    double X = c->log_X_mean, X2 = c->log_X2_mean, Z = c->log_Z_mean, ZX = c->log_ZX_mean,
           Z2 = c->log_Z2_mean, dZ2 = c->log_dZ2_mean;
    double dZ = (X + t) + midL;
    double nX = X + T;
    double nX2 = X2 + T2;
    double nZ = lae(Z, dZ);
    double nZX = lae(ZX + T, (X2 + tT) + midL);
    double sq = 2.0 * midL;
    double nZ2 = lae(lae(Z2, ((ORC_LOG2 + ZX) + t) + midL), (X2 + t2) + sq);
    double ndZ2 = lae(dZ2, (X2 + t2) + sq);
    c->log_L = log_L_next;
    c->log_X_mean = nX;
    c->log_X2_mean = nX2;
    c->log_Z_mean = nZ;
    c->log_Z2_mean = nZ2;
    c->log_ZX_mean = nZX;
    c->log_dZ_mean = dZ;
    c->log_dZ2_mean = ndZ2;
}

/* compute_evidence_stats (shrinkage_statistics.py:131-157), static scan; per-sample
 * outputs optional (out may be NULL). */
void orc_compute_evidence_stats(const double *log_L, const double *num_live, long N, orc_evcalc *final,
                                orc_evcalc *out) {
    orc_evcalc c;
    orc_evcalc_init(&c);
    for (long i = 0; i < N; ++i) {
        orc_evcalc_update(&c, num_live[i], log_L[i]);
        if (out) out[i] = c;
    }
    *final = c;
}

/* linear_to_log_stats (internals/stats.py:55-74) */
void orc_linear_to_log_stats(double log_f_mean, double log_f2_mean, double *mu, double *var) {
    *mu = 2.0 * log_f_mean - 0.5 * log_f2_mean;
    double s = log_f2_mean - 2.0 * log_f_mean;
    const double eps = 2.220446049250313e-16;
    *var = s > eps ? s : eps;
    if (isnan(s)) *var = s;
}

/* sample_evidence (utils.py:433-484): S replicas of log Z with the shrinkage drawn instead
 * of averaged.  Replica s: keys split(split(key, S)[s], M); per sample i, in order,
 * log T = log(uniform(key_i)) / n_i (T ~ Beta(n_i, 1)), next X = X T,
 * dZ = (X - next X) L_i in LogSpace (signed_logaddexp, log_semiring.py:28-48), Z += dZ. */
void orc_sample_evidence(uint32_t k0, uint32_t k1, const long *num_live, const double *log_L, long M, int S,
                         double *log_Z_out) {
    okey key = {k0, k1};
    for (int s = 0; s < S; ++s) {
        okey ks = key_fold(key, (uint64_t)s);
        double log_Z = -INFINITY, log_X = 0.0;
        for (long i = 0; i < M; ++i) {
            okey ki = key_fold(ks, (uint64_t)i);
            double u = uniform_f64(ki, 0, 0.0, 1.0);
            double log_T = log(u) / (double)num_live[i];
            double log_nX = log_X + log_T;
            /* X - next X: signed_logaddexp(log_X, +1, log_nX, -1) */
            double delta = -fabs(log_nX - log_X);
            double amax = log_X > log_nX ? log_X : log_nX;
            double log_dX = isnan(delta) ? log_X + log_nX : amax + log1p(-exp(delta));
            double log_dZ = log_dX + log_L[i];
            log_Z = lae(log_Z, log_dZ);
            log_X = log_nX;
        }
        log_Z_out[s] = log_Z;
    }
}

/* ------------------------------------------------------- tree counting ---- */

/* count_crossed_edges (internals/tree_structure.py:33-108).  num_samples < 0 means the
 * static variant; otherwise the +inf-padded dynamic variant.  Outputs [N]. */
void orc_count_crossed_edges(const long *sender, const double *log_L, long N, long num_samples,
                             long *samples_indices, long *num_live_points) {
    double *nodes = (double *)malloc(sizeof(double) * (size_t)(N + 1));
    long *perm = (long *)malloc(sizeof(long) * (size_t)(N + 1));
    long *deg = (long *)calloc((size_t)(N + 1), sizeof(long));
    nodes[0] = -INFINITY;
    for (long i = 0; i < N; ++i) nodes[i + 1] = log_L[i];
    orc_stable_argsort(nodes, N + 1, perm);
    /* out_degree.at[max(sender, 0)].add(1): scatter updates outside [0, N] are dropped (jax) */
    for (long i = 0; i < N; ++i) {
        long sd = sender[i] > 0 ? sender[i] : 0;
        if (sd <= N) deg[sd] += 1;
    }
    long fake = num_samples >= 0 ? (N - num_samples) : 0;
    long stop = num_samples >= 0 ? num_samples : N + 1;
    long crossed = 1;
    long *cs = (long *)malloc(sizeof(long) * (size_t)(N + 1));
    for (long i = 0; i < N + 1; ++i) {
        if (i < stop) {
            crossed += deg[perm[i]] - 1;
            cs[i] = crossed;
        } else {
            cs[i] = fake; /* empty_fill */
        }
    }
    for (long i = 0; i < N; ++i) {
        samples_indices[i] = perm[i + 1] - 1;
        num_live_points[i] = cs[i] - fake;
    }
    free(nodes); free(perm); free(deg); free(cs);
}

/* ---------------------------------------------------------- termination ---- */

typedef struct {
    int has_ess; double ess;
    int has_evidence_uncert; double evidence_uncert;
    int has_dlogZ; double dlogZ;
    int has_max_samples; double max_samples;
    int has_max_nlik; double max_nlik;
    int has_log_L_contour; double log_L_contour;
    int has_efficiency; double efficiency_threshold;
    int has_rtol; double rtol;
    int has_atol; double atol;
    int has_peak_XL; double peak_XL_frac;
} orc_term_cond;

typedef struct {
    long num_samples_used;
    orc_evcalc ev;
    orc_evcalc ev_rem;
    long num_likelihood_evaluations;
    double log_L_contour;
    double efficiency;
    int plateau;
    int no_seed_points;
    double relative_spread;
    double absolute_spread;
    double peak_log_XL;
} orc_term_reg;

/* create_init_termination_register (nested_samplers/common/initialisation.py:87-108) */
void orc_term_reg_init(orc_term_reg *r) {
    memset(r, 0, sizeof(*r));
    orc_evcalc_init(&r->ev);
    orc_evcalc_init(&r->ev_rem);
    r->log_L_contour = -INFINITY;
    r->efficiency = 0.0;
    r->relative_spread = INFINITY;
    r->absolute_spread = INFINITY;
    r->peak_log_XL = -INFINITY;
}

/* determine_termination for a single TerminationCondition
 * (nested_samplers/common/termination.py:13-147). Returns done; *reason gets the bits. */
int orc_determine_termination(const orc_term_cond *tc, const orc_term_reg *r, long *reason) {
    int done = 0;
    long rs = 0;
#define SETBIT(cond, bit) do { if (cond) { done = 1; rs += (1L << (bit)); } } while (0)
    if (tc->has_max_samples) SETBIT((double)r->num_samples_used >= tc->max_samples, 0);
    if (tc->has_evidence_uncert) {
        double mu, var;
        orc_linear_to_log_stats(r->ev_rem.log_Z_mean, r->ev_rem.log_Z2_mean, &mu, &var);
        SETBIT(var <= tc->evidence_uncert * tc->evidence_uncert, 1);
    }
    if (tc->has_dlogZ) {
        double m1, v1, m0, v0;
        orc_linear_to_log_stats(r->ev_rem.log_Z_mean, r->ev_rem.log_Z2_mean, &m1, &v1);
        orc_linear_to_log_stats(r->ev.log_Z_mean, r->ev.log_Z2_mean, &m0, &v0);
        SETBIT((m1 - m0) < tc->dlogZ, 2);
    }
    if (tc->has_ess) {
        double ess = exp(2.0 * r->ev_rem.log_Z_mean - r->ev_rem.log_dZ2_mean);
        SETBIT(ess >= tc->ess, 3);
    }
    if (tc->has_max_nlik) SETBIT((double)r->num_likelihood_evaluations >= tc->max_nlik, 4);
    if (tc->has_log_L_contour) SETBIT(r->log_L_contour >= tc->log_L_contour, 5);
    if (tc->has_efficiency) SETBIT(r->efficiency < tc->efficiency_threshold, 6);
    SETBIT(r->plateau, 7);
    if (tc->has_rtol) SETBIT(r->relative_spread < tc->rtol, 8);
    if (tc->has_atol) SETBIT(r->absolute_spread < tc->atol, 9);
    SETBIT(r->no_seed_points, 10);
    if (tc->has_peak_XL) {
        double log_XL = r->ev.log_X_mean + r->ev.log_L;
        SETBIT(log_XL < r->peak_log_XL + log(tc->peak_XL_frac), 11);
    }
#undef SETBIT
    *reason = rs;
    return done;
}

/* --------------------------------------------------------- the NS run ---- */

typedef struct {
    int num_live_points;      /* n, already rounded (round_up_num_live_points) */
    int shell_size;           /* int(n * shell_fraction) */
    long max_samples;         /* store size, already rounded (round_up_max_samples) */
    double init_efficiency_threshold;
    orc_slice_cfg slice;
    int uniform_max_evals;    /* UniformSampler.max_likelihood_evals (100) */
} orc_ns_cfg;

typedef struct {
    /* store (SampleCollection, nested_samplers/common/types.py:116-121) */
    long *sender;
    double *log_L;
    double *U;
    long *nevals;
    int *phantom;
    long next_sample_idx;
    long num_samples;
    uint32_t key0, key1;
    long termination_reason;
    orc_term_reg reg;
    long iterations;
} orc_ns_state;

typedef struct {
    long *sender;
    double *U;
    double *log_Lc;
    double *log_L;
    long *nevals;
} live_set;

/* _add_samples_to_state (sharded_static.py:40-85) with dynamic_update_slice clamping. */
static void add_samples(orc_ns_state *st, long cap, int D, long cnt, const long *sender,
                        const double *log_L, const double *U, const long *nevals, int is_phantom) {
    if (cnt <= 0) return;
    long start = st->next_sample_idx;
    if (start > cap - cnt) start = cap - cnt;
    if (start < 0) start = 0;
    for (long i = 0; i < cnt; ++i) {
        st->sender[start + i] = sender[i];
        st->log_L[start + i] = log_L[i];
        memcpy(st->U + (start + i) * D, U + i * D, sizeof(double) * D);
        st->nevals[start + i] = nevals[i];
        st->phantom[start + i] = is_phantom;
    }
    st->next_sample_idx = (st->next_sample_idx + cnt) % cap;
    st->num_samples += cnt;
}

static void sort_live(live_set *lv, int n, int D) {
    long *perm = (long *)malloc(sizeof(long) * (size_t)n);
    orc_stable_argsort(lv->log_L, n, perm);
    long *s2 = (long *)malloc(sizeof(long) * (size_t)n);
    double *U2 = (double *)malloc(sizeof(double) * (size_t)n * D);
    double *c2 = (double *)malloc(sizeof(double) * (size_t)n);
    double *l2 = (double *)malloc(sizeof(double) * (size_t)n);
    long *e2 = (long *)malloc(sizeof(long) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        long p = perm[i];
        s2[i] = lv->sender[p];
        memcpy(U2 + (size_t)i * D, lv->U + p * D, sizeof(double) * D);
        c2[i] = lv->log_Lc[p];
        l2[i] = lv->log_L[p];
        e2[i] = lv->nevals[p];
    }
    memcpy(lv->sender, s2, sizeof(long) * n);
    memcpy(lv->U, U2, sizeof(double) * (size_t)n * D);
    memcpy(lv->log_Lc, c2, sizeof(double) * n);
    memcpy(lv->log_L, l2, sizeof(double) * n);
    memcpy(lv->nevals, e2, sizeof(long) * n);
    free(perm); free(s2); free(U2); free(c2); free(l2); free(e2);
}

/* _collect_shell (sharded_static.py:210-324). sampler: 0 uniform, 1 slice. */
static void collect_shell(const orc_model *m, const orc_ns_cfg *cfg, orc_ns_state *st, live_set *lv,
                          int sampler) {
    int n = cfg->num_live_points, s = cfg->shell_size, D = m->D;
    int K = sampler == 1 ? cfg->slice.num_phantom : 0;
    long cap = cfg->max_samples;
    /* discard the shell */
    long *d_sender = (long *)malloc(sizeof(long) * s);
    double *d_logL = (double *)malloc(sizeof(double) * s);
    memcpy(d_sender, lv->sender, sizeof(long) * s);
    memcpy(d_logL, lv->log_L, sizeof(double) * s);
    add_samples(st, cap, D, s, lv->sender, lv->log_L, lv->U, lv->nevals, 0);
    okey key = {st->key0, st->key1};
    okey nkey = key_fold(key, 0), sample_key = key_fold(key, 1);
    st->key0 = nkey.k0; st->key1 = nkey.k1;
    double Lstar = lv->log_L[s - 1];
    /* get_samples: split(sample_key, s); chain c uses keys[c] (sampler state = sorted live) */
    double *nU = (double *)malloc(sizeof(double) * (size_t)s * D);
    double *nL = (double *)malloc(sizeof(double) * s);
    long *nE = (long *)malloc(sizeof(long) * s);
    double *pU = (double *)malloc(sizeof(double) * (size_t)s * (K > 0 ? K : 1) * D);
    double *pL = (double *)malloc(sizeof(double) * (size_t)s * (K > 0 ? K : 1));
    for (int c = 0; c < s; ++c) {
        okey kc = key_fold(sample_key, (uint64_t)c);
        if (sampler == 1)
            orc_slice_get_sample(m, &cfg->slice, kc.k0, kc.k1, Lstar, lv->U, lv->log_L, n, nU + (size_t)c * D,
                                 &nL[c], &nE[c], pU + (size_t)c * K * D, pL + (size_t)c * K);
        else
            orc_uniform_get_sample(m, kc.k0, kc.k1, Lstar, cfg->uniform_max_evals, nU + (size_t)c * D, &nL[c],
                                   &nE[c]);
    }
    long sender_idx = st->next_sample_idx - 1;
    for (int c = 0; c < s; ++c) {
        lv->sender[c] = sender_idx;
        memcpy(lv->U + (size_t)c * D, nU + (size_t)c * D, sizeof(double) * D);
        lv->log_L[c] = nL[c];
        lv->log_Lc[c] = Lstar;
        lv->nevals[c] = nE[c];
    }
    sort_live(lv, n, D);
    if (K > 0) {
        long np = (long)s * K;
        long *ps = (long *)malloc(sizeof(long) * np);
        long *pe = (long *)calloc((size_t)(np > 0 ? np : 1), sizeof(long));
        for (long i = 0; i < np; ++i) ps[i] = sender_idx;
        add_samples(st, cap, D, np, ps, pL, pU, pe, 1);
        free(ps); free(pe);
    }
    /* termination register update (sharded_static.py:281-323) */
    orc_term_reg *r = &st->reg;
    orc_evcalc ev = r->ev;
    for (int i = 0; i < s; ++i) orc_evcalc_update(&ev, (double)n, d_logL[i]);
    orc_evcalc evr = ev;
    for (int i = 0; i < n; ++i) orc_evcalc_update(&evr, (double)(n - i), lv->log_L[i]);
    long sumE = 0, sumLive = 0;
    for (int c = 0; c < s; ++c) sumE += nE[c];
    for (int i = 0; i < n; ++i) sumLive += lv->nevals[i];
    double peak = ev.log_X_mean + ev.log_L;
    double old_peak = r->peak_log_XL;
    r->num_samples_used = st->num_samples;
    r->ev = ev;
    r->ev_rem = evr;
    r->num_likelihood_evaluations += sumE;
    r->log_L_contour = Lstar;
    r->efficiency = (double)n / (double)sumLive;
    int plateau = 1;
    for (int i = 0; i < n; ++i) if (!(lv->log_L[i] == lv->log_L[0])) { plateau = 0; break; }
    r->plateau = plateau;
    r->absolute_spread = fabs(lv->log_L[n - 1] - lv->log_L[0]);
    r->relative_spread = 2.0 * r->absolute_spread / fabs(lv->log_L[0] + lv->log_L[n - 1]);
    r->no_seed_points = lv->log_L[s - 1] >= lv->log_L[n - 1];
    r->peak_log_XL = (isnan(peak) || isnan(old_peak)) ? NAN : (peak > old_peak ? peak : old_peak);
    free(d_sender); free(d_logL); free(nU); free(nL); free(nE); free(pU); free(pL);
}

/* _main_ns_thread (sharded_static.py:427-574). */
static long main_ns_thread(const orc_model *m, const orc_ns_cfg *cfg, orc_ns_state *st, live_set *lv,
                           orc_term_cond tc, int sampler, long max_iterations) {
    int s = cfg->shell_size, n = cfg->num_live_points;
    int K = sampler == 1 ? cfg->slice.num_phantom : 0;
    long space = (long)s * (1 + K);
    if (tc.has_max_samples) {
        double lim = (double)(cfg->max_samples - space);
        if (lim < tc.max_samples) tc.max_samples = lim;
    }
    st->reg.no_seed_points = lv->log_L[s - 1] >= lv->log_L[n - 1];
    long reason = 0;
    long it = 0;
    while (!orc_determine_termination(&tc, &st->reg, &reason)) {
        if (max_iterations > 0 && it >= max_iterations) break;
        okey key = {st->key0, st->key1};
        okey k1 = key_fold(key, 0);
        st->key0 = k1.k0; st->key1 = k1.k1;
        collect_shell(m, cfg, st, lv, sampler);
        okey key2 = {st->key0, st->key1};
        okey k3 = key_fold(key2, 0);
        st->key0 = k3.k0; st->key1 = k3.k1;
        ++it;
    }
    orc_determine_termination(&tc, &st->reg, &reason);
    st->iterations += it;
    return reason;
}

/* create_init_state (nested_samplers/common/initialisation.py:20-84). */
static void create_init_state(const orc_model *m, const orc_ns_cfg *cfg, orc_ns_state *st, live_set *lv,
                              uint32_t k0, uint32_t k1) {
    int n = cfg->num_live_points, D = m->D;
    long cap = cfg->max_samples;
    for (long i = 0; i < cap; ++i) {
        st->sender[i] = 0;
        st->log_L[i] = INFINITY;
        st->nevals[i] = 0;
        st->phantom[i] = 0;
    }
    memset(st->U, 0, sizeof(double) * (size_t)cap * D);
    okey key = {k0, k1};
    okey nkey = key_fold(key, 0), sample_key = key_fold(key, 1);
    for (int i = 0; i < n; ++i) {
        okey ki = key_fold(sample_key, (uint64_t)i);
        orc_uniform_get_sample(m, ki.k0, ki.k1, -INFINITY, 0, lv->U + (size_t)i * D, &lv->log_L[i], &lv->nevals[i]);
        lv->sender[i] = 0;
        lv->log_Lc[i] = -INFINITY;
    }
    sort_live(lv, n, D);
    st->key0 = nkey.k0;
    st->key1 = nkey.k1;
    st->next_sample_idx = 0;
    st->num_samples = 0;
    st->iterations = 0;
}

/* ShardedStaticNestedSampler._run (sharded_static.py:775-851), with the caller's
 * term_cond already clamped as NestedSampler.__call__ does (public.py:153-170).
 * The store buffers in st must hold cfg->max_samples entries.  Returns the
 * termination reason.  The final live set is also returned through lv_out_* if
 * non-NULL (only the init live set when init_only != 0). */
long orc_ns_run(const orc_model *m, const orc_ns_cfg *cfg, const orc_term_cond *tc, uint32_t k0,
                uint32_t k1, orc_ns_state *st, long max_iterations, int init_only, double *live_U_out,
                double *live_logL_out) {
    int n = cfg->num_live_points, D = m->D;
    live_set lv;
    lv.sender = (long *)malloc(sizeof(long) * n);
    lv.U = (double *)malloc(sizeof(double) * (size_t)n * D);
    lv.log_Lc = (double *)malloc(sizeof(double) * n);
    lv.log_L = (double *)malloc(sizeof(double) * n);
    lv.nevals = (long *)malloc(sizeof(long) * n);
    create_init_state(m, cfg, st, &lv, k0, k1);
    orc_term_reg_init(&st->reg);
    long reason = 0;
    if (!init_only) {
        if (cfg->init_efficiency_threshold > 0.0) {
            orc_term_cond utc;
            memset(&utc, 0, sizeof(utc));
            utc.has_efficiency = 1; utc.efficiency_threshold = cfg->init_efficiency_threshold;
            utc.has_dlogZ = 1; utc.dlogZ = 0.0;
            utc.has_max_samples = 1; utc.max_samples = (double)cfg->max_samples;
            main_ns_thread(m, cfg, st, &lv, utc, 0, max_iterations);
        }
        reason = main_ns_thread(m, cfg, st, &lv, *tc, 1, max_iterations);
        add_samples(st, cfg->max_samples, D, n, lv.sender, lv.log_L, lv.U, lv.nevals, 0);
    }
    if (live_U_out) memcpy(live_U_out, lv.U, sizeof(double) * (size_t)n * D);
    if (live_logL_out) memcpy(live_logL_out, lv.log_L, sizeof(double) * n);
    st->termination_reason = reason;
    free(lv.sender); free(lv.U); free(lv.log_Lc); free(lv.log_L); free(lv.nevals);
    return reason;
}

/* One shell of the slice sampler from a given live set (get_samples,
 * sharded_static.py:88-129), for chain-level parity checks. */
void orc_slice_shell(const orc_model *m, const orc_slice_cfg *cfg, uint32_t k0, uint32_t k1, double Lstar,
                     const double *live_U, const double *live_logL, long n, long num_chains, double *U_out,
                     double *logL_out, long *nevals_out) {
    okey key = {k0, k1};
    int D = m->D, K = cfg->num_phantom;
    double *pU = (double *)malloc(sizeof(double) * (size_t)(K > 0 ? K : 1) * D);
    double *pL = (double *)malloc(sizeof(double) * (size_t)(K > 0 ? K : 1));
    for (long c = 0; c < num_chains; ++c) {
        okey kc = key_fold(key, (uint64_t)c);
        orc_slice_get_sample(m, cfg, kc.k0, kc.k1, Lstar, live_U, live_logL, n, U_out + c * D, &logL_out[c],
                             &nevals_out[c], pU, pL);
    }
    free(pU); free(pL);
}

/* orc_slice_shell that also reports, per chain, the smallest |log L - L*| over its accept
 * tests: a chain of another implementation whose likelihoods differ by less than that from
 * these FP64 ones makes every decision this chain makes. */
void orc_slice_shell_margin(const orc_model *m, const orc_slice_cfg *cfg, uint32_t k0, uint32_t k1, double Lstar,
                            const double *live_U, const double *live_logL, long n, long num_chains, double *U_out,
                            double *logL_out, long *nevals_out, double *margin_out) {
    okey key = {k0, k1};
    int D = m->D, K = cfg->num_phantom;
    double *pU = (double *)malloc(sizeof(double) * (size_t)(K > 0 ? K : 1) * D);
    double *pL = (double *)malloc(sizeof(double) * (size_t)(K > 0 ? K : 1));
    for (long c = 0; c < num_chains; ++c) {
        okey kc = key_fold(key, (uint64_t)c);
        margin_out[c] = INFINITY;
        orc_margin_sink = &margin_out[c];
        orc_slice_get_sample(m, cfg, kc.k0, kc.k1, Lstar, live_U, live_logL, n, U_out + c * D, &logL_out[c],
                             &nevals_out[c], pU, pL);
        orc_margin_sink = NULL;
    }
    free(pU); free(pL);
}

/* ------------------------------------------------------------ results ---- */

typedef struct {
    double log_Z_mean, log_Z_uncert, ESS, H_mean;
    long total_num_samples, total_phantom_samples, total_num_likelihood_evaluations;
    double log_efficiency;
} orc_results;

/* _to_results with trim=True (sharded_static.py:652-773).  Per-sample outputs are in
 * sorted order; X outputs are U->X transformed samples. */
void orc_to_results(const orc_model *m, const orc_ns_state *st, long cap, orc_results *res,
                    long *samples_indices, long *num_live, double *log_L_sorted, double *log_dp_mean,
                    double *log_X_mean, double *U_sorted) {
    int D = m->D;
    long N = st->num_samples < cap ? st->num_samples : cap;
    orc_count_crossed_edges(st->sender, st->log_L, N, -1, samples_indices, num_live);
    double *nl = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    orc_evcalc *per = (orc_evcalc *)malloc(sizeof(orc_evcalc) * (size_t)(N > 0 ? N : 1));
    long total_evals = 0, total_phantom = 0;
    for (long i = 0; i < N; ++i) {
        long si = samples_indices[i];
        log_L_sorted[i] = st->log_L[si];
        nl[i] = (double)num_live[i];
        total_evals += st->nevals[si];
        total_phantom += st->phantom[i] ? 1 : 0;
        if (U_sorted) memcpy(U_sorted + i * D, st->U + si * D, sizeof(double) * D);
    }
    orc_evcalc fin;
    orc_compute_evidence_stats(log_L_sorted, nl, N, &fin, per);
    double mu, var;
    orc_linear_to_log_stats(fin.log_Z_mean, fin.log_Z2_mean, &mu, &var);
    double uncert = sqrt(var);
    double pf = (double)total_phantom / (double)N;
    double k = pf / (1.0 - pf);
    uncert *= sqrt(1.0 + k);
    double ess = exp(2.0 * fin.log_Z_mean - fin.log_dZ2_mean) / (1.0 + k);
    /* normalise_log_space(log_dZ_mean) with a logsumexp (max-shifted) */
    double mx = -INFINITY;
    for (long i = 0; i < N; ++i) if (per[i].log_dZ_mean > mx) mx = per[i].log_dZ_mean;
    double se = 0;
    for (long i = 0; i < N; ++i) se += exp(per[i].log_dZ_mean - mx);
    double norm = isinf(mx) ? mx : mx + log(se);
    double h1 = 0, h2 = 0;
    for (long i = 0; i < N; ++i) {
        double ld = isinf(norm) && norm < 0 ? -INFINITY : per[i].log_dZ_mean - norm;
        log_dp_mean[i] = ld;
        log_X_mean[i] = per[i].log_X_mean;
        double L = isinf(ld) && ld < 0 ? 0.0 : log_L_sorted[i];
        h1 += exp(ld) * L;
        h2 += exp(ld) * (-per[i].log_X_mean);
    }
    double H_inst = -(h1 - mu);
    double H_stab = -h2;
    res->log_Z_mean = mu;
    res->log_Z_uncert = uncert;
    res->ESS = ess;
    res->H_mean = isfinite(H_inst) ? H_inst : H_stab;
    res->total_num_samples = N;
    res->total_phantom_samples = total_phantom;
    res->total_num_likelihood_evaluations = total_evals;
    res->log_efficiency = log((double)N) - log((double)total_evals);
    free(nl); free(per);
}

/* ------------------------------------------- evidence-gradient oracle ---- */

/* Reweighted fixed-dead-point evidence (experimental/evidence_maximisation.py:151-160, :213):
 * log Z(theta) = logsumexp_i(log L_theta(U_i) + log w_i), log w_i = log_dp_i - log L_i + log Z.
 * Linear-Gaussian family with prior w = tau * ndtri(U); theta = (log tau, log sigma).
 * Returns log Z(theta) and its exact gradient (FP64). */
void orc_blr_reweighted(const double *Phi, const double *y, int N, int P, const double *U, const double *log_w,
                        long M, double log_tau, double log_sigma, double *log_Z, double *grad) {
    double tau = exp(log_tau), sigma = exp(log_sigma);
    double *lv = (double *)malloc(sizeof(double) * (size_t)(M > 0 ? M : 1));
    double *g_tau = (double *)malloc(sizeof(double) * (size_t)(M > 0 ? M : 1));
    double *g_sig = (double *)malloc(sizeof(double) * (size_t)(M > 0 ? M : 1));
    double w[256], z[256];
    double *r = (double *)malloc(sizeof(double) * (size_t)N);
    for (long i = 0; i < M; ++i) {
        for (int j = 0; j < P; ++j) {
            z[j] = ORC_SQRT2 * orc_erfinv(2.0 * U[i * P + j] - 1.0);
            w[j] = tau * z[j];
        }
        double ss = 0;
        for (int a = 0; a < N; ++a) {
            double acc = y[a];
            for (int j = 0; j < P; ++j) acc -= Phi[(size_t)a * P + j] * w[j];
            r[a] = acc;
            ss += acc * acc;
        }
        double ll = -0.5 * N * log(2.0 * ORC_PI * sigma * sigma) - 0.5 * ss / (sigma * sigma);
        /* d ll / d log sigma = -N + ss / sigma^2 */
        g_sig[i] = -N + ss / (sigma * sigma);
        /* d ll / d log tau = (1/sigma^2) r . (Phi w) */
        double rp = 0;
        for (int a = 0; a < N; ++a) {
            double pw = 0;
            for (int j = 0; j < P; ++j) pw += Phi[(size_t)a * P + j] * w[j];
            rp += r[a] * pw;
        }
        g_tau[i] = rp / (sigma * sigma);
        lv[i] = ll + log_w[i];
    }
    double mx = -INFINITY;
    for (long i = 0; i < M; ++i) if (lv[i] > mx) mx = lv[i];
    double se = 0, gt = 0, gs = 0;
    for (long i = 0; i < M; ++i) {
        double e = exp(lv[i] - mx);
        se += e;
        gt += e * g_tau[i];
        gs += e * g_sig[i];
    }
    *log_Z = mx + log(se);
    grad[0] = gt / se;
    grad[1] = gs / se;
    free(lv); free(g_tau); free(g_sig); free(r);
}

/* --------------------------------------------- threaded CPU baseline ---- */

typedef struct {
    const orc_model *models;
    const orc_ns_cfg *cfgs;
    const orc_term_cond *tcs;
    const uint32_t *keys;
    int num_runs;
    int next;
    pthread_mutex_t mu;
    double *log_Z;
    long *nevals;
    long *reasons;
    long max_iterations;
    double *seconds;
    long *iterations;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *j = (batch_job *)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int r = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (r >= j->num_runs) break;
        const orc_model *m = &j->models[r];
        const orc_ns_cfg *cfg = &j->cfgs[r];
        long cap = cfg->max_samples;
        orc_ns_state st;
        memset(&st, 0, sizeof(st));
        st.sender = (long *)malloc(sizeof(long) * cap);
        st.log_L = (double *)malloc(sizeof(double) * cap);
        st.U = (double *)malloc(sizeof(double) * (size_t)cap * m->D);
        st.nevals = (long *)malloc(sizeof(long) * cap);
        st.phantom = (int *)malloc(sizeof(int) * cap);
        struct timespec t0, t1;
        clock_gettime(CLOCK_MONOTONIC, &t0);
        j->reasons[r] = orc_ns_run(m, cfg, &j->tcs[r], j->keys[2 * r], j->keys[2 * r + 1], &st, j->max_iterations, 0,
                                   NULL, NULL);
        clock_gettime(CLOCK_MONOTONIC, &t1);
        if (j->seconds) j->seconds[r] = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
        if (j->iterations) j->iterations[r] = st.iterations;
        long N = st.num_samples < cap ? st.num_samples : cap;
        long *si = (long *)malloc(sizeof(long) * N), *nl = (long *)malloc(sizeof(long) * N);
        double *ls = (double *)malloc(sizeof(double) * N), *dp = (double *)malloc(sizeof(double) * N),
               *lx = (double *)malloc(sizeof(double) * N);
        orc_results res;
        orc_to_results(m, &st, cap, &res, si, nl, ls, dp, lx, NULL);
        j->log_Z[r] = res.log_Z_mean;
        j->nevals[r] = res.total_num_likelihood_evaluations;
        free(si); free(nl); free(ls); free(dp); free(lx);
        free(st.sender); free(st.log_L); free(st.U); free(st.nevals); free(st.phantom);
    }
    return NULL;
}

/* Runs independent NS problems on num_threads host threads (CPU baseline). */
void orc_ns_run_batch(const orc_model *models, const orc_ns_cfg *cfgs, const orc_term_cond *tcs,
                      const uint32_t *keys, int num_runs, int num_threads, double *log_Z, long *nevals,
                      long *reasons, long max_iterations, double *seconds, long *iterations) {
    batch_job j;
    j.models = models; j.cfgs = cfgs; j.tcs = tcs; j.keys = keys; j.num_runs = num_runs; j.next = 0;
    j.log_Z = log_Z; j.nevals = nevals; j.reasons = reasons;
    j.max_iterations = max_iterations; j.seconds = seconds; j.iterations = iterations;
    pthread_mutex_init(&j.mu, NULL);
    if (num_threads < 1) num_threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * num_threads);
    for (int t = 0; t < num_threads; ++t) pthread_create(&th[t], NULL, batch_worker, &j);
    for (int t = 0; t < num_threads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&j.mu);
}

/* =====================================================================================
 * fp32 kernel-arithmetic mode.
 *
 * The device chains compute in fp32 (U, directions, interval, log-likelihoods relative to
 * the run's FP64 offset) and use the elementary functions of gbns_fmath.h, which are built
 * from correctly rounded IEEE operations only.  This section restates the same chain
 * algorithm (uni_slice_sampler.py:114-273, :343-441; bases.py:63-75; random.py:34-84) in
 * exactly the kernels' fp32 operation order, so that each chain's evaluation count,
 * accepted point and log-likelihood can be compared bit for bit.  It differs from the FP64
 * restatement above only in precision and in the order of the fp32 reductions the kernels
 * perform (the likelihood's sum of squares, the direction's and the gradient's norms, the
 * reflection's dot product: sequential per thread, or a butterfly across the 32 lanes of a
 * warp in the warp-cooperative correlated-Gaussian kernel); the RNG stream, the seed choice, the
 * accept test and the shrink rule are the same.
 * ===================================================================================== */

#include "../jaxns_gb300/csrc/gbns_fmath.h"

typedef struct {
    int D;
    int family;               /* ORC_LIK_MVN or ORC_LIK_SHELLS */
    const int *prior_kind;    /* [D] */
    const float *prior_a;     /* [D] fp32, as the device holds it */
    const float *prior_b;     /* [D] */
    const float *p;           /* fp32 parameters in the device layout: MVN [mu, Linv (row-major lower), c0];
                                 shells [c1, c2, R, w, norm] */
    int variant;              /* 0: one thread per chain; 32 / 64: warp-cooperative MVN kernel of that DMAX */
} orc32_model;

static inline float o32_uniform(okey k) { return gbns_fm_u64_to_float(bits64(k, 0) >> 12) * 0x1p-52f; }

static inline float o32_quantile(const orc32_model *m, int j, float u) {
    if (m->prior_kind[j] == ORC_PRIOR_UNIFORM) return fmaf(m->prior_b[j], u, m->prior_a[j]);
    return fmaf(m->prior_b[j], gbns_fm_ndtri(u), m->prior_a[j]);
}

/* Sum of the squared rows z_i (i < D) of the warp kernel's register tile: rows 8g..8g+7
 * (and 32+8g.. for DMAX 64) summed per lane group g in order, then (S0 + S1) + (S2 + S3). */
static float o32_warp_sumsq(const float *z, int D, int dmax) {
    float S[4];
    for (int g = 0; g < 4; ++g) {
        float s = 0.0f;
        for (int p = 0; p < dmax / 32; ++p) {
            if (32 * p >= D) continue;
            for (int rr = 0; rr < 8; ++rr) {
                int row = 32 * p + 8 * g + rr;
                float a = row < D ? z[row] : 0.0f;
                s = fmaf(a, a, s);
            }
        }
        S[g] = s;
    }
    return (S[0] + S[1]) + (S[2] + S[3]);
}

/* 32-lane butterfly sum (__shfl_xor over 16, 8, 4, 2, 1); every lane ends with this value */
static float o32_butterfly(const float *a_in) {
    float a[32], b[32];
    memcpy(a, a_in, sizeof a);
    for (int o = 16; o > 0; o >>= 1) {
        for (int l = 0; l < 32; ++l) b[l] = a[l] + a[l ^ o];
        memcpy(a, b, sizeof a);
    }
    return a[0];
}

/* log L(u) - offset, fp32, of the point u = u0 + t d (Model.forward, framework/model.py:167;
 * NaN -> -inf, framework/ops.py:323-325) */
static float o32_loglik_line(const orc32_model *m, const float *u0, const float *d, float t) {
    int D = m->D;
    float x[128];
    for (int j = 0; j < D; ++j) x[j] = o32_quantile(m, j, fmaf(t, d[j], u0[j]));
    float v;
    if (m->family == ORC_LIK_MVN) {
        const float *mu = m->p, *Linv = m->p + D;
        float z[128];
        for (int j = 0; j < D; ++j) x[j] = x[j] - mu[j];
        for (int i = 0; i < D; ++i) {
            float acc = 0.0f;
            for (int j = 0; j <= i; ++j) acc = fmaf(Linv[i * D + j], x[j], acc);
            z[i] = acc;
        }
        float s;
        if (m->variant == 0) {
            s = 0.0f;
            for (int i = 0; i < D; ++i) s = fmaf(z[i], z[i], s);
        } else {
            s = o32_warp_sumsq(z, D, m->variant);
        }
        v = -0.5f * s;
    } else {
        const float *c1 = m->p, *c2 = m->p + D;
        float R = m->p[2 * D], w = m->p[2 * D + 1];
        float r1 = 0.0f, r2 = 0.0f;
        for (int j = 0; j < D; ++j) {
            float e1 = x[j] - c1[j], e2 = x[j] - c2[j];
            r1 = fmaf(e1, e1, r1);
            r2 = fmaf(e2, e2, r2);
        }
        float iw = 1.0f / w; /* the kernels multiply by the width's reciprocal */
        float z1 = (sqrtf(r1) - R) * iw, z2 = (sqrtf(r2) - R) * iw;
        float s1 = -0.5f * z1 * z1, s2 = -0.5f * z2 * z2;
        float mx = fmaxf(s1, s2), dd = s1 - s2;
        v = (dd != dd) ? s1 + s2 : mx + gbns_fm_log1p(gbns_fm_exp(-fabsf(dd)));
    }
    return (v != v) ? -INFINITY : v;
}

float orc32_forward(const orc32_model *m, const float *U) {
    float zero[128];
    memset(zero, 0, sizeof zero);
    return o32_loglik_line(m, U, zero, 0.0f);
}

void orc32_forward_batch(const orc32_model *m, const float *U, long B, float *out) {
    for (long b = 0; b < B; ++b) out[b] = orc32_forward(m, U + b * m->D);
}

/* U-space gradient of log L - offset in the thread kernel's fp32 arithmetic (jax.grad of
 * Model.forward through the prior quantile: Uniform dx/du = b, Normal dx/du = b sqrt(2 pi)
 * exp(z^2 / 2)); correlated Gaussian -Linv^T Linv (x - mu), shells the softmax-weighted radial
 * terms. */
static void o32_grad_u(const orc32_model *m, const float *u, float *g) {
    int D = m->D;
    float x[128], dxdu[128];
    for (int j = 0; j < D; ++j) {
        if (m->prior_kind[j] == ORC_PRIOR_UNIFORM) {
            x[j] = fmaf(m->prior_b[j], u[j], m->prior_a[j]);
            dxdu[j] = m->prior_b[j];
        } else {
            float z = gbns_fm_ndtri(u[j]);
            x[j] = fmaf(m->prior_b[j], z, m->prior_a[j]);
            dxdu[j] = m->prior_b[j] * 2.5066282746310002f * gbns_fm_exp(0.5f * z * z);
        }
    }
    if (m->family == ORC_LIK_MVN) {
        const float *mu = m->p, *Linv = m->p + D;
        float e[128], zz[128];
        for (int j = 0; j < D; ++j) e[j] = x[j] - mu[j];
        for (int i = 0; i < D; ++i) {
            float acc = 0.0f;
            for (int j = 0; j <= i; ++j) acc = fmaf(Linv[i * D + j], e[j], acc);
            zz[i] = acc;
        }
        for (int q = 0; q < D; ++q) {
            float acc = 0.0f;
            for (int i = q; i < D; ++i) acc = fmaf(Linv[i * D + q], zz[i], acc);
            g[q] = -acc * dxdu[q];
        }
    } else {
        const float *c1 = m->p, *c2 = m->p + D;
        float R = m->p[2 * D], w = m->p[2 * D + 1];
        float r1 = 0.f, r2 = 0.f;
        for (int j = 0; j < D; ++j) {
            float e1 = x[j] - c1[j], e2 = x[j] - c2[j];
            r1 = fmaf(e1, e1, r1);
            r2 = fmaf(e2, e2, r2);
        }
        r1 = sqrtf(r1);
        r2 = sqrtf(r2);
        float z1 = (r1 - R) / w, z2 = (r2 - R) / w;
        float s1 = -0.5f * z1 * z1, s2 = -0.5f * z2 * z2, mx = fmaxf(s1, s2);
        float q1 = gbns_fm_exp(s1 - mx), q2 = gbns_fm_exp(s2 - mx), tot = q1 + q2;
        float f1 = (q1 / tot) * (-z1 / w) / r1, f2 = (q2 / tot) * (-z2 / w) / r2;
        for (int j = 0; j < D; ++j) g[j] = (f1 * (x[j] - c1[j]) + f2 * (x[j] - c2[j])) * dxdu[j];
    }
}

/* sum over the dimensions of p_j q_j in the order of the kernel that runs the chain: one fmaf
 * chain in dimension order (thread per chain), or, in the warp-cooperative kernel, lane l
 * holding dimensions l and l + 32 forms fmaf(p_l, q_l, p_{l+32} q_{l+32}) and the 32 lanes
 * are summed by the xor butterfly.  Used for the gradient's norm and the reflection's dot
 * product and norm (uni_slice_sampler.py:202-214, :255-269). */
static float o32_dot_dims(const orc32_model *m, const float *p, const float *q) {
    int D = m->D;
    if (m->variant == 0) {
        float s = 0.0f;
        for (int j = 0; j < D; ++j) s = fmaf(p[j], q[j], s);
        return s;
    }
    float a[32];
    for (int l = 0; l < 32; ++l) {
        float p0 = l < D ? p[l] : 0.0f, q0 = l < D ? q[l] : 0.0f;
        int hi = m->variant > 32 && l + 32 < D;
        float p1 = hi ? p[l + 32] : 0.0f, q1 = hi ? q[l + 32] : 0.0f;
        a[l] = fmaf(p0, q0, p1 * q1);
    }
    return o32_butterfly(a);
}

/* _sample_direction (uni_slice_sampler.py:23-38): D normals, normalised by one reciprocal of
 * the norm (sum of squares sequential per thread, or the warp kernel's butterfly). */
static void o32_direction(const orc32_model *m, okey k, float *d) {
    int D = m->D;
    if (D == 1) { d[0] = 1.0f; return; }
    float v[128];
    for (int j = 0; j < D; ++j) v[j] = gbns_fm_normal_from_mantissa(bits64(k, (uint64_t)j) >> 12);
    float ss;
    if (m->variant == 0) {
        ss = 0.0f;
        for (int j = 0; j < D; ++j) ss = fmaf(v[j], v[j], ss);
    } else {
        float a[32];
        for (int l = 0; l < 32; ++l) {
            float v0 = l < D ? v[l] : 0.0f;
            float v1 = (m->variant > 32 && l + 32 < D) ? v[l + 32] : 0.0f;
            a[l] = fmaf(v1, v1, v0 * v0);
        }
        ss = o32_butterfly(a);
    }
    float inv = 1.0f / sqrtf(ss);
    for (int j = 0; j < D; ++j) d[j] = v[j] * inv;
}

/* linspace(0.5, 1, S)[j] in fp32 */
static float o32_alpha(int j, int S) {
    if (S == 1) return 0.5f;
    if (j == S - 1) return 1.0f;
    float step = (float)j / (float)(S - 1);
    return 0.5f * (1.0f - step) + step;
}

/* One chain (UniDimSliceSampler.get_sample) in the kernels' fp32 arithmetic: chain key kc =
 * split(sample_key, s)[c]; returns the accepted point, its log L (relative) and the number
 * of evaluations.  Phantoms: [K, D] and [K]. */
void orc32_slice_chain(const orc32_model *m, const orc_slice_cfg *cfg, uint32_t k0, uint32_t k1, float Lstar,
                       const float *live_U, const float *live_L, long n, long max_evals_per_slice, float *U_out,
                       float *L_out, long *E_out, float *ph_U, float *ph_L) {
    int D = m->D, S = cfg->num_slices, K = cfg->num_phantom;
    okey kc = {k0, k1};
    okey chain_key = key_fold(kc, 0), seed_key = key_fold(kc, 1);
    /* m = #live points above the contour (the live set is sorted ascending) */
    long lo = 0, hi = n;
    while (lo < hi) {
        long mid = (lo + hi) >> 1;
        if (live_L[mid] > Lstar) hi = mid; else lo = mid + 1;
    }
    long mm = n - lo, idx = 0;
    if (mm > 0) {
        /* resample_indicies (random.py:34-75) in its exact integer form k = ceil(m (1 - U)) */
        uint64_t M52 = bits64(seed_key, 0) >> 12;
        uint64_t q = (1ull << 52) - M52;
        unsigned __int128 prod = (unsigned __int128)(uint64_t)mm * q;
        uint64_t kk = (uint64_t)(prod >> 52);
        if ((uint64_t)prod & ((1ull << 52) - 1)) kk += 1;
        idx = (n - mm) + (long)kk - 1;
    }
    float u0[128], d[128];
    memcpy(u0, live_U + idx * D, sizeof(float) * D);
    float logL0 = live_L[idx];
    okey slices_key = key_fold(chain_key, 1);
    o32_direction(m, key_fold(chain_key, 0), d);
    long total = 0;
    for (int j = 0; j < S; ++j) {
        okey B = key_fold(slices_key, (uint64_t)j);
        okey ck = key_fold(B, 0), tk = key_fold(B, 2), after = key_fold(B, 3);
        float alpha = o32_alpha(j, S);
        int climb = 0;
        if (cfg->gradient_slice) {
            /* gradient_slice (uni_slice_sampler.py:202-214) */
            float g[128];
            o32_grad_u(m, u0, g);
            ++total;
            float gn = sqrtf(o32_dot_dims(m, g, g));
            if (gn != 0.0f && isfinite(gn)) {
                climb = 1;
                for (int q = 0; q < D; ++q) d[q] = g[q] / gn;
            }
        }
        /* _slice_bounds (uni_slice_sampler.py:41-64) with one reciprocal per component */
        float t1r = INFINITY, t1l = -INFINITY, t0r = INFINITY, t0l = -INFINITY;
        for (int q = 0; q < D; ++q) {
            float rc = 1.0f / d[q];
            float t1 = (1.0f - u0[q]) * rc, t0 = -u0[q] * rc;
            t1r = fminf(t1r, t1 >= 0.f ? t1 : INFINITY);
            t1l = fmaxf(t1l, t1 <= 0.f ? t1 : -INFINITY);
            t0r = fminf(t0r, t0 >= 0.f ? t0 : INFINITY);
            t0l = fmaxf(t0l, t0 <= 0.f ? t0 : -INFINITY);
        }
        float right = fminf(t0r, t1r), left = climb ? 0.0f : fmaxf(t0l, t1l);
        long in_slice = 0;
        float t = 0.0f, logL;
        for (;;) {
            float u = o32_uniform(tk);
            t = fmaf(u, right - left, left);
            logL = o32_loglik_line(m, u0, d, t);
            ++total;
            ++in_slice;
            int accept = (logL > Lstar) || ((logL0 == Lstar) && (logL == Lstar));
            if (accept || in_slice >= max_evals_per_slice) break;
            /* _shrink_interval (uni_slice_sampler.py:92-111) and the next pick */
            okey Bs = ck;
            ck = key_fold(Bs, 0);
            tk = key_fold(Bs, 1);
            if (t < 0.f) left = t;
            if (t > 0.f) right = t;
            if (cfg->midpoint_shrink) {
                if (t < 0.f) left = alpha * left;
                if (t > 0.f) right = alpha * right;
            }
        }
        for (int q = 0; q < D; ++q) u0[q] = fmaf(t, d[q], u0[q]);
        logL0 = logL;
        int p = j - (S - 1 - K);
        if (K > 0 && p >= 0 && j < S - 1) {
            memcpy(ph_U + (size_t)p * D, u0, sizeof(float) * D);
            ph_L[p] = logL;
        }
        if (cfg->gradient_guided) {
            /* Householder reflection at the accepted point (uni_slice_sampler.py:255-269) */
            ++total;
            if (j + 1 < S) {
                float g[128];
                o32_grad_u(m, u0, g);
                float gn = sqrtf(o32_dot_dims(m, g, g));
                if (!(gn >= 1e-10f) || isinf(gn)) {
                    o32_direction(m, key_fold(after, 0), d);
                } else {
                    float gu[128];
                    for (int q = 0; q < D; ++q) gu[q] = g[q] / gn;
                    float dot = o32_dot_dims(m, d, gu);
                    for (int q = 0; q < D; ++q) d[q] = fmaf(-2.0f * dot, gu[q], d[q]);
                    float dn = sqrtf(o32_dot_dims(m, d, d));
                    for (int q = 0; q < D; ++q) d[q] = d[q] / dn;
                }
            }
        } else if (j + 1 < S) {
            o32_direction(m, after, d);
        }
    }
    memcpy(U_out, u0, sizeof(float) * D);
    *L_out = logL0;
    *E_out = total;
}

/* One shell: chains c = 0..num_chains-1 with keys split(sample_key, .)[c] (get_samples,
 * sharded_static.py:88-129).  ph_U: [num_chains, K, D], ph_L: [num_chains, K] (may be NULL
 * when K = 0). */
void orc32_slice_shell(const orc32_model *m, const orc_slice_cfg *cfg, uint32_t k0, uint32_t k1, float Lstar,
                       const float *live_U, const float *live_L, long n, long num_chains, long max_evals_per_slice,
                       float *U_out, float *L_out, long *E_out, float *ph_U, float *ph_L) {
    okey key = {k0, k1};
    int D = m->D, K = cfg->num_phantom;
    for (long c = 0; c < num_chains; ++c) {
        okey kc = key_fold(key, (uint64_t)c);
        orc32_slice_chain(m, cfg, kc.k0, kc.k1, Lstar, live_U, live_L, n, max_evals_per_slice, U_out + c * D,
                          &L_out[c], &E_out[c], ph_U ? ph_U + (size_t)c * K * D : NULL,
                          ph_L ? ph_L + (size_t)c * K : NULL);
    }
}

/* The elementary functions of gbns_fmath.h (for their accuracy tests) */
float orc32_fm_exp(float x) { return gbns_fm_exp(x); }
float orc32_fm_log(float x) { return gbns_fm_log(x); }
float orc32_fm_log1p(float x) { return gbns_fm_log1p(x); }
float orc32_fm_ndtri(float u) { return gbns_fm_ndtri(u); }
float orc32_fm_ndtri_d(double u) { return gbns_fm_ndtri_d(u); }
float orc32_fm_normal_from_bits(uint64_t b) { return gbns_fm_normal_from_mantissa(b >> 12); }
double orc_fm_log64(double x) { return gbns_fm_log64(x); }
double orc_fm_ndtri64(double p) { return gbns_fm_ndtri64(p); }

/* Model.transform and Model.log_prob_prior (framework/model.py:155-187) of M sample rows, as
 * _to_results applies them to the sorted samples (sharded_static.py:744-745), in the
 * arithmetic of the device's prior transform: Uniform q = fma(b, u, a), Normal
 * q = fma(b, Phi^-1(u), a) with the AS 241 PPND16 quantile, X = c + A q row by row over
 * [row_start, d] when A is given (the MultivariateNormalTriL blocks), and the density summed
 * per lane (dimension d on lane d mod 32, in dimension order), then over the 32 lanes by the
 * xor butterfly, plus log_det and log L when given.  U is fp32 (U32) or FP64 (U64). */
void orc_prior_transform(int D, const int *kind, const double *a, const double *b, const double *log_norm,
                         const double *A, const int *row_start, const double *c, double log_det, const float *U32,
                         const double *U64, long M, const double *log_L, double *X, double *out) {
    double *q = (double *)malloc(sizeof(double) * (size_t)(D > 0 ? D : 1));
    for (long row = 0; row < M; ++row) {
        double part[32], tmp[32];
        for (int l = 0; l < 32; ++l) part[l] = 0.0;
        for (int d = 0; d < D; ++d) {
            const double u = U32 ? (double)U32[row * D + d] : U64[row * D + d];
            double ld;
            if (kind[d] == ORC_PRIOR_NORMAL) {
                const double z = gbns_fm_ndtri64(u);
                q[d] = fma(b[d], z, a[d]);
                ld = fma(-0.5 * z, z, log_norm[d]);
            } else {
                q[d] = fma(b[d], u, a[d]);
                ld = (q[d] >= a[d] && q[d] <= a[d] + b[d]) ? log_norm[d] : -INFINITY;
            }
            part[d & 31] += ld;
        }
        if (X) {
            for (int d = 0; d < D; ++d) {
                if (!A) {
                    X[row * D + d] = q[d];
                    continue;
                }
                double acc = c[d];
                for (int k = row_start[d] > 0 ? row_start[d] : 0; k <= d; ++k) acc = fma(A[(size_t)d * D + k], q[k], acc);
                X[row * D + d] = acc;
            }
        }
        for (int m = 16; m >= 1; m >>= 1) {
            for (int l = 0; l < 32; ++l) tmp[l] = part[l] + part[l ^ m];
            memcpy(part, tmp, sizeof part);
        }
        if (out) out[row] = (log_L ? log_L[row] : 0.0) + (part[0] + log_det);
    }
    free(q);
}
