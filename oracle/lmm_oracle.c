/*
 * lmm_oracle.c -- CPU restatement (FP64) of finmath-lib's LIBOR Market Model
 * Monte Carlo path.  TEST INFRASTRUCTURE ONLY (parity reference + timed CPU baseline); the
 * CUDA product never calls into this file.  See lmm_oracle.h for the parity status.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -fPIC -shared (Java never contracts
 * a*b+c into an FMA, so neither may this file).
 *
 * Citations are to finmath-lib: M: = src/main/java/net/finmath/.
 */
#include "lmm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ======================================================================== */
/* MT19937.  The reference wraps org.apache.commons.math3.random.MersenneTwister
 * (M:randomnumbers/MersenneTwister.java:24-51).  commons-math3 3.6.1 is a compiled
 * dependency that is absent from the reference tree; its published algorithm is:
 *   - MersenneTwister(long seed): key = {high 32 bits, low 32 bits} of the seed,
 *     then the MT19937 init_by_array procedure of Matsumoto & Nishimura (2002);
 *   - next(bits): one tempered 32-bit MT19937 word, shifted right by 32-bits;
 *   - nextDouble(): (next(26) << 26 | next(26)) * 2^-52.
 * The core recurrence and seeding below follow Matsumoto & Nishimura (1998/2002).
 */
#define MT_N 624
#define MT_M 397

static void mt_init_genrand(orc_mt19937* s, uint32_t seed)
{
    s->mt[0] = seed;
    for (int i = 1; i < MT_N; i++) {
        uint32_t prev = s->mt[i - 1];
        s->mt[i] = (uint32_t)(1812433253u * (prev ^ (prev >> 30)) + (uint32_t)i);
    }
    s->mti = MT_N;
}

static void mt_init_by_array(orc_mt19937* s, const uint32_t* key, int key_len)
{
    mt_init_genrand(s, 19650218u);
    int i = 1, j = 0;
    for (int k = (MT_N > key_len ? MT_N : key_len); k != 0; k--) {
        uint32_t prev = s->mt[i - 1];
        s->mt[i] = (uint32_t)((s->mt[i] ^ ((prev ^ (prev >> 30)) * 1664525u)) + key[j] + (uint32_t)j);
        i++;
        j++;
        if (i >= MT_N) { s->mt[0] = s->mt[MT_N - 1]; i = 1; }
        if (j >= key_len) j = 0;
    }
    for (int k = MT_N - 1; k != 0; k--) {
        uint32_t prev = s->mt[i - 1];
        s->mt[i] = (uint32_t)((s->mt[i] ^ ((prev ^ (prev >> 30)) * 1566083941u)) - (uint32_t)i);
        i++;
        if (i >= MT_N) { s->mt[0] = s->mt[MT_N - 1]; i = 1; }
    }
    s->mt[0] = 0x80000000u;
    s->mti = MT_N;
}

void orc_mt_seed_long(orc_mt19937* s, int64_t seed)
{
    uint64_t u = (uint64_t)seed;
    uint32_t key[2] = { (uint32_t)(u >> 32), (uint32_t)(u & 0xffffffffu) };
    mt_init_by_array(s, key, 2);
}

static void mt_regenerate(orc_mt19937* s)
{
    uint32_t* mt = s->mt;
    int k;
    for (k = 0; k < MT_N - MT_M; k++) {
        uint32_t y = (mt[k] & 0x80000000u) | (mt[k + 1] & 0x7fffffffu);
        mt[k] = mt[k + MT_M] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    for (; k < MT_N - 1; k++) {
        uint32_t y = (mt[k] & 0x80000000u) | (mt[k + 1] & 0x7fffffffu);
        mt[k] = mt[k + (MT_M - MT_N)] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    uint32_t y = (mt[MT_N - 1] & 0x80000000u) | (mt[0] & 0x7fffffffu);
    mt[MT_N - 1] = mt[MT_M - 1] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    s->mti = 0;
}

uint32_t orc_mt_next_word(orc_mt19937* s)
{
    if (s->mti >= MT_N) mt_regenerate(s);
    uint32_t y = s->mt[s->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

double orc_mt_next_double(orc_mt19937* s)
{
    uint64_t high = (uint64_t)(orc_mt_next_word(s) >> 6) << 26;
    uint64_t low = (uint64_t)(orc_mt_next_word(s) >> 6);
    return (double)(high | low) * 0x1.0p-52;
}

void orc_mt_words(int64_t seed, int64_t skip, int64_t count, uint32_t* out)
{
    orc_mt19937 s;
    orc_mt_seed_long(&s, seed);
    for (int64_t i = 0; i < skip; i++) (void)orc_mt_next_word(&s);
    for (int64_t i = 0; i < count; i++) out[i] = orc_mt_next_word(&s);
}

void orc_mt_doubles(int64_t seed, int64_t skip, int64_t count, double* out)
{
    orc_mt19937 s;
    orc_mt_seed_long(&s, seed);
    for (int64_t i = 0; i < 2 * skip; i++) (void)orc_mt_next_word(&s);
    for (int64_t i = 0; i < count; i++) out[i] = orc_mt_next_double(&s);
}

void orc_mt_seeded_state(int64_t seed, uint32_t* out624)
{
    orc_mt19937 s;
    orc_mt_seed_long(&s, seed);
    memcpy(out624, s.mt, sizeof(s.mt));
}

/* ======================================================================== */
/* Wichura AS241, M:functions/NormalDistribution.java:67-162.  The coefficients are
 * those of the published algorithm (Applied Statistics 37(3), 1988). */
double orc_icdf_wichura(double p)
{
    const double split1 = 0.425, split2 = 5.0, const1 = 0.180625, const2 = 1.6;
    const double a0 = 3.3871328727963666080e+00, a1 = 1.3314166789178437745e+02,
                 a2 = 1.9715909503065514427e+03, a3 = 1.3731693765509461125e+04,
                 a4 = 4.5921953931549871457e+04, a5 = 6.7265770927008700853e+04,
                 a6 = 3.3430575583588128105e+04, a7 = 2.5090809287301226727e+03;
    const double b1 = 4.2313330701600911252e+01, b2 = 6.8718700749205790830e+02,
                 b3 = 5.3941960214247511077e+03, b4 = 2.1213794301586595867e+04,
                 b5 = 3.9307895800092710610e+04, b6 = 2.8729085735721942674e+04,
                 b7 = 5.2264952788528545610e+03;
    const double c0 = 1.42343711074968357734e+00, c1 = 4.63033784615654529590e+00,
                 c2 = 5.76949722146069140550e+00, c3 = 3.64784832476320460504e+00,
                 c4 = 1.27045825245236838258e+00, c5 = 2.41780725177450611770e-01,
                 c6 = 2.27238449892691845833e-02, c7 = 7.74545014278341407640e-04;
    const double d1 = 2.05319162663775882187e+00, d2 = 1.67638483018380384940e+00,
                 d3 = 6.89767334985100004550e-01, d4 = 1.48103976427480074590e-01,
                 d5 = 1.51986665636164571966e-02, d6 = 5.47593808499534494600e-04,
                 d7 = 1.05075007164441684324e-09;
    const double e0 = 6.65790464350110377720e+00, e1 = 5.46378491116411436990e+00,
                 e2 = 1.78482653991729133580e+00, e3 = 2.96560571828504891230e-01,
                 e4 = 2.65321895265761230930e-02, e5 = 1.24266094738807843860e-03,
                 e6 = 2.71155556874348757815e-05, e7 = 2.01033439929228813265e-07;
    const double f1 = 5.99832206555887937690e-01, f2 = 1.36929880922735805310e-01,
                 f3 = 1.48753612908506148525e-02, f4 = 7.86869131145613259100e-04,
                 f5 = 1.84631831751005468180e-05, f6 = 1.42151175831644588870e-07,
                 f7 = 2.04426310338993978564e-15;

    double q = p - 0.5;
    if (fabs(q) <= split1) {
        double r = const1 - q * q;
        double num = (((((((a7 * r + a6) * r + a5) * r + a4) * r + a3) * r + a2) * r + a1) * r + a0);
        double den = (((((((b7 * r + b6) * r + b5) * r + b4) * r + b3) * r + b2) * r + b1) * r + 1.0);
        return q * num / den;
    }
    double r = (q < 0.0) ? p : 1.0 - p;
    if (r <= 0.0) return 0.0;
    r = sqrt(-log(r));
    double v;
    if (r <= split2) {
        r -= const2;
        v = (((((((c7 * r + c6) * r + c5) * r + c4) * r + c3) * r + c2) * r + c1) * r + c0)
            / (((((((d7 * r + d6) * r + d5) * r + d4) * r + d3) * r + d2) * r + d1) * r + 1.0);
    } else {
        r -= split2;
        v = (((((((e7 * r + e6) * r + e5) * r + e4) * r + e3) * r + e2) * r + e1) * r + e0)
            / (((((((f7 * r + f6) * r + f5) * r + f4) * r + f3) * r + f2) * r + f1) * r + 1.0);
    }
    if (q < 0.0) v = -v;
    return v;
}

/* ======================================================================== */
/* TimeDiscretizationFromArray (M:time/TimeDiscretizationFromArray.java). */
static const double kTick = 1.0 / (365.0 * 24.0); /* :39 */

double orc_round_to_tick(double t) { return rint(t / kTick) * kTick; } /* :387-389 */

int orc_binary_search(const double* a, int n, double key)
{
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (int)(((unsigned)lo + (unsigned)hi) >> 1);
        double v = a[mid];
        if (v < key) lo = mid + 1;
        else if (v > key) hi = mid - 1;
        else return mid; /* exact values only; no NaN on the grid */
    }
    return -(lo + 1);
}

int orc_time_index(const double* times, int n, double t) { return orc_binary_search(times, n, orc_round_to_tick(t)); } /* :272-274 */

void orc_time_discretization(double initial, int n, double dt, double* out) /* :210-217 */
{
    for (int i = 0; i <= n; i++) out[i] = orc_round_to_tick(initial + (double)i * dt);
}

/* ======================================================================== */
/* BrownianMotionFromMersenneRandomNumbers.doGenerateBrownianMotion
 * (M:montecarlo/BrownianMotionFromMersenneRandomNumbers.java:141-191):
 * one MT stream, loop path -> time -> factor, dW = ICDF(u) * sqrt(dt). */
void orc_brownian_increments(const double* times, int T, int F, int P, int seed, double* out)
{
    orc_mt19937 s;
    orc_mt_seed_long(&s, (int64_t)seed); /* int seed widened to long (:147) */
    double* sq = (double*)malloc(sizeof(double) * (size_t)T);
    for (int t = 0; t < T; t++) sq[t] = sqrt(times[t + 1] - times[t]);
    for (int p = 0; p < P; p++)
        for (int t = 0; t < T; t++)
            for (int k = 0; k < F; k++) {
                double u = orc_mt_next_double(&s);
                out[((size_t)t * F + k) * (size_t)P + p] = orc_icdf_wichura(u) * sq[t];
            }
    free(sq);
}

/* ======================================================================== */
/* Linear algebra.  commons-math3 EigenDecomposition / SingularValueDecomposition are
 * compiled third-party code; here: cyclic Jacobi (symmetric eigenproblem) and
 * one-sided Jacobi (SVD), both textbook methods (Golub & Van Loan, ch. 8). */
int orc_eigen_symmetric(int n, const double* Ain, double* evals, double* V)
{
    double* A = (double*)malloc(sizeof(double) * (size_t)n * n);
    memcpy(A, Ain, sizeof(double) * (size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) V[i * n + j] = (i == j) ? 1.0 : 0.0;
    int sweep;
    for (sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                if (i != j) off += A[i * n + j] * A[i * n + j];
                else diag += A[i * n + i] * A[i * n + i];
            }
        if (off <= 1e-300 || off <= 1e-34 * diag) break;
        /* an element below 2^-53 of the matrix's diagonal norm is rounding noise: rotating
         * it changes nothing the factor matrix keeps, and a sweep without a rotation ends
         * the iteration (rank-deficient and clustered spectra otherwise never meet the
         * relative criterion above) */
        const double tiny = 0x1.0p-53 * sqrt(diag);
        int rotated = 0;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = A[p * n + q];
                if (apq == 0.0 || fabs(apq) <= tiny) continue;
                rotated = 1;
                double app = A[p * n + p], aqq = A[q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
        if (!rotated) break;
    }
    for (int i = 0; i < n; i++) evals[i] = A[i * n + i];
    free(A);
    return sweep;
}

/* LinearAlgebra.getFactorMatrixUsingCommonsMath (M:functions/LinearAlgebra.java:392-445):
 * eigenvectors of the F largest eigenvalues (stable descending sort), sign convention
 * "first entry positive", scaled by sqrt(max(lambda,0) / |v|^2). */
void orc_factor_matrix(const double* corr, int n, int F, double* out)
{
    double* ev = (double*)malloc(sizeof(double) * (size_t)n);
    double* V = (double*)malloc(sizeof(double) * (size_t)n * n);
    int* idx = (int*)malloc(sizeof(int) * (size_t)n);
    orc_eigen_symmetric(n, corr, ev, V);
    for (int i = 0; i < n; i++) idx[i] = i;
    /* stable insertion sort, descending */
    for (int i = 1; i < n; i++) {
        int v = idx[i], j = i - 1;
        while (j >= 0 && ev[idx[j]] < ev[v]) { idx[j + 1] = idx[j]; j--; }
        idx[j + 1] = v;
    }
    for (int f = 0; f < F; f++) {
        int e = idx[f];
        double lambda = ev[e];
        double sign = V[0 * n + e] > 0.0 ? 1.0 : -1.0;
        double norm2 = 0.0;
        for (int r = 0; r < n; r++) norm2 += V[r * n + e] * V[r * n + e];
        lambda = lambda > 0.0 ? lambda : 0.0;
        for (int r = 0; r < n; r++) out[r * F + f] = sign * sqrt(lambda / norm2) * V[r * n + e];
    }
    free(ev);
    free(V);
    free(idx);
}

/* LinearAlgebra.factorReductionUsingCommonsMath (M:functions/LinearAlgebra.java:454-482). */
void orc_factor_reduction(const double* corr, int n, int F, double* out)
{
    double* fm = (double*)malloc(sizeof(double) * (size_t)n * F);
    double* red = (double*)malloc(sizeof(double) * (size_t)n * n);
    orc_factor_matrix(corr, n, F, fm);
    for (int r = 0; r < n; r++) {
        double s2 = 0.0;
        for (int f = 0; f < F; f++) s2 += fm[r * F + f] * fm[r * F + f];
        if (s2 != 0.0) {
            for (int f = 0; f < F; f++) fm[r * F + f] = fm[r * F + f] / sqrt(s2);
        } else {
            for (int f = 0; f < F; f++) fm[r * F + f] = 1.0;
        }
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            double s = 0.0;
            for (int f = 0; f < F; f++) s += fm[i * F + f] * fm[j * F + f];
            red[i * n + j] = s;
        }
    orc_factor_matrix(red, n, F, out);
    free(fm);
    free(red);
}

/* One-sided Jacobi SVD of A (m x n): A V = U diag(s).  Returns U (m x n), s (n), V (n x n). */
static void svd_one_sided_jacobi(int m, int n, const double* A, double* U, double* s, double* V)
{
    memcpy(U, A, sizeof(double) * (size_t)m * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) V[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        int rotated = 0;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double alpha = 0.0, beta = 0.0, gamma = 0.0;
                for (int k = 0; k < m; k++) {
                    double up = U[k * n + p], uq = U[k * n + q];
                    alpha += up * up;
                    beta += uq * uq;
                    gamma += up * uq;
                }
                if (gamma == 0.0 || fabs(gamma) <= 0x1.0p-52 * sqrt(alpha * beta)) continue;
                rotated = 1;
                double zeta = (beta - alpha) / (2.0 * gamma);
                double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
                for (int k = 0; k < m; k++) {
                    double up = U[k * n + p], uq = U[k * n + q];
                    U[k * n + p] = c * up - sn * uq;
                    U[k * n + q] = sn * up + c * uq;
                }
                for (int k = 0; k < n; k++) {
                    double vp = V[k * n + p], vq = V[k * n + q];
                    V[k * n + p] = c * vp - sn * vq;
                    V[k * n + q] = sn * vp + c * vq;
                }
            }
        if (!rotated) break;
    }
    for (int j = 0; j < n; j++) {
        double nn = 0.0;
        for (int k = 0; k < m; k++) nn += U[k * n + j] * U[k * n + j];
        s[j] = sqrt(nn);
        if (s[j] > 0.0)
            for (int k = 0; k < m; k++) U[k * n + j] = U[k * n + j] / s[j];
    }
}

/* Pseudo-inverse solve with the cutoff of an SVD-based least-squares solver:
 * singular values <= max(max(m,n) * s_max * 2^-52, sqrt(2^-1022)) are dropped. */
int orc_lstsq_pinv(int m, int n, int k, const double* A, const double* B, double* X)
{
    /* One-sided Jacobi needs at least as many rows as columns; pad with zero rows. */
    int mm = m > n ? m : n;
    double* Ap = (double*)calloc((size_t)mm * n, sizeof(double));
    memcpy(Ap, A, sizeof(double) * (size_t)m * n);
    double* U = (double*)malloc(sizeof(double) * (size_t)mm * n);
    double* s = (double*)malloc(sizeof(double) * (size_t)n);
    double* V = (double*)malloc(sizeof(double) * (size_t)n * n);
    svd_one_sided_jacobi(mm, n, Ap, U, s, V);
    double smax = 0.0;
    for (int j = 0; j < n; j++) smax = s[j] > smax ? s[j] : smax;
    double tol = (double)(m > n ? m : n) * smax * 0x1.0p-52;
    double tmin = sqrt(0x1.0p-1022);
    if (tol < tmin) tol = tmin;
    for (int c = 0; c < k; c++) {
        for (int i = 0; i < n; i++) {
            double acc = 0.0;
            for (int j = 0; j < n; j++) {
                if (!(s[j] > tol)) continue;
                double utb = 0.0;
                for (int r = 0; r < m; r++) utb += U[r * n + j] * B[r * k + c];
                acc += V[i * n + j] * (utb / s[j]);
            }
            X[i * k + c] = acc;
        }
    }
    free(Ap);
    free(U);
    free(s);
    free(V);
    return 0;
}

/* ======================================================================== */
/* LIBORCorrelationModelExponentialDecay.initialize
 * (M:montecarlo/interestrate/models/covariance/LIBORCorrelationModelExponentialDecay.java:102-134). */
void orc_exp_decay_correlation(const double* tenor, int N, int F, double a, double* factor, double* corr)
{
    if (a < 0.0) a = 0.0;
    for (int r = 0; r < N; r++)
        for (int c = 0; c < N; c++) corr[r * N + c] = exp(-a * fabs(tenor[r] - tenor[c]));
    orc_factor_reduction(corr, N, F, factor);
    for (int c1 = 0; c1 < N; c1++) {
        for (int c2 = 0; c2 < c1; c2++) {
            double s = 0.0;
            for (int f = 0; f < F; f++) s += factor[c1 * F + f] * factor[c2 * F + f];
            corr[c1 * N + c2] = s;
            corr[c2 * N + c1] = s;
        }
        corr[c1 * N + c1] = 1.0;
    }
}

/* LIBORVolatilityModelFourParameterExponentialForm.getVolatility
 * (…/covariance/LIBORVolatilityModelFourParameterExponentialForm.java:168-194):
 * sigma = ((a + b*tau) * exp(c*(-tau))) + d for tau = T_j - t_i > 0, else 0. */
void orc_vol_abcd(const double* times, int T, const double* tenor, int N,
                  double a, double b, double c, double d, double* vol)
{
    for (int i = 0; i < T; i++)
        for (int j = 0; j < N; j++) {
            double tau = tenor[j] - times[i];
            double v = 0.0;
            if (!(tau <= 0.0)) v = ((b * tau + a) * exp(c * -tau)) + d;
            vol[i * N + j] = v;
        }
}

/* LIBORCovarianceModelFromVolatilityAndCorrelation.getFactorLoading / getCovariance
 * (…/covariance/LIBORCovarianceModelFromVolatilityAndCorrelation.java:48-57, 83-93). */
void orc_covariance_tables(int T, int N, int F, const double* vol, const double* factor,
                           const double* corr, double* loadings, double* variance)
{
    for (int i = 0; i < T; i++)
        for (int j = 0; j < N; j++) {
            double s = vol[i * N + j];
            for (int f = 0; f < F; f++) loadings[((size_t)i * N + j) * F + f] = s * factor[j * F + f];
            variance[i * N + j] = (s * s) * corr[j * N + j];
        }
}

/* ForwardCurveInterpolation value: LINEAR on values, CONSTANT extrapolation
 * (M:interpolation/RationalFunctionInterpolation.java:184-225, 278-300). */
double orc_curve_forward(const double* x, const double* y, int n, double t)
{
    int idx = orc_binary_search(x, n, t);
    if (idx >= 0) return y[idx];
    int iv = -idx - 2;
    if (iv < 0) return y[0];
    if (iv > n - 2) return y[n - 1];
    double slope = (y[iv + 1] - y[iv]) / (x[iv + 1] - x[iv]);
    double dx = t - x[iv];
    double v = 0.0;
    v += y[iv] * 1.0;
    v += slope * dx;
    return v;
}

/* DiscountCurveFromForwardCurve.getDiscountFactor
 * (M:marketdata/model/curves/DiscountCurveFromForwardCurve.java:115-140). */
double orc_discount_factor_from_forward_curve(const double* x, const double* y, int n,
                                              double payment_offset, double maturity)
{
    double time = 0.0, df = 1.0;
    while (time < maturity) {
        double m = payment_offset < maturity - time ? payment_offset : maturity - time;
        df /= 1.0 + orc_curve_forward(x, y, n, time) * m * 1.0;
        time += payment_offset;
    }
    return df;
}

/* LIBORMarketModelFromCovarianceModel.getNumeraireDefaultableZeroBondAsOfTimeZero
 * (…/models/LIBORMarketModelFromCovarianceModel.java:915-944): a chain of
 * Scalar.discount steps (M:stochastic/Scalar.java:321-328). */
void orc_numeraire_discount_chain(const double* tenor, int N, const double* df, double* out)
{
    double adj = df[0];
    out[0] = adj;
    for (int i = 0; i < N; i++) {
        double step = tenor[i + 1] - tenor[i];
        double r = (df[i] / df[i + 1] - 1.0) / step;
        if (adj == 0.0) adj = r * 0.0;
        else adj = 1.0 / (r * (step / adj) + 1.0 / adj);
        out[i + 1] = adj;
    }
}

/* ======================================================================== */
/* The simulation. */
struct orc_sim {
    orc_lmm m;
    int P;
    int* obs_slot;        /* [T+1] -> slot or -1 */
    int nobs;
    double* states;       /* [nobs][N][P] */
    double* numeraire;    /* [N+1][P] unadjusted spot numeraire at tenor times */
    uint8_t* num_det;     /* [N+1] deterministic flag */
    int* tenor_tidx;      /* [N+1] process time index used for L_l(T_l) */
    double* times_copy;
    double* tenor_copy;
};

/* LIBORMarketModelFromCovarianceModel.getDrift (:1125-1191) for components first..N-1 of the
 * state L at simulation step i: SPOT sums the measure-change terms of l <= j (the running sum
 * is updated before component j reads it), TERMINAL those of l > j (walking down from N-1, the
 * sum is read before j adds to it); LOGNORMAL multiplies the one-step transform by L and adds
 * -variance/2.  Scalar(+-delta).discount(L, delta) = 1/(L*(delta/(+-delta)) + 1/(+-delta))
 * (M:stochastic/Scalar.java:321-328). */
static void orc_drift(const orc_lmm* m, int i, int first, const double* L, double* mu)
{
    const int N = m->N, F = m->F;
    const double* lam = m->loadings + (size_t)i * N * F;
    const double* var = m->variance + (size_t)i * N;
    const int lognormal = m->state_space == 0;
    double S[64];
    for (int k = 0; k < F; k++) S[k] = 0.0;
    if (m->measure == 0) {
        for (int j = first; j < N; j++) {
            const double delta = m->tenor[j + 1] - m->tenor[j];
            double os = 1.0 / (L[j] * (delta / delta) + 1.0 / delta);
            if (lognormal) os = os * L[j];
            const double* lj = lam + (size_t)j * F;
            for (int k = 0; k < F; k++) S[k] = S[k] + os * lj[k];
            double d = 0.0;
            for (int k = 0; k < F; k++) d = d + S[k] * lj[k];
            mu[j] = d;
        }
    } else {
        for (int j = N - 1; j >= first; j--) {
            const double delta = m->tenor[j + 1] - m->tenor[j];
            double os = 1.0 / (L[j] * (delta / -delta) + 1.0 / -delta);
            if (lognormal) os = os * L[j];
            const double* lj = lam + (size_t)j * F;
            double d = 0.0;
            for (int k = 0; k < F; k++) d = d + S[k] * lj[k];
            mu[j] = d;
            for (int k = 0; k < F; k++) S[k] = S[k] + os * lj[k];
        }
    }
    if (lognormal)
        for (int j = first; j < N; j++) mu[j] = mu[j] + var[j] * -0.5;
}

/* applyStateSpaceTransform (:1200-1212): exp for LOGNORMAL, then the cap (Math.min). */
static double orc_transform(const orc_lmm* m, double y)
{
    double v = m->state_space == 0 ? exp(y) : y;
    if (!isinf(m->libor_cap) && v > m->libor_cap) v = m->libor_cap;
    return v;
}

/* Terminal-measure numeraire at tenor index l from the state L at the process time index of
 * T_l (getNumerairetUnAdjustedAtLIBORIndex :1029-1048): prod_{m=l}^{N-1} 1/(1 + L_m delta_m),
 * as Scalar.discount steps while the value is deterministic (time index 0) and as
 * RandomVariableFromDoubleArray.discount (x / (1 + L delta), :1308-1333) afterwards. */
static double orc_terminal_numeraire(const orc_lmm* m, int l, const double* L, int deterministic)
{
    const int N = m->N;
    double x = 1.0;
    for (int k = l; k < N; k++) {
        const double delta = m->tenor[k + 1] - m->tenor[k];
        if (deterministic || k == l) x = 1.0 / (L[k] * (delta / x) + 1.0 / x);
        else x = x / (1.0 + L[k] * delta);
    }
    return x;
}

static int first_alive_component(const double* tenor, int N1, double t)
{
    /* LIBORMarketModelFromCovarianceModel.getDrift (:1127-1130) */
    int idx = orc_time_index(tenor, N1, t);
    int first = idx + 1;
    if (first < 0) first = -first - 1 + 1;
    return first;
}

orc_sim* orc_simulate(const orc_lmm* m, int P, const double* dW, const uint8_t* observe, int threads)
{
    const int T = m->T, N = m->N, F = m->F;
    orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
    s->m = *m;
    s->P = P;
    s->times_copy = (double*)malloc(sizeof(double) * (size_t)(T + 1));
    s->tenor_copy = (double*)malloc(sizeof(double) * (size_t)(N + 1));
    memcpy(s->times_copy, m->times, sizeof(double) * (size_t)(T + 1));
    memcpy(s->tenor_copy, m->tenor, sizeof(double) * (size_t)(N + 1));
    s->m.times = s->times_copy;
    s->m.tenor = s->tenor_copy;
    s->obs_slot = (int*)malloc(sizeof(int) * (size_t)(T + 1));
    s->nobs = 0;
    for (int t = 0; t <= T; t++) s->obs_slot[t] = (observe == NULL || observe[t]) ? s->nobs++ : -1;
    s->states = (double*)malloc(sizeof(double) * (size_t)s->nobs * N * P);
    s->numeraire = (double*)malloc(sizeof(double) * (size_t)(N + 1) * P);
    s->num_det = (uint8_t*)calloc((size_t)(N + 1), 1);
    s->tenor_tidx = (int*)malloc(sizeof(int) * (size_t)(N + 1));
    /* getNumerairetUnAdjustedAtLIBORIndex (:1050-1066): L_{l}(T_{l}) at the process index of T_l,
     * rounded up when T_l is not on the grid. */
    for (int l = 0; l <= N; l++) {
        int ti = orc_time_index(m->times, T + 1, m->tenor[l]);
        if (ti < 0) ti = -ti - 1;
        s->tenor_tidx[l] = ti;
    }
    /* deterministic numeraire flags.  SPOT: N(T_0) = 1; N(T_{l+1}) deterministic iff N(T_l) is
     * and L_l is read at index 0.  TERMINAL: N(T_N) = 1 and N(T_l) with all rates read at index 0. */
    if (m->measure == 0) {
        s->num_det[0] = 1;
        for (int l = 0; l < N; l++) s->num_det[l + 1] = (uint8_t)(s->num_det[l] && s->tenor_tidx[l] == 0);
    } else {
        for (int l = 0; l <= N; l++) s->num_det[l] = (uint8_t)(l == N || s->tenor_tidx[l] == 0);
    }

    int* first = (int*)malloc(sizeof(int) * (size_t)T);
    double* dt = (double*)malloc(sizeof(double) * (size_t)T);
    for (int i = 0; i < T; i++) {
        first[i] = first_alive_component(m->tenor, N + 1, m->times[i]);
        dt[i] = m->times[i + 1] - m->times[i];
    }
    const int functional = (m->scheme == 1 || m->scheme == 3);
    const int pc = (m->scheme == 2 || m->scheme == 3);
    const int lognormal = (m->state_space == 0);
    const int terminal = (m->measure == 1);
    const int general = pc || !lognormal || terminal;
    const int capped = !isinf(m->libor_cap);

#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static)
#endif
    for (int p = 0; p < P; p++) {
        double L[256], Y[256], S[64], fixed_libor[257];
        if (general) {
            /* the general Euler step (EulerSchemeFromProcessModel.java:170-326) for any scheme,
             * measure and state space */
            double mu0[256], mu1[256], Ln[256];
            for (int j = 0; j < N; j++) {
                const double f = m->initial_forwards[j];
                Y[j] = lognormal ? log(f > 0.0 ? f : 0.0) : f;
                L[j] = orc_transform(m, Y[j]);
            }
            if (s->obs_slot[0] >= 0)
                for (int j = 0; j < N; j++) s->states[((size_t)s->obs_slot[0] * N + j) * P + p] = L[j];
            for (int l = 0; l < N; l++)
                if (s->tenor_tidx[l] == 0) fixed_libor[l] = L[l];
            if (terminal) {
                for (int l = 0; l <= N; l++)
                    if (s->tenor_tidx[l] == 0) s->numeraire[(size_t)l * P + p] = orc_terminal_numeraire(m, l, L, 1);
            }
            for (int n = 1; n <= T; n++) {
                const int i = n - 1;
                const double* lam = m->loadings + (size_t)i * N * F;
                orc_drift(m, i, first[i], L, mu0);
                for (int j = 0; j < N; j++) Ln[j] = L[j];
                for (int j = first[i]; j < N; j++) {
                    double y = functional ? (lognormal ? log(L[j]) : L[j]) : Y[j];
                    y = y + mu0[j] * dt[i];
                    for (int k = 0; k < F; k++) y = y + dW[((size_t)i * F + k) * (size_t)P + p] * lam[(size_t)j * F + k];
                    Y[j] = y;
                    Ln[j] = orc_transform(m, y);
                }
                if (pc) {
                    /* corrector (:292-314): state += ((mu(predictor) - mu)/2) dt, transform again */
                    orc_drift(m, i, first[i], Ln, mu1);
                    for (int j = first[i]; j < N; j++) {
                        Y[j] = Y[j] + ((mu1[j] - mu0[j]) / 2.0) * dt[i];
                        Ln[j] = orc_transform(m, Y[j]);
                    }
                }
                for (int j = 0; j < N; j++) L[j] = Ln[j];
                if (s->obs_slot[n] >= 0)
                    for (int j = 0; j < N; j++) s->states[((size_t)s->obs_slot[n] * N + j) * P + p] = L[j];
                for (int l = 0; l < N; l++)
                    if (s->tenor_tidx[l] == n) fixed_libor[l] = L[l];
                if (terminal)
                    for (int l = 0; l <= N; l++)
                        if (s->tenor_tidx[l] == n) s->numeraire[(size_t)l * P + p] = orc_terminal_numeraire(m, l, L, 0);
            }
            if (!terminal) {
                double Nv = 1.0;
                s->numeraire[p] = 1.0;
                for (int l = 0; l < N; l++) {
                    const double delta = m->tenor[l + 1] - m->tenor[l];
                    const double Ll = fixed_libor[l];
                    if (s->num_det[l]) Nv = Ll * (delta * Nv) + Nv;
                    else Nv = Nv * (1.0 + Ll * delta);
                    s->numeraire[(size_t)(l + 1) * P + p] = Nv;
                }
            } else if (s->tenor_tidx[N] > T) {
                s->numeraire[(size_t)N * P + p] = 1.0;
            }
            continue;
        }
        /* initial state: Y0 = log(max(f,0)), L = cap(exp(Y0)) (:1081-1093, EulerScheme :186-190) */
        for (int j = 0; j < N; j++) {
            double f = m->initial_forwards[j];
            Y[j] = log(f > 0.0 ? f : 0.0);
            double v = exp(Y[j]);
            if (capped && v > m->libor_cap) v = m->libor_cap; /* Math.min(v, cap) */
            L[j] = v;
        }
        if (s->obs_slot[0] >= 0)
            for (int j = 0; j < N; j++) s->states[((size_t)s->obs_slot[0] * N + j) * P + p] = L[j];
        for (int l = 0; l < N; l++)
            if (s->tenor_tidx[l] == 0) fixed_libor[l] = L[l];

        for (int n = 1; n <= T; n++) {
            const int i = n - 1;
            const double* lam = m->loadings + (size_t)i * N * F;
            const double* var = m->variance + (size_t)i * N;
            for (int k = 0; k < F; k++) S[k] = 0.0;
            for (int j = first[i]; j < N; j++) {
                const double delta = m->tenor[j + 1] - m->tenor[j];
                const double Lj = L[j];
                /* Scalar(delta).discount(L, delta) = 1/(L*(delta/delta) + 1/delta), then * L (:1149-1153) */
                double os = (1.0 / (Lj * (delta / delta) + 1.0 / delta)) * Lj;
                const double* lj = lam + (size_t)j * F;
                for (int k = 0; k < F; k++) S[k] = S[k] + os * lj[k];          /* :1156-1158 */
                double mu = 0.0;
                for (int k = 0; k < F; k++) mu = mu + S[k] * lj[k];            /* :1159 */
                mu = mu + var[j] * -0.5;                                         /* :1183-1189 */
                /* EulerSchemeFromProcessModel (:235-255) */
                double y = functional ? log(Lj) : Y[j];
                y = y + mu * dt[i];
                for (int k = 0; k < F; k++) y = y + dW[((size_t)i * F + k) * (size_t)P + p] * lj[k];
                Y[j] = y;
                double v = exp(y);
                if (capped && v > m->libor_cap) v = m->libor_cap; /* Math.min(v, cap) */
                L[j] = v;
            }
            if (s->obs_slot[n] >= 0)
                for (int j = 0; j < N; j++) s->states[((size_t)s->obs_slot[n] * N + j) * P + p] = L[j];
            for (int l = 0; l < N; l++)
                if (s->tenor_tidx[l] == n) fixed_libor[l] = L[l];
        }
        /* spot numeraire (LIBORMarketModelFromCovarianceModel.java:1050-1066 with Scalar.accrue
         * M:stochastic/Scalar.java:316-318 and RandomVariableFromDoubleArray.accrue :1279-1305) */
        double Nv = 1.0;
        s->numeraire[p] = 1.0;
        for (int l = 0; l < N; l++) {
            const double delta = m->tenor[l + 1] - m->tenor[l];
            const double Ll = fixed_libor[l];
            if (s->num_det[l]) Nv = Ll * (delta * Nv) + Nv;
            else Nv = Nv * (1.0 + Ll * delta);
            s->numeraire[(size_t)(l + 1) * P + p] = Nv;
        }
    }
    free(first);
    free(dt);
    return s;
}

void orc_sim_free(orc_sim* s)
{
    if (!s) return;
    free(s->obs_slot);
    free(s->states);
    free(s->numeraire);
    free(s->num_det);
    free(s->tenor_tidx);
    free(s->times_copy);
    free(s->tenor_copy);
    free(s);
}

int orc_sim_process_value(const orc_sim* s, int time_index, int component, double* out)
{
    if (time_index < 0 || time_index > s->m.T || component < 0 || component >= s->m.N) return -1;
    int slot = s->obs_slot[time_index];
    if (slot < 0) return -2;
    memcpy(out, s->states + ((size_t)slot * s->m.N + component) * s->P, sizeof(double) * (size_t)s->P);
    return 0;
}

/* RandomVariableFromDoubleArray.getAverage (M:montecarlo/RandomVariableFromDoubleArray.java:287-308). */
double orc_kahan_average(const double* x, int64_t n)
{
    double sum = 0.0, err = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double v = x[i] - err;
        double ns = sum + v;
        err = (ns - sum) - v;
        sum = ns;
    }
    return sum / (double)n;
}

/* getVariance (:332-354) / getStandardError (:419-428). */
double orc_standard_error(const double* x, int64_t n)
{
    if (n <= 1) return 0.0;
    double avg = orc_kahan_average(x, n);
    double sum = 0.0, err = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double v = (x[i] - avg) * (x[i] - avg) - err;
        double ns = sum + v;
        err = (ns - sum) - v;
        sum = ns;
    }
    double var = sum / (double)n;
    return sqrt(var) / sqrt((double)n);
}

static double orc_numeraire_at_zero(const orc_sim* s);

/* getNumeraire(time) at a tenor time (:860-876, :915-944). out[P]; returns 1 if deterministic. */
/* getNumerairetUnAdjusted at a tenor time (LIBORMarketModelFromCovarianceModel.java:1017-1074) */
int orc_sim_numeraire_unadjusted(const orc_sim* s, double time, double* out)
{
    const int P = s->P, N = s->m.N;
    int l = orc_time_index(s->m.tenor, N + 1, time);
    if (l < 0) return -1;
    const double* Nu = s->numeraire + (size_t)l * P;
    for (int p = 0; p < P; p++) out[p] = s->num_det[l] ? Nu[0] : Nu[p];
    return s->num_det[l];
}

int orc_sim_numeraire(const orc_sim* s, double time, double* out)
{
    const int P = s->P, N = s->m.N;
    int l = orc_time_index(s->m.tenor, N + 1, time);
    if (l < 0) return -1; /* off-tenor numeraire interpolation is not part of this path */
    const double* Nu = s->numeraire + (size_t)l * P;
    int det = s->num_det[l];
    if (s->m.discount_chain == NULL) {
        for (int p = 0; p < P; p++) out[p] = det ? Nu[0] : Nu[p];
        return det;
    }
    const double pd = s->m.discount_chain[l];
    /* nonDefaultableZeroBond = mean(N(T)^-1 * N(0)) (:869-874); N(0) = 1 under SPOT */
    const double N0 = s->numeraire[0];
    if (det) {
        double a = N0 * (1.0 / Nu[0]);
        double v = (1.0 / pd) * (Nu[0] * a);
        for (int p = 0; p < P; p++) out[p] = v;
        return 1;
    }
    double* tmp = (double*)malloc(sizeof(double) * (size_t)P);
    for (int p = 0; p < P; p++) tmp[p] = (1.0 / Nu[p]) * N0;
    double a = orc_kahan_average(tmp, P);
    free(tmp);
    for (int p = 0; p < P; p++) out[p] = (Nu[p] * a) / pd;
    return 0;
}

/* getLIBOR(process.getTimeIndex(min(time, start)), startIndex) for a single-period forward
 * (LIBORMarketModelFromCovarianceModel.getForwardRate :1238-1288, ROUND_NEAREST). */
static const double* sim_forward(const orc_sim* s, double time, double start, double end)
{
    const int T = s->m.T, N = s->m.N;
    int si = orc_time_index(s->m.tenor, N + 1, start);
    int ei = orc_time_index(s->m.tenor, N + 1, end);
    if (si < 0 || ei != si + 1) return NULL;
    double t = time < start ? time : start;
    int ti = orc_time_index(s->m.times, T + 1, t);
    if (ti < 0) {
        ti = -ti - 2;
        if (t - s->m.times[ti] > s->m.times[ti + 1] - t) ti++;
    }
    int slot = s->obs_slot[ti];
    if (slot < 0) return NULL;
    return s->states + ((size_t)slot * N + si) * s->P;
}

int orc_swaption(const orc_sim* s, double exercise, int nper, const double* fixing, const double* payment,
                 const double* period_length, const double* strike, double notional,
                 double* value, double* stderr_out, double* per_path)
{
    const int P = s->P;
    double* v = (double*)calloc((size_t)P, sizeof(double));
    double* num = (double*)malloc(sizeof(double) * (size_t)P);
    const double w = 1.0 / (double)P;
    /* Swaption.getValue (M:montecarlo/interestrate/products/Swaption.java:137-199) */
    for (int per = nper - 1; per >= 0; per--) {
        double fix = fixing[per], pay = payment[per], K = strike[per];
        if (pay <= 0.0) break;
        double plen = period_length ? period_length[per] : pay - fix;
        const double* L = sim_forward(s, exercise, fix, pay);
        if (!L) { free(v); free(num); return -1; }
        double disc_date = fix > exercise ? fix : exercise;
        for (int p = 0; p < P; p++) {
            double payoff = ((L[p] - K) * plen) * notional;
            double x = v[p] + payoff;
            x = x / (1.0 + L[p] * (pay - disc_date));
            x = x * 1.0; /* discounting adjustment of identical forward and discount curves */
            v[p] = x;
        }
    }
    if (orc_sim_numeraire(s, exercise, num) < 0) { free(v); free(num); return -2; }
    const double num0 = orc_numeraire_at_zero(s);
    for (int p = 0; p < P; p++) {
        double x = isnan(v[p]) ? v[p] : (v[p] > 0.0 ? v[p] : 0.0); /* Math.max(v, 0.0) */
        x = x / num[p];
        x = x * w;
        x = x * num0;  /* numeraire at evaluation time 0 (1 under SPOT) */
        x = x / w;
        v[p] = x;
    }
    *value = orc_kahan_average(v, P);
    if (stderr_out) *stderr_out = orc_standard_error(v, P);
    if (per_path) memcpy(per_path, v, sizeof(double) * (size_t)P);
    free(v);
    free(num);
    return 0;
}

#define MAXB 6
#define MAXPER 128

/* MonteCarloConditionalExpectationRegression (M:montecarlo/conditionalexpectation/
 * MonteCarloConditionalExpectationRegression.java:98-150).  basis[b] NULL = the constant 1. */
static void regression_ce(int P, int nb, double** basis, const double* y, double* out)
{
    double G[MAXB * MAXB], rhs[MAXB], beta[MAXB];
    double* tmp = (double*)malloc(sizeof(double) * (size_t)P);
    for (int i = 0; i < nb; i++)
        for (int j = i; j < nb; j++) {
            double g;
            if (!basis[i] && !basis[j]) g = 1.0 * 1.0;
            else {
                for (int p = 0; p < P; p++) {
                    double a = basis[i] ? basis[i][p] : 1.0;
                    double b = basis[j] ? basis[j][p] : 1.0;
                    tmp[p] = a * b;
                }
                g = orc_kahan_average(tmp, P);
            }
            G[i * nb + j] = g;
            G[j * nb + i] = g;
        }
    for (int i = 0; i < nb; i++) {
        for (int p = 0; p < P; p++) tmp[p] = y[p] * (basis[i] ? basis[i][p] : 1.0);
        rhs[i] = orc_kahan_average(tmp, P);
    }
    orc_lstsq_pinv(nb, nb, 1, G, rhs, beta);
    for (int p = 0; p < P; p++) {
        double ce = (basis[0] ? basis[0][p] : 1.0) * beta[0];
        for (int i = 1; i < nb; i++) ce = ce + (basis[i] ? basis[i][p] : 1.0) * beta[i];
        out[p] = ce;
    }
    free(tmp);
}

/* What the AAD reverse sweep needs of the forward valuation, per exercise date (in the
 * order the backward induction visits them): the period, the conditional expectation X of
 * the trigger, the continuation values Y and underlying Z the choice picks from, and the
 * five non-constant basis functions. */
typedef struct {
    int ne;
    int per[MAXPER];
    double* X;   /* [ne][P] */
    double* Y;   /* [ne][P] */
    double* Z;   /* [ne][P] */
    double* B;   /* [ne][MAXB - 1][P] */
} berm_record;

static int bermudan_core(const orc_sim* s, int nper, const uint8_t* exercisable, const double* fixing,
                         const double* period_length, const double* payment, const double* notional,
                         const double* strike, int callable, int basis_id,
                         double* value, double* stderr_out, double* per_path, double* exercise_time,
                         berm_record* rec)
{
    const int P = s->P, N = s->m.N;
    const double w = 1.0 / (double)P;
    double* values = (double*)calloc((size_t)P, sizeof(double));
    double* under = (double*)calloc((size_t)P, sizeof(double));
    double* ex = (double*)malloc(sizeof(double) * (size_t)P);
    double* num = (double*)malloc(sizeof(double) * (size_t)P);
    double* trig = (double*)malloc(sizeof(double) * (size_t)P);
    double* ce = (double*)malloc(sizeof(double) * (size_t)P);
    double* b[MAXB];
    for (int i = 0; i < MAXB; i++) b[i] = (double*)malloc(sizeof(double) * (size_t)P);
    for (int p = 0; p < P; p++) ex[p] = INFINITY;
    int rc = 0;
    /* BermudanSwaption.getValues (M:montecarlo/interestrate/products/BermudanSwaption.java:91-157) */
    for (int per = nper - 1; per >= 0; per--) {
        const double fix = fixing[per], plen = period_length[per], pay = payment[per];
        const double* L = sim_forward(s, fix, fix, fix + plen);
        if (!L || orc_sim_numeraire(s, pay, num) < 0) { rc = -1; goto done; }
        for (int p = 0; p < P; p++) {
            double payoff = ((L[p] - strike[per]) * plen) * notional[per];
            payoff = payoff / num[p];
            payoff = payoff * w;
            if (callable) under[p] = under[p] + payoff;
            else values[p] = values[p] + payoff;
        }
        if (!exercisable[per]) continue;
        for (int p = 0; p < P; p++) trig[p] = values[p] - under[p];
        /* basis functions at the exercise date */
        double* basis[MAXB];
        basis[0] = NULL;
        if (orc_sim_numeraire(s, fix, num) < 0) { rc = -2; goto done; }
        if (basis_id == 0) {
            /* BermudanSwaption.getBasisFunctions (:215-252) */
            int fi = orc_binary_search(fixing, nper, fix);
            if (fi < 0) fi = -fi;
            if (fi >= nper) fi = nper - 1;
            const double* rs = sim_forward(s, fix, fix, payment[fi]);
            if (!rs) { rc = -3; goto done; }
            const double dts = payment[fi] - fix;
            const double tl0 = fixing[fi], tl1 = payment[nper - 1];
            for (int p = 0; p < P; p++) {
                double ds = 1.0 / (rs[p] * dts + 1.0);
                b[0][p] = ds;
                b[1][p] = ds * ds;
            }
            /* forward rate from fixing[fi] to the last payment: single period primitive or accrual */
            int si = orc_time_index(s->m.tenor, N + 1, tl0);
            int ei = orc_time_index(s->m.tenor, N + 1, tl1);
            if (si < 0 || ei < 0 || ei <= si) { rc = -4; goto done; }
            for (int p = 0; p < P; p++) b[2][p] = 0.0;
            if (ei == si + 1) {
                const double* ll = sim_forward(s, fix, tl0, tl1);
                for (int p = 0; p < P; p++) b[2][p] = ll[p];
            } else {
                for (int q = si; q < ei; q++) {
                    double sub = s->m.tenor[q + 1] - s->m.tenor[q];
                    const double* lq = sim_forward(s, fix, s->m.tenor[q], s->m.tenor[q + 1]);
                    if (!lq) { rc = -5; goto done; }
                    for (int p = 0; p < P; p++) {
                        if (q == si) b[2][p] = lq[p] * sub + 1.0;
                        else b[2][p] = b[2][p] * (1.0 + lq[p] * sub);
                    }
                }
                for (int p = 0; p < P; p++) b[2][p] = (b[2][p] - 1.0) / (tl1 - tl0);
            }
            for (int p = 0; p < P; p++) {
                double dl = 1.0 / (b[2][p] * (tl1 - tl0) + 1.0);
                b[2][p] = dl;
                b[3][p] = dl * dl;
                b[4][p] = 1.0 / num[p];
            }
            basis[1] = b[0]; basis[2] = b[1]; basis[3] = b[2]; basis[4] = b[3]; basis[5] = b[4];
        } else {
            /* {1, S, S^2, N, N^2, S*N}: S = par rate of the remaining periods from L_j(T_ex),
             * S = (prod g_q - 1) / sum_s d_s prod_{r>s} g_r, g_q = 1 + L_q d_q, by the forward
             * recursion B = B g, H = H g + d (b[0] = B, b[5] = H). */
            for (int q = per; q < nper; q++) {
                const double* lq = sim_forward(s, fix, fixing[q], payment[q]);
                if (!lq) { rc = -6; goto done; }
                const double dq = period_length[q];
                for (int p = 0; p < P; p++) {
                    double g = 1.0 + lq[p] * dq;
                    if (q == per) { b[0][p] = g; b[5][p] = dq; }
                    else { b[0][p] = b[0][p] * g; b[5][p] = b[5][p] * g + dq; }
                }
            }
            for (int p = 0; p < P; p++) {
                double S = (b[0][p] - 1.0) / b[5][p];
                double Nn = num[p];
                b[0][p] = S;
                b[1][p] = S * S;
                b[2][p] = Nn;
                b[3][p] = Nn * Nn;
                b[4][p] = S * Nn;
            }
            basis[1] = b[0]; basis[2] = b[1]; basis[3] = b[2]; basis[4] = b[3]; basis[5] = b[4];
        }
        regression_ce(P, 6, basis, trig, ce);
        if (rec) {
            const int r = rec->ne++;
            const size_t P_ = (size_t)P;
            rec->per[r] = per;
            memcpy(rec->X + r * P_, ce, sizeof(double) * P_);
            memcpy(rec->Y + r * P_, values, sizeof(double) * P_);
            memcpy(rec->Z + r * P_, under, sizeof(double) * P_);
            for (int i = 1; i < MAXB; i++) memcpy(rec->B + ((size_t)r * (MAXB - 1) + i - 1) * P_, basis[i], sizeof(double) * P_);
        }
        for (int p = 0; p < P; p++) {
            int cont = ce[p] >= 0.0;
            values[p] = cont ? values[p] : under[p];
            ex[p] = cont ? ex[p] : fix;
        }
    }
    {
        const double num0 = orc_numeraire_at_zero(s);  /* 1 under SPOT */
        for (int p = 0; p < P; p++) values[p] = (values[p] * num0) / w;
    }
    *value = orc_kahan_average(values, P);
    if (stderr_out) *stderr_out = orc_standard_error(values, P);
    if (per_path) memcpy(per_path, values, sizeof(double) * (size_t)P);
    if (exercise_time) memcpy(exercise_time, ex, sizeof(double) * (size_t)P);
done:
    free(values); free(under); free(ex); free(num); free(trig); free(ce);
    for (int i = 0; i < MAXB; i++) free(b[i]);
    return rc;
}

int orc_bermudan(const orc_sim* s, int nper, const uint8_t* exercisable, const double* fixing,
                 const double* period_length, const double* payment, const double* notional,
                 const double* strike, int callable, int basis_id,
                 double* value, double* stderr_out, double* per_path, double* exercise_time)
{
    return bermudan_core(s, nper, exercisable, fixing, period_length, payment, notional, strike, callable, basis_id,
                         value, stderr_out, per_path, exercise_time, NULL);
}

/* getStandardDeviation (RandomVariableFromDoubleArray.java:395-404 with getVariance :333-355) */
static double orc_standard_deviation(const double* x, int64_t n)
{
    if (n <= 1) return 0.0;
    double avg = orc_kahan_average(x, n);
    double sum = 0.0, err = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double v = (x[i] - avg) * (x[i] - avg) - err;
        double ns = sum + v;
        err = (ns - sum) - v;
        sum = ns;
    }
    return sqrt(sum / (double)n);
}

/* The adjoint weights that the reference's RandomVariableDifferentiableAAD gives the
 * Bermudan's discounted cash flows.  The value is F = mean(values * N(0) / w) with
 * values built by BermudanSwaption.getValues (BermudanSwaption.java:91-157) from the cash
 * flows c[k][p] = ((L_k - K_k) d_k) n_k / N(T_pay) times the weight w = 1/P; the reverse
 * sweep of that operator graph follows RandomVariableDifferentiableAAD.java:
 *   CHOOSE  values = X.choose(Y, Z): Y gets the adjoint where X >= 0, Z where X < 0
 *           (:171-208 with the partial derivatives of :396-444); X gets
 *           ZERO (method 0): nothing;
 *           DISCRETE_DELTA (method 1): (Y - Z) 1{-eps/2 <= X < eps/2} / eps with
 *           eps = width * X.getStandardDeviation() (:409-429; the factory's default width
 *           is 0.05, RandomVariableDifferentiableAADFactory.java:67-68);
 *   CONDITIONAL_EXPECTATION  the trigger X = E[values - under | basis]: its argument gets
 *           the conditional expectation of the adjoint, with the same basis (:188-192);
 *   AVERAGE  getAverage returns a double, so the numeraire adjustment is a constant (:771).
 * omega[k][p] = dF/dc[k][p] / w: the gradient of F is then the path mean of
 * sum_k omega[k][p] dc[k][p]/dtheta, the cash flows differentiated with the adjustment held. */
int orc_bermudan_aad(const orc_sim* s, int nper, const uint8_t* exercisable, const double* fixing,
                     const double* period_length, const double* payment, const double* notional,
                     const double* strike, int callable, int basis_id, int method, double width,
                     double* value, double* omega)
{
    const int P = s->P;
    const size_t P_ = (size_t)P;
    if (nper > MAXPER) return -10;
    int ne = 0;
    for (int k = 0; k < nper; k++) ne += exercisable[k] ? 1 : 0;
    berm_record rec;
    rec.ne = 0;
    rec.X = (double*)malloc(sizeof(double) * P_ * (size_t)(ne > 0 ? ne : 1));
    rec.Y = (double*)malloc(sizeof(double) * P_ * (size_t)(ne > 0 ? ne : 1));
    rec.Z = (double*)malloc(sizeof(double) * P_ * (size_t)(ne > 0 ? ne : 1));
    rec.B = (double*)malloc(sizeof(double) * P_ * (MAXB - 1) * (size_t)(ne > 0 ? ne : 1));
    double* vbar = (double*)malloc(sizeof(double) * P_);
    double* ubar = (double*)malloc(sizeof(double) * P_);
    double* xbar = (double*)malloc(sizeof(double) * P_);
    double* dbar = (double*)malloc(sizeof(double) * P_);
    int rc = bermudan_core(s, nper, exercisable, fixing, period_length, payment, notional, strike, callable, basis_id,
                           value, NULL, NULL, NULL, &rec);
    if (rc == 0) {
        const double num0 = orc_numeraire_at_zero(s);
        for (int p = 0; p < P; p++) { vbar[p] = num0; ubar[p] = 0.0; }
        /* the backward induction recorded its dates from the last period down: replay them upward */
        int r = rec.ne - 1;
        for (int k = 0; k < nper; k++) {
            if (exercisable[k]) {
                const double* X = rec.X + (size_t)r * P_;
                const double* Y = rec.Y + (size_t)r * P_;
                const double* Z = rec.Z + (size_t)r * P_;
                double eps = 0.0;
                if (method == 1) eps = width * orc_standard_deviation(X, P);
                for (int p = 0; p < P; p++) {
                    double xb = 0.0;
                    if (method == 1) {
                        if (isinf(eps)) xb = vbar[p] * (Y[p] - Z[p]);
                        else if (eps > 0.0)
                            xb = (X[p] + eps / 2 >= 0.0 && X[p] - eps / 2 < 0.0) ? vbar[p] * (Y[p] - Z[p]) / eps : 0.0;
                    }
                    xbar[p] = xb;
                    const int cont = X[p] >= 0.0;
                    ubar[p] = ubar[p] + (cont ? 0.0 : vbar[p]);
                    vbar[p] = cont ? vbar[p] : 0.0;
                }
                if (method == 1) {
                    double* basis[MAXB];
                    basis[0] = NULL;
                    for (int i = 1; i < MAXB; i++) basis[i] = rec.B + ((size_t)r * (MAXB - 1) + i - 1) * P_;
                    regression_ce(P, 6, basis, xbar, dbar);
                    for (int p = 0; p < P; p++) {
                        vbar[p] = vbar[p] + dbar[p];
                        ubar[p] = ubar[p] - dbar[p];
                    }
                }
                r--;
            }
            for (int p = 0; p < P; p++) omega[(size_t)k * P_ + p] = callable ? ubar[p] : vbar[p];
        }
    }
    free(rec.X); free(rec.Y); free(rec.Z); free(rec.B);
    free(vbar); free(ubar); free(xbar); free(dbar);
    return rc;
}

/* Value of the Bermudan with the exercise time of every path given (decisions frozen):
 * the mean over paths of the realised, numeraire-discounted cash flows.  Central finite
 * differences of this function with common random numbers are the exact pathwise
 * derivative with frozen exercise decisions -- the quantity an adjoint computes. */
int orc_bermudan_frozen(const orc_sim* s, int nper, const double* fixing, const double* period_length,
                        const double* payment, const double* notional, const double* strike, int callable,
                        const double* exercise_time, double* value)
{
    const int P = s->P;
    double* x = (double*)calloc((size_t)P, sizeof(double));
    double* num = (double*)malloc(sizeof(double) * (size_t)P);
    int rc = 0;
    for (int per = 0; per < nper; per++) {
        const double fix = fixing[per];
        const double* L = sim_forward(s, fix, fix, fix + period_length[per]);
        if (!L || orc_sim_numeraire(s, payment[per], num) < 0) { rc = -1; break; }
        for (int p = 0; p < P; p++) {
            const int paid = callable ? (fix >= exercise_time[p]) : (fix < exercise_time[p]);
            if (paid) x[p] += ((L[p] - strike[per]) * period_length[per]) * notional[per] / num[p];
        }
    }
    if (!rc) *value = orc_kahan_average(x, P) * orc_numeraire_at_zero(s);
    free(x);
    free(num);
    return rc;
}

/* The (adjusted, deterministic) numeraire at evaluation time 0 that product values are
 * multiplied by (AbstractLIBORMonteCarloProduct: values * N(0) / w(0)); exactly 1 under SPOT. */
static double orc_numeraire_at_zero(const orc_sim* s)
{
    double* tmp = (double*)malloc(sizeof(double) * (size_t)s->P);
    orc_sim_numeraire(s, s->m.tenor[0], tmp);
    const double v = tmp[0];
    free(tmp);
    return v;
}
