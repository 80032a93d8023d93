/*
 * lmm_oracle.h -- CPU restatement of finmath-lib's Monte Carlo LIBOR Market Model
 * path (FP64).  TEST INFRASTRUCTURE ONLY: the oracle is the parity reference for the
 * CUDA library and the timed CPU baseline.  Product code never links, loads or calls it.
 *
 * Every function restates the reference's arithmetic in the reference's operation
 * order (no fused multiply-add; compile with -ffp-contract=off).  File:line citations
 * refer to finmath-lib's src/main/java/net/finmath/ tree.
 *
 * Parity status of this oracle:
 *   - MT19937 core and init_by_array seeding: pinned against numpy's independent
 *     MT19937 implementation (tests/golden/make_golden.py).
 *   - commons-math3 3.6.1 glue (long seed split into two key words, nextDouble from
 *     two 26-bit draws): restated from the published algorithm of that library;
 *     the reference's own Java run could not be executed (no JDK), so this part is
 *     "parity unpinned" against Java.
 *   - Pseudo-inverse least squares: pinned against the known-answer tests in
 *     src/test/java/net/finmath/functions/LinearAlgebraTest.java.
 *   - Everything downstream (ICDF, Euler, numeraire, products) follows the Java
 *     sources line by line; the reference's tests hold no golden values for them.
 */
#ifndef LMM_ORACLE_H
#define LMM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- MT19937 (commons-math3 MersenneTwister(long) + BitsStreamGenerator.nextDouble) */
typedef struct {
    uint32_t mt[624];
    int mti;
} orc_mt19937;

void     orc_mt_seed_long(orc_mt19937* s, int64_t seed);
uint32_t orc_mt_next_word(orc_mt19937* s);
double   orc_mt_next_double(orc_mt19937* s);
/* Words/doubles of the stream of `seed`, skipping `skip` words/doubles first. */
void orc_mt_words(int64_t seed, int64_t skip, int64_t count, uint32_t* out);
void orc_mt_doubles(int64_t seed, int64_t skip, int64_t count, double* out);
/* The seeded 624-word state array (before the first regeneration). */
void orc_mt_seeded_state(int64_t seed, uint32_t* out624);

/* ---- NormalDistribution.inverseCumulativeNormalDistributionWichura (AS241) */
double orc_icdf_wichura(double p);

/* ---- TimeDiscretizationFromArray */
double orc_round_to_tick(double t);
/* java.util.Arrays.binarySearch on a sorted array (found: index; else -(ins)-1). */
int orc_binary_search(const double* a, int n, double key);
/* getTimeIndex: binary search of the tick-rounded key. */
int orc_time_index(const double* times, int n, double t);
/* TimeDiscretizationFromArray(initial, numberOfTimeSteps, deltaT): n+1 times. */
void orc_time_discretization(double initial, int n, double dt, double* out);

/* ---- BrownianMotionFromMersenneRandomNumbers.doGenerateBrownianMotion: dW[T][F][P] */
void orc_brownian_increments(const double* times, int T, int F, int P, int seed, double* out);

/* ---- Linear algebra */
int orc_eigen_symmetric(int n, const double* A, double* evals, double* evecs /* column j = vector j */);
void orc_factor_matrix(const double* corr, int n, int F, double* out /* [n][F] */);
void orc_factor_reduction(const double* corr, int n, int F, double* out /* [n][F] */);
/* Least-squares solve A x = b via the SVD pseudo-inverse (one-sided Jacobi).
 * A is m x n row-major, b has m entries (k right-hand sides laid out [m][k]). */
int orc_lstsq_pinv(int m, int n, int k, const double* A, const double* B, double* X /* [n][k] */);

/* ---- Covariance model pieces */
/* LIBORCorrelationModelExponentialDecay: factor matrix [N][F] and reduced correlation [N][N]. */
void orc_exp_decay_correlation(const double* tenor, int N, int F, double a, double* factor, double* corr);
/* LIBORVolatilityModelFourParameterExponentialForm: vol[T][N] (time index x libor index). */
void orc_vol_abcd(const double* times, int T, const double* tenor, int N,
                  double a, double b, double c, double d, double* vol);
/* LIBORCovarianceModelFromVolatilityAndCorrelation: loadings[T][N][F] and variance[T][N]. */
void orc_covariance_tables(int T, int N, int F, const double* vol, const double* factor,
                           const double* corr, double* loadings, double* variance);
/* DiscountCurveFromForwardCurve.getDiscountFactor for a forward curve given by
 * nodes (LINEAR interpolation on values, CONSTANT extrapolation) and payment offset. */
double orc_curve_forward(const double* nodes, const double* values, int n, double t);
double orc_discount_factor_from_forward_curve(const double* nodes, const double* values, int n,
                                              double payment_offset, double maturity);
/* Deterministic numeraire adjustment chain P^d(T_i) (LIBORMarketModelFromCovarianceModel.java:915-944). */
void orc_numeraire_discount_chain(const double* tenor, int N, const double* df_at_tenor, double* out);

/* ---- The LMM process and products */
typedef struct {
    int T;                          /* number of simulation time steps */
    const double* times;            /* T+1 simulation times */
    int N;                          /* number of forward rates (libor periods) */
    const double* tenor;            /* N+1 tenor times */
    int F;                          /* number of factors */
    const double* loadings;         /* [T][N][F] */
    const double* variance;         /* [T][N] */
    const double* initial_forwards; /* [N] */
    const double* discount_chain;   /* [N+1] P^d(T_i), or NULL for no discount curve */
    double libor_cap;               /* +inf disables the cap */
    int scheme;                     /* 0 = EULER, 1 = EULER_FUNCTIONAL, 2 = PREDICTOR_CORRECTOR,
                                       3 = PREDICTOR_CORRECTOR_FUNCTIONAL */
    int measure;                    /* 0 = SPOT, 1 = TERMINAL */
    int state_space;                /* 0 = LOGNORMAL, 1 = NORMAL */
} orc_lmm;

typedef struct orc_sim orc_sim;

/* Euler process over dW[T][F][P]; keeps the forward vector at the observed time
 * indices (observe[T+1] != 0) and the spot numeraire at every tenor time. */
orc_sim* orc_simulate(const orc_lmm* m, int P, const double* dW, const uint8_t* observe, int threads);
void     orc_sim_free(orc_sim* s);
/* getProcessValue(timeIndex, component) for an observed time index. */
int orc_sim_process_value(const orc_sim* s, int time_index, int component, double* out);
/* getNumeraire(time) (adjusted) at a tenor time; returns 1 if deterministic. */
int orc_sim_numeraire(const orc_sim* s, double time, double* out);
int orc_sim_numeraire_unadjusted(const orc_sim* s, double time, double* out);
/* Kahan average (RandomVariableFromDoubleArray.getAverage). */
double orc_kahan_average(const double* x, int64_t n);
double orc_standard_error(const double* x, int64_t n);

/* Swaption.getValue(0, model) per path, then average / standard error. */
int orc_swaption(const orc_sim* s, double exercise, int nper, const double* fixing, const double* payment,
                 const double* period_length /* or NULL */, const double* strike, double notional,
                 double* value, double* stderr_out, double* per_path /* or NULL */);

/* BermudanSwaption.getValues(0, model).  basis_id 0 = the reference's built-in basis
 * {1, P_short, P_short^2, P_long, P_long^2, 1/N}; 1 = {1, S, S^2, N, N^2, S*N}. */
int orc_bermudan(const orc_sim* s, int nper, const uint8_t* exercisable, const double* fixing,
                 const double* period_length, const double* payment, const double* notional,
                 const double* strike, int callable, int basis_id,
                 double* value, double* stderr_out, double* per_path /* or NULL */,
                 double* exercise_time /* or NULL */);
/* The reference AAD's adjoint weights of the Bermudan's discounted cash flows (method 0:
 * diracDeltaApproximationMethod ZERO, 1: DISCRETE_DELTA with the given width per standard
 * deviation); omega [nper][P]. */
int orc_bermudan_aad(const orc_sim* s, int nper, const uint8_t* exercisable, const double* fixing,
                     const double* period_length, const double* payment, const double* notional,
                     const double* strike, int callable, int basis_id, int method, double width,
                     double* value, double* omega);

/* Bermudan value with frozen per-path exercise times (for finite differences of the
 * pathwise derivative). */
int orc_bermudan_frozen(const orc_sim* s, int nper, const double* fixing, const double* period_length,
                        const double* payment, const double* notional, const double* strike, int callable,
                        const double* exercise_time, double* value);

#ifdef __cplusplus
}
#endif
#endif
