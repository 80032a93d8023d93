/*
 * lmm_gb300.h -- C ABI of the GB300-native LIBOR Market Model Monte Carlo library.
 *
 * This is the drop-in boundary a finmath-lib host binds (JNI / Panama FFM / ctypes):
 * plain C types, host pointers and sizes, no CUDA or torch types.  Every entry point
 * names the finmath-lib interface it replaces (file:line in finmath-lib's
 * src/main/java/net/finmath/ tree).
 *
 * Conventions
 *   - Every function returns an int status: LMM_OK (0) or a negative LMM_ERR_* code;
 *     lmm_last_error() returns a thread-local message for the last failure.  A finmath
 *     shim maps these to CalculationException (valuation path) or
 *     IllegalArgumentException (invalid arguments).
 *   - Host arrays are caller-owned and copied on input; device memory is owned by the
 *     handle and released by the matching *_destroy.
 *   - A handle is used by one thread at a time (the Java shim serialises per handle,
 *     as finmath's lazy initialisation is synchronized); different handles may be used
 *     concurrently.  Each handle enqueues its work on its own CUDA stream.
 *   - Arrays of random variables are [index][path] row-major: one contiguous path
 *     vector per (time, component), i.e. RandomVariable.getRealizations() layout.
 */
#ifndef LMM_GB300_H
#define LMM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LMM_OK 0
#define LMM_ERR_INVALID (-1)   /* invalid argument or unsupported configuration */
#define LMM_ERR_NOMEM (-2)     /* device or host allocation failed */
#define LMM_ERR_CUDA (-3)      /* CUDA runtime error (message holds the CUDA error string) */
#define LMM_ERR_TIMEOUT (-4)   /* a bounded device-side wait gave up */
#define LMM_ERR_STATE (-5)     /* call out of order (e.g. value requested before simulation) */

/* Precision forms of the path. */
#define LMM_PRECISION_FP64 0   /* plain FP64: the parity form */
#define LMM_PRECISION_MIXED 1  /* FP32 log-space paths, FP64 numeraire / regression / sums */

/* Discretisation schemes: EulerSchemeFromProcessModel.Scheme (montecarlo/process/EulerSchemeFromProcessModel.java:68-73). */
#define LMM_SCHEME_EULER 0
#define LMM_SCHEME_EULER_FUNCTIONAL 1
#define LMM_SCHEME_PREDICTOR_CORRECTOR 2             /* FP64 only */
#define LMM_SCHEME_PREDICTOR_CORRECTOR_FUNCTIONAL 3  /* FP64 only */

/* LIBORMarketModelFromCovarianceModel.Measure and .StateSpace
 * (…/interestrate/models/LIBORMarketModelFromCovarianceModel.java:1148-1189, :1081-1093).
 * TERMINAL and NORMAL are FP64 only, and the adjoint takes SPOT, LOGNORMAL and the Euler
 * schemes. */
#define LMM_MEASURE_SPOT 0
#define LMM_MEASURE_TERMINAL 1
#define LMM_STATE_SPACE_LOGNORMAL 0
#define LMM_STATE_SPACE_NORMAL 1

/* Regression bases of the Bermudan swaption. */
#define LMM_BASIS_REFERENCE 0  /* BermudanSwaption.getBasisFunctions: {1, P_short, P_short^2, P_long, P_long^2, 1/N} (…/products/BermudanSwaption.java:215-252) */
#define LMM_BASIS_SWAPRATE 1   /* a RegressionBasisFunctionsProvider giving {1, S, S^2, N, N^2, S*N} (conditionalexpectation/RegressionBasisFunctionsProvider.java:28) */

const char* lmm_last_error(void);
int lmm_version(void);

/* ---------------------------------------------------------------- host-side model setup
 * Tables a finmath shim can equally take from its own Java objects. */

/* TimeDiscretizationFromArray(initial, numberOfTimeSteps, deltaT) with tick rounding
 * (time/TimeDiscretizationFromArray.java:210-217, 387-389).  out has num_steps+1 entries. */
int lmm_time_discretization(double initial, int num_steps, double dt, double* out_times);

/* LinearAlgebra.factorReduction (functions/LinearAlgebra.java:380-482): n x n
 * correlation -> n x num_factors factor matrix (row-major). */
int lmm_factor_reduction(const double* correlation, int n, int num_factors, double* out_factors);

/* LIBORCorrelationModelExponentialDecay (…/covariance/LIBORCorrelationModelExponentialDecay.java:102-134):
 * rho_ij = exp(-a |T_i - T_j|) reduced to num_factors; outputs the factor matrix
 * [num_periods][num_factors] and the reduced correlation [num_periods][num_periods]. */
int lmm_correlation_exponential_decay(const double* tenor, int num_periods, int num_factors, double a,
                                      double* out_factor_matrix, double* out_correlation);

/* LIBORVolatilityModelFourParameterExponentialForm.getVolatility
 * (…/covariance/LIBORVolatilityModelFourParameterExponentialForm.java:168-194): out [num_steps][num_periods]. */
int lmm_volatility_four_parameter(const double* times, int num_steps, const double* tenor, int num_periods,
                                  double a, double b, double c, double d, double* out_volatility);

/* LIBORCovarianceModelFromVolatilityAndCorrelation.getFactorLoading / getCovariance
 * (…/covariance/LIBORCovarianceModelFromVolatilityAndCorrelation.java:48-57, 83-93):
 * loadings [num_steps][num_periods][num_factors], variance [num_steps][num_periods]. */
int lmm_covariance_tables(int num_steps, int num_periods, int num_factors, const double* volatility,
                          const double* factor_matrix, const double* correlation, double* out_loadings,
                          double* out_variance);

/* ForwardCurveInterpolation (LINEAR on values, CONSTANT extrapolation) value at t
 * (marketdata/model/curves/ForwardCurveInterpolation.java:224-233, 298-346). */
int lmm_forward_curve_value(const double* nodes, const double* values, int num_nodes, double t, double* out);

/* DiscountCurveFromForwardCurve.getDiscountFactor (marketdata/model/curves/DiscountCurveFromForwardCurve.java:115-140). */
int lmm_discount_factor_from_forward_curve(const double* nodes, const double* values, int num_nodes,
                                           double payment_offset, double maturity, double* out);

/* The deterministic numeraire adjustment P^d(T_i) chain of
 * LIBORMarketModelFromCovarianceModel.getNumeraireDefaultableZeroBondAsOfTimeZero
 * (…/models/LIBORMarketModelFromCovarianceModel.java:915-944); df has num_periods+1 entries. */
int lmm_numeraire_discount_chain(const double* tenor, int num_periods, const double* discount_factors,
                                 double* out_chain);

/* x solving A x = b (A n x n, row-major) by the SVD pseudo-inverse with the cutoff
 * max(n sigma_max 2^-52, sqrt(2^-1022)): new SingularValueDecomposition(A).getSolver().solve(b)
 * as MonteCarloConditionalExpectationRegression.getLinearRegressionParameters uses it
 * (montecarlo/conditionalexpectation/MonteCarloConditionalExpectationRegression.java:125-147,
 * commons-math3 3.6.1).  Host computation, n <= 64. */
int lmm_solve_svd(int n, const double* A, const double* b, double* x);

/* ---------------------------------------------------------------- Brownian motion */
typedef struct lmm_brownian lmm_brownian;

/* new BrownianMotionFromMersenneRandomNumbers(timeDiscretization, numberOfFactors, numberOfPaths, seed)
 * (montecarlo/BrownianMotionFromMersenneRandomNumbers.java:69-103).  Generation is lazy,
 * as in the reference (:123-131): it runs at the first increment request or simulation. */
int lmm_brownian_create(const double* times, int num_times, int num_factors, int num_paths, int seed,
                        int precision, lmm_brownian** out);
/* getBrownianIncrement(timeIndex, factor) (:123-136): num_paths doubles. */
int lmm_brownian_get_increment(lmm_brownian* bm, int time_index, int factor, double* out_host);
/* getCloneWithModifiedSeed(seed) (:106-109) in place: the increments are regenerated
 * lazily with the new seed, reusing the device allocation; processes built on this
 * Brownian motion re-simulate on their next use. */
int lmm_brownian_set_seed(lmm_brownian* bm, int seed);
/* doGenerateBrownianMotion (:141-191), explicit trigger. */
int lmm_brownian_generate(lmm_brownian* bm);
int lmm_brownian_destroy(lmm_brownian* bm);

/* The MT19937 stream of commons-math3 MersenneTwister(seed).nextDouble() as used by
 * randomnumbers/MersenneTwister.java:42-51, values [offset, offset+count) generated on
 * the GPU by the same partitioned generator. */
int lmm_mt19937_uniforms(int64_t seed, int64_t offset, int64_t count, double* out_host);

/* The same stream computed on the host by one GF(2) jump of `skip` words followed by
 * sequential generation: tempered 32-bit words [skip, skip+count).  A check of the jump
 * polynomials that needs no GPU; not a production path. */
int lmm_mt19937_words_host(int64_t seed, uint64_t skip, uint64_t count, uint32_t* out);

/* Tempered words [chunk * stride_words, + count) of the same stream, reached on the host the
 * way a generator block reaches its chunk: one GF(2) jump x^(d 8^j stride) per nonzero
 * base-8 digit d (position j) of the chunk index.  A check of the chunk jump polynomials
 * that needs no GPU; not a production path. */
int lmm_mt19937_chunk_words_host(int64_t seed, uint64_t stride_words, uint64_t chunk, uint64_t count,
                                 uint32_t* out);

/* ---------------------------------------------------------------- LMM process */
typedef struct {
    int num_steps;                  /* T: simulation time steps */
    const double* times;            /* T+1 simulation times (the Brownian motion's grid) */
    int num_periods;                /* N: forward rates */
    const double* tenor;            /* N+1 tenor times */
    int num_factors;                /* F */
    const double* factor_loadings;  /* [T][N][F]  lambda_{i,j,k} = sigma_{i,j} f_{j,k} */
    const double* variance;         /* [T][N]     getCovariance(t_i, j, j) */
    const double* initial_forwards; /* [N]        forward curve at T_j over the period */
    const double* discount_chain;   /* [N+1]      P^d(T_l), or NULL for no discount curve */
    double libor_cap;               /* liborCap property (default 1e5); +inf disables */
    int scheme;                     /* LMM_SCHEME_* */
    int measure;                    /* LMM_MEASURE_* */
    int state_space;                /* LMM_STATE_SPACE_* */
    const double* volatility;       /* [T][N] sigma_{i,j}, optional: the leaves of the vegas
                                       (NULL: sqrt(variance), i.e. rho_jj = 1) */
} lmm_model_desc;

typedef struct lmm_process lmm_process;

/* LIBORMarketModelFromCovarianceModel.of(...) (…/models/LIBORMarketModelFromCovarianceModel.java:283, 388-444)
 * + new EulerSchemeFromProcessModel(model, brownianMotion) (montecarlo/process/EulerSchemeFromProcessModel.java:101-123)
 * + new LIBORMonteCarloSimulationFromLIBORModel(process) (montecarlo/interestrate/LIBORMonteCarloSimulationFromLIBORModel.java:32-37).
 * The process keeps a reference to bm (which must outlive it) and uses bm's precision. */
int lmm_process_create(const lmm_model_desc* model, lmm_brownian* bm, lmm_process** out);
/* Restrict storage to the time indices in mask[T+1] (non-zero = keep).  The default is
 * every time index (the reference materialises all).  Products need the tenor times. */
int lmm_process_set_observed_times(lmm_process* proc, const uint8_t* mask);
/* doPrecalculateProcess (EulerSchemeFromProcessModel.java:170-326), explicit trigger;
 * the getters below trigger it lazily. */
int lmm_process_simulate(lmm_process* proc);
/* getProcessValue(timeIndex, component) (:132-146) == getLIBOR(timeIndex, liborIndex)
 * (LIBORMarketModelFromCovarianceModel.java:1308-1312): num_paths doubles. */
int lmm_process_get_value(lmm_process* proc, int time_index, int component, double* out_host);
/* LIBORMonteCarloSimulationFromLIBORModel.getNumeraire(time) (:153-155) at a tenor time: num_paths doubles. */
int lmm_process_get_numeraire(lmm_process* proc, double time, double* out_host);
int lmm_process_destroy(lmm_process* proc);

/* ---------------------------------------------------------------- products */
typedef struct {
    double exercise_date;
    int num_periods;
    const double* fixing_dates;     /* [n] */
    const double* payment_dates;    /* [n] */
    const double* period_lengths;   /* [n] or NULL (payment - fixing) */
    const double* swaprates;        /* [n] */
    double notional;
} lmm_swaption_desc;

/* Swaption.getValue(evaluationTime 0, model) (montecarlo/interestrate/products/Swaption.java:137-199),
 * then getAverage / getStandardError (montecarlo/AbstractMonteCarloProduct.java:82-104). */
int lmm_swaption_get_value(lmm_process* proc, const lmm_swaption_desc* product, double* out_value,
                           double* out_error);

/* The same values for n_products swaptions on each of n_processes processes (a calibration's
 * trial models, which share one Brownian motion): the simulations, the fused swaption kernels and
 * the mean / variance reductions are queued on the processes' streams without a host round
 * trip, then each process's results come back in one copy.  out_values[n_processes][n_products];
 * out_errors likewise, or NULL. */
int lmm_swaption_values_batch(int n_processes, lmm_process* const* processes, int n_products,
                              const lmm_swaption_desc* products, double* out_values, double* out_errors);

typedef struct {
    int num_periods;
    const uint8_t* is_exercise_date;  /* [n] isPeriodStartDateExerciseDate */
    const double* fixing_dates;       /* [n] */
    const double* period_lengths;     /* [n] */
    const double* payment_dates;      /* [n] */
    const double* notionals;          /* [n] periodNotionals */
    const double* swaprates;          /* [n] */
    int is_callable;                  /* isCallable */
    int basis;                        /* LMM_BASIS_* */
} lmm_bermudan_desc;

/* BermudanSwaption.getValues(evaluationTime 0, model) (montecarlo/interestrate/products/BermudanSwaption.java:91-157):
 * value and error (standard error).  out_values_host (optional, num_paths doubles)
 * receives the per-path values (the "value" random variable). */
int lmm_bermudan_get_value(lmm_process* proc, const lmm_bermudan_desc* product, double* out_value,
                           double* out_error, double* out_values_host);

/* Mean and standard error of num_values doubles already in device memory (d_values),
 * computed with the same compensated reduction as the product entry points, without
 * allocating anything.  No counterpart in finmath-lib: it exists for callers that must
 * not allocate device memory on their valuation path -- a pricing service that reserves
 * its whole device budget at start-up and forbids allocator calls afterwards (a JVM host
 * sharing one GPU between several engines, each held to a fixed slice), or code running
 * where an allocator call would stall other work on the device.  Its scratch is one fixed
 * 8,208-byte array per GPU inside the library (held until the process exits), so:
 *   - num_values must be in [1, 2^30]; larger inputs are rejected with LMM_ERR_INVALID;
 *   - every call shares that array: calls that overlap on the GPU (different streams, or
 *     different host threads on one device) race and must be serialised by the caller;
 *   - the call copies its two results to the host and waits for them, so it must not be
 *     made while any stream is being captured into a graph (the capture would be
 *     invalidated); graph users call it between graph launches;
 *   - the first call on a device looks up the array's device address (which may load the
 *     library's GPU code on that device);
 *   - the looked-up address is kept for the life of the process: the library must not be
 *     used on a device after cudaDeviceReset there.
 * stream is a cudaStream_t (NULL = the legacy default stream); d_values must be ready in
 * stream order.  The call waits for the two results and writes them to host memory. */
int lmm_values_mean_stderr_noalloc(const double* d_values, int64_t num_values, void* stream, double* out_mean,
                                   double* out_error);

/* BermudanSwaption value and its gradient, as RandomVariableDifferentiable.getGradient()
 * (montecarlo/automaticdifferentiation/RandomVariableDifferentiable.java:56-75) gives it for
 * the initial forwards and the volatility-matrix entries as leaves
 * (LIBORMarketModelNormalAADSensitivitiesTest.java:343-355, 431-434).  A hand-written adjoint
 * of the Euler step (LOGNORMAL: in log coordinates; NORMAL, FP64 processes, uncapped: on the
 * forwards themselves) replays each path backward from checkpoints written every
 * checkpoint_stride steps (1..16); the steps between checkpoints are recomputed by the
 * path kernel's own step, so the stride trades memory for time without changing a bit of
 * the result (LOGNORMAL SPOT Euler processes; other FP64 forms replay in plain FP64);
 * exercise decisions are frozen from the forward valuation.  freeze_numeraire_adjustment = 1 treats the numeraire adjustment's path
 * average as a constant, as the reference's AAD does (RandomVariableDifferentiableAAD
 * getAverage returns a double); 0 differentiates through it (the derivative that central
 * finite differences of the value measure).
 * out_deltas[N] = d value / d initial forward j; out_vegas[T][N] = d value / d sigma_{i,j}
 * (zero where sigma_{i,j} does not enter: t_i >= T_j). */
int lmm_bermudan_get_gradient(lmm_process* proc, const lmm_bermudan_desc* product, int checkpoint_stride,
                              int freeze_numeraire_adjustment, double* out_value, double* out_error,
                              double* out_deltas, double* out_vegas);

/* The same gradient with RandomVariableDifferentiableAADFactory's diracDeltaApproximationMethod
 * (montecarlo/automaticdifferentiation/backward/RandomVariableDifferentiableAADFactory.java:
 * 60-72): LMM_DIRAC_ZERO is lmm_bermudan_get_gradient (exercise decisions frozen);
 * LMM_DIRAC_DISCRETE_DELTA (the reference's default, width 0.05) runs the reference AAD's
 * reverse sweep over the backward induction (RandomVariableDifferentiableAAD.java:171-208,
 * 396-429): each choice passes (Y - Z) 1{-eps/2 <= X < eps/2} / eps, eps = dirac_width x the
 * trigger's standard deviation, to its trigger, and the trigger's conditional expectation
 * hands that adjoint to its argument through the same regression; the resulting weights of
 * the cash flows seed the adjoint of the Euler scheme.  FP64 processes only. */
#define LMM_DIRAC_ZERO 0
#define LMM_DIRAC_DISCRETE_DELTA 1
int lmm_bermudan_get_gradient_aad(lmm_process* proc, const lmm_bermudan_desc* product, int checkpoint_stride,
                                  int freeze_numeraire_adjustment, int dirac_method, double dirac_width,
                                  double* out_value, double* out_error, double* out_deltas, double* out_vegas);

/* Gradients of the European products the reference's sensitivity test differentiates
 * (LIBORMarketModelNormalAADSensitivitiesTest.java:127-165): Swaption.getValue
 * (montecarlo/interestrate/products/Swaption.java:137-199) and Caplet.getValue
 * (montecarlo/interestrate/products/Caplet.java:100-147).  Their payoffs are floored at 0,
 * whose AAD derivative is 1 where the argument is >= 0 (RandomVariableDifferentiableAAD.java:
 * 324-331), so the gradient is pathwise: per path the derivative of the value to every
 * state of the product's observation date (the swaption's forwards at the exercise date and
 * the fixings of its numeraire; the caplet's fixing L_m(T_m) and the fixings of N(T_{m+1})),
 * the numeraire adjustment held constant, then the adjoint of the Euler scheme back to the
 * initial forwards and the volatility matrix (as lmm_bermudan_get_gradient).  FP64
 * processes; the LOGNORMAL or NORMAL state space.  The swaption's value and error are the
 * plain valuation's (the same kernel and reduction).  The caplet's period [maturity,
 * maturity + period_length] must be a tenor period; daycount is its day count fraction. */
int lmm_swaption_get_gradient(lmm_process* proc, const lmm_swaption_desc* product, int checkpoint_stride,
                              double* out_value, double* out_error, double* out_deltas, double* out_vegas);
int lmm_caplet_get_gradient(lmm_process* proc, double maturity, double period_length, double strike,
                            double daycount_fraction, int checkpoint_stride, double* out_deltas, double* out_vegas);

/* ---------------------------------------------------------------- portfolio batch
 * A portfolio of Bermudan swaptions valued, with their deltas and vegas, on one shared
 * simulation: the per-product work (regression, backward induction, adjoint) is recorded
 * once into a CUDA graph whose launch values the whole portfolio.  finmath-lib values a
 * portfolio product by product on a shared LIBORMonteCarloSimulationFromLIBORModel
 * (AbstractMonteCarloProduct.getValues, montecarlo/AbstractMonteCarloProduct.java:87-104);
 * this is that loop, batched. */
typedef struct {
    int num_products;
    const lmm_bermudan_desc* products;  /* [num_products] */
    int with_greeks;                     /* 0: values and errors only */
    int checkpoint_stride;               /* adjoint checkpoint stride, 1..16 */
    int concurrency;                     /* products in flight (independent branches of the graph), 1..16 */
    int adjoint_threads;                 /* paths per adjoint block: 64, 128 or 256 */
    int gram_blocks;                     /* blocks per exercise date in the Gram pass (0: automatic) */
} lmm_portfolio_desc;

typedef struct lmm_portfolio lmm_portfolio;

/* Validates every product, allocates per-branch scratch, and records the graph. */
int lmm_portfolio_create(lmm_process* proc, const lmm_portfolio_desc* desc, lmm_portfolio** out);
/* One graph launch: out_values/out_errors [n]; out_deltas [n][N] and out_vegas [n][T][N] (with
 * greeks, else may be NULL); out_latency_ms [n] = completion time of each product measured on
 * the device from the start of the launch (may be NULL); out_total_ms the device time of the
 * whole launch (may be NULL). */
int lmm_portfolio_run(lmm_portfolio* pf, double* out_values, double* out_errors, double* out_deltas, double* out_vegas,
                      double* out_latency_ms, double* out_total_ms);
int lmm_portfolio_destroy(lmm_portfolio* pf);

/* ---------------------------------------------------------------- instrumentation */
/* Per-kernel launch counts and (when enabled) CUDA-event times of this library's kernels. */
int lmm_stats_enable_timing(int enable);
int lmm_stats_reset(void);
/* Fills names[i] (static strings), launches[i], total_ms[i] for up to max entries; returns the count. */
int lmm_stats_get(int max, const char** names, int64_t* launches, double* total_ms);
/* Bytes this library has copied from host to device since it was loaded (tables, states,
 * parameters): the difference across a call is that call's host-to-device traffic. */
int lmm_stats_h2d_bytes(int64_t* out);
/* Bytes reserved from the device and in use in the current device's default stream-ordered
 * memory pool, the pool every allocation of this library comes from: the difference across
 * a call is that call's pool traffic. */
int lmm_stats_pool_bytes(int64_t* out_reserved, int64_t* out_used);
/* The CUDA stream (as an opaque pointer) on which a process enqueues its work. */
int lmm_process_stream(lmm_process* proc, void** out_stream);
/* A FP64 fused-multiply-add throughput probe (DFMA/s), used to report the FP64 roofline. */
int lmm_probe_fp64_fma_rate(double* out_fma_per_second);

/* Self-check of the FP64 path kernel's small-argument exp (table-driven, |d| <= 1) and
 * Newton reciprocal against CUDA's exp and correctly rounded division on n grid points:
 * the largest errors in ulps.  A test of the device arithmetic; not a production path. */
int lmm_fp64_math_check(int64_t n, double* max_ulp_exp, double* max_ulp_rcp);

#ifdef __cplusplus
}
#endif
#endif /* LMM_GB300_H */
