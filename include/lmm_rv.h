/* lmm_rv.h -- device random variables: the C ABI behind a GPU RandomVariableFactory.
 *
 * Replaces, for a Java shim over JNI / Panama FFM, the elementwise algebra of
 *   net.finmath.montecarlo.RandomVariableFromDoubleArray
 *     (montecarlo/RandomVariableFromDoubleArray.java: getAverage :287-308, getVariance
 *      :332-354, getStandardError :419-428, scalar operations :743-1020, random-variable
 *      operations :1028-1486)
 * and the factory net.finmath.montecarlo.RandomVariableFactory (RandomVariableFactory.java:56-94).
 *
 * An lmm_rv is immutable: it is either deterministic (one value, the reference's
 * valueIfNonStochastic) or holds n realizations in device memory, with a filtration time.
 * Every operation returns a new lmm_rv, as the reference's operations return new objects;
 * an operation on two random variables takes the later filtration time.  FP64 semantics
 * are the reference's: every + - * / rounds separately, min/max follow Math.min/Math.max
 * (NaN wins, -0.0 < +0.0), choose selects on trigger >= 0.  exp, log, pow, sin and cos are
 * CUDA's (within 1-2 ulp of the reference's Math functions).  Averages are compensated
 * sums, as the reference's Kahan sums.  Work is enqueued on one library stream in call
 * order; host reads synchronise.  Status codes as lmm_gb300.h. */
#ifndef LMM_RV_H
#define LMM_RV_H

#include <stdint.h>

#include "lmm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lmm_rv lmm_rv;

/* operation codes */
enum {
    /* x op y for a random variable or a double y */
    LMM_RV_ADD = 0,       /* x + y   add            :773, :1028 */
    LMM_RV_SUB = 1,       /* x - y   sub            :788, :1061 */
    LMM_RV_BUS = 2,       /* y - x   bus            :803, :1094 */
    LMM_RV_MULT = 3,      /* x * y   mult           :818, :1124 */
    LMM_RV_DIV = 4,       /* x / y   div            :833, :1157 */
    LMM_RV_VID = 5,       /* y / x   vid            :848, :1187 */
    LMM_RV_CAP = 6,       /* min(x, y)  cap         :743, :1217 */
    LMM_RV_FLOOR = 7,     /* max(x, y)  floor       :758, :1246 */
    LMM_RV_POW = 8,       /* x^y (double y only)    :863 */
    /* unary (the double argument is ignored) */
    LMM_RV_SQUARED = 16,  /* x * x                  :889 */
    LMM_RV_SQRT = 17,     /*                        :904 */
    LMM_RV_EXP = 18,      /*                        :949 */
    LMM_RV_LOG = 19,      /*                        :979 */
    LMM_RV_SIN = 20,      /*                        :994 */
    LMM_RV_COS = 21,      /*                        :1009 */
    LMM_RV_INVERT = 22,   /* 1 / x                  :919 */
    LMM_RV_ABS = 23,      /*                        :934 */
    LMM_RV_ISNAN = 24,    /* 1.0 if NaN else 0.0    :1486 */
    LMM_RV_EXPM1 = 25,    /* exp(x) - 1             :964 */
    /* lmm_rv_apply3(x, op, a, b, c) */
    LMM_RV_ACCRUE = 32,      /* x * (1 + a * c)            accrue(rate a, period c)    :1279 */
    LMM_RV_DISCOUNT = 33,    /* x / (1.0 + a * c)          discount(rate a, period c)  :1308 */
    LMM_RV_CHOOSE = 34,      /* x >= 0 ? a : b             choose (x the trigger)      :1342 */
    LMM_RV_ADD_PRODUCT = 35, /* x + a * b, or x + a * c when b is NULL   addProduct     :1366, :1395 */
    LMM_RV_ADD_RATIO = 36,   /* x + a / b                  addRatio                    :1440 */
    LMM_RV_SUB_RATIO = 37    /* x - a / b                  subRatio                    :1463 */
};

/* createRandomVariable(time, value): a deterministic random variable */
int lmm_rv_create_constant(double time, double value, lmm_rv** out);
/* createRandomVariable(time, values[]): n realizations copied from host memory */
int lmm_rv_create(double time, const double* host, int64_t n, lmm_rv** out);
int lmm_rv_destroy(lmm_rv* x);
/* the CUDA stream (opaque) on which every random-variable operation is enqueued */
int lmm_rv_stream(void** out_stream);
/* filtration time, number of realizations (0 when deterministic), deterministic flag and,
 * when deterministic, the value (any output may be NULL) */
int lmm_rv_describe(const lmm_rv* x, double* out_time, int64_t* out_n, int* out_deterministic, double* out_value);
/* getRealizations(): n values (one value when deterministic) into host memory */
int lmm_rv_get(const lmm_rv* x, double* out_host);

/* binary operation with a double argument, or a unary operation (argument ignored) */
int lmm_rv_apply_scalar(const lmm_rv* x, int op, double y, lmm_rv** out);
/* binary operation x op y of two random variables (LMM_RV_ADD .. LMM_RV_FLOOR) */
int lmm_rv_apply(const lmm_rv* x, int op, const lmm_rv* y, lmm_rv** out);
/* the three-argument operations LMM_RV_ACCRUE .. LMM_RV_SUB_RATIO */
int lmm_rv_apply3(const lmm_rv* x, int op, const lmm_rv* a, const lmm_rv* b, double c, lmm_rv** out);

/* The float class, RandomVariableFromFloatArray (montecarlo/RandomVariableFromFloatArray.java):
 * FP32 realizations; + - * / in FP32 arithmetic, square root and the transcendental functions
 * in FP64 rounded to FP32, the deterministic forms in FP64, as the reference computes them
 * (:755-1486).  The receiver of an operation decides the class of its result; a
 * deterministic double-class receiver (a Scalar, type priority 0) hands the operation to a
 * float-class operand.  Reductions read the floats as doubles (:311-430).
 * lmm_rv_create_float: n FP32 realizations; lmm_rv_create_constant_float: a deterministic
 * value of the float class; lmm_rv_to_float: RandomVariableFromFloatArray(RandomVariable),
 * the realizations rounded to FP32 (:38-45, :214-220); lmm_rv_is_float: 1 for the float
 * class; lmm_rv_get_float: the FP32 realizations (lmm_rv_get widens them, :222-228). */
int lmm_rv_create_float(double time, const float* host, int64_t n, lmm_rv** out);
int lmm_rv_create_constant_float(double time, double value, lmm_rv** out);
int lmm_rv_to_float(const lmm_rv* x, lmm_rv** out);
int lmm_rv_is_float(const lmm_rv* x, int* out);
int lmm_rv_get_float(const lmm_rv* x, float* out_host);

/* getQuantile, getQuantileExpectation and getHistogram(intervalPoints)
 * (stochastic/RandomVariable.java:219-269; RandomVariableFromDoubleArray.java:446-553 and the
 * float class's :470-520): the realizations sorted on the device as java.util.Arrays.sort
 * orders them, the element at (int) Math.round((n + 1) q - 1) clamped to [0, n - 1], the
 * plain mean of the sorted range between two such indices, and the share of realizations in
 * each interval (out has num_points + 1 entries; the reference's deterministic case kept). */
int lmm_rv_quantile(const lmm_rv* x, double quantile, double* out);
int lmm_rv_quantile_expectation(const lmm_rv* x, double quantile_start, double quantile_end, double* out);
int lmm_rv_histogram(const lmm_rv* x, const double* interval_points, int num_points, double* out);

/* getAverage, getVariance, getStandardError, getMin / getMax (:257-283) */
int lmm_rv_average(const lmm_rv* x, double* out);
int lmm_rv_variance(const lmm_rv* x, double* out);
int lmm_rv_standard_error(const lmm_rv* x, double* out);
int lmm_rv_min_max(const lmm_rv* x, double* out_min, double* out_max);

/* The simulation's process values and numeraire as device random variables, without a
 * host round trip: LIBORModelMonteCarloSimulationModel.getLIBOR(timeIndex, liborIndex)
 * (LIBORMonteCarloSimulationFromLIBORModel.java:123-126, the FP32 states of the mixed form
 * widened to FP64) and getNumeraire(time) (:153-155, with the discount-curve adjustment of
 * LIBORMarketModelFromCovarianceModel.java:860-876). */
int lmm_process_get_value_rv(lmm_process* proc, int time_index, int component, lmm_rv** out);
int lmm_process_get_numeraire_rv(lmm_process* proc, double time, lmm_rv** out);
/* The numeraire before the discount-curve adjustment at a tenor time,
 * getNumerairetUnAdjusted (LIBORMarketModelFromCovarianceModel.java:968-1015): the building
 * block of getNumeraire between tenor times, where the reference discounts the next tenor
 * time's unadjusted numeraire with the short forward rate and re-applies the adjustment. */
int lmm_process_get_numeraire_unadjusted_rv(lmm_process* proc, double time, lmm_rv** out);

#ifdef __cplusplus
}
#endif

#endif /* LMM_RV_H */
