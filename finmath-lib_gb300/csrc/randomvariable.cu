// randomvariable.cu -- device random variables (lmm_rv.h): the elementwise algebra of
// RandomVariableFromDoubleArray (montecarlo/RandomVariableFromDoubleArray.java) on GB300.
//
// A random variable is one deterministic value or n FP64 realizations in device memory, or
// of the float class (RandomVariableFromFloatArray.java): FP32 realizations, FP32 arithmetic
// for + - * / and the rest in FP64 rounded to FP32, as the reference's float class computes.
// Each operation is one streaming kernel over its operands (an HBM-bound pass: 8 bytes read
// per stochastic operand and 8 written per realization), launched on one library stream.
// Deterministic operands are broadcast as kernel arguments; an operation whose operands
// are all deterministic is evaluated on the host with the same formula.  This translation
// unit is compiled with -fmad=false and the host side with -ffp-contract=off, so that every
// + - * / rounds separately, as the reference's Java does.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "lmm_internal.h"
#include "lmm_rv.h"
#include "reduce.cuh"

struct lmm_rv {
    double time = 0.0;
    int64_t n = 0;          // 0: deterministic
    double value = 0.0;     // the deterministic value
    double* d = nullptr;    // n FP64 realizations (device), nullptr when deterministic or FP32
    float* f = nullptr;     // n FP32 realizations (device) of the float class
    int fp32 = 0;           // RandomVariableFromFloatArray class (deterministic ones included)
};

namespace lmm {
namespace {

constexpr int kRvThreads = 256;

cudaStream_t rv_stream()
{
    static cudaStream_t s = nullptr;
    static std::once_flag once;
    std::call_once(once, [] { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); });
    return s;
}

// Math.min / Math.max: a NaN operand gives NaN, and -0.0 is below +0.0
__host__ __device__ __forceinline__ double java_min(double a, double b)
{
    if (a != a) return a;
    if (b != b) return b;
    if (a < b) return a;
    if (b < a) return b;
    return signbit(a) ? a : b;
}
__host__ __device__ __forceinline__ double java_max(double a, double b)
{
    if (a != a) return a;
    if (b != b) return b;
    if (a > b) return a;
    if (b > a) return b;
    return signbit(a) ? b : a;
}

// Math.pow where its special cases differ from C's pow: a NaN exponent gives NaN, and
// |x| = 1 with an infinite exponent gives NaN.  Java's pow (fdlibm's e_pow) also answers
// the exponents +-1, 2 and 0.5 exactly: x, 1/x, x*x and, for x >= +0, sqrt(x); so do these,
// which keeps x.pow(2.0) == x.squared() and x.pow(0.5) == x.sqrt() bit for bit.
__host__ __device__ __forceinline__ double java_pow(double x, double y)
{
    if (y != y) return y;
    if (fabs(x) == 1.0 && isinf(y)) return y - y;  // NaN
    if (y == 1.0) return x;
    if (y == -1.0) return 1.0 / x;
    if (y == 2.0) return x * x;
    if (y == 0.5 && !signbit(x)) return sqrt(x);
    return pow(x, y);
}

// One realization of operation OP; a, b are the operands' realizations (or values), c the
// double argument, has_b whether b is given (addProduct with a double factor otherwise).
template <int OP>
__host__ __device__ __forceinline__ double rv_op(double x, double a, double b, double c, bool has_b)
{
    switch (OP) {
        case LMM_RV_ADD: return x + a;
        case LMM_RV_SUB: return x - a;
        case LMM_RV_BUS: return a - x;
        case LMM_RV_MULT: return x * a;
        case LMM_RV_DIV: return x / a;
        case LMM_RV_VID: return a / x;
        case LMM_RV_CAP: return java_min(x, a);
        case LMM_RV_FLOOR: return java_max(x, a);
        case LMM_RV_POW: return java_pow(x, a);
        case LMM_RV_SQUARED: return x * x;
        case LMM_RV_SQRT: return sqrt(x);
        case LMM_RV_EXP: return exp(x);
        case LMM_RV_LOG: return log(x);
        case LMM_RV_SIN: return sin(x);
        case LMM_RV_COS: return cos(x);
        case LMM_RV_INVERT: return 1.0 / x;
        case LMM_RV_ABS: return fabs(x);
        case LMM_RV_ISNAN: return (x != x) ? 1.0 : 0.0;
        case LMM_RV_EXPM1: return expm1(x);
        case LMM_RV_ACCRUE: return x * (1 + a * c);
        case LMM_RV_DISCOUNT: return x / (1.0 + a * c);
        case LMM_RV_CHOOSE: return x >= 0.0 ? a : b;
        case LMM_RV_ADD_PRODUCT: return has_b ? x + a * b : x + a * c;
        case LMM_RV_ADD_RATIO: return x + a / b;
        case LMM_RV_SUB_RATIO: return x - a / b;
        default: return x;
    }
}

struct Operand {
    const double* p;  // FP64 realizations, or nullptr
    const float* pf;  // FP32 realizations, or nullptr (both null: the value v)
    double v;
};

__device__ __forceinline__ double load(const Operand& o, int64_t i)
{
    return o.p ? __ldg(o.p + i) : o.pf ? (double)__ldg(o.pf + i) : o.v;
}
// an operand as the float class reads it: (float) get(i)
__device__ __forceinline__ float loadf(const Operand& o, int64_t i)
{
    return o.pf ? __ldg(o.pf + i) : o.p ? (float)__ldg(o.p + i) : (float)o.v;
}

// Math.min / Math.max on floats (NaN wins, -0.0f below +0.0f)
__host__ __device__ __forceinline__ float java_minf(float a, float b)
{
    if (a != a) return a;
    if (b != b) return b;
    if (a < b) return a;
    if (b < a) return b;
    return signbit(a) ? a : b;
}
__host__ __device__ __forceinline__ float java_maxf(float a, float b)
{
    if (a != a) return a;
    if (b != b) return b;
    if (a > b) return a;
    if (b > a) return b;
    return signbit(a) ? b : a;
}

// One realization of operation OP in the float class (RandomVariableFromFloatArray.java:
// 755-1486): x the receiver as a float, a and b the operands as (float) get(i), c the double
// argument; xd the receiver's double value when it is deterministic (xdet), which floor reads
// unrounded (:1249).  + - * / in FP32, square root and the transcendentals in FP64 rounded to
// FP32 ((float) Math.f), pow with its exponent (the operand a) first rounded to FP32.
template <int OP>
__device__ __forceinline__ float rv_op_f32(float x, float a, float b, double c, bool has_b, double xd, bool xdet)
{
    switch (OP) {
        case LMM_RV_ADD: return x + a;
        case LMM_RV_SUB: return x - a;
        case LMM_RV_BUS: return a - x;
        case LMM_RV_MULT: return x * a;
        case LMM_RV_DIV: return x / a;
        case LMM_RV_VID: return a / x;
        case LMM_RV_CAP: return java_minf(x, a);
        case LMM_RV_FLOOR: return xdet ? (float)java_max(xd, (double)a) : java_maxf(x, a);
        case LMM_RV_POW: return (float)java_pow((double)x, (double)a);  // a: the exponent as (float) exponent
        case LMM_RV_SQUARED: return x * x;
        case LMM_RV_SQRT: return (float)sqrt((double)x);
        case LMM_RV_EXP: return (float)exp((double)x);
        case LMM_RV_LOG: return (float)log((double)x);
        case LMM_RV_SIN: return (float)sin((double)x);
        case LMM_RV_COS: return (float)cos((double)x);
        case LMM_RV_INVERT: return 1.0f / x;
        case LMM_RV_ABS: return fabsf(x);
        case LMM_RV_ISNAN: return (x != x) ? 1.0f : 0.0f;
        case LMM_RV_EXPM1: return (float)exp((double)x) - 1.0f;  // the interface's exp().sub(1.0)
        case LMM_RV_ACCRUE: return x * (1.0f + a * (float)c);
        case LMM_RV_DISCOUNT: return x / (1.0f + a * (float)c);
        case LMM_RV_CHOOSE: return x >= 0.0f ? a : b;
        case LMM_RV_ADD_PRODUCT: return has_b ? x + a * b : x + a * (float)c;
        case LMM_RV_ADD_RATIO: return x + a / b;
        case LMM_RV_SUB_RATIO: return x - a / b;
        default: return x;
    }
}

// Four independent elements per thread per iteration (strided by the grid) keep enough
// loads in flight to stream at HBM bandwidth.
template <int OP>
__global__ void __launch_bounds__(kRvThreads) rv_kernel(Operand x, Operand a, Operand b, double c, bool has_b, double* out,
                                                        int64_t n)
{
    const int64_t stride = (int64_t)gridDim.x * kRvThreads;
    for (int64_t i0 = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i0 < n; i0 += 4 * stride) {
        double r[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t i = i0 + k * stride;
            r[k] = i < n ? rv_op<OP>(load(x, i), load(a, i), load(b, i), c, has_b) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t i = i0 + k * stride;
            if (i < n) out[i] = r[k];
        }
    }
}

template <int OP>
__global__ void __launch_bounds__(kRvThreads) rv_kernel_f32(Operand x, Operand a, Operand b, double c, bool has_b,
                                                            bool xdet, float* out, int64_t n)
{
    const int64_t stride = (int64_t)gridDim.x * kRvThreads;
    for (int64_t i0 = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i0 < n; i0 += 4 * stride) {
        float r[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t i = i0 + k * stride;
            r[k] = i < n ? rv_op_f32<OP>(loadf(x, i), loadf(a, i), loadf(b, i), c, has_b, x.v, xdet) : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t i = i0 + k * stride;
            if (i < n) out[i] = r[k];
        }
    }
}

int rv_blocks(int64_t n)
{
    static int cap = 0;
    if (!cap) {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 152;
        cap = sms * 8;
    }
    const int64_t need = (n + 4 * kRvThreads - 1) / (4 * kRvThreads);
    return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

template <int OP>
void launch_op(const Operand& x, const Operand& a, const Operand& b, double c, bool has_b, double* out, int64_t n)
{
    rv_kernel<OP><<<rv_blocks(n), kRvThreads, 0, rv_stream()>>>(x, a, b, c, has_b, out, n);
}

template <int OP>
void launch_op_f32(const Operand& x, const Operand& a, const Operand& b, double c, bool has_b, bool xdet, float* out,
                   int64_t n)
{
    rv_kernel_f32<OP><<<rv_blocks(n), kRvThreads, 0, rv_stream()>>>(x, a, b, c, has_b, xdet, out, n);
}

template <int OP>
double host_op(double x, double a, double b, double c, bool has_b)
{
    return rv_op<OP>(x, a, b, c, has_b);
}

#define LMM_RV_OPS(X)                                                                                                     \
    X(LMM_RV_ADD) X(LMM_RV_SUB) X(LMM_RV_BUS) X(LMM_RV_MULT) X(LMM_RV_DIV) X(LMM_RV_VID) X(LMM_RV_CAP) X(LMM_RV_FLOOR)     \
    X(LMM_RV_POW) X(LMM_RV_SQUARED) X(LMM_RV_SQRT) X(LMM_RV_EXP) X(LMM_RV_LOG) X(LMM_RV_SIN) X(LMM_RV_COS)                \
    X(LMM_RV_INVERT) X(LMM_RV_ABS) X(LMM_RV_ISNAN) X(LMM_RV_EXPM1) X(LMM_RV_ACCRUE) X(LMM_RV_DISCOUNT) X(LMM_RV_CHOOSE)  \
    X(LMM_RV_ADD_PRODUCT) X(LMM_RV_ADD_RATIO) X(LMM_RV_SUB_RATIO)

bool valid_op(int op)
{
    switch (op) {
#define LMM_RV_CASE(o) case o:
        LMM_RV_OPS(LMM_RV_CASE)
#undef LMM_RV_CASE
        return true;
        default: return false;
    }
}

// evaluate op: on the host when every operand is deterministic, else one kernel
int dispatch(int op, const Operand& x, const Operand& a, const Operand& b, double c, bool has_b, double* out, int64_t n,
             double* host_out)
{
    if (n == 0) {
        switch (op) {
#define LMM_RV_CASE(o) \
    case o: *host_out = host_op<o>(x.v, a.v, b.v, c, has_b); return LMM_OK;
            LMM_RV_OPS(LMM_RV_CASE)
#undef LMM_RV_CASE
            default: return fail(LMM_ERR_INVALID, "unknown random-variable operation");
        }
    }
    switch (op) {
#define LMM_RV_CASE(o) \
    case o: launch_op<o>(x, a, b, c, has_b, out, n); break;
        LMM_RV_OPS(LMM_RV_CASE)
#undef LMM_RV_CASE
        default: return fail(LMM_ERR_INVALID, "unknown random-variable operation");
    }
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

// the same operation in the float class (float realizations out)
int dispatch_f32(int op, const Operand& x, const Operand& a, const Operand& b, double c, bool has_b, bool xdet,
                 float* out, int64_t n)
{
    switch (op) {
#define LMM_RV_CASE(o) \
    case o: launch_op_f32<o>(x, a, b, c, has_b, xdet, out, n); break;
        LMM_RV_OPS(LMM_RV_CASE)
#undef LMM_RV_CASE
        default: return fail(LMM_ERR_INVALID, "unknown random-variable operation");
    }
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

// block partial sums of x, or of (x - m)^2 when centered: each thread runs the
// reference's Kahan loop over its elements (four FP64 operations per value; this GPU's
// FP64 pipe, not HBM, bounds a reduction), the threads' (sum, -compensation) pairs are
// merged as double-doubles in a fixed tree
template <typename T>
__global__ void __launch_bounds__(kRvThreads) rv_sum_kernel(const T* x, int64_t n, int centered, double m,
                                                            double* partials)
{
    double sum = 0.0, err = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRvThreads) {
        const double xi = (double)x[i];
        const double v = (centered ? (xi - m) * (xi - m) : xi) - err;
        const double t = sum + v;
        err = (t - sum) - v;
        sum = t;
    }
    dd acc = block_dd_sum(dd{sum, -err});
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = acc.hi;
        partials[2 * blockIdx.x + 1] = acc.lo;
    }
}

__global__ void __launch_bounds__(kRvThreads) rv_finish_kernel(const double* partials, int blocks, int64_t n, double* out)
{
    dd acc{0.0, 0.0};
    for (int b = threadIdx.x; b < blocks; b += kRvThreads) acc = dd_add(acc, dd{partials[2 * b], partials[2 * b + 1]});
    acc = block_dd_sum(acc);
    if (threadIdx.x == 0) *out = (acc.hi + acc.lo) / (double)n;
}

// Math.min / Math.max over the realizations (tree order; NaN propagates, -0.0 < +0.0)
template <typename T>
__global__ void __launch_bounds__(kRvThreads) rv_minmax_kernel(const T* x, int64_t n, double* partials)
{
    __shared__ double smin[kRvThreads], smax[kRvThreads];
    double mn = (double)x[0], mx = (double)x[0];
    for (int64_t i = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRvThreads) {
        mn = java_min(mn, (double)x[i]);
        mx = java_max(mx, (double)x[i]);
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int h = kRvThreads / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            smin[threadIdx.x] = java_min(smin[threadIdx.x], smin[threadIdx.x + h]);
            smax[threadIdx.x] = java_max(smax[threadIdx.x], smax[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = smin[0];
        partials[2 * blockIdx.x + 1] = smax[0];
    }
}

// float states (mixed form) widened to FP64
__global__ void __launch_bounds__(kRvThreads) rv_widen_kernel(const float* src, double* out, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRvThreads)
        out[i] = (double)src[i];
}

// RandomVariableFromFloatArray(RandomVariable): the realizations rounded to FP32 (:214-220)
__global__ void __launch_bounds__(kRvThreads) rv_narrow_kernel(const double* src, float* out, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRvThreads)
        out[i] = (float)src[i];
}

// getNumeraire with the discount-curve adjustment (LIBORMarketModelFromCovarianceModel.java:869-874):
// Scalar.div on a deterministic numeraire date (invert, then multiply), else (N a) / P^d
__global__ void __launch_bounds__(kRvThreads) rv_numeraire_kernel(const double* num, const double* adj, double pd, int det,
                                                                  double* out, int64_t n)
{
    const double a = *adj;
    for (int64_t i = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRvThreads)
        out[i] = det ? (1.0 / pd) * (num[i] * a) : (num[i] * a) / pd;
}

int rv_alloc(double time, int64_t n, lmm_rv** out, bool fp32 = false)
{
    lmm_rv* r = new lmm_rv;
    r->time = time;
    r->n = n;
    r->fp32 = fp32 ? 1 : 0;
    if (n > 0) {
        void* p = nullptr;
        const int rc = device_alloc(&p, (fp32 ? sizeof(float) : sizeof(double)) * (size_t)n, rv_stream(),
                                    "cudaMallocAsync (random variable)");
        if (rc) {
            delete r;
            return rc;
        }
        if (fp32) r->f = static_cast<float*>(p);
        else r->d = static_cast<double*>(p);
    }
    *out = r;
    return LMM_OK;
}

Operand operand(const lmm_rv* r)
{
    const bool stoch = r && r->n > 0;
    return Operand{stoch ? r->d : nullptr, stoch ? r->f : nullptr, r ? r->value : 0.0};
}

int64_t common_size(const lmm_rv* x, const lmm_rv* a, const lmm_rv* b, bool* ok)
{
    int64_t n = 0;
    *ok = true;
    for (const lmm_rv* r : {x, a, b}) {
        if (!r || r->n == 0) continue;
        if (n != 0 && r->n != n) *ok = false;
        n = r->n;
    }
    return n;
}

double later_time(const lmm_rv* x, const lmm_rv* a, const lmm_rv* b)
{
    double t = x->time;
    if (a && a->time > t) t = a->time;
    if (b && b->time > t) t = b->time;
    return t;
}

bool stoch_fp32(const lmm_rv* r) { return r && r->n > 0 && r->fp32; }

int copy_rv(const lmm_rv* src, double time, lmm_rv** out);

int apply_any(const lmm_rv* x, int op, const lmm_rv* a, const lmm_rv* b, double c, bool has_b, lmm_rv** out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    if (!valid_op(op)) return fail(LMM_ERR_INVALID, "unknown random-variable operation");
    bool ok;
    const int64_t n = common_size(x, a, b, &ok);
    if (!ok) return fail(LMM_ERR_INVALID, "random variables of different sizes");
    // the class of the result: the receiver's; a deterministic double-class receiver (the
    // role of Scalar, type priority 0) hands the operation to a float-class operand
    // (RandomVariableFromFloatArray.java's type-priority checks)
    const bool f32 = x->fp32 || (x->n == 0 && (stoch_fp32(a) || stoch_fp32(b)));
    if (f32 && n > 0) {
        // a deterministic trigger returns the chosen random variable itself
        if (op == LMM_RV_CHOOSE && x->n == 0) return copy_rv(x->value >= 0.0 ? a : b, later_time(x, a, b), out);
        // the float class's deterministic-operand forms (:1266-1320, :1350-1420): accrue and
        // discount by a deterministic rate multiply / divide by (1 + r dt) formed in double,
        // addProduct with deterministic factors adds their double product
        lmm_rv k;
        k.time = later_time(x, a, b);
        if ((op == LMM_RV_ACCRUE || op == LMM_RV_DISCOUNT) && a && a->n == 0 && x->n > 0) {
            k.value = 1.0 + a->value * c;
            return apply_any(x, op == LMM_RV_ACCRUE ? LMM_RV_MULT : LMM_RV_DIV, &k, nullptr, 0.0, false, out);
        }
        if (op == LMM_RV_ADD_PRODUCT && x->n > 0) {
            if (has_b && a->n == 0 && b->n == 0) {
                k.value = a->value * b->value;
                return apply_any(x, LMM_RV_ADD, &k, nullptr, 0.0, false, out);
            }
            if (has_b && b->n == 0) return apply_any(x, op, a, nullptr, b->value, false, out);
            if (has_b && a->n == 0) return apply_any(x, op, b, nullptr, a->value, false, out);
            if (!has_b && a->n == 0) {
                k.value = a->value * c;
                return apply_any(x, LMM_RV_ADD, &k, nullptr, 0.0, false, out);
            }
        }
    }
    lmm_rv* r = nullptr;
    int rc = rv_alloc(later_time(x, a, b), n, &r, f32);
    if (rc) return rc;
    if (f32 && n > 0) rc = dispatch_f32(op, operand(x), operand(a), operand(b), c, has_b, x->fp32 && x->n == 0, r->f, n);
    else rc = dispatch(op, operand(x), operand(a), operand(b), c, has_b, r->d, n, &r->value);
    if (rc) {
        lmm_rv_destroy(r);
        return rc;
    }
    *out = r;
    return LMM_OK;
}

// a copy of src (same class and values) with the filtration time given
int copy_rv(const lmm_rv* src, double time, lmm_rv** out)
{
    lmm_rv* r = nullptr;
    int rc = rv_alloc(time, src->n, &r, src->fp32 != 0);
    if (rc) return rc;
    r->value = src->value;
    if (src->n > 0) {
        const cudaError_t e = src->fp32 ? cudaMemcpyAsync(r->f, src->f, sizeof(float) * (size_t)src->n,
                                                          cudaMemcpyDeviceToDevice, rv_stream())
                                        : cudaMemcpyAsync(r->d, src->d, sizeof(double) * (size_t)src->n,
                                                          cudaMemcpyDeviceToDevice, rv_stream());
        if (e != cudaSuccess) {
            lmm_rv_destroy(r);
            return cuda_fail(e, "random-variable copy");
        }
    }
    *out = r;
    return LMM_OK;
}

// order the library stream after the work so far on src, and src after the copy that follows
struct StreamHandoff {
    cudaEvent_t before = nullptr, after = nullptr;
    cudaStream_t src;
    explicit StreamHandoff(cudaStream_t s) : src(s)
    {
        cudaEventCreateWithFlags(&before, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&after, cudaEventDisableTiming);
        cudaEventRecord(before, src);
        cudaStreamWaitEvent(rv_stream(), before, 0);
    }
    ~StreamHandoff()
    {
        cudaEventRecord(after, rv_stream());
        cudaStreamWaitEvent(src, after, 0);  // the source buffers outlive the copy
        cudaEventDestroy(before);
        cudaEventDestroy(after);
    }
};

}  // namespace

// ------------------------------------------------------------------ quantiles and histograms
// A sorted copy of the realizations, as java.util.Arrays.sort orders them (ascending, every
// NaN last): NaNs are first mapped to the positive quiet NaN (the radix order of a NaN with
// the sign bit set would put it first), then CUB's radix sort orders the keys.
template <typename T>
__global__ void __launch_bounds__(kRvThreads) rv_canonical_nan_kernel(const T* x, T* out, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * kRvThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRvThreads) {
        const T v = x[i];
        out[i] = v != v ? (T)NAN : v;
    }
}

// count of sorted values <= the running maximum of the interval points (getHistogram's
// forward-only scan over the sorted realizations, RandomVariableFromDoubleArray.java:528-543)
template <typename T>
__global__ void rv_count_le_kernel(const T* sorted, int64_t n, const double* points, int m, int64_t* counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double bound = points[0];
    for (int k = 1; k <= i; k++) bound = points[k] > bound ? points[k] : bound;
    int64_t lo = 0, hi = n;  // first index whose value is not <= bound
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if ((double)sorted[mid] <= bound) lo = mid + 1;
        else hi = mid;
    }
    counts[i] = lo;
}

template <typename T>
int sorted_copy(const T* src, int64_t n, T** out)
{
    *out = nullptr;
    if (n > (int64_t)INT32_MAX) return fail(LMM_ERR_INVALID, "quantiles of more than 2^31 - 1 realizations");
    T* keys = nullptr;
    T* sorted = nullptr;
    void* temp = nullptr;
    size_t temp_bytes = 0;
    int rc = device_alloc(reinterpret_cast<void**>(&keys), sizeof(T) * (size_t)n, rv_stream(), "cudaMallocAsync (sort keys)");
    if (!rc) rc = device_alloc(reinterpret_cast<void**>(&sorted), sizeof(T) * (size_t)n, rv_stream(),
                               "cudaMallocAsync (sorted realizations)");
    cudaError_t e = cudaSuccess;
    if (!rc) {
        rv_canonical_nan_kernel<T><<<rv_blocks(n), kRvThreads, 0, rv_stream()>>>(src, keys, n);
        e = cub::DeviceRadixSort::SortKeys(nullptr, temp_bytes, keys, sorted, (int)n, 0, 8 * (int)sizeof(T), rv_stream());
    }
    if (!rc && e == cudaSuccess) rc = device_alloc(&temp, temp_bytes, rv_stream(), "cudaMallocAsync (sort scratch)");
    if (!rc && e == cudaSuccess)
        e = cub::DeviceRadixSort::SortKeys(temp, temp_bytes, keys, sorted, (int)n, 0, 8 * (int)sizeof(T), rv_stream());
    if (temp) cudaFreeAsync(temp, rv_stream());
    if (keys) cudaFreeAsync(keys, rv_stream());
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "random-variable sort");
    if (rc) {
        if (sorted) cudaFreeAsync(sorted, rv_stream());
        return rc;
    }
    *out = sorted;
    return LMM_OK;
}

// Math.round(double) as an int (floor(x + 1/2) without the double rounding of x + 0.5; NaN -> 0)
int64_t java_round(double x)
{
    if (x != x) return 0;
    const double r = std::floor(x);
    return (int64_t)(x - r >= 0.5 ? r + 1.0 : r);
}

// (int) Math.round((size + 1) * quantile - 1) clamped to [0, size - 1] (:457, :489-490)
int64_t quantile_index(int64_t n, double q)
{
    int64_t k = (int64_t)(int32_t)java_round((double)(n + 1) * q - 1);
    return std::min(std::max(k, (int64_t)0), n - 1);
}

// the sorted values [i0, i1] of x widened to doubles on the host
int sorted_range(const lmm_rv* x, int64_t i0, int64_t i1, std::vector<double>* out)
{
    const size_t cnt = (size_t)(i1 - i0 + 1);
    out->assign(cnt, 0.0);
    if (x->fp32) {
        float* sorted = nullptr;
        int rc = sorted_copy<float>(x->f, x->n, &sorted);
        if (rc) return rc;
        std::vector<float> tmp(cnt);
        cudaError_t e = cudaMemcpyAsync(tmp.data(), sorted + i0, sizeof(float) * cnt, cudaMemcpyDeviceToHost, rv_stream());
        cudaFreeAsync(sorted, rv_stream());
        if (e == cudaSuccess) e = cudaStreamSynchronize(rv_stream());
        if (e != cudaSuccess) return cuda_fail(e, "random-variable quantile");
        for (size_t k = 0; k < cnt; k++) (*out)[k] = (double)tmp[k];
        return LMM_OK;
    }
    double* sorted = nullptr;
    int rc = sorted_copy<double>(x->d, x->n, &sorted);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(out->data(), sorted + i0, sizeof(double) * cnt, cudaMemcpyDeviceToHost, rv_stream());
    cudaFreeAsync(sorted, rv_stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(rv_stream());
    return e == cudaSuccess ? LMM_OK : cuda_fail(e, "random-variable quantile");
}

template <typename T>
int histogram_counts(const T* src, int64_t n, const double* h_points, int m, std::vector<int64_t>* counts)
{
    T* sorted = nullptr;
    int rc = sorted_copy<T>(src, n, &sorted);
    if (rc) return rc;
    double* d_points = nullptr;
    int64_t* d_counts = nullptr;
    rc = device_alloc(reinterpret_cast<void**>(&d_points), sizeof(double) * (size_t)m, rv_stream(),
                      "cudaMallocAsync (histogram points)");
    if (!rc) rc = device_alloc(reinterpret_cast<void**>(&d_counts), sizeof(int64_t) * (size_t)m, rv_stream(),
                               "cudaMallocAsync (histogram counts)");
    cudaError_t e = cudaSuccess;
    if (!rc) {
        e = cudaMemcpyAsync(d_points, h_points, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice, rv_stream());
        if (e == cudaSuccess) {
            rv_count_le_kernel<T><<<(m + 127) / 128, 128, 0, rv_stream()>>>(sorted, n, d_points, m, d_counts);
            e = cudaGetLastError();
        }
        counts->assign((size_t)m, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(counts->data(), d_counts, sizeof(int64_t) * (size_t)m, cudaMemcpyDeviceToHost, rv_stream());
        if (e == cudaSuccess) e = cudaStreamSynchronize(rv_stream());
    }
    cudaFreeAsync(sorted, rv_stream());
    if (d_points) cudaFreeAsync(d_points, rv_stream());
    if (d_counts) cudaFreeAsync(d_counts, rv_stream());
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "random-variable histogram");
    return rc;
}

int rv_from_device(double time, const void* src, int fp32, int64_t n, cudaStream_t src_stream, lmm_rv** out)
{
    lmm_rv* r = nullptr;
    int rc = rv_alloc(time, n, &r);
    if (rc) return rc;
    {
        StreamHandoff h(src_stream);
        if (fp32) {
            const int blocks = rv_blocks(n);
            rv_widen_kernel<<<blocks, kRvThreads, 0, rv_stream()>>>(static_cast<const float*>(src), r->d, n);
        } else {
            cudaMemcpyAsync(r->d, src, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, rv_stream());
        }
    }
    LMM_CUDA(cudaGetLastError());
    *out = r;
    return LMM_OK;
}

int rv_numeraire(double time, const double* d_num, const double* d_adj, int has_discount, int det, double pd, int64_t n,
                 cudaStream_t src_stream, lmm_rv** out)
{
    lmm_rv* r = nullptr;
    int rc = rv_alloc(time, n, &r);
    if (rc) return rc;
    {
        StreamHandoff h(src_stream);
        if (has_discount)
            rv_numeraire_kernel<<<rv_blocks(n), kRvThreads, 0, rv_stream()>>>(d_num, d_adj, pd, det, r->d, n);
        else
            cudaMemcpyAsync(r->d, d_num, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, rv_stream());
    }
    LMM_CUDA(cudaGetLastError());
    *out = r;
    return LMM_OK;
}

}  // namespace lmm

using namespace lmm;

extern "C" {

int lmm_rv_create_constant(double time, double value, lmm_rv** out)
{
    if (!out) return fail(LMM_ERR_INVALID, "null argument");
    lmm_rv* r = new lmm_rv;
    r->time = time;
    r->value = value;
    *out = r;
    return LMM_OK;
}

int lmm_rv_create(double time, const double* host, int64_t n, lmm_rv** out)
{
    if (!out || (!host && n > 0)) return fail(LMM_ERR_INVALID, "null argument");
    if (n < 1) return fail(LMM_ERR_INVALID, "a stochastic random variable needs at least one realization");
    lmm_rv* r = nullptr;
    int rc = rv_alloc(time, n, &r);
    if (rc) return rc;
    const cudaError_t e = cudaMemcpyAsync(r->d, host, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, rv_stream());
    if (e != cudaSuccess) {
        lmm_rv_destroy(r);
        return cuda_fail(e, "cudaMemcpyAsync (random variable)");
    }
    count_h2d(sizeof(double) * (size_t)n);
    *out = r;
    return LMM_OK;
}

int lmm_rv_stream(void** out_stream)
{
    if (!out_stream) return fail(LMM_ERR_INVALID, "null argument");
    *out_stream = (void*)rv_stream();
    return LMM_OK;
}

int lmm_rv_destroy(lmm_rv* x)
{
    if (!x) return LMM_OK;
    if (x->d) cudaFreeAsync(x->d, rv_stream());
    if (x->f) cudaFreeAsync(x->f, rv_stream());
    delete x;
    return LMM_OK;
}

int lmm_rv_create_float(double time, const float* host, int64_t n, lmm_rv** out)
{
    if (!out || (!host && n > 0)) return fail(LMM_ERR_INVALID, "null argument");
    if (n < 1) return fail(LMM_ERR_INVALID, "a stochastic random variable needs at least one realization");
    lmm_rv* r = nullptr;
    int rc = rv_alloc(time, n, &r, true);
    if (rc) return rc;
    const cudaError_t e = cudaMemcpyAsync(r->f, host, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, rv_stream());
    if (e != cudaSuccess) {
        lmm_rv_destroy(r);
        return cuda_fail(e, "cudaMemcpyAsync (random variable)");
    }
    count_h2d(sizeof(float) * (size_t)n);
    // the host buffer may be released once the call returns
    LMM_CUDA(cudaStreamSynchronize(rv_stream()));
    *out = r;
    return LMM_OK;
}

int lmm_rv_create_constant_float(double time, double value, lmm_rv** out)
{
    if (!out) return fail(LMM_ERR_INVALID, "null argument");
    lmm_rv* r = new lmm_rv;
    r->time = time;
    r->value = value;
    r->fp32 = 1;
    *out = r;
    return LMM_OK;
}

int lmm_rv_to_float(const lmm_rv* x, lmm_rv** out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    if (x->fp32 || x->n == 0) {
        int rc = copy_rv(x, x->time, out);
        if (!rc) (*out)->fp32 = 1;
        return rc;
    }
    lmm_rv* r = nullptr;
    int rc = rv_alloc(x->time, x->n, &r, true);
    if (rc) return rc;
    rv_narrow_kernel<<<rv_blocks(x->n), kRvThreads, 0, rv_stream()>>>(x->d, r->f, x->n);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        lmm_rv_destroy(r);
        return cuda_fail(e, "random-variable narrowing");
    }
    *out = r;
    return LMM_OK;
}

int lmm_rv_is_float(const lmm_rv* x, int* out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    *out = x->fp32;
    return LMM_OK;
}

int lmm_rv_get_float(const lmm_rv* x, float* out_host)
{
    if (!x || !out_host) return fail(LMM_ERR_INVALID, "null argument");
    if (!x->fp32 || x->n == 0) return fail(LMM_ERR_INVALID, "not a stochastic random variable of the float class");
    LMM_CUDA(cudaMemcpyAsync(out_host, x->f, sizeof(float) * (size_t)x->n, cudaMemcpyDeviceToHost, rv_stream()));
    LMM_CUDA(cudaStreamSynchronize(rv_stream()));
    return LMM_OK;
}

int lmm_rv_describe(const lmm_rv* x, double* out_time, int64_t* out_n, int* out_deterministic, double* out_value)
{
    if (!x) return fail(LMM_ERR_INVALID, "null argument");
    if (out_time) *out_time = x->time;
    if (out_n) *out_n = x->n;
    if (out_deterministic) *out_deterministic = x->n == 0;
    if (out_value) *out_value = x->value;
    return LMM_OK;
}

int lmm_rv_get(const lmm_rv* x, double* out_host)
{
    if (!x || !out_host) return fail(LMM_ERR_INVALID, "null argument");
    if (x->n == 0) {
        *out_host = x->value;
        return LMM_OK;
    }
    if (x->fp32) {
        // getRealizations of the float class: the floats widened to doubles (:222-228)
        std::vector<float> tmp((size_t)x->n);
        LMM_CUDA(cudaMemcpyAsync(tmp.data(), x->f, sizeof(float) * (size_t)x->n, cudaMemcpyDeviceToHost, rv_stream()));
        LMM_CUDA(cudaStreamSynchronize(rv_stream()));
        for (int64_t i = 0; i < x->n; i++) out_host[i] = (double)tmp[(size_t)i];
        return LMM_OK;
    }
    LMM_CUDA(cudaMemcpyAsync(out_host, x->d, sizeof(double) * (size_t)x->n, cudaMemcpyDeviceToHost, rv_stream()));
    LMM_CUDA(cudaStreamSynchronize(rv_stream()));
    return LMM_OK;
}

int lmm_rv_apply_scalar(const lmm_rv* x, int op, double y, lmm_rv** out)
{
    if (op >= LMM_RV_ACCRUE) return fail(LMM_ERR_INVALID, "three-argument operation: use lmm_rv_apply3");
    lmm_rv c;  // y as a deterministic operand
    c.value = y;
    c.time = x ? x->time : 0.0;
    return apply_any(x, op, &c, nullptr, 0.0, false, out);
}

int lmm_rv_apply(const lmm_rv* x, int op, const lmm_rv* y, lmm_rv** out)
{
    if (!y) return fail(LMM_ERR_INVALID, "null argument");
    if (op > LMM_RV_FLOOR) return fail(LMM_ERR_INVALID, "not a binary random-variable operation");
    return apply_any(x, op, y, nullptr, 0.0, false, out);
}

int lmm_rv_apply3(const lmm_rv* x, int op, const lmm_rv* a, const lmm_rv* b, double c, lmm_rv** out)
{
    if (op < LMM_RV_ACCRUE) return fail(LMM_ERR_INVALID, "not a three-argument random-variable operation");
    if (!a) return fail(LMM_ERR_INVALID, "null argument");
    const bool needs_b = op == LMM_RV_CHOOSE || op == LMM_RV_ADD_RATIO || op == LMM_RV_SUB_RATIO;
    if (needs_b && !b) return fail(LMM_ERR_INVALID, "null argument");
    return apply_any(x, op, a, b, c, b != nullptr, out);
}

static int reduce_sum(const lmm_rv* x, bool centered, double center, double* out)
{
    const int blocks = (int)std::min<int64_t>((x->n + kRvThreads - 1) / kRvThreads, 1024);
    double* scratch = nullptr;
    int arc = device_alloc(reinterpret_cast<void**>(&scratch), sizeof(double) * (2 * (size_t)blocks + 1), rv_stream(),
                           "cudaMallocAsync (reduction scratch)");
    if (arc) return arc;
    if (x->fp32) rv_sum_kernel<float><<<blocks, kRvThreads, 0, rv_stream()>>>(x->f, x->n, centered ? 1 : 0, center, scratch);
    else rv_sum_kernel<double><<<blocks, kRvThreads, 0, rv_stream()>>>(x->d, x->n, centered ? 1 : 0, center, scratch);
    rv_finish_kernel<<<1, kRvThreads, 0, rv_stream()>>>(scratch, blocks, x->n, scratch + 2 * blocks);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, scratch + 2 * blocks, sizeof(double), cudaMemcpyDeviceToHost, rv_stream());
    cudaFreeAsync(scratch, rv_stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(rv_stream());
    return e == cudaSuccess ? LMM_OK : cuda_fail(e, "random-variable reduction");
}

int lmm_rv_average(const lmm_rv* x, double* out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    if (x->n == 0) {
        *out = x->value;
        return LMM_OK;
    }
    return reduce_sum(x, false, 0.0, out);
}

int lmm_rv_variance(const lmm_rv* x, double* out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    if (x->n <= 1) {
        *out = 0.0;
        return LMM_OK;
    }
    double avg = 0.0;
    const int rc = reduce_sum(x, false, 0.0, &avg);  // getVariance centres on getAverage (two passes)
    if (rc) return rc;
    return reduce_sum(x, true, avg, out);
}

int lmm_rv_standard_error(const lmm_rv* x, double* out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    if (x->n == 0) {
        *out = 0.0;
        return LMM_OK;
    }
    double var = 0.0;
    const int rc = lmm_rv_variance(x, &var);
    if (rc) return rc;
    *out = std::sqrt(var) / std::sqrt((double)x->n);  // getStandardDeviation() / Math.sqrt(size())
    return LMM_OK;
}

int lmm_rv_min_max(const lmm_rv* x, double* out_min, double* out_max)
{
    if (!x || !out_min || !out_max) return fail(LMM_ERR_INVALID, "null argument");
    if (x->n == 0) {
        *out_min = *out_max = x->value;
        return LMM_OK;
    }
    const int blocks = (int)std::min<int64_t>((x->n + kRvThreads - 1) / kRvThreads, 1024);
    double* scratch = nullptr;
    int arc = device_alloc(reinterpret_cast<void**>(&scratch), sizeof(double) * 2 * (size_t)blocks, rv_stream(),
                           "cudaMallocAsync (min/max scratch)");
    if (arc) return arc;
    if (x->fp32) rv_minmax_kernel<float><<<blocks, kRvThreads, 0, rv_stream()>>>(x->f, x->n, scratch);
    else rv_minmax_kernel<double><<<blocks, kRvThreads, 0, rv_stream()>>>(x->d, x->n, scratch);
    std::vector<double> h(2 * (size_t)blocks);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), scratch, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, rv_stream());
    cudaFreeAsync(scratch, rv_stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(rv_stream());
    if (e != cudaSuccess) return cuda_fail(e, "random-variable min/max");
    double mn = h[0], mx = h[1];
    for (int b = 1; b < blocks; b++) {
        mn = java_min(mn, h[2 * b]);
        mx = java_max(mx, h[2 * b + 1]);
    }
    *out_min = mn;
    *out_max = mx;
    return LMM_OK;
}

int lmm_rv_quantile(const lmm_rv* x, double quantile, double* out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    if (x->n == 0) {
        *out = x->value;
        return LMM_OK;
    }
    const int64_t k = quantile_index(x->n, quantile);
    std::vector<double> v;
    int rc = sorted_range(x, k, k, &v);
    if (rc) return rc;
    *out = v[0];
    return LMM_OK;
}

int lmm_rv_quantile_expectation(const lmm_rv* x, double quantile_start, double quantile_end, double* out)
{
    if (!x || !out) return fail(LMM_ERR_INVALID, "null argument");
    if (x->n == 0) {
        *out = x->value;
        return LMM_OK;
    }
    if (quantile_start > quantile_end) std::swap(quantile_start, quantile_end);
    const int64_t i0 = quantile_index(x->n, quantile_start), i1 = quantile_index(x->n, quantile_end);
    std::vector<double> v;
    int rc = sorted_range(x, i0, i1, &v);
    if (rc) return rc;
    double sum = 0.0;  // the reference's plain loop, in index order (:492-496)
    for (double y : v) sum += y;
    *out = sum / (double)(i1 - i0 + 1);
    return LMM_OK;
}

int lmm_rv_histogram(const lmm_rv* x, const double* interval_points, int num_points, double* out)
{
    if (!x || !out || (num_points > 0 && !interval_points) || num_points < 0)
        return fail(LMM_ERR_INVALID, "null argument");
    std::fill(out, out + num_points + 1, 0.0);
    if (x->n == 0) {
        // the reference's deterministic case (:506-520): a 1 at the first interval point the
        // value exceeds, and always a 1 in the last entry
        for (int i = 0; i < num_points; i++)
            if (x->value > interval_points[i]) {
                out[i] = 1.0;
                break;
            }
        out[num_points] = 1.0;
        return LMM_OK;
    }
    std::vector<int64_t> le;
    if (num_points > 0) {
        int rc = x->fp32 ? histogram_counts<float>(x->f, x->n, interval_points, num_points, &le)
                         : histogram_counts<double>(x->d, x->n, interval_points, num_points, &le);
        if (rc) return rc;
    }
    int64_t prev = 0;
    for (int i = 0; i < num_points; i++) {
        out[i] = (double)(le[(size_t)i] - prev);
        prev = le[(size_t)i];
    }
    out[num_points] = (double)(x->n - prev);
    for (int i = 0; i <= num_points; i++) out[i] /= (double)x->n;
    return LMM_OK;
}

}  // extern "C"
