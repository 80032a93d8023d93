// host_model.cpp -- host-side model construction (finmath-lib setup classes).
//
// These are the pieces of finmath-lib that run once per model on the host: time grids
// with tick rounding, exponential-decay correlation and its factor reduction, the
// four-parameter volatility, covariance tables, forward/discount curves, the
// deterministic numeraire-adjustment chain, and the small SVD solve of a regression.  A Java shim can take the same tables from
// finmath's own objects; C/C++/Python callers use these.  Compiled without FMA
// contraction (-ffp-contract=off), as the reference's Java never fuses.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lmm_internal.h"

namespace {

const double kTick = 1.0 / (365.0 * 24.0);  // TimeDiscretizationFromArray.java:39

double round_to_tick(double t) { return std::rint(t / kTick) * kTick; }  // :387-389

int binary_search(const double* a, int n, double key)
{
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (int)(((unsigned)lo + (unsigned)hi) >> 1);
        if (a[mid] < key) lo = mid + 1;
        else if (a[mid] > key) hi = mid - 1;
        else return mid;
    }
    return -(lo + 1);
}

// Cyclic Jacobi eigen-decomposition of a symmetric matrix; V columns are eigenvectors.
void eigen_symmetric(int n, const double* Ain, std::vector<double>& ev, std::vector<double>& V)
{
    std::vector<double> A(Ain, Ain + (size_t)n * n);
    ev.assign(n, 0.0);
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                const double a = A[(size_t)i * n + j];
                if (i != j) off += a * a;
                else diag += a * a;
            }
        if (off <= 1e-300 || off <= 1e-34 * diag) break;
        // an element below 2^-53 of the diagonal norm is rounding noise: rotating it changes
        // nothing the factor matrix keeps, and a sweep without a rotation ends the iteration
        // (rank-deficient and clustered spectra otherwise never meet the relative criterion)
        const double tiny = 0x1.0p-53 * std::sqrt(diag);
        bool rotated = false;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = A[(size_t)p * n + q];
                if (apq == 0.0 || std::fabs(apq) <= tiny) continue;
                rotated = true;
                const double theta = (A[(size_t)q * n + q] - A[(size_t)p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = c * akp - s * akq;
                    A[(size_t)k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = c * apk - s * aqk;
                    A[(size_t)q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - s * vkq;
                    V[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
        if (!rotated) break;
    }
    for (int i = 0; i < n; i++) ev[i] = A[(size_t)i * n + i];
}

// LinearAlgebra.getFactorMatrixUsingCommonsMath (functions/LinearAlgebra.java:392-445).
void factor_matrix(const double* corr, int n, int F, double* out)
{
    std::vector<double> ev, V;
    eigen_symmetric(n, corr, ev, V);
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return ev[a] > ev[b]; });
    for (int f = 0; f < F; f++) {
        const int e = idx[f];
        double lambda = ev[e];
        const double sign = V[(size_t)0 * n + e] > 0.0 ? 1.0 : -1.0;
        double norm2 = 0.0;
        for (int r = 0; r < n; r++) norm2 += V[(size_t)r * n + e] * V[(size_t)r * n + e];
        lambda = std::max(lambda, 0.0);
        for (int r = 0; r < n; r++) out[(size_t)r * F + f] = sign * std::sqrt(lambda / norm2) * V[(size_t)r * n + e];
    }
}

// A = U diag(s) V^T of a square n x n matrix by one-sided Jacobi rotations on the columns
// of U (initially A), V accumulating the rotations; s the column norms, U normalised.
void svd_jacobi(int n, const double* A, std::vector<double>& U, std::vector<double>& s, std::vector<double>& V)
{
    U.assign(A, A + (size_t)n * n);
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        bool rotated = false;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double alpha = 0.0, beta = 0.0, gamma = 0.0;
                for (int k = 0; k < n; k++) {
                    const double up = U[(size_t)k * n + p], uq = U[(size_t)k * n + q];
                    alpha += up * up;
                    beta += uq * uq;
                    gamma += up * uq;
                }
                if (gamma == 0.0 || std::fabs(gamma) <= 0x1.0p-52 * std::sqrt(alpha * beta)) continue;
                rotated = true;
                const double zeta = (beta - alpha) / (2.0 * gamma);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double cs = 1.0 / std::sqrt(1.0 + t * t), sn = cs * t;
                for (int k = 0; k < n; k++) {
                    const double up = U[(size_t)k * n + p], uq = U[(size_t)k * n + q];
                    U[(size_t)k * n + p] = cs * up - sn * uq;
                    U[(size_t)k * n + q] = sn * up + cs * uq;
                    const double vp = V[(size_t)k * n + p], vq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = cs * vp - sn * vq;
                    V[(size_t)k * n + q] = sn * vp + cs * vq;
                }
            }
        if (!rotated) break;
    }
    s.assign(n, 0.0);
    for (int j = 0; j < n; j++) {
        double nn = 0.0;
        for (int k = 0; k < n; k++) nn += U[(size_t)k * n + j] * U[(size_t)k * n + j];
        s[j] = std::sqrt(nn);
        if (s[j] > 0.0)
            for (int k = 0; k < n; k++) U[(size_t)k * n + j] = U[(size_t)k * n + j] / s[j];
    }
}

}  // namespace

extern "C" {

int lmm_solve_svd(int n, const double* A, const double* b, double* x)
{
    if (!A || !b || !x || n < 1 || n > 64) return lmm::fail(LMM_ERR_INVALID, "lmm_solve_svd: bad arguments (1 <= n <= 64)");
    std::vector<double> U, s, V;
    svd_jacobi(n, A, U, s, V);
    double smax = 0.0;
    for (int j = 0; j < n; j++) smax = std::max(smax, s[j]);
    // the solver's cutoff: max(n sigma_max 2^-52, sqrt(the smallest normal double))
    const double tol = std::max((double)n * smax * 0x1.0p-52, std::sqrt(0x1.0p-1022));
    std::vector<double> w(n, 0.0);
    for (int j = 0; j < n; j++) {
        if (!(s[j] > tol)) continue;
        double utb = 0.0;
        for (int r = 0; r < n; r++) utb += U[(size_t)r * n + j] * b[r];
        w[j] = utb / s[j];
    }
    for (int i = 0; i < n; i++) {
        double acc = 0.0;
        for (int j = 0; j < n; j++) acc += V[(size_t)i * n + j] * w[j];
        x[i] = acc;
    }
    return LMM_OK;
}

int lmm_time_discretization(double initial, int num_steps, double dt, double* out_times)
{
    if (num_steps < 0 || !out_times) return lmm::fail(LMM_ERR_INVALID, "lmm_time_discretization: bad arguments");
    for (int i = 0; i <= num_steps; i++) out_times[i] = round_to_tick(initial + (double)i * dt);
    return LMM_OK;
}

int lmm_factor_reduction(const double* corr, int n, int F, double* out)
{
    if (!corr || !out || n <= 0 || F <= 0 || F > n) return lmm::fail(LMM_ERR_INVALID, "lmm_factor_reduction: need 0 < F <= n");
    std::vector<double> fm((size_t)n * F), red((size_t)n * n);
    factor_matrix(corr, n, F, fm.data());
    // LinearAlgebra.factorReductionUsingCommonsMath (:454-482): renormalise rows, re-factor F F^T
    for (int r = 0; r < n; r++) {
        double s2 = 0.0;
        for (int f = 0; f < F; f++) s2 += fm[(size_t)r * F + f] * fm[(size_t)r * F + f];
        for (int f = 0; f < F; f++)
            fm[(size_t)r * F + f] = (s2 != 0.0) ? fm[(size_t)r * F + f] / std::sqrt(s2) : 1.0;
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            double s = 0.0;
            for (int f = 0; f < F; f++) s += fm[(size_t)i * F + f] * fm[(size_t)j * F + f];
            red[(size_t)i * n + j] = s;
        }
    factor_matrix(red.data(), n, F, out);
    return LMM_OK;
}

int lmm_correlation_exponential_decay(const double* tenor, int N, int F, double a, double* factor, double* corr)
{
    if (!tenor || !factor || !corr || N <= 0 || F <= 0 || F > N)
        return lmm::fail(LMM_ERR_INVALID, "lmm_correlation_exponential_decay: need 0 < F <= N");
    a = std::max(a, 0.0);
    for (int r = 0; r < N; r++)
        for (int c = 0; c < N; c++) corr[(size_t)r * N + c] = std::exp(-a * std::fabs(tenor[r] - tenor[c]));
    int rc = lmm_factor_reduction(corr, N, F, factor);
    if (rc) return rc;
    for (int c1 = 0; c1 < N; c1++) {
        for (int c2 = 0; c2 < c1; c2++) {
            double s = 0.0;
            for (int f = 0; f < F; f++) s += factor[(size_t)c1 * F + f] * factor[(size_t)c2 * F + f];
            corr[(size_t)c1 * N + c2] = s;
            corr[(size_t)c2 * N + c1] = s;
        }
        corr[(size_t)c1 * N + c1] = 1.0;
    }
    return LMM_OK;
}

int lmm_volatility_four_parameter(const double* times, int T, const double* tenor, int N, double a, double b,
                                  double c, double d, double* vol)
{
    if (!times || !tenor || !vol || T <= 0 || N <= 0) return lmm::fail(LMM_ERR_INVALID, "lmm_volatility_four_parameter: bad arguments");
    for (int i = 0; i < T; i++)
        for (int j = 0; j < N; j++) {
            const double tau = tenor[j] - times[i];
            vol[(size_t)i * N + j] = (tau <= 0.0) ? 0.0 : ((b * tau + a) * std::exp(c * -tau)) + d;
        }
    return LMM_OK;
}

int lmm_covariance_tables(int T, int N, int F, const double* vol, const double* factor, const double* corr,
                          double* loadings, double* variance)
{
    if (!vol || !factor || !corr || !loadings || !variance || T <= 0 || N <= 0 || F <= 0)
        return lmm::fail(LMM_ERR_INVALID, "lmm_covariance_tables: bad arguments");
    for (int i = 0; i < T; i++)
        for (int j = 0; j < N; j++) {
            const double s = vol[(size_t)i * N + j];
            for (int f = 0; f < F; f++) loadings[((size_t)i * N + j) * F + f] = s * factor[(size_t)j * F + f];
            variance[(size_t)i * N + j] = (s * s) * corr[(size_t)j * N + j];
        }
    return LMM_OK;
}

int lmm_forward_curve_value(const double* x, const double* y, int n, double t, double* out)
{
    if (!x || !y || !out || n <= 0) return lmm::fail(LMM_ERR_INVALID, "lmm_forward_curve_value: empty curve");
    const int idx = binary_search(x, n, t);
    if (idx >= 0) { *out = y[idx]; return LMM_OK; }
    const int iv = -idx - 2;
    if (iv < 0) { *out = y[0]; return LMM_OK; }
    if (iv > n - 2) { *out = y[n - 1]; return LMM_OK; }
    const double slope = (y[iv + 1] - y[iv]) / (x[iv + 1] - x[iv]);
    double v = 0.0;
    v += y[iv] * 1.0;
    v += slope * (t - x[iv]);
    *out = v;
    return LMM_OK;
}

int lmm_discount_factor_from_forward_curve(const double* x, const double* y, int n, double po, double maturity,
                                           double* out)
{
    if (!(po > 0.0)) return lmm::fail(LMM_ERR_INVALID, "discount curve from forward curve needs a positive payment offset");
    double time = 0.0, df = 1.0;
    while (time < maturity) {
        double f = 0.0;
        const int rc = lmm_forward_curve_value(x, y, n, time, &f);
        if (rc) return rc;
        df /= 1.0 + f * std::min(po, maturity - time) * 1.0;
        time += po;
    }
    *out = df;
    return LMM_OK;
}

int lmm_numeraire_discount_chain(const double* tenor, int N, const double* df, double* out)
{
    if (!tenor || !df || !out || N <= 0) return lmm::fail(LMM_ERR_INVALID, "lmm_numeraire_discount_chain: bad arguments");
    double adj = df[0];
    out[0] = adj;
    for (int i = 0; i < N; i++) {
        const double step = tenor[i + 1] - tenor[i];
        const double r = (df[i] / df[i + 1] - 1.0) / step;
        adj = (adj == 0.0) ? r * 0.0 : 1.0 / (r * (step / adj) + 1.0 / adj);  // Scalar.discount
        out[i + 1] = adj;
    }
    return LMM_OK;
}

}  // extern "C"
