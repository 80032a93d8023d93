// lmm_internal.h -- shared declarations of the GB300 LMM library (host + device).
#pragma once

#include <cmath>
#include <cstddef>
#include <cstring>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "lmm_gb300.h"
#include "lmm_rv.h"

namespace lmm {

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define LMM_CUDA(call)                                                   \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return ::lmm::cuda_fail(e_, #call);       \
    } while (0)

// Kernel-launch bookkeeping: every launch of a library kernel bumps a counter and,
// when timing is enabled, is bracketed by CUDA events on the launching stream.
enum KernelId : int {
    K_MT_JUMP_GENERATE = 0,
    K_PATHS_FP64,
    K_PATHS_FP32,
    K_NUMERAIRE_FINISH,
    K_SWAPTION,
    K_BERMUDAN_STEP,
    K_BERMUDAN_SOLVE,
    K_VALUE_REDUCE,
    K_ADJOINT,
    K_PORTFOLIO,        // one launch of a recorded portfolio graph
    K_MISC,
    K_COUNT
};
const char* kernel_name(int id);
struct KernelTimer {
    KernelTimer(int id, cudaStream_t s, int launches = 1);
    ~KernelTimer();
    int id;
    cudaStream_t stream;
    cudaEvent_t start = nullptr;
};
bool timing_enabled();
// host-to-device bytes copied by the library (every table and parameter upload)
void count_h2d(size_t bytes);
// Every device allocation of the library: cudaMallocAsync on stream s, failures mapped to
// LMM_ERR_NOMEM / LMM_ERR_CUDA with a message.  With LMM_FAULT_INJECT_ALLOC=n in the
// environment (read once), every allocation after the first n fails as an out-of-memory
// would, without calling the allocator: the host-side fault injection the tests use.
int device_alloc(void** p, size_t bytes, cudaStream_t s, const char* what);

// ---------------------------------------------------------------- MT19937 (host side)
constexpr int kMtN = 624;
constexpr int kMtM = 397;
constexpr int kPolyWords = 312;            // 19937-bit GF(2) polynomials, 64-bit words
constexpr int kMtDegree = 19937;
constexpr int kJumpWindow = kMtDegree + kMtN - 1;  // raw words needed by one jump (20560)

// Seeded 624-word array of commons-math3 MersenneTwister(long seed).
void mt_seeded_state(int64_t seed, uint32_t out[kMtN]);
// Chunk jumps by base-8 digits: polynomial [j * 7 + (d - 1)] = x^(d 8^j stride) mod phi for
// the digit values d = 1..7 of the digit positions j < ndigits (cached per stride).
constexpr int kJumpDigitBits = 3;
constexpr int kJumpBase = 1 << kJumpDigitBits;
const std::vector<uint64_t>& mt_jump_digit_polynomials(uint64_t stride_words, int ndigits);

// ---------------------------------------------------------------- device launchers
constexpr int kMaxJumps = 32;  // jump polynomial lists: 7 per base-8 digit, so at most 4 digits
struct RngPlan {
    int64_t chunks = 0;
    int64_t chunk_values = 0;
    int ndigits = 0;      // base-8 digits of the largest chunk index
    // set-bit positions of the jump polynomials x^(d 8^j stride) mod phi, as 16-bit indices
    // packed four to a word; list j * 7 + d - 1 starts at index bit_off[j * 7 + d - 1] (a
    // multiple of 8)
    std::vector<uint64_t> polys;
    int bit_off[kMaxJumps] = {};
    int bit_cnt[kMaxJumps] = {};
    int tile_k = 1;       // paths per increments tile
    int smem_bytes = 0;   // dynamic shared memory of a generator block
};
// Chunking of a stream of num_values values (2 words each) over the resident CTAs, for
// values_per_path increments per path of elem_bytes each (1 and 8 for plain uniforms).
int plan_mt_generate(int64_t num_values, int values_per_path, int elem_bytes, RngPlan* plan);

struct RngLaunch {
    const RngPlan* plan;
    const uint32_t* d_seeded;  // [624] seeded state
    const uint64_t* d_jumps;   // plan->polys on the device
    int64_t num_values;        // values in the stream (normals or uniforms)
    int values_per_path;       // T*F for Brownian increments (1 for plain uniforms)
    int num_paths;             // P (row stride of the [T*F][P] layout)
    int num_factors;           // F
    int mode;                  // 0 uniforms (double), 1 increments fp64, 2 increments fp32
    const double* d_sqrt_dt;   // [T] (mode 1)
    const float* d_sqrt_dt32;  // [T] (mode 2)
    void* d_out;
};
int launch_mt_generate(const RngLaunch& a, cudaStream_t s, int* num_launches);

struct PathLaunch {
    int T, N, F, P;
    int scheme;                // 0 EULER, 1 EULER_FUNCTIONAL, 2 PREDICTOR_CORRECTOR, 3 ..._FUNCTIONAL
    int measure;               // 0 SPOT, 1 TERMINAL
    int state_space;           // 0 LOGNORMAL, 1 NORMAL
    const int* d_tenor_tidx;   // [N+1] process time index of each tenor time (TERMINAL numeraire)
    double libor_cap;          // +inf: no cap
    const double* d_loadings;  // [T][N][F]
    const double* d_variance;  // [T][N]
    const double* d_dt;        // [T]
    const int* d_first;        // [T] first alive component at t_i
    const double* d_delta;     // [N] period lengths
    const double* d_inv_delta; // [N] 1.0 / delta (delta/delta == 1.0 exactly for the validated tenor)
    const double* d_var_half_dt; // [T][N] (variance * -0.5) * dt_i, the drift's deterministic part of a step
    const float* d_inv_delta32;// [N] 1/delta in FP32 (mixed form)
    const float* d_dt32;       // [T] time steps in FP32 (mixed form)
    const float* d_init32;     // [N] initial forwards max(f, 0) in FP32 (mixed form)
    const double* d_exp_tab;   // [2 kExpTableHalf + 1] exp(k/kExpTableHalf) (FP64 form, see fp64math.cuh)
    const float* d_rows_df;    // [T][N][fp64_df_pitch(FMAX)] FP64 fast kernel rows as double-float pairs:
                               // loadings hi [FMAX], lo [FMAX], drift term (hi, lo), 1/delta (hi, lo)
    const float* d_dt_df;      // [T][2] time steps as double-float pairs
    const double* d_init;      // [N] initial forwards
    const double* d_init_state;// [N] exp(log(max(f, 0))): the transformed initial state of the lognormal model
    const int* d_obs_slot;     // [T+1] observation slot or -1
    const void* d_dw;          // [T][F][P] fp64 or fp32
    void* d_states;            // [nobs][N][P] fp64 or fp32
    double* d_numeraire;       // [N+1][P] unadjusted spot numeraire
    double* d_inv_numeraire;   // [N+1][P] its reciprocal 1/N (nullptr: not kept)
    double* d_inv_num_partials;// [blocks][N][2] double-double partial sums of 1/N(T_{l+1})
    int num_det_prefix;        // numeraire deterministic for l < num_det_prefix
    void* d_ckpt;              // [T/stride+1][N][P] path state every ckpt_stride steps (nullptr: none)
    int ckpt_stride;           // forward rates L every ckpt_stride steps (in the path precision)
    // the adjoint's replay (FP64 fast kernel): steps [rp_n0, rp_n_stop) from rp_ckpt [N][P],
    // the rates of components below rp_n_eff into rp_seg [rp_n_stop - rp_n0 + 1][N][P]
    int rp_n0, rp_n_stop, rp_n_eff;
    const double* rp_ckpt;
    double* rp_seg;
};
int launch_paths_fp64(const PathLaunch& a, cudaStream_t s, int* blocks_out);
// The adjoint's replay of the steps [n0, n_stop) of an FP64 process from its checkpoint at
// n0 with the fast path kernel's own step (bit for bit the stored rates): seg[n - n0][j][p]
// for the components j < n_eff.  Returns kReplayNotFast where the simulation did not run the
// fast kernel (another scheme, measure or state space, or EULER with a cap).
struct ReplaySegment {
    int n0, n_stop, n_eff;
    const double* ckpt;  // [N][P]
    double* seg;         // [n_stop - n0 + 1][N][P]
};
constexpr int kReplayNotFast = -1000;
int launch_replay_fp64(const PathLaunch& a, const ReplaySegment& r, cudaStream_t s);
// row pitch (floats) of the FP64 fast kernel's double-float rows, and the FMAX the launcher
// instantiates for N forward rates and F factors
__host__ __device__ constexpr int fp64_df_pitch(int fmax) { return (2 * fmax + 4 + 3) / 4 * 4; }
int paths_fp64_fmax(int N, int F);
// rows32: [T][N][pitch] FP32 component rows of the mixed path kernel, pitch =
// paths_fp32_rows(N, F, &fmax): the F loadings, zeros up to fmax, then at fmax the drift's
// deterministic part of the step, (variance * -0.5) * dt_i, and at fmax + 1 the 1/delta_j
int paths_fp32_rows(int N, int F, int* fmax);
int launch_paths_fp32(const PathLaunch& a, const float* rows32, cudaStream_t s, int* blocks_out);
int path_blocks(int P);
// exp(k/kExpTableHalf) for |k| <= kExpTableHalf, rounded to FP64 from extended precision
// (the table of exp_small in fp64math.cuh)
constexpr int kExpTableHalf = 256;
// forward rates of a model: the FP64 form takes up to 80 (the fast path kernels and the mixed
// form up to 64, the general FP64 path kernel beyond)
constexpr int kMaxForwardRates = 80;
void fp64_exp_table(double out[2 * kExpTableHalf + 1]);

// device random variables (randomvariable.cu) from process buffers: a copy (FP32 states
// widened) or the adjusted numeraire, ordered after the work so far on src_stream
int rv_from_device(double time, const void* src, int fp32, int64_t n, cudaStream_t src_stream, lmm_rv** out);
int rv_numeraire(double time, const double* d_num, const double* d_adj, int has_discount, int det, double pd, int64_t n,
                 cudaStream_t src_stream, lmm_rv** out);

// numeraire adjustment: adj[l] = mean over paths of 1/N_l (or the deterministic value)
int launch_numeraire_finish(const double* d_partials, int blocks, int N, int P, const double* d_numeraire,
                            const uint8_t* d_det, double* d_adj, cudaStream_t s);

struct ProductView {
    int P, N, T;
    int state_fp32;              // states stored as float
    const void* d_states;        // [nobs][N][P]
    const int* h_obs_slot;       // host copy [T+1]
    const double* d_numeraire;   // [N+1][P]
    const double* d_inv_numeraire;  // [N+1][P] 1/N, kept by the mixed form (else nullptr)
    const double* d_num_adj;     // [N+1] mean of 1/N (or deterministic value)
    const double* h_discount;    // [N+1] P^d chain (nullptr = none)
    const uint8_t* h_num_det;    // [N+1]
};

struct SwaptionLaunch {
    int nper;
    int period_slot[kMaxForwardRates];   // observation slot of min(exercise, fixing) per period
    int num_index;                       // tenor index of the exercise date
    int period_index[kMaxForwardRates];  // tenor index of each period
    double period_length[kMaxForwardRates];
    double disc_dt[kMaxForwardRates];    // payment - max(fixing, exercise)
    double strike[kMaxForwardRates];
    double notional;
};
int launch_swaption(const ProductView& v, const SwaptionLaunch& a, double* d_values, cudaStream_t s);
// Adjoint seeds of a European product (FP64 states): d value_p / d L_j(t) / P for every
// component j at the product's observation slot (the fixings of frozen components and the
// forwards of alive ones), the cross-path numeraire adjustment held constant (the reference
// AAD's getAverage).  Swaption.getValue (Swaption.java:137-199) and Caplet.getValue
// (Caplet.java:100-147) have pathwise derivatives: floor(0) differentiates to 1 where its
// argument is >= 0 (RandomVariableDifferentiableAAD.java:324-331).
struct CapletSeed {
    int slot;           // observation slot of the maturity (fixing) time
    int index;          // tenor index m of the period; paid at T_{m+1}
    double strike, daycount;
};
int launch_swaption_seeds(const ProductView& v, const SwaptionLaunch& a, int exercise_slot, const double* h_delta,
                          double* d_seeds, cudaStream_t s);
int launch_caplet_seeds(const ProductView& v, const CapletSeed& c, const double* h_delta, double* d_seeds,
                        cudaStream_t s);

// mean and standard error of d_values[P] (Kahan-equivalent compensated sums)
int reduce_mean_stderr(const double* d_values, int P, double* d_scratch, size_t scratch_bytes, double* h_mean,
                       double* h_stderr, cudaStream_t s);

struct BermudanPeriod {
    int libor_slot;      // observation slot of the fixing index
    int libor_index;     // tenor index of the period
    int pay_num_index;   // tenor index of the payment date (numeraire)
    int ex_slot;         // observation slot of the exercise index (exercisable periods)
    int ex_num_index;    // tenor index of the exercise date
    int exercisable;
    double period_length, strike, notional, fixing;
    // basis 0 (reference built-in)
    int short_index;     // tenor index of the short forward
    double short_dt;     // payment[fi] - fixing
    int long_first, long_last;  // tenor indices [first, last) of the long rate
    double long_dt;      // last payment - fixing[fi]
    // basis 1 (swap rate + numeraire)
    int swap_first, swap_last;  // product periods [first, last) of the remaining swap
};
struct BermudanLaunch {
    int nper, callable, basis;
    std::vector<BermudanPeriod> per;
};
struct BermudanScratch {
    double* d_values;     // [P]
    double* d_under;      // [P]
    double* d_ex;         // [P]
    double* d_basis;      // [ne][5][P] basis functions of every exercise date
    double* d_gram;       // [ne][gram blocks][20][2] Gram partial sums
    double* d_svd;        // [ne][80] U, s, V and cutoff of every exercise date
    double* d_partials;   // [blocks][6][2] X^T y partial sums of one date
    double* d_beta;       // [ne][6]
    BermudanPeriod* d_per;          // [nper]
    int* d_ex_period;               // [ne]
    const double* d_tenor_delta;    // [N]
    const int* d_period_index;      // [nper]
    const double* d_period_length;  // [nper]
    int tables_on_device = 0;       // d_per / d_ex_period already hold this product's tables
    int gram_blocks = 0;            // Gram blocks per exercise date (0: automatic)
    double* d_rec = nullptr;        // FP64 form, optional: [2][ne][P] trigger X and Y - Z per date
};
// scratch of the discrete-delta AAD weights of a Bermudan's cash flows (launch_bermudan_dd_weights)
struct BermudanDdScratch {
    const double* d_rec;      // [2][ne][P] from the forward valuation
    const void* d_basis;      // [ne][5][P]: doubles (FP64 form) or floats (mixed form)
    int basis_fp32;
    const double* d_svd;      // [ne][80]
    double* d_moments;        // [ne][64][2]
    double* d_mean;           // [ne]
    double* d_eps;            // [ne]
    double* d_betap;          // [ne][6]
    double* d_vbar;           // [P]
    double* d_ubar;           // [P]
    double* d_omega;          // [nper][P] the weights
    double* d_partials;       // [blocks][6][2] + completion counter (zero on entry)
};
int launch_bermudan_dd_weights(const BermudanLaunch& a, const BermudanDdScratch& sc, int P, double num0, double width,
                               cudaStream_t s);
int reduce_mean_var_device(const double* d_values, int P, double* d_scratch, double* d_out2, cudaStream_t s);
int launch_timestamp(unsigned long long* d_out, cudaStream_t s);
int bermudan_blocks(int P);
int bermudan_gram_blocks(int P, int ne, bool fp32);
// capacity (in blocks) of the Gram partials buffer for any exercise-date count <= 64
inline int bermudan_gram_capacity(int P) { return 4 * bermudan_blocks(P) + 64; }

struct AdjointLaunch {
    int T, N, F, P, nper, stride, callable, freeze_adjustment, fp32, T_slot, blocks;
    int threads;        // adjoint threads per block (64, 128, 256)
    int t_end, n_eff;   // reverse sweep from time index t_end over components 0..n_eff-1
    int normal;         // NORMAL state space (FP64 form): the state is L itself
    double cap;
    const double* h_discount;      // [N+1] or nullptr
    const uint8_t* h_num_det;      // [N+1]
    const double* h_delta;         // [N]
    const BermudanPeriod* d_per;   // [nper]
    const void* d_states;          // [nobs][N][P]
    const double* d_numeraire;     // [N+1][P]
    const double* d_inv_numeraire; // [N+1][P] 1/N
    const double* d_num_adj;       // [N+1]
    const double* d_ex;            // [P] exercise time of the forward valuation
    const int* d_first;            // [T]
    const double* d_init;          // [N]
    const void* d_dw;              // [T][F][P]
    const void* d_ckpt;            // [T/stride+1][N][P] forward rates every stride steps
    void* d_seg;                   // stride > 1: [stride+1][N][P] replayed forward rates of a segment
    void* d_ybar;                  // stride > 1: [N][P] adjoint of log L between segments
    const void *d_lam, *d_f, *d_sigma, *d_var_half, *d_inv_delta, *d_dt;  // tables in the path precision
    const PathLaunch* path64;      // FP64 processes: the path kernel's launch (the replay runs its own step)
    const float* d_rows32;         // FP32 processes: the mixed path kernel's component rows [T][N][pitch]
    const float* d_dt32;           // and its time steps [T] (the replay runs the path kernel's own step)
    double *d_abar, *d_abar_partials, *d_seeds, *d_value_partials, *d_value_out;
    double* d_nb;                  // [N+1][P] adjoints of the adjusted numeraires (scratch)
    double *d_vega_partials, *d_delta_partials, *d_vegas, *d_deltas;
    const double* d_omega;         // nullptr, or [nper][P] the cash flows' AAD weights (FP64 form)
};
int adjoint_blocks(int P, int threads, int fp32);
// scratch of one adjoint evaluation: per-warp partial rows and the segment buffers of stride > 1
struct AdjointScratch {
    int blocks, warps;
    size_t vega_partials, delta_partials;  // doubles
    size_t seg_bytes, ybar_bytes;
    size_t nb_doubles;                     // the d_nb scratch
};
AdjointScratch adjoint_scratch(int T, int N, int P, int threads, int stride, int fp32);
// row pitch (elements) of the factor table f[T][N][pitch] the reverse kernel reads
int adjoint_f_pitch(int N, int F, int fp32);
int launch_adjoint(const AdjointLaunch& a, cudaStream_t s);
// the reverse sweeps and Greek sums alone, from seeds already in d_seeds (d value / d L_j at t_end)
int launch_adjoint_sweeps(const AdjointLaunch& a, cudaStream_t s);
int launch_bermudan(const ProductView& v, const BermudanLaunch& a, const BermudanScratch& sc, cudaStream_t s,
                    int* launches);

}  // namespace lmm
