// mt19937_jump.cpp -- host side of the partitioned MT19937 stream.
//
// finmath-lib draws every Brownian increment from ONE MersenneTwister stream in
// path -> time -> factor order (BrownianMotionFromMersenneRandomNumbers.java:167-178,
// MersenneTwister.java:26-51 wrapping commons-math3's MersenneTwister(long)).  To split
// that stream across thread blocks without changing a single bit, each block starts
// from the state at its chunk offset, reached by a jump: the MT19937 state transition A
// is linear over GF(2), so A^J = g(A) with g = x^J mod phi, phi the characteristic
// polynomial of A (Haramoto, Matsumoto, Nishimura, Panneton, L'Ecuyer, "Efficient
// jump ahead for F2-linear random number generators", INFORMS J. Computing 2008).
//
// Here: phi is recovered once with Berlekamp-Massey from a 2*19937-bit output
// sequence (phi is primitive, so the minimal polynomial of any nonzero output bit
// sequence is phi itself).  Chunk c starts at word offset c * stride; with the base-8
// digits d_j of c that is the product of the jumps x^(d_j 8^j stride) mod phi, so a
// block applies at most one jump per nonzero digit.  Those 7 polynomials per digit are
// computed by square-and-multiply-by-x, squaring and GF(2) products modulo phi, and
// cached per chunk stride.  The device applies g(A) to a state as an XOR of the windows
// x[i..i+623] of the raw word sequence for which g_i = 1.
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>

#include "lmm_internal.h"

namespace lmm {

// ------------------------------------------------------------------ seeding
static void init_genrand(uint32_t* mt, uint32_t s)
{
    mt[0] = s;
    for (int i = 1; i < kMtN; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
}

void mt_seeded_state(int64_t seed, uint32_t out[kMtN])
{
    // commons-math3 MersenneTwister(long): key {hi, lo}, then init_by_array.
    const uint64_t u = (uint64_t)seed;
    const uint32_t key[2] = {(uint32_t)(u >> 32), (uint32_t)u};
    uint32_t* mt = out;
    init_genrand(mt, 19650218u);
    int i = 1, j = 0;
    for (int k = kMtN; k != 0; k--) {
        mt[i] = (mt[i] ^ ((mt[i - 1] ^ (mt[i - 1] >> 30)) * 1664525u)) + key[j] + (uint32_t)j;
        i++;
        j++;
        if (i >= kMtN) { mt[0] = mt[kMtN - 1]; i = 1; }
        if (j >= 2) j = 0;
    }
    for (int k = kMtN - 1; k != 0; k--) {
        mt[i] = (mt[i] ^ ((mt[i - 1] ^ (mt[i - 1] >> 30)) * 1566083941u)) - (uint32_t)i;
        i++;
        if (i >= kMtN) { mt[0] = mt[kMtN - 1]; i = 1; }
    }
    mt[0] = 0x80000000u;
}

// Raw (untempered) word sequence x[n], x[0..623] = the given state.
static void mt_raw_sequence(const uint32_t* state, size_t count, std::vector<uint32_t>& x)
{
    x.resize(count);
    for (size_t n = 0; n < count; n++) {
        if (n < (size_t)kMtN) { x[n] = state[n]; continue; }
        uint32_t y = (x[n - kMtN] & 0x80000000u) | (x[n - kMtN + 1] & 0x7fffffffu);
        x[n] = x[n - (kMtN - kMtM)] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
}

// ------------------------------------------------------------------ GF(2) polynomials
using Poly = std::vector<uint64_t>;

static inline int get_bit(const Poly& p, size_t i) { return (int)((p[i >> 6] >> (i & 63)) & 1u); }
static inline void flip_bit(Poly& p, size_t i) { p[i >> 6] ^= (uint64_t)1 << (i & 63); }

// p ^= q << shift (bits), p sized large enough
static void xor_shifted(Poly& p, const Poly& q, size_t qbits, size_t shift)
{
    const size_t ws = shift >> 6, bs = shift & 63;
    const size_t qw = (qbits + 63) >> 6;
    for (size_t i = 0; i < qw; i++) {
        uint64_t v = q[i];
        if (!v) continue;
        p[i + ws] ^= v << bs;
        if (bs && i + ws + 1 < p.size()) p[i + ws + 1] ^= v >> (64 - bs);
    }
}

struct Phi {
    Poly coeff;   // degree 19937, bit i = coefficient of x^i (19938 bits)
};

static Phi compute_phi()
{
    // Output bit sequence: most significant bit of the raw words of an arbitrary state.
    uint32_t st[kMtN];
    mt_seeded_state(5489, st);
    const size_t nbits = 2 * (size_t)kMtDegree;
    std::vector<uint32_t> x;
    mt_raw_sequence(st, nbits, x);
    // Berlekamp-Massey over GF(2).  sr = reversed bit sequence so that the discrepancy is
    // an aligned-direction inner product.
    const size_t W = (nbits + 63) / 64 + 2;
    Poly sr(W, 0);
    for (size_t n = 0; n < nbits; n++)
        if (x[n] >> 31) { size_t j = nbits - 1 - n; sr[j >> 6] |= (uint64_t)1 << (j & 63); }
    auto window = [&](size_t off, size_t w) -> uint64_t {  // 64 bits of sr starting at bit off + 64 w
        size_t b = off + 64 * w;
        size_t i = b >> 6, s = b & 63;
        uint64_t lo = i < W ? sr[i] : 0, hi = (i + 1) < W ? sr[i + 1] : 0;
        return s ? ((lo >> s) | (hi << (64 - s))) : lo;
    };
    Poly C(W, 0), B(W, 0), Tmp;
    C[0] = 1;
    B[0] = 1;
    size_t L = 0, m = 1, LB = 0;  // LB: degree bound of B
    for (size_t n = 0; n < nbits; n++) {
        // d = sum_{i=0..L} C_i s_{n-i};  s_{n-i} = sr[nbits-1-n+i]
        const size_t off = nbits - 1 - n;
        const size_t nw = (L + 1 + 63) / 64;
        uint64_t acc = 0;
        for (size_t w = 0; w < nw; w++) {
            uint64_t c = C[w];
            if (w == nw - 1 && ((L + 1) & 63)) c &= (((uint64_t)1 << ((L + 1) & 63)) - 1);
            acc ^= c & window(off, w);
        }
        int d = __builtin_parityll(acc);
        if (!d) { m++; continue; }
        if (2 * L <= n) {
            Tmp = C;
            xor_shifted(C, B, LB + 1, m);
            LB = L;
            L = n + 1 - L;
            B = Tmp;
            m = 1;
        } else {
            xor_shifted(C, B, LB + 1, m);
            m++;
        }
    }
    if (L != (size_t)kMtDegree) throw std::runtime_error("MT19937 characteristic polynomial: unexpected degree");
    Phi phi;
    phi.coeff.assign(kPolyWords + 1, 0);
    // phi(x) = x^L C(1/x): phi_i = C_{L-i}
    for (size_t i = 0; i <= L; i++)
        if (get_bit(C, L - i)) flip_bit(phi.coeff, i);
    return phi;
}

static const Phi& phi()
{
    static Phi p;
    static std::once_flag once;
    std::call_once(once, [] { p = compute_phi(); });
    return p;
}

// r = r^2 mod phi (r has kPolyWords words, degree < 19937)
static void poly_square_mod(Poly& r)
{
    const Phi& f = phi();
    Poly sq(2 * kPolyWords + 2, 0);
    for (int i = 0; i < kPolyWords; i++) {
        uint64_t v = r[i];
        if (!v) continue;
        // spread 32-bit halves into 64-bit words (bit k -> bit 2k)
        for (int h = 0; h < 2; h++) {
            uint64_t t = (v >> (32 * h)) & 0xffffffffu;
            t = (t | (t << 16)) & 0x0000ffff0000ffffULL;
            t = (t | (t << 8)) & 0x00ff00ff00ff00ffULL;
            t = (t | (t << 4)) & 0x0f0f0f0f0f0f0f0fULL;
            t = (t | (t << 2)) & 0x3333333333333333ULL;
            t = (t | (t << 1)) & 0x5555555555555555ULL;
            sq[2 * i + h] = t;
        }
    }
    // reduce bits >= 19937 from the top
    for (size_t i = 2 * (size_t)(kMtDegree - 1); i >= (size_t)kMtDegree; i--) {
        if (get_bit(sq, i)) xor_shifted(sq, f.coeff, kMtDegree + 1, i - kMtDegree);
    }
    r.assign(sq.begin(), sq.begin() + kPolyWords);
    // clear bits >= 19937 in the last word (they are zero after reduction)
}

// r = r * x mod phi
static void poly_mulx_mod(Poly& r)
{
    const Phi& f = phi();
    uint64_t carry = 0;
    for (int i = 0; i < kPolyWords; i++) {
        uint64_t v = r[i];
        r[i] = (v << 1) | carry;
        carry = v >> 63;
    }
    // degree 19937 bit lives in word 311, bit 33 (19937 = 311*64 + 33)
    if ((r[kMtDegree >> 6] >> (kMtDegree & 63)) & 1u) {
        for (int i = 0; i < kPolyWords; i++) r[i] ^= f.coeff[i];
        r[kMtDegree >> 6] &= ~((uint64_t)1 << (kMtDegree & 63));
    }
}

static Poly poly_x_pow(uint64_t e)
{
    Poly r(kPolyWords, 0);
    r[0] = 1;
    int top = 63;
    while (top >= 0 && !((e >> top) & 1u)) top--;
    for (int b = top; b >= 0; b--) {
        poly_square_mod(r);
        if ((e >> b) & 1u) poly_mulx_mod(r);
    }
    return r;
}

// a b mod phi over GF(2): the shifted copies of b for the set bits of a, then the
// reduction of the bits >= 19937 from the top
static Poly poly_mul_mod(const Poly& a, const Poly& b)
{
    const Phi& f = phi();
    Poly prod(2 * kPolyWords + 2, 0);
    for (int i = 0; i < kPolyWords; i++) {
        uint64_t v = a[i];
        while (v) {
            const int k = __builtin_ctzll(v);
            v &= v - 1;
            xor_shifted(prod, b, kMtDegree, (size_t)i * 64 + (size_t)k);
        }
    }
    for (size_t i = 2 * (size_t)(kMtDegree - 1); i >= (size_t)kMtDegree; i--)
        if (get_bit(prod, i)) xor_shifted(prod, f.coeff, kMtDegree + 1, i - kMtDegree);
    prod.resize(kPolyWords);
    return prod;
}

const std::vector<uint64_t>& mt_jump_digit_polynomials(uint64_t stride_words, int ndigits)
{
    static std::mutex mu;
    static std::map<uint64_t, std::vector<uint64_t>> cache;
    std::lock_guard<std::mutex> lock(mu);
    constexpr int per = kJumpBase - 1;
    std::vector<uint64_t>& v = cache[stride_words];
    if (v.size() >= (size_t)ndigits * per * kPolyWords) return v;
    v.clear();
    Poly g1 = poly_x_pow(stride_words);  // x^(8^j stride) for the digit j
    for (int j = 0; j < ndigits; j++) {
        Poly g[kJumpBase];
        g[1] = g1;
        for (int d = 2; d < kJumpBase; d++) {
            if (d % 2 == 0) {
                g[d] = g[d / 2];
                poly_square_mod(g[d]);  // x^(2e) = (x^e)^2
            } else {
                g[d] = poly_mul_mod(g[d - 1], g[1]);
            }
        }
        for (int d = 1; d < kJumpBase; d++) v.insert(v.end(), g[d].begin(), g[d].end());
        g1 = g[kJumpBase / 2];
        poly_square_mod(g1);  // x^(8^(j+1) stride)
    }
    return v;
}

// the raw state after the jump g applied to st (in place)
static void apply_jump(uint32_t* st, const Poly& g)
{
    std::vector<uint32_t> x;
    mt_raw_sequence(st, (size_t)kJumpWindow, x);
    for (int w = 0; w < kMtN; w++) {
        uint32_t acc = 0;
        for (int i = 0; i < kMtDegree; i++)
            if (get_bit(g, (size_t)i)) acc ^= x[(size_t)i + w];
        st[w] = acc;
    }
}

static void tempered_words(const uint32_t* st, uint64_t count, uint32_t* out);

// Host restatement of the device jump (used to check the jump polynomials without a GPU):
// the tempered words [skip, skip+count) of MersenneTwister(seed), reached by one jump.
void mt_words_after_jump(int64_t seed, uint64_t skip, uint64_t count, uint32_t* out)
{
    uint32_t st[kMtN];
    mt_seeded_state(seed, st);
    if (skip > 0) apply_jump(st, poly_x_pow(skip));
    tempered_words(st, count, out);
}

// The same for the start of chunk `chunk` of a partition with `stride_words` words per
// chunk, reached as the device reaches it: one jump per nonzero base-8 digit of the chunk.
void mt_words_at_chunk(int64_t seed, uint64_t stride_words, uint64_t chunk, uint64_t count, uint32_t* out)
{
    uint32_t st[kMtN];
    mt_seeded_state(seed, st);
    int ndigits = 0;
    while (ndigits < 21 && (chunk >> (kJumpDigitBits * ndigits)) != 0) ndigits++;
    if (ndigits > 0) {
        const std::vector<uint64_t>& v = mt_jump_digit_polynomials(stride_words, ndigits);
        for (int j = 0; j < ndigits; j++) {
            const int d = (int)((chunk >> (kJumpDigitBits * j)) & (kJumpBase - 1));
            if (!d) continue;
            const size_t off = ((size_t)j * (kJumpBase - 1) + (size_t)(d - 1)) * kPolyWords;
            apply_jump(st, Poly(v.begin() + off, v.begin() + off + kPolyWords));
        }
    }
    tempered_words(st, count, out);
}

static void tempered_words(const uint32_t* st, uint64_t count, uint32_t* out)
{
    std::vector<uint32_t> x;
    mt_raw_sequence(st, (size_t)kMtN + count, x);
    for (uint64_t k = 0; k < count; k++) {
        uint32_t y = x[kMtN + k];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        out[k] = y;
    }
}

}  // namespace lmm

extern "C" int lmm_mt19937_chunk_words_host(int64_t seed, uint64_t stride_words, uint64_t chunk, uint64_t count,
                                            uint32_t* out)
{
    if (!out) return lmm::fail(LMM_ERR_INVALID, "null argument");
    if (stride_words == 0 && chunk > 0) return lmm::fail(LMM_ERR_INVALID, "a chunk stride of zero words");
    try {
        lmm::mt_words_at_chunk(seed, stride_words, chunk, count, out);
    } catch (const std::exception& e) {
        return lmm::fail(LMM_ERR_INVALID, e.what());
    }
    return LMM_OK;
}

extern "C" int lmm_mt19937_words_host(int64_t seed, uint64_t skip, uint64_t count, uint32_t* out)
{
    if (!out) return lmm::fail(LMM_ERR_INVALID, "null argument");
    try {
        lmm::mt_words_after_jump(seed, skip, count, out);
    } catch (const std::exception& e) {
        return lmm::fail(LMM_ERR_INVALID, e.what());
    }
    return LMM_OK;
}
