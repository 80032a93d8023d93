// unroll_range.cuh -- fully unrolled loops over the forward-rate components whose
// first (or last) live index is known only at run time.
//
// The path state lives in registers, so a component loop must be unrolled with
// compile-time indices.  A plain unrolled loop guarded by `if (j >= first)` tends to be
// if-converted: the dead components then still issue, predicated off, which costs issue
// slots in the FP32 kernels.  These helpers enter the unrolled sequence through a jump
// table (a fall-through switch on the run-time start) instead.
#pragma once

#include <type_traits>

namespace lmm {

#define LMM_UP_CASE(J)                                                   \
    case J:                                                              \
        if constexpr (J < NMAX) body(std::integral_constant<int, J>{}); \
        [[fallthrough]];

// body(J) for J = j0 .. NMAX-1, ascending (J a std::integral_constant)
template <int NMAX, typename Body>
__device__ __forceinline__ void for_up_from(int j0, Body&& body)
{
    static_assert(NMAX <= 64, "at most 64 components");
    switch (j0) {
    LMM_UP_CASE(0)
    LMM_UP_CASE(1)
    LMM_UP_CASE(2)
    LMM_UP_CASE(3)
    LMM_UP_CASE(4)
    LMM_UP_CASE(5)
    LMM_UP_CASE(6)
    LMM_UP_CASE(7)
    LMM_UP_CASE(8)
    LMM_UP_CASE(9)
    LMM_UP_CASE(10)
    LMM_UP_CASE(11)
    LMM_UP_CASE(12)
    LMM_UP_CASE(13)
    LMM_UP_CASE(14)
    LMM_UP_CASE(15)
    LMM_UP_CASE(16)
    LMM_UP_CASE(17)
    LMM_UP_CASE(18)
    LMM_UP_CASE(19)
    LMM_UP_CASE(20)
    LMM_UP_CASE(21)
    LMM_UP_CASE(22)
    LMM_UP_CASE(23)
    LMM_UP_CASE(24)
    LMM_UP_CASE(25)
    LMM_UP_CASE(26)
    LMM_UP_CASE(27)
    LMM_UP_CASE(28)
    LMM_UP_CASE(29)
    LMM_UP_CASE(30)
    LMM_UP_CASE(31)
    LMM_UP_CASE(32)
    LMM_UP_CASE(33)
    LMM_UP_CASE(34)
    LMM_UP_CASE(35)
    LMM_UP_CASE(36)
    LMM_UP_CASE(37)
    LMM_UP_CASE(38)
    LMM_UP_CASE(39)
    LMM_UP_CASE(40)
    LMM_UP_CASE(41)
    LMM_UP_CASE(42)
    LMM_UP_CASE(43)
    LMM_UP_CASE(44)
    LMM_UP_CASE(45)
    LMM_UP_CASE(46)
    LMM_UP_CASE(47)
    LMM_UP_CASE(48)
    LMM_UP_CASE(49)
    LMM_UP_CASE(50)
    LMM_UP_CASE(51)
    LMM_UP_CASE(52)
    LMM_UP_CASE(53)
    LMM_UP_CASE(54)
    LMM_UP_CASE(55)
    LMM_UP_CASE(56)
    LMM_UP_CASE(57)
    LMM_UP_CASE(58)
    LMM_UP_CASE(59)
    LMM_UP_CASE(60)
    LMM_UP_CASE(61)
    LMM_UP_CASE(62)
    LMM_UP_CASE(63)
    default:
        break;
    }
}

#define LMM_DOWN_CASE(J)                                                      \
    case J:                                                                   \
        if constexpr (J < NMAX) {                                             \
            body(std::integral_constant<int, J>{});                          \
            if (J <= j0) break;                                               \
        }                                                                     \
        [[fallthrough]];

// body(J) for J = j_hi down to j0 (nothing when j_hi < j0)
template <int NMAX, typename Body>
__device__ __forceinline__ void for_down_to(int j_hi, int j0, Body&& body)
{
    static_assert(NMAX <= 64, "at most 64 components");
    if (j_hi < j0) return;
    switch (j_hi) {
    LMM_DOWN_CASE(63)
    LMM_DOWN_CASE(62)
    LMM_DOWN_CASE(61)
    LMM_DOWN_CASE(60)
    LMM_DOWN_CASE(59)
    LMM_DOWN_CASE(58)
    LMM_DOWN_CASE(57)
    LMM_DOWN_CASE(56)
    LMM_DOWN_CASE(55)
    LMM_DOWN_CASE(54)
    LMM_DOWN_CASE(53)
    LMM_DOWN_CASE(52)
    LMM_DOWN_CASE(51)
    LMM_DOWN_CASE(50)
    LMM_DOWN_CASE(49)
    LMM_DOWN_CASE(48)
    LMM_DOWN_CASE(47)
    LMM_DOWN_CASE(46)
    LMM_DOWN_CASE(45)
    LMM_DOWN_CASE(44)
    LMM_DOWN_CASE(43)
    LMM_DOWN_CASE(42)
    LMM_DOWN_CASE(41)
    LMM_DOWN_CASE(40)
    LMM_DOWN_CASE(39)
    LMM_DOWN_CASE(38)
    LMM_DOWN_CASE(37)
    LMM_DOWN_CASE(36)
    LMM_DOWN_CASE(35)
    LMM_DOWN_CASE(34)
    LMM_DOWN_CASE(33)
    LMM_DOWN_CASE(32)
    LMM_DOWN_CASE(31)
    LMM_DOWN_CASE(30)
    LMM_DOWN_CASE(29)
    LMM_DOWN_CASE(28)
    LMM_DOWN_CASE(27)
    LMM_DOWN_CASE(26)
    LMM_DOWN_CASE(25)
    LMM_DOWN_CASE(24)
    LMM_DOWN_CASE(23)
    LMM_DOWN_CASE(22)
    LMM_DOWN_CASE(21)
    LMM_DOWN_CASE(20)
    LMM_DOWN_CASE(19)
    LMM_DOWN_CASE(18)
    LMM_DOWN_CASE(17)
    LMM_DOWN_CASE(16)
    LMM_DOWN_CASE(15)
    LMM_DOWN_CASE(14)
    LMM_DOWN_CASE(13)
    LMM_DOWN_CASE(12)
    LMM_DOWN_CASE(11)
    LMM_DOWN_CASE(10)
    LMM_DOWN_CASE(9)
    LMM_DOWN_CASE(8)
    LMM_DOWN_CASE(7)
    LMM_DOWN_CASE(6)
    LMM_DOWN_CASE(5)
    LMM_DOWN_CASE(4)
    LMM_DOWN_CASE(3)
    LMM_DOWN_CASE(2)
    LMM_DOWN_CASE(1)
    LMM_DOWN_CASE(0)
    default:
        break;
    }
}

#undef LMM_UP_CASE
#undef LMM_DOWN_CASE

}  // namespace lmm
