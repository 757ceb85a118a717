// The compensated FP32 operator of the mixed-precision solvers on pinned
// (near-singular) pressure systems: q = (I + N) p with N = S A S - I stored as
// FP32 entries plus an 8-bit correction each, and the row accumulated in
// float-float arithmetic.
//
// Why: on a pressure system pinned at one cell (pure Neumann walls plus the
// reference's cell-0 pin) the FP32 inner CG needs 15-30% more iterations than
// FP64 CG at a 1e-8 tolerance.  Rounding the entries of S A S to FP32, and
// summing a row in FP32, each perturb the inner operator by about one FP32
// rounding per term; with the slow mode of such a system that puts the true
// residual's floor near 2.5e-8, above the tolerance, and the last decade
// stalls.  An operator accurate to ~2^-31 per term lowers the floor below the
// tolerance: each stored entry u gets k = round((a - u) / (ulp(u) / 128)), an
// int8 (|k| <= 64), so u + k ulp(u)/128 equals a to ~2^-31 of u, and each
// product is summed with its rounding error carried (TwoSum, and the exact
// product error from an FMA).  The vectors stay FP32: their rounding does not
// move the floor.  Measured in a bit-faithful numpy emulation of the inner
// iteration: a 128x128 cavity system with a random right-hand side takes 769
// iterations this way, 944 with FP32 entries and FP32 sums, 762 in FP64; a
// 256x256 one 1536, 1988 and 1528.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace simall {

// The 8-bit correction of an FP64 value a against its FP32 rounding u:
// (a - u) in units of 2^(E - 157) = ulp(u) / 128, E u's biased exponent; 0
// where u is 0, not finite or below 2^-96 (the unit would leave FP32's normal
// range).  The same operations on the host and the device: an exact FP64
// difference, a multiplication by a power of two and a round-to-nearest-even.
__host__ __device__ inline int8_t ff_correction(double a, float u)
{
    const float au = u < 0.0f ? -u : u;
    if (!(au >= 1.2621774483536189e-29f) || !(au <= 3.4028234663852886e38f))  // [2^-96, FLT_MAX]
        return 0;
    uint32_t bits = 0;
    memcpy(&bits, &u, sizeof bits);
    const int E = static_cast<int>((bits >> 23) & 0xffu);
    const double k = rint((a - static_cast<double>(u)) * ldexp(1.0, 157 - E));
    return static_cast<int8_t>(k > 127.0 ? 127 : (k < -127.0 ? -127 : k));
}

// The correction's value, exact in FP32: k 2^(E - 157), E u's biased exponent
// (the float whose exponent field is E - 30).
__device__ __forceinline__ float ff_low(float u, int8_t k)
{
    const int ebits = __float_as_int(u) & 0x7f800000;
    const float unit = __int_as_float((ebits > (31 << 23) ? ebits : (31 << 23)) - (30 << 23));
    return __fmul_rn(static_cast<float>(k), unit);
}

// Float-float accumulator.
struct FFAcc {
    float hi, lo;
};

__device__ __forceinline__ FFAcc ff_start(float v) { return FFAcc{v, 0.0f}; }

// acc += (uh + ul) v: the product uh v as a rounded value plus its exact error
// (FMA), added to hi with TwoSum; ul v is summed into lo with the errors.
// Every operation is explicitly rounded, so the compiler cannot contract it.
__device__ __forceinline__ void ff_add(FFAcc &acc, float uh, float ul, float v)
{
    const float th = __fmul_rn(uh, v);
    const float tl = __fmaf_rn(uh, v, -th);
    const float s = __fadd_rn(acc.hi, th);
    const float bb = __fsub_rn(s, acc.hi);
    const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(th, bb));
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(err, __fmaf_rn(ul, v, tl)));
}

__device__ __forceinline__ float ff_value(const FFAcc &acc) { return __fadd_rn(acc.hi, acc.lo); }

}  // namespace simall
