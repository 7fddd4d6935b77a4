// ieee_bits.h -- IEEE-754 double comparisons evaluated on the bit pattern.
//
// GB300's FP64 pipe issues about two lanes per clock per SM (1/64 of FP32),
// and FP64 compares, minimum/maximum and conversions run on it like FP64
// arithmetic.  The reference-mode kernels are FP64 end to end and are bound
// by that pipe, so their compares go through these predicates instead: plain
// 64-bit integer tests on the ALU.  Each one returns exactly what the IEEE
// comparison returns for every input -- NaNs (any payload, either sign),
// signed zeros (-0 == +0) and infinities included -- so replacing an FP64
// compare with one of these changes no result bit.
//
// Bit layout: sign bit 63, exponent 62..52, mantissa 51..0.  With the sign
// bit clear, the bit patterns of +0 .. +inf increase with the value; NaNs lie
// above +inf (0x7FF0000000000001 .. 0x7FFFFFFFFFFFFFFF) and, with the sign
// bit set, above -inf.
//
// Plain C++ as well as CUDA, so the predicates are tested on the host
// against the compiler's own double comparisons.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define TAM_HD __host__ __device__ __forceinline__
#else
#define TAM_HD inline
#endif

namespace tam {
namespace ieee {

constexpr uint64_t SIGN = 0x8000000000000000ull;
constexpr uint64_t PINF = 0x7FF0000000000000ull;  // +inf; |x| bits above this are NaN

TAM_HD uint64_t bits(double x)
{
#if defined(__CUDA_ARCH__)
    // an opaque move: the compiler would otherwise fold the integer tests
    // below back into FP64 compares
    uint64_t b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return b;
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

// x != x
TAM_HD bool is_nan(double x) { return (bits(x) & ~SIGN) > PINF; }
// x == 0.0 (either zero)
TAM_HD bool is_zero(double x) { return (bits(x) << 1) == 0; }
// x > 0.0: +min denormal .. +inf
TAM_HD bool gt_zero(double x) { return bits(x) - 1u < PINF; }
// x >= 0.0: +0 .. +inf, or -0
TAM_HD bool ge_zero(double x)
{
    const uint64_t b = bits(x);
    return b <= PINF || b == SIGN;
}
// x < 0.0: -min denormal .. -inf
TAM_HD bool lt_zero(double x) { return bits(x) - (SIGN + 1u) < PINF; }

// Compares against a constant c > 0 (finite, not NaN), passed as its bit
// pattern cb = bits(c).  The caller guarantees c > 0; use the general forms
// below otherwise.
// x >= c: cb <= bits(x) <= +inf
TAM_HD bool ge_pos(double x, uint64_t cb) { return bits(x) - cb <= PINF - cb; }
// x < c: +0 .. below cb, or any negative non-NaN value (-0 .. -inf)
TAM_HD bool lt_pos(double x, uint64_t cb)
{
    const uint64_t b = bits(x);
    return b < cb || b - SIGN <= PINF;
}

// General forms: a key that orders all non-NaN doubles like their values, with
// -0 and +0 equal (sign-magnitude to two's complement).
TAM_HD int64_t key(double x)
{
    const uint64_t b = bits(x);
    const int64_t m = (int64_t)(b & ~SIGN);
    return (b & SIGN) ? -m : m;
}
TAM_HD bool lt(double a, double b) { return !is_nan(a) && !is_nan(b) && key(a) < key(b); }
TAM_HD bool le(double a, double b) { return !is_nan(a) && !is_nan(b) && key(a) <= key(b); }
TAM_HD bool eq(double a, double b) { return !is_nan(a) && !is_nan(b) && key(a) == key(b); }

TAM_HD double from_bits(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

// 0.5 * x with IEEE round-to-nearest-even, on the bit pattern.  A biased
// exponent of 2..2046 is lowered by one (exact); zeros, denormals and the
// smallest normal binade shift their significand right by one and round
// half to even (the significand and the exponent field are contiguous, so
// the shift covers both); infinities pass through.  Bit-identical to the
// FP64 multiply for every non-NaN input; a NaN stays a NaN.
TAM_HD double half(double x)
{
    const uint64_t b = bits(x), s = b & SIGN, m = b & ~SIGN;
    const uint64_t e = m >> 52;
    uint64_t r;
    if (e >= 2u) r = e == 0x7FFu ? m : m - (1ull << 52);
    else r = (m >> 1) + (m & (m >> 1) & 1u);
    return from_bits(s | r);
}

// 2.0 * half(s), given h = half(s), on the bit pattern.  When half(s) was
// exact (biased exponent of s at least 2, or s infinite) it is s itself;
// otherwise h is a denormal or zero and its doubling shifts the
// significand left by one (exact).  Bit-identical to the FP64 multiply for
// every non-NaN input.
TAM_HD double twice_half(double s, double h)
{
    const uint64_t sb = bits(s);
    if (((sb & ~SIGN) >> 52) >= 2u) return s;
    const uint64_t hb = bits(h);
    return from_bits((hb & SIGN) | ((hb & ~SIGN) << 1));
}

}  // namespace ieee
}  // namespace tam

#undef TAM_HD
