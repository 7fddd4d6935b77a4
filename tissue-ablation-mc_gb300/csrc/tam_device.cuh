// tam_device.cuh -- device-side building blocks shared by the transport and
// heat kernels: Philox4x32-10, uniform conversion, device error bits and the
// round-to-nearest FP64 helpers used where the arithmetic must follow the
// reference statement by statement (no fused multiply-add contraction).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tam {

// Device error word bits (read by the host after each hot call).
enum : unsigned {
    DEVERR_STEP_CAP = 1u << 0,    // a packet exceeded its loop cap (was killed)
    DEVERR_NAN = 1u << 1,         // a packet direction or a temperature became NaN
    DEVERR_NEG_T = 1u << 2,       // negative kelvin (src/3dFD.f90:179-182, thermalConst_mod.f90:20-23)
    DEVERR_EVENT_OVF = 1u << 3,   // event list overflow
    DEVERR_SYNC_TIMEOUT = 1u << 4, // a bounded wait on an asynchronous copy gave up
};

// Truncated constants of src/constants.f90:13 (promoted to FP64).
constexpr double PI_R = 3.141592;
constexpr double TWOPI_R = 6.283185;

// ---------------------------------------------------------------- Philox --
// Philox4x32-10 (Salmon et al., SC'11).  Counter layout per packet event:
// {event, packet_lo, packet_hi, stream}; key {seed_lo, seed_hi}.
struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                     uint32_t k0, uint32_t k1)
{
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

// The same generator with the ten round keys given (rk[2r], rk[2r + 1]: the
// key of round r, i.e. the key plus r times the Weyl increments): from a
// kernel parameter block they are constant-bank operands of the rounds'
// XORs, and no round adds to the key.
__device__ __forceinline__ U4 philox4x32_10_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const uint32_t *rk)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ rk[2 * r], n2 = hi0 ^ c3 ^ rk[2 * r + 1];
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return U4{c0, c1, c2, c3};
}
__host__ __device__ inline void philox_round_keys(uint64_t seed, uint32_t *rk)
{
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r, k0 += 0x9E3779B9u, k1 += 0xBB67AE85u) {
        rk[2 * r] = k0;
        rk[2 * r + 1] = k1;
    }
}

template <typename Real> struct Uniform;
// FP64: u = (x + 0.5) 2^-32, exact in (0,1).
template <> struct Uniform<double> {
    __device__ __forceinline__ static double from(uint32_t x) { return ((double)x + 0.5) * 0x1p-32; }
};
// FP32: u = ((x >> 9) + 0.5) 2^-23: k + 0.5 is exact in FP32 for k < 2^23, so
// u lies on a 2^-23 grid strictly inside (0,1), the largest value 1 - 2^-24.
// (24 bits would round k + 0.5 to even above 2^23 and could give u = 1.)
template <> struct Uniform<float> {
    // (k + 1/2) 2^-23 for k = x >> 9, exactly: the float 1 + k 2^-23 built
    // from its bits, minus 1 - 2^-24 (an exact difference), in place of an
    // integer-to-float conversion
    __device__ __forceinline__ static float from(uint32_t x)
    {
        return __uint_as_float(0x3f800000u | (x >> 9)) - 0x1.fffffep-1f;
    }
};

// ------------------------------------------- exact FP64 helpers (no FMA) --
__device__ __forceinline__ double ADD(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double SUB(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double MUL(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double DIV(double a, double b) { return __ddiv_rn(a, b); }

// ------------------------------------------------------- math dispatch --
template <typename Real> struct M;
template <> struct M<float> {
    __device__ __forceinline__ static float log(float x) { return __logf(x); }
    // -log(u) for u in (0,1), never below 1 - u (> 0): the fast logarithm's
    // absolute error near 1 could otherwise give 0 or a negative value
    __device__ __forceinline__ static float neglog(float u) { return fmaxf(-__logf(u), 1.f - u); }
    __device__ __forceinline__ static void sincos(float x, float *s, float *c) { __sincosf(x, s, c); }
    __device__ __forceinline__ static float sqrt(float x) { return sqrtf(x); }
    __device__ __forceinline__ static float acos(float x) { return acosf(x); }
    __device__ __forceinline__ static float div(float a, float b) { return __fdividef(a, b); }
    __device__ __forceinline__ static float rcp(float a) { return __frcp_rn(a); }  // correctly rounded 1/a
    __device__ __forceinline__ static float abs(float a) { return fabsf(a); }
};
template <> struct M<double> {
    __device__ __forceinline__ static double log(double x) { return ::log(x); }
    __device__ __forceinline__ static double neglog(double u) { return -::log(u); }
    __device__ __forceinline__ static void sincos(double x, double *s, double *c) { ::sincos(x, s, c); }
    __device__ __forceinline__ static double sqrt(double x) { return ::sqrt(x); }
    __device__ __forceinline__ static double acos(double x) { return ::acos(x); }
    __device__ __forceinline__ static double div(double a, double b) { return a / b; }
    __device__ __forceinline__ static double rcp(double a) { return 1.0 / a; }
    __device__ __forceinline__ static double abs(double a) { return fabs(a); }
};

}  // namespace tam
