// transport_common.cuh -- device pieces of the photon transport shared by
// the single-pass kernel (transport.cu) and the batched kernel
// (transport_batch.cu): the HG deflection of src/stokes.f90 in its FP64 and
// FP32 forms, the Fresnel reflectance, and the incremental DDA's per-axis
// set-up and position reconstruction.
#pragma once

#include "tam_device.cuh"
#include "tam_kernels.h"

namespace tam {
namespace {

template <typename Real> struct MatR {
    Real mut, mua, alb, g, g2, n;
};

// HG deflection with the arithmetic of src/stokes.f90:6-153 (PI/TWOPI are
// the truncated constants of src/constants.f90:13).  Leaves the direction
// unchanged when the sampled cosine is exactly +-1 (the `goto 100`).
template <typename Real>
__device__ __forceinline__ bool stokes(Real hgg, Real g2, Real u0, Real u1, Real &cost, Real &sint, Real &phi,
                                       Real &cosp, Real &sinp)
{
    const Real PI = (Real)PI_R, TWOPI = (Real)TWOPI_R;
    const Real one = (Real)1;
    if (hgg == (Real)0) {
        cost = (Real)2 * u0 - one;
        Real s2 = one - cost * cost;
        sint = s2 <= (Real)0 ? (Real)0 : M<Real>::sqrt(s2);
        phi = TWOPI * u1;
        M<Real>::sincos(phi, &sinp, &cosp);
        return true;
    }
    const Real costp = cost, sintp = sint, phip = phi;
    const Real t = M<Real>::div(one - g2, one - hgg + (Real)2 * hgg * u0);
    Real bmu = M<Real>::div((one + g2) - t * t, (Real)2 * hgg);
    Real cosb2 = bmu * bmu;
    if (M<Real>::abs(bmu) > one) {
        bmu = bmu > one ? one : -one;
        cosb2 = one;
    }
    if (bmu == one || bmu == -one) return false;  // direction unchanged
    const Real sinbt = M<Real>::sqrt(one - cosb2);
    const Real ri1 = TWOPI * u1;
    const bool upper = ri1 > PI;
    const Real ang = upper ? TWOPI - ri1 : ri1;
    Real sa, ca;
    M<Real>::sincos(ang, &sa, &ca);
    Real cosi2 = (Real)0, sini2;
    cost = costp * bmu + sintp * sinbt * ca;
    if (M<Real>::abs(cost) < one) {
        sint = M<Real>::abs(M<Real>::sqrt(one - cost * cost));
        sini2 = M<Real>::div(sa * sintp, sint);
        const Real bott = sint * sinbt;
        cosi2 = M<Real>::div(costp, bott) - M<Real>::div(cost * bmu, bott);
    } else {
        sint = (Real)0;
        sini2 = (Real)0;
        if (cost >= one) cosi2 = -one;
        if (cost <= -one) cosi2 = one;
    }
    Real cosdph = -cosi2 * ca + sini2 * sa * bmu;
    if (M<Real>::abs(cosdph) > one) cosdph = cosdph > one ? one : -one;
    const Real dph = M<Real>::acos(cosdph);
    phi = upper ? phip + dph : phip - dph;
    if (phi > TWOPI) phi = phi - TWOPI;
    if (phi < (Real)0) phi = phi + TWOPI;
    M<Real>::sincos(phi, &sinp, &cosp);
    return true;
}

// PTX approximate forms (relative error ~2^-22) for the FP32 path, whose
// results are checked statistically against the FP64 path.
__device__ __forceinline__ float rcp_ax(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_ax(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_ax(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// FP32 form of the same HG deflection.  The azimuth is carried as the pair
// (cos phi, sin phi) and rotated by the deflection angle dph, since
// phi' = phi +- dph (src/stokes.f90:136-140) gives
//   cos phi' = cos phi cos dph -+ sin phi sin dph,  sin dph = sqrt(1 - cos^2 dph),
// which replaces acos(cosdph) and the sincos of phi by one square root; the
// pair is renormalised so that rounding cannot drift over many scatters.
// Every sampled quantity (t, bmu, ang, cost, cosdph) follows the reference's
// formulas; only the evaluation of phi differs.
__device__ __forceinline__ bool stokes_f32(float hgg, float g2, float u0, float u1, float &cost, float &sint, float &cp,
                                           float &sp)
{
    const float PI = (float)PI_R, TWOPI = (float)TWOPI_R;
    if (hgg == 0.f) {
        cost = 2.f * u0 - 1.f;
        const float s2 = 1.f - cost * cost;
        sint = s2 <= 0.f ? 0.f : sqrt_ax(s2);
        __sincosf(TWOPI * u1, &sp, &cp);
        return true;
    }
    const float costp = cost, sintp = sint;
    const float t = __fdividef(1.f - g2, 1.f - hgg + 2.f * hgg * u0);
    const float bmu = __fdividef((1.f + g2) - t * t, 2.f * hgg);
    if (fabsf(bmu) >= 1.f) return false;  // clamped to +-1: direction unchanged
    const float sinbt = sqrt_ax(1.f - bmu * bmu);
    const float ri1 = TWOPI * u1;
    const bool upper = ri1 > PI;
    float sa, ca;
    __sincosf(upper ? TWOPI - ri1 : ri1, &sa, &ca);
    cost = costp * bmu + sintp * sinbt * ca;
    float sini2, cosi2;
    if (fabsf(cost) < 1.f) {
        sint = sqrt_ax(1.f - cost * cost);
        const float rs = rcp_ax(sint);
        sini2 = sa * sintp * rs;
        cosi2 = (costp - cost * bmu) * rs * rcp_ax(sinbt);
    } else {
        sint = 0.f;
        sini2 = 0.f;
        cosi2 = cost >= 1.f ? -1.f : 1.f;
    }
    float cosdph = -cosi2 * ca + sini2 * sa * bmu;
    cosdph = fminf(fmaxf(cosdph, -1.f), 1.f);
    float sdph = sqrt_ax(1.f - cosdph * cosdph);
    sdph = upper ? sdph : -sdph;
    const float ncp = cp * cosdph - sp * sdph, nsp = sp * cosdph + cp * sdph;
    const float rn = rsqrt_ax(ncp * ncp + nsp * nsp);
    cp = ncp * rn;
    sp = nsp * rn;
    return true;
}

// Unpolarised Fresnel reflectance n1 -> n2 at incidence cosine cosi.
template <typename Real> __device__ __forceinline__ Real fresnel(Real n1, Real n2, Real cosi)
{
    if (n1 == n2) return (Real)0;
    if (cosi > (Real)1) cosi = (Real)1;
    const Real sini = M<Real>::sqrt((Real)1 - cosi * cosi);
    const Real st = n1 / n2 * sini;
    if (st >= (Real)1) return (Real)1;
    const Real ct = M<Real>::sqrt((Real)1 - st * st);
    const Real rs = M<Real>::div(n1 * cosi - n2 * ct, n1 * cosi + n2 * ct);
    const Real rp = M<Real>::div(n1 * ct - n2 * cosi, n1 * ct + n2 * cosi);
    return (Real)0.5 * (rs * rs + rp * rp);
}

template <typename Real> __device__ __forceinline__ Real clamp0h(Real f, Real h)
{
    return f < (Real)0 ? (Real)0 : (f > h ? h : f);
}

// Voxel steps per warp vote of the flight phase: the votes are a sizeable
// share of a step, and a lane that stops early only idles for the rest (its
// packet's walk does not depend on when the event batch runs).  Measured on
// the 200^3 bench pass: 2 -> 190.5, 4 -> 193.5, 6 -> 189.9 Mphotons/s.
#ifndef TAM_VSTEPS
#define TAM_VSTEPS 4
#endif

// Dead lanes of a warp that make it draw new packets: the launch code runs
// for the dead lanes only, so refilling them together spends fewer of its
// warp instructions per packet, while they idle in the flight phase meanwhile.
// On the 200^3 bench pass: 1 -> 516.2, 2 -> 513.4, 4 -> 526.3, 8 -> 573.2 ms
// per 1e8 packets.
#ifndef TAM_REFILL_MIN
#define TAM_REFILL_MIN 2
#endif

enum : int { M_DEAD = 0, M_FLY = 1, M_SCAT = 2, M_FACE = 3 };  // M_SCAT, M_FACE: waiting for the event batch

// Per-flight DDA set-up from the in-cell position f and direction n of one
// axis: td = cell width along the ray, tm = distance to the next face.
template <typename Real>
__device__ __forceinline__ void axis_setup(Real n, Real f, Real h, Real BIG, Real &td, Real &tm, int &sg)
{
    // the reciprocal only for a component that is not zero: an FP64 1/0
    // takes the division's slow special-case path, and the reference medium
    // launches every packet with x and y components of zero
    if (n != (Real)0) {
        const Real inv = M<Real>::rcp(n);
        td = h * M<Real>::abs(inv);
        tm = n > (Real)0 ? (h - f) * inv : (n < (Real)0 ? -f * inv : BIG);
    } else {
        td = BIG;
        tm = BIG;
    }
    tm = tm < (Real)0 ? (Real)0 : tm;
    sg = n > (Real)0 ? 1 : -1;
}
// FP32: approximate reciprocal; |n| below 1e-30 counts as parallel to the
// faces (its reciprocal would overflow and turn 0 * inf into NaN).
template <>
__device__ __forceinline__ void axis_setup<float>(float n, float f, float h, float BIG, float &td, float &tm, int &sg)
{
    const float inv = rcp_ax(n);
    const bool par = fabsf(n) < 1e-30f;
    td = par ? BIG : h * fabsf(inv);
    tm = par ? BIG : (n > 0.f ? h - f : -f) * inv;
    tm = tm < 0.f ? 0.f : tm;
    sg = n > 0.f ? 1 : -1;
}

// In-cell position of one axis at distance t along the flight.
template <typename Real> __device__ __forceinline__ Real axis_pos(Real n, Real f, Real h, Real tm, Real t)
{
    const Real r = n > (Real)0 ? h - (tm - t) * n : (n < (Real)0 ? -(tm - t) * n : f);
    return clamp0h(r, h);
}

}  // namespace
}  // namespace tam
