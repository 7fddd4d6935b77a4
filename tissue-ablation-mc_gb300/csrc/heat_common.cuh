// heat_common.cuh -- device helpers shared by the fused heat-step kernels
// (heat.cu: cp.async form; heat_tma.cu: TMA form).
#pragma once

#include "tam_device.cuh"
#include "tam_kernels.h"

namespace tam {
namespace {

constexpr int FX = FX_TILE, FY = FY_TILE;

template <typename Real> struct Pt {
    Real T, e, k, r, h;  // temperature, Kahan compensation (true T = T - e), k, rho, c
};

template <typename Real, bool KAHAN>
__device__ __forceinline__ Pt<Real> ld(const Real *T, const float *E, const Real *K, const Real *R, const Real *C,
                                       int64_t v)
{
    Pt<Real> p;
    p.T = __ldg(T + v);
    p.e = KAHAN ? (Real)__ldg(E + v) : (Real)0;
    p.k = __ldg(K + v);
    p.r = __ldg(R + v);
    p.h = __ldg(C + v);
    return p;
}

// face diffusivity k_f / (rho_f c_f) with arithmetic face means
template <typename Real> __device__ __forceinline__ Real falpha(const Pt<Real> &a, const Pt<Real> &b)
{
    const Real kf = (Real)0.5 * (a.k + b.k), rf = (Real)0.5 * (a.r + b.r), cf = (Real)0.5 * (a.h + b.h);
    return M<Real>::div(kf, rf * cf);
}

// (true neighbour - true centre) for an interior neighbour
template <typename Real> __device__ __forceinline__ Real tdiff(const Pt<Real> &n, const Pt<Real> &c)
{
    return (n.T - c.T) - (n.e - c.e);
}

template <typename Real> __device__ __forceinline__ Real cst(const FusedArgs &a, int i);
template <> __device__ __forceinline__ float cst<float>(const FusedArgs &a, int i) { return a.fc[i]; }
template <> __device__ __forceinline__ double cst<double>(const FusedArgs &a, int i) { return a.dc[i]; }

// The step's source multiplier x dt and end time: from the launch's constants,
// or from device memory for steps replayed from a CUDA graph (the same values,
// rounded the same way).
template <typename Real> __device__ __forceinline__ Real step_pdt(const FusedArgs &a)
{
    return a.sv ? (Real)a.sv->pdt : cst<Real>(a, FC_PDT);
}
__device__ __forceinline__ double step_tnew(const FusedArgs &a) { return a.sv ? a.sv->t_new : a.t_new; }

// Laplacian term of one boundary face f (x-, x+, y-, y+, z-, z+): the ghost
// carries the voxel's own properties, so the face diffusivity is k/(rho c);
// (ghost - true centre) is the Dirichlet value minus the true temperature, or
// -h d / k (T - T_amb) for a convective (Robin) face.
template <typename Real>
__device__ __noinline__ Real ghost_term(const FusedArgs &a, int f, Real T, Real e, Real k, Real r, Real h)
{
    Real d;
    if (a.bc_type[f] == BC_ROBIN) d = -(cst<Real>(a, FC_BCHD + f) / k) * ((T - cst<Real>(a, FC_BCTA + f)) - e);
    else d = (cst<Real>(a, FC_BCT + f) - T) + e;
    return cst<Real>(a, f < 2 ? FC_CX : (f < 4 ? FC_CY : FC_CZ)) * (k / (r * h)) * d;
}

// Sum of the ghost terms of the boundary faces in mask gm (bit f = face f),
// one out-of-line call for all of a voxel's boundary faces.
__device__ __noinline__ float ghost_faces(const FusedArgs &a, unsigned gm, float T, float e, float k, float r,
                                          float h)
{
    float g = 0.f;
    for (int f = 0; f < 6; ++f)
        if (gm >> f & 1u) g += ghost_term<float>(a, f, T, e, k, r, h);
    return g;
}

// Arrhenius damage (FP64 exponent ln A - Ea/RT, src/3dFD.f90:450-461 with
// every crossed threshold stamped) and ablation of the optics for one voxel
// whose new true temperature is Tt.  Kept out of line so that no FP64 work is
// scheduled for the voxels that never reach it.
template <typename Real>
__device__ __noinline__ void rare_update(const FusedArgs &a, int64_t v, int64_t ni, double Tt, double t_new)
{
    if (a.arrhenius && Tt >= a.T_lo && Tt < a.T_hi) {
        const double o = a.omega[v];
        const double on = o + a.dt * exp(a.lnA - a.Ea / (a.Rgas * Tt));
        a.omega[v] = on;
#pragma unroll
        for (int t = 0; t < 3; ++t)
            if (o < a.thr[t] && on >= a.thr[t]) a.thres[v + t * ni] = t_new;
    }
    if (Tt >= a.T_abl && a.mat[v] != 0) {
        a.mat[v] = 0;  // optics -> air
        ((Real *)a.J)[v] = (Real)0;
        atomicAdd(a.n_ablated, 1ull);
    }
}

// (T - e) >= hi + lo for a double threshold split into floats (hi, lo),
// decided as the FP64 comparison of the exact T - e decides it: near the
// threshold T - hi is exact (Sterbenz), so only an error of ~1e-12 K remains.
__device__ __forceinline__ bool ge_ff(float T, float e, float hi, float lo) { return (T - hi) - (e + lo) >= 0.f; }

// FP32 form of rare_update from the Kahan pair (T, e), true temperature T - e.
// The exponent ln A - (Ea/R)/(T - e) is a difference of two numbers near 200
// whose FP32 rounding alone would put ~1e-5 relative error on the rate, so it
// is evaluated in float-float arithmetic (about 44 significant bits): the
// quotient's remainder comes exactly from one FMA, the difference from an
// error-free TwoSum (Knuth), and exp(hi + lo) = expf(hi) (1 + lo).  Only the
// damage sum itself is FP64 (one conversion and one add); threshold tests
// compare the non-negative doubles by their bit patterns, which order the same
// way.  Exponents beyond expf's range take the FP64 path, and so does every
// voxel when arr_fp64 is set (FP64 exponent ln A - Ea/RT of T - e).
// `o_pre` is the voxel's damage integral when the caller loaded it early
// (have_o), so that its latency overlapped the step's arithmetic.
__device__ __noinline__ void rare_update_f32(const FusedArgs &a, int64_t v, int64_t ni, float T, float e,
                                            double t_new, bool have_o = false, double o_pre = 0.0)
{
    if (a.arr_fp64) {
        rare_update<float>(a, v, ni, (double)T - (double)e, t_new);
        return;
    }
    if (a.arrhenius && ge_ff(T, e, a.fc[FC_TLO], a.fc[FC_TLO_LO]) && !ge_ff(T, e, a.fc[FC_THI], a.fc[FC_THI_LO])) {
        const float ear = a.fc[FC_EAR_HI], lna = a.fc[FC_LNA_HI];
        const float yh = __fdiv_rn(ear, T);
        // (Ea/R) - yh (T - e) = [ear - yh T] + ear_lo + yh e; the bracket is exact
        const float r = (__fmaf_rn(-yh, T, ear) + a.fc[FC_EAR_LO]) + yh * e;
        const float yl = __fdiv_rn(r, T);
        const float s = lna - yh, bb = s - lna;
        const float err = (lna - (s - bb)) + (-yh - bb);
        const float xl = (err + a.fc[FC_LNA_LO]) - yl;
        double inc;
        if (s < 80.f) {
            const float ex = expf(s);
            inc = (double)(a.fc[FC_DT] * __fmaf_rn(ex, xl, ex));
        } else {
            inc = a.dt * exp(a.lnA - a.Ea / (a.Rgas * ((double)T - (double)e)));
        }
        const double o = have_o ? o_pre : a.omega[v];
        const double on = o + inc;
        a.omega[v] = on;
        const long long ob = __double_as_longlong(o), nb = __double_as_longlong(on);
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const long long tb = __double_as_longlong(a.thr[t]);
            if (ob < tb && nb >= tb) a.thres[v + t * ni] = t_new;
        }
    }
    if (ge_ff(T, e, a.fc[FC_TABL], a.fc[FC_TABL_LO]) && a.mat[v] != 0) {
        a.mat[v] = 0;  // optics -> air
        ((float *)a.J)[v] = 0.f;
        atomicAdd(a.n_ablated, 1ull);
    }
}

}  // namespace
}  // namespace tam
