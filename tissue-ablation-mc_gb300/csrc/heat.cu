// heat.cu -- explicit heat diffusion, Arrhenius damage and ablation on sm_103a.
//
// Two families of kernels:
//  * reference path (FP64, reference array layout with halos): the stencil of
//    src/3dFD.f90:113-187, Arrhenius of src/3dFD.f90:424-466 and the property
//    / ablation update of src/3dFD.f90:312-361, each evaluated with explicit
//    round-to-nearest operations in the reference's order of evaluation so
//    the result matches the Fortran arithmetic (no FMA contraction), with
//    compares on the integer pipe (ieee_bits.h) because these kernels are
//    bound by GB300's narrow FP64 pipe; an FP32 form of the stencil reads
//    FP32 copies of the fields and adds its increments to the FP64
//    temperatures;
//  * fused config-mode step: stencil + latent-heat clamp + Arrhenius (exponent
//    ln A - Ea/RT in FP64, or float-float in the FP32 form) + ablation in one
//    pass, with FP32 storage and a Kahan-compensated temperature, or plain
//    FP64.  Each thread marches a (x, y) column through a z-chunk keeping the
//    z-neighbours in registers; this cp.async form with per-voxel k, rho, c
//    serves the FP64 step and FP32 grids whose properties were uploaded per
//    voxel on rows TMA cannot copy (class-table steps: heat_tma.cu with TMA,
//    batch.cu with cp.async staging for any row pitch).
#include <algorithm>
#include <atomic>
#include <cstdio>

#include "heat_common.cuh"
#include "ieee_bits.h"

namespace tam {

namespace {

// ------------------------------------------------------- reference path --
// Bit patterns of the positive constants the reference kernels compare
// against (ieee::ge_pos / lt_pos).
constexpr uint64_t B_0_53 = 0x3FE0F5C28F5C28F6ull;  // 0.53
constexpr uint64_t B_0_75 = 0x3FE8000000000000ull;  // 0.75
constexpr uint64_t B_1 = 0x3FF0000000000000ull;     // 1.0
constexpr uint64_t B_316 = 0x4073C00000000000ull;   // 316.0
constexpr uint64_t B_373 = 0x4077500000000000ull;   // 373.0
constexpr uint64_t B_1E4 = 0x40C3880000000000ull;   // 10000.0

struct H {
    int64_t hx, hy;
    __device__ __forceinline__ int64_t operator()(int i, int j, int k) const
    {
        return (int64_t)i + hx * ((int64_t)j + hy * (int64_t)k);
    }
};

// Face term of src/3dFD.f90:119-132: a = 0.5*(kM/(dM*cM))*(1/d^2).  The
// products with 0.5 are formed on the bit pattern (ieee::half, bit-identical
// to the FP64 multiply): a fifth of the stencil's FP64 operations move off
// GB300's narrow FP64 pipe.
__device__ __forceinline__ double ref_face(double kc, double kn, double dc, double dn, double cc, double cn,
                                           double id2)
{
    const double kh = ieee::half(ADD(kc, kn));
    const double dh = ieee::half(ADD(dc, dn));
    const double ch = ieee::half(ADD(cc, cn));
    return MUL(ieee::half(DIV(kh, MUL(dh, ch))), id2);
}

// u = a*T- - 2b*T + d*T+ with b = 0.5(a+d)   (src/3dFD.f90:130-132); 2b from
// a + d on the bit pattern (ieee::twice_half: the FP64 products' bits)
__device__ __forceinline__ double ref_axis(double a, double d, double tm, double t, double tp)
{
    const double s = ADD(a, d);
    const double b2 = ieee::twice_half(s, ieee::half(s));
    return ADD(SUB(MUL(a, tm), MUL(b2, t)), MUL(d, tp));
}

// Source, latent-heat clamp and physicality check of one voxel
// (src/3dFD.f90:166-183); c: halo index, q: interior index.
__device__ __forceinline__ void ref_update(const RefHeatArgs &a, int64_t c, int64_t q, double T, double cc,
                                           double u_xx, double u_yy, double u_zz)
{
    const double J = a.J[q];
    const double tempIncrease = MUL(a.delt, ADD(ADD(u_xx, u_yy), u_zz));
    const double energyIncrease =
        ADD(MUL(MUL(MUL(a.laserOn, J), a.delt), a.vvox), MUL(MUL(cc, a.mvox), tempIncrease));
    const double heat = ADD(ADD(T, tempIncrease), MUL(MUL(a.laserOn, a.coeff[c]), J));
    double tn = heat;
    // compares on the bit patterns (ieee_bits.h); Q is read only at 373 K and above
    if (ieee::ge_pos(T, B_373)) {
        const double Qv = a.Q[q];
        if (ieee::lt(Qv, a.qvapor) && ieee::gt_zero(energyIncrease)) {
            const double qn = ADD(Qv, energyIncrease);
            a.Q[q] = ieee::lt(qn, a.qvapor) ? qn : a.qvapor;
            tn = 373.0;
        }
    } else if (ieee::lt_zero(T)) {
        atomicOr(a.err, DEVERR_NEG_T);
    }
    if (ieee::is_nan(tn)) atomicOr(a.err, DEVERR_NAN);
    a.tn[c] = tn;
}

// The FP32 form of the same update: the step's increment and source term in
// FP32, added to the FP64 temperature in FP64 (so no compensation is
// needed), and the FP32 copy of the result written beside it; the
// latent-heat branch, rare, stays FP64.
__device__ __forceinline__ void ref_update_f32(const RefHeatArgs &a, int64_t c, int64_t q, double T, float cc,
                                               float u_xx, float u_yy, float u_zz)
{
    const double J = a.J[q];
    const float inc = (float)a.delt * ((u_xx + u_yy) + u_zz);
    const float src = (float)a.laserOn * a.p32[3 * a.nh + c] * (float)J;
    const double heat = T + (double)(inc + src);
    double tn = heat;
    if (ieee::ge_pos(T, B_373)) {
        const double Qv = a.Q[q];
        if (ieee::lt(Qv, a.qvapor)) {
            const double energyIncrease = a.laserOn * J * a.delt * a.vvox + (double)cc * a.mvox * (double)inc;
            if (ieee::gt_zero(energyIncrease)) {
                const double qn = Qv + energyIncrease;
                a.Q[q] = ieee::lt(qn, a.qvapor) ? qn : a.qvapor;
                tn = 373.0;
            }
        }
    } else if (ieee::lt_zero(T)) {
        atomicOr(a.err, DEVERR_NEG_T);
    }
    if (ieee::is_nan(tn)) atomicOr(a.err, DEVERR_NAN);
    a.tn[c] = tn;
    a.sn[c] = (float)tn;
}

// Face terms and axis sums of the reference stencil in the working precision
// F: double keeps the Fortran's operations and order (bit parity); float is
// the precision form, on FP32 copies of the properties and temperatures.
template <typename F> struct RefOps;
template <> struct RefOps<double> {
    static __device__ __forceinline__ double face(double kc, double kn, double dc, double dn, double cc, double cn,
                                                  double id2)
    {
        return ref_face(kc, kn, dc, dn, cc, cn, id2);
    }
    static __device__ __forceinline__ double axis(double a, double d, double tm, double t, double tp)
    {
        return ref_axis(a, d, tm, t, tp);
    }
};
template <> struct RefOps<float> {
    static __device__ __forceinline__ float face(float kc, float kn, float dc, float dn, float cc, float cn, float id2)
    {
        const float kh = 0.5f * (kc + kn), dh = 0.5f * (dc + dn), ch = 0.5f * (cc + cn);
        return 0.5f * __fdividef(kh, dh * ch) * id2;
    }
    // a (T- - T) + d (T+ - T): the reference's a T- - 2b T + d T+ with b = (a + d)/2
    static __device__ __forceinline__ float axis(float a, float d, float tm, float t, float tp)
    {
        return a * (tm - t) + d * (tp - t);
    }
};

// The reference stencil (src/3dFD.f90:113-187) with every face coefficient
// computed once: a face term is symmetric in its two voxels (IEEE addition
// and multiplication commute), so a voxel's plus face is its neighbour's
// minus face, bit for bit.  Blocks of 32 x 8 columns march REF_ZC planes:
// the x plus face comes from the next lane (shuffle), the y plus face from
// the next row (shared memory), the z plus face becomes the next plane's
// minus face; only the tile's last lane, last row and last plane compute
// theirs.  Three divisions per voxel instead of six.  F = double: the parity
// form; F = float: the FP32 form of reference mode.
constexpr int REF_ZC = 8;
template <typename F> __global__ void __launch_bounds__(256) ref_stencil_kernel(const RefHeatArgs a0)
{
    // the iteration's laserOn from device memory when replayed from a graph
    RefHeatArgs a = a0;
    if (a0.laser_dev) a.laserOn = *a0.laser_dev;
    using O = RefOps<F>;
    __shared__ F s_fy[8][32];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.x * 32 + tx + 1, j = blockIdx.y * 8 + ty + 1;
    const bool in = i <= a.nx && j <= a.ny;
    // lanes past the last interior cell load a halo cell (their faces are the
    // neighbours' plus faces) or, further out, a clamped one that is never used
    const int ic = min(i, a.nx + 1), jc = min(j, a.ny + 1);
    const int k0 = blockIdx.z * REF_ZC + 1, k1 = min(a.nz, k0 + REF_ZC - 1);
    const H I{a.nx + 2, a.ny + 2};
    // the fields the stencil reads: FP64 for the parity form, the FP32
    // copies for the precision form (whose update still adds to the FP64 T)
    const F *K, *D, *C, *tt;
    if constexpr (sizeof(F) == 8) {
        K = a.kappa, D = a.density, C = a.heatcap, tt = a.t0;
    } else {
        K = a.p32, D = a.p32 + a.nh, C = a.p32 + 2 * a.nh, tt = a.s0;
    }
    const F idx2 = (F)a.idx2, idy2 = (F)a.idy2, idz2 = (F)a.idz2;
    int64_t c = I(ic, jc, k0);
    const int64_t sz = (int64_t)(a.nx + 2) * (a.ny + 2), sy = a.nx + 2;
    F kc = K[c], dc = D[c], cc = C[c];
    F fzm = O::face(kc, K[c - sz], dc, D[c - sz], cc, C[c - sz], idz2);
    for (int k = k0; k <= k1; ++k, c += sz) {
        const F kp = K[c + sz], dp = D[c + sz], cp = C[c + sz];
        const F fzp = O::face(kc, kp, dc, dp, cc, cp, idz2);
        const F fym = O::face(kc, K[c - sy], dc, D[c - sy], cc, C[c - sy], idy2);
        const F fxm = O::face(kc, K[c - 1], dc, D[c - 1], cc, C[c - 1], idx2);
        s_fy[ty][tx] = fym;
        F fxp = __shfl_down_sync(0xffffffffu, fxm, 1);
        if (tx == 31 && ic <= a.nx) fxp = O::face(kc, K[c + 1], dc, D[c + 1], cc, C[c + 1], idx2);
        __syncthreads();
        F fyp = 0;
        if (ty < 7) fyp = s_fy[ty + 1][tx];
        else if (jc <= a.ny) fyp = O::face(kc, K[c + sy], dc, D[c + sy], cc, C[c + sy], idy2);
        __syncthreads();  // the row is read before the next plane overwrites it
        if (in) {
            const F t = tt[c];
            const F u_zz = O::axis(fzm, fzp, tt[c - sz], t, tt[c + sz]);
            const F u_yy = O::axis(fym, fyp, tt[c - sy], t, tt[c + sy]);
            const F u_xx = O::axis(fxm, fxp, tt[c - 1], t, tt[c + 1]);
            const int64_t q = (int64_t)(i - 1) + (int64_t)a.nx * ((int64_t)(j - 1) + (int64_t)a.ny * (int64_t)(k - 1));
            if constexpr (sizeof(F) == 8) ref_update(a, c, q, t, cc, u_xx, u_yy, u_zz);
            else ref_update_f32(a, c, q, a.t0[c], cc, u_xx, u_yy, u_zz);
        }
        fzm = fzp;
        kc = kp;
        dc = dp;
        cc = cp;
    }
}

// Arrhenius damage of one voxel: T and rk its temperature and extinction,
// q its interior index.
__device__ __forceinline__ void arrhenius_voxel(const RefArrheniusArgs &a, int64_t q, double T, double rk)
{
    const int64_t ni = (int64_t)a.nx * a.ny * a.nz;
    double om = a.tissue[q];
    // src/3dFD.f90:450-452 with A=3.1d98, dE=6.3d5, R=8.314d0 (compares on
    // the bit patterns, ieee_bits.h)
    if (ieee::ge_pos(T, B_316) && ieee::lt_pos(T, B_373) && ieee::ge_zero(rk)) {
        om = ADD(om, MUL(MUL(a.delt, 3.1e98), exp(-DIV(6.3e5, MUL(8.314, T)))));
        a.tissue[q] = om;
    }
    // src/3dFD.f90:455-461, with the damage tested before each threshold
    // time is loaded (the conditions are pure, so the order of the two tests
    // changes nothing): below 0.53 no threshold time is read at all
    double *t1 = a.thres + q, *t2 = a.thres + q + ni, *t3 = a.thres + q + 2 * ni;
    auto now = [&]() { return a.time_dev ? *a.time_dev : a.time; };  // replayed from a graph: this iteration's clock
    if (ieee::ge_pos(om, B_0_53) && ieee::is_zero(*t1)) *t1 = now();
    else if (ieee::ge_pos(om, B_1) && ieee::is_zero(*t2)) *t2 = now();
    else if (ieee::ge_pos(om, B_1E4) && ieee::is_zero(*t3)) *t3 = now();
}

__global__ void ref_arrhenius_kernel(const RefArrheniusArgs a)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int z = blockIdx.z + 1;
    if (x > a.nx || y > a.ny) return;
    const H I{a.nx + 2, a.ny + 2};
    const int64_t q = (int64_t)(x - 1) + (int64_t)a.nx * ((int64_t)(y - 1) + (int64_t)a.ny * (int64_t)(z - 1));
    const int64_t c = I(x, y, z);
    arrhenius_voxel(a, q, a.temp[c], a.rhokap[c]);
}

// src/thermalConst_mod.f90 with explicit rounding (the reference evaluates
// each product and sum separately).
__device__ __forceinline__ double air_cond(double T)
{
    return ADD(MUL(-0.188521, exp(-MUL(0.000367259, SUB(T, 273.15)))), 0.212453);
}
__device__ __forceinline__ double air_dens(double T) { return DIV(101.325e3, MUL(287.058, T)); }
__device__ __forceinline__ double skin_dens(double w) { return DIV(1000.0, ADD(w, MUL(0.649, 0.25))); }
__device__ __forceinline__ double skin_cap(double w) { return MUL(1000.0, ADD(MUL(4.2, w), MUL(1.09, 0.25))); }
__device__ __forceinline__ double skin_cond(double w, double rho)
{
    return MUL(rho, ADD(MUL(6.28e-4, w), MUL(1.17e-4, 0.25)));
}

// setupThermalCoeff (src/3dFD.f90:312-361) as a parallel map.  The
// reference sweeps k, j, i sequentially and its 6-neighbour test reads the
// already-updated rhokap of the (i-1), (j-1), (k-1) neighbours and the old
// rhokap of the (i+1), (j+1), (k+1) ones.  Because rhokap values are 0 or
// >= mu_protein and only ever go to zero, a backward neighbour is zero after
// its own update iff it was zero or is ablated (it cannot become isolated
// while this voxel is non-zero), so the sweep equals:
//   zero_new(v) = abl(v) | !(rk_old(v) > 0) |
//                 [AND_back (rk_old(b)==0 | abl(b))] & [AND_fwd rk_old(f)==0]
// with ghost neighbours counting as zero.  rhokap is double-buffered.
// FP32 copies of one voxel's new properties, for the FP32 form of the stencil
__device__ __forceinline__ void store_p32(const RefPropsArgs &a, int64_t c, double kk, double dn, double hc, double cf)
{
    a.p32[c] = (float)kk;
    a.p32[a.nh + c] = (float)dn;
    a.p32[2 * a.nh + c] = (float)hc;
    a.p32[3 * a.nh + c] = (float)cf;
}

// The property update of voxel (i, j, k): c its halo index, q its interior
// index, T its temperature.
__device__ __forceinline__ void props_voxel(const RefPropsArgs &a, int i, int j, int k, int64_t c, int64_t q, double T)
{
    const H I{a.nx + 2, a.ny + 2};
    const double abl_T = a.abl_T;
    // WaterContent = getWaterContent(Q, watercontent)  (src/3dFD.f90:328).
    // Compares run on the bit patterns (ieee_bits.h), and a zero Q gives
    // 0.75 - 0.75 * (0 / qvapor) = 0.75 exactly unless qvapor is 0 or NaN,
    // so the FP64 division is skipped for it.
    const double Qv = a.Q[q];
    double wa = 0.75;
    if (!ieee::is_zero(Qv) || ieee::is_zero(a.qvapor) || ieee::is_nan(a.qvapor))
        wa = SUB(0.75, MUL(0.75, DIV(Qv, a.qvapor)));
    double w = ieee::lt_pos(wa, B_0_75) ? wa : 0.75;
    const double wo = a.water[q];
    w = ieee::lt(w, wo) ? w : wo;
    w = ieee::gt_zero(w) ? w : 0.0;
    a.water[q] = w;

    const double *rk = a.rk_old;
    // the loads the common case needs (this voxel's extinction, the -x
    // neighbour's extinction and temperature; all inside the halo) issued
    // together instead of one after another
    const double rkc = rk[c], rkxm = rk[I(i - 1, j, k)], txm = a.temp[I(i - 1, j, k)];
    const bool abl = ieee::le(abl_T, T);
    bool zero = abl || !ieee::gt_zero(rkc);
    if (!zero) {
        // backward neighbours (already swept): zero if zero before or ablated now
        bool iso = true;
        if (i > 1) iso = iso && (ieee::is_zero(rkxm) || ieee::le(abl_T, txm));
        else iso = iso && ieee::is_zero(rkxm);
        if (j > 1) iso = iso && (ieee::is_zero(rk[I(i, j - 1, k)]) || ieee::le(abl_T, a.temp[I(i, j - 1, k)]));
        else iso = iso && ieee::is_zero(rk[I(i, j - 1, k)]);
        if (k > 1) iso = iso && (ieee::is_zero(rk[I(i, j, k - 1)]) || ieee::le(abl_T, a.temp[I(i, j, k - 1)]));
        else iso = iso && ieee::is_zero(rk[I(i, j, k - 1)]);
        // forward neighbours (not yet swept): old values
        iso = iso && ieee::is_zero(rk[I(i + 1, j, k)]) && ieee::is_zero(rk[I(i, j + 1, k)]) &&
              ieee::is_zero(rk[I(i, j, k + 1)]);
        zero = iso;
    }
    if (!zero) {
        if (a.reuse && ieee::eq(w, wo)) {
            // the water content is what the previous call's skin branch saw:
            // its properties are still in place and would come out bit for bit
            // the same, so only the ping-pong copy of rhokap is written
            a.rk_new[c] = rkc;
            return;
        }
        const double dn = skin_dens(w);
        const double hc = skin_cap(w);
        const double kk = skin_cond(w, dn), cf = DIV(a.delt, MUL(dn, hc));
        a.density[c] = dn;
        a.rk_new[c] = ADD(MUL(w, a.mu_water), a.mu_protein);
        a.heatcap[c] = hc;
        a.kappa[c] = kk;
        a.coeff[c] = cf;
        if (a.p32) store_p32(a, c, kk, dn, hc, cf);
    } else {
        if (ieee::lt_zero(T)) atomicOr(a.err, DEVERR_NEG_T);
        const double dn = air_dens(T);
        const double hc = 1.006e3;
        const double kk = air_cond(T);
        a.density[c] = dn;
        a.heatcap[c] = hc;
        a.rk_new[c] = 0.0;
        a.kappa[c] = kk;
        a.alpha[c] = DIV(kk, MUL(dn, hc));
        const double cf = DIV(a.delt, MUL(air_dens(T), hc));
        a.coeff[c] = cf;
        if (a.p32) store_p32(a, c, kk, dn, hc, cf);
    }
}

__global__ void ref_props_kernel(const RefPropsArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > a.nx || j > a.ny) return;
    const H I{a.nx + 2, a.ny + 2};
    const int64_t c = I(i, j, k);
    const int64_t q = (int64_t)(i - 1) + (int64_t)a.nx * ((int64_t)(j - 1) + (int64_t)a.ny * (int64_t)(k - 1));
    props_voxel(a, i, j, k, c, q, a.temp[c]);
}

// Arrhenius then the property update, voxel by voxel: the coupled loop's
// order, one read of T and rhokap for both
__global__ void ref_damage_props_kernel(const RefArrheniusArgs d, const RefPropsArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > a.nx || j > a.ny) return;
    const H I{a.nx + 2, a.ny + 2};
    const int64_t c = I(i, j, k);
    const int64_t q = (int64_t)(i - 1) + (int64_t)a.nx * ((int64_t)(j - 1) + (int64_t)a.ny * (int64_t)(k - 1));
    const double T = a.temp[c];
    arrhenius_voxel(d, q, T, a.rk_old[c]);
    props_voxel(a, i, j, k, c, q, T);
}

// FP32 copies of the temperature (into both ping-pong buffers, halo
// included) and of the four properties the FP32 stencil reads.
__global__ void ref_shadow_kernel(int64_t nh, const double *T, float *ta, float *tb, const double *kappa,
                                  const double *density, const double *heatcap, const double *coeff, float *p32)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nh; c += (int64_t)gridDim.x * blockDim.x) {
        const float t = (float)T[c];
        ta[c] = t;
        tb[c] = t;
        p32[c] = (float)kappa[c];
        p32[nh + c] = (float)density[c];
        p32[2 * nh + c] = (float)heatcap[c];
        p32[3 * nh + c] = (float)coeff[c];
    }
}

__global__ void ref_finalize_kernel(int nx, int ny, int nz, const double *rk, double *tissue)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > nx || j > ny) return;
    const H I{nx + 2, ny + 2};
    if (rk[I(i, j, k)] <= 0.1)
        tissue[(int64_t)(i - 1) + (int64_t)nx * ((int64_t)(j - 1) + (int64_t)ny * (int64_t)(k - 1))] = -1.0;
}

dim3 ref_grid(int nx, int ny, int nz) { return dim3((nx + 31) / 32, (ny + 7) / 8, nz); }

// --------------------------------------------------------- fused path --
// cp.async (LDGSTS) of one 4- or 8-byte element into shared memory.
template <int BYTES> __device__ __forceinline__ void cp_async(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(BYTES));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// One z level of the block's tile in shared memory: FX x FY voxels plus a
// one-cell halo in x and y (the 7-point stencil never reads the corners).
constexpr int NSTAGE = 4;
template <typename Real> struct Plane {
    Real T[FY + 2][FX + 2];
    float e[FY + 2][FX + 2];
    Real k[FY + 2][FX + 2];
    Real r[FY + 2][FX + 2];
    Real h[FY + 2][FX + 2];
    Real J[FY][FX];
};

template <typename Real, bool KAHAN> __device__ __forceinline__ Pt<Real> get(const Plane<Real> &P, int i, int j)
{
    Pt<Real> q;
    q.T = P.T[i][j];
    q.e = KAHAN ? (Real)P.e[i][j] : (Real)0;
    q.k = P.k[i][j];
    q.r = P.r[i][j];
    q.h = P.h[i][j];
    return q;
}

// Issue the asynchronous copies of one voxel's T, Kahan term, k, rho, c.
template <typename Real, bool KAHAN>
__device__ __forceinline__ void stage_cell(Plane<Real> &P, int i, int j, const Real *T, const float *E,
                                           const Real *K, const Real *R, const Real *C, int64_t v)
{
    cp_async<sizeof(Real)>(&P.T[i][j], T + v);
    if (KAHAN) cp_async<4>(&P.e[i][j], E + v);
    cp_async<sizeof(Real)>(&P.k[i][j], K + v);
    cp_async<sizeof(Real)>(&P.r[i][j], R + v);
    cp_async<sizeof(Real)>(&P.h[i][j], C + v);
}

// 2.5-D blocking: a block owns an FX x FY column of the grid for zchunk
// planes.  Planes stream through a ring of NSTAGE shared-memory stages filled
// with cp.async two planes ahead of the one being updated (own voxels, the
// x/y halo staged by the edge threads, and J), so HBM latency overlaps the
// compute of earlier planes; one barrier per plane.  Per voxel the kernel
// reads T, the Kahan term, k, rho, c and J once from HBM and writes T and the
// Kahan term once.  Interior voxels take a branch-free path; faces on the
// grid boundary are handled by ghost_term.
template <typename Real, bool KAHAN>
__global__ void __launch_bounds__(FX *FY, KAHAN ? 4 : 2) fused_kernel(const FusedArgs a, int zchunk)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Plane<Real> *S = reinterpret_cast<Plane<Real> *>(smem_raw);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = blockIdx.x * FX + tx, y = blockIdx.y * FY + ty;
    const bool in = x < a.nx && y < a.ny;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(a.nz, z0 + zchunk);
    const int64_t sy = a.nx, sz = (int64_t)a.nx * a.ny, ni = sz * a.nz;
    const Real *T = (const Real *)a.T_in, *K = (const Real *)a.k, *R = (const Real *)a.rho,
               *C = (const Real *)a.c;
    Real *To = (Real *)a.T_out;
    Real *J = (Real *)a.J, *Q = (Real *)a.Q;
    const float *E = a.Tc_in;
    float *Eo = a.Tc_out;
    const Real cx = cst<Real>(a, FC_CX), cy = cst<Real>(a, FC_CY), cz = cst<Real>(a, FC_CZ);
    const Real dt = cst<Real>(a, FC_DT), Pdt = step_pdt<Real>(a);
    const double t_new = step_tnew(a);
    const bool src_on = Pdt != (Real)0;
    // halo cells this thread stages for every plane
    const bool hL = tx == 0 && x >= 1 && y < a.ny;
    const bool hR = tx == FX - 1 && x + 1 < a.nx && y < a.ny;
    const bool hB = ty == 0 && y >= 1 && x < a.nx;
    const bool hT = ty == FY - 1 && y + 1 < a.ny && x < a.nx;
    const bool xy_inner = x > 0 && x < a.nx - 1 && y > 0 && y < a.ny - 1;
    const int64_t vxy = (int64_t)x + sy * y;

    // copies of plane zz into its stage (no-op outside the grid)
    auto stage = [&](int zz) {
        if (zz >= 0 && zz < a.nz) {
            Plane<Real> &P = S[(zz + NSTAGE) % NSTAGE];
            const int64_t v = vxy + sz * zz;
            if (in) {
                stage_cell<Real, KAHAN>(P, ty + 1, tx + 1, T, E, K, R, C, v);
                if (src_on) cp_async<sizeof(Real)>(&P.J[ty][tx], J + v);
            }
            if (hL) stage_cell<Real, KAHAN>(P, ty + 1, 0, T, E, K, R, C, v - 1);
            if (hR) stage_cell<Real, KAHAN>(P, ty + 1, FX + 1, T, E, K, R, C, v + 1);
            if (hB) stage_cell<Real, KAHAN>(P, 0, tx + 1, T, E, K, R, C, v - sy);
            if (hT) stage_cell<Real, KAHAN>(P, FY + 1, tx + 1, T, E, K, R, C, v + sy);
        }
        cp_async_commit();
    };

    // prologue: planes z0-1, z0, z0+1 in flight
    stage(z0 - 1);
    stage(z0);
    stage(z0 + 1);
    cp_async_wait<1>();  // z0-1 and z0 have landed
    __syncthreads();
    Pt<Real> prv{}, cur{};
    Real am_z = 0;
    if (in) {
        cur = get<Real, KAHAN>(S[(z0 + NSTAGE) % NSTAGE], ty + 1, tx + 1);
        if (z0 > 0) {
            prv = get<Real, KAHAN>(S[(z0 - 1 + NSTAGE) % NSTAGE], ty + 1, tx + 1);
            am_z = falpha(cur, prv);
        }
    }
    unsigned errbits = 0;
    for (int z = z0; z < z1; ++z) {
        const int64_t v = vxy + sz * z;
        const bool has_n = z + 1 < a.nz;
        stage(z + 2);        // two planes ahead
        cp_async_wait<1>();  // plane z+1 has landed (for this thread's copies)
        __syncthreads();     // ... and for every thread's copies
        const Plane<Real> &P = S[z % NSTAGE];
        Pt<Real> nxt{};
        if (in && has_n) nxt = get<Real, KAHAN>(S[(z + 1) % NSTAGE], ty + 1, tx + 1);
        Real ap_z = am_z;
        if (in) {
            const Real Jv = src_on ? P.J[ty][tx] : (Real)0;
            Real lap;
            if (xy_inner && z > 0 && has_n) {
                ap_z = falpha(cur, nxt);
                const Pt<Real> ym = get<Real, KAHAN>(P, ty, tx + 1), yp = get<Real, KAHAN>(P, ty + 2, tx + 1);
                const Pt<Real> xm = get<Real, KAHAN>(P, ty + 1, tx), xp = get<Real, KAHAN>(P, ty + 1, tx + 2);
                lap = cz * (am_z * tdiff(prv, cur) + ap_z * tdiff(nxt, cur)) +
                      cy * (falpha(cur, ym) * tdiff(ym, cur) + falpha(cur, yp) * tdiff(yp, cur)) +
                      cx * (falpha(cur, xm) * tdiff(xm, cur) + falpha(cur, xp) * tdiff(xp, cur));
            } else {
                // a face of this voxel lies on the grid boundary
                lap = (Real)0;
                if (z > 0) lap += cz * am_z * tdiff(prv, cur);
                else lap += ghost_term<Real>(a, 4, cur.T, cur.e, cur.k, cur.r, cur.h);
                if (has_n) {
                    ap_z = falpha(cur, nxt);
                    lap += cz * ap_z * tdiff(nxt, cur);
                } else {
                    lap += ghost_term<Real>(a, 5, cur.T, cur.e, cur.k, cur.r, cur.h);
                }
                if (y > 0) {
                    const Pt<Real> nb = get<Real, KAHAN>(P, ty, tx + 1);
                    lap += cy * falpha(cur, nb) * tdiff(nb, cur);
                } else {
                    lap += ghost_term<Real>(a, 2, cur.T, cur.e, cur.k, cur.r, cur.h);
                }
                if (y < a.ny - 1) {
                    const Pt<Real> nb = get<Real, KAHAN>(P, ty + 2, tx + 1);
                    lap += cy * falpha(cur, nb) * tdiff(nb, cur);
                } else {
                    lap += ghost_term<Real>(a, 3, cur.T, cur.e, cur.k, cur.r, cur.h);
                }
                if (x > 0) {
                    const Pt<Real> nb = get<Real, KAHAN>(P, ty + 1, tx);
                    lap += cx * falpha(cur, nb) * tdiff(nb, cur);
                } else {
                    lap += ghost_term<Real>(a, 0, cur.T, cur.e, cur.k, cur.r, cur.h);
                }
                if (x < a.nx - 1) {
                    const Pt<Real> nb = get<Real, KAHAN>(P, ty + 1, tx + 2);
                    lap += cx * falpha(cur, nb) * tdiff(nb, cur);
                } else {
                    lap += ghost_term<Real>(a, 1, cur.T, cur.e, cur.k, cur.r, cur.h);
                }
            }

            const Real dT = dt * lap;
            const Real rc = cur.r * cur.h;
            const Real sPJ = Pdt * Jv;  // P J dt
            const Real src = src_on ? M<Real>::div(sPJ, rc) : (Real)0;
            Real Tn, En = (Real)0;
            bool clamped = false;
            if (a.boil && cur.T >= cst<Real>(a, FC_TBOIL)) {
                const Real qv = cst<Real>(a, FC_LW) * cur.r * cst<Real>(a, FC_VVOX);
                const Real Qv = Q[v];
                if (Qv < qv) {
                    const Real Ein = (sPJ + rc * dT) * cst<Real>(a, FC_VVOX);
                    if (Ein > (Real)0) {
                        const Real qn = Qv + Ein;
                        Q[v] = qn < qv ? qn : qv;
                        Tn = cst<Real>(a, FC_TBOIL);
                        if (KAHAN) En = cst<Real>(a, FC_TBOIL_E);
                        clamped = true;
                    }
                }
            }
            if (!clamped) {
                const Real inc = dT + src;
                if (KAHAN) {
                    const Real yk = inc - cur.e;
                    const Real t = cur.T + yk;
                    En = (t - cur.T) - yk;
                    Tn = t;
                } else {
                    Tn = cur.T + inc;
                }
            }
            To[v] = Tn;
            if (KAHAN) Eo[v] = (float)En;
            // screen in the storage precision; FP64 only for voxels inside the
            // damage window or at the ablation threshold
            const Real Ts = Tn - En;
            if (!(Ts == Ts)) errbits |= DEVERR_NAN;
            else if (Ts < (Real)0) errbits |= DEVERR_NEG_T;
            if (Ts >= cst<Real>(a, FC_SCREEN)) {
                if constexpr (sizeof(Real) == 4) rare_update_f32(a, v, ni, Tn, (float)En, t_new);
                else rare_update<Real>(a, v, ni, (double)Tn - (double)En, t_new);
            }
        }
        prv = cur;
        cur = nxt;
        am_z = ap_z;
    }
    cp_async_wait<0>();
    if (errbits) atomicOr(a.err, errbits);
}

}  // namespace

void fill_fused_consts(FusedArgs &a)
{
    double *d = a.dc;
    d[FC_CX] = a.opscale / (a.dx * a.dx);
    d[FC_CY] = a.opscale / (a.dy * a.dy);
    d[FC_CZ] = a.opscale / (a.dz * a.dz);
    d[FC_DT] = a.dt;
    d[FC_PDT] = a.P * a.dt;
    d[FC_VVOX] = a.vvox;
    d[FC_TBOIL] = a.T_boil;
    d[FC_LW] = a.lw;
    // screening thresholds a little below the exact ones (|T - true T| <= a few ulp)
    d[FC_TLO_S] = a.T_lo - 0.01;
    d[FC_TABL_S] = a.T_abl - 0.01;
    d[FC_SCREEN] = a.arrhenius ? std::min(d[FC_TLO_S], d[FC_TABL_S]) : d[FC_TABL_S];
    for (int f = 0; f < 6; ++f) {
        d[FC_BCT + f] = a.bc_T[f];
        d[FC_BCHD + f] = a.bc_h[f] * (f < 2 ? a.dx : (f < 4 ? a.dy : a.dz));
        d[FC_BCTA + f] = a.bc_Tamb[f];
    }
    d[FC_LNA_HI] = a.lnA;
    d[FC_LNA_LO] = 0.0;
    d[FC_EAR_HI] = a.Ea / a.Rgas;
    d[FC_EAR_LO] = 0.0;
    d[FC_TLO] = a.T_lo;
    d[FC_THI] = a.T_hi;
    d[FC_TABL] = a.T_abl;
    d[FC_TBOIL_E] = 0.0;  // the FP64 forms clamp to T_boil itself
    for (int i = 0; i < FC_N; ++i) a.fc[i] = (float)d[i];
    a.fc[FC_LNA_LO] = (float)(d[FC_LNA_HI] - (double)a.fc[FC_LNA_HI]);
    a.fc[FC_EAR_LO] = (float)(d[FC_EAR_HI] - (double)a.fc[FC_EAR_HI]);
    a.fc[FC_TLO_LO] = (float)(d[FC_TLO] - (double)a.fc[FC_TLO]);
    a.fc[FC_THI_LO] = (float)(d[FC_THI] - (double)a.fc[FC_THI]);
    a.fc[FC_TABL_LO] = (float)(d[FC_TABL] - (double)a.fc[FC_TABL]);
    a.fc[FC_TBOIL_E] = (float)((double)a.fc[FC_TBOIL] - d[FC_TBOIL]);
}

namespace {

template <typename Real, bool KAHAN>
cudaError_t launch_fused_t(const FusedArgs &a0, cudaStream_t s)
{
    FusedArgs a = a0;
    fill_fused_consts(a);
    const int bx = (a.nx + FX - 1) / FX, by = (a.ny + FY - 1) / FY;
    // enough z-chunks to fill every SM several times over
    int64_t want = 152 * 8;
    int chunks = (int)((want + (int64_t)bx * by - 1) / ((int64_t)bx * by));
    if (chunks < 1) chunks = 1;
    if (chunks > a.nz) chunks = a.nz;
    int zchunk = (a.nz + chunks - 1) / chunks;
    if (zchunk > 16) zchunk = 16;
    if (a.zchunk > 0) zchunk = a.zchunk;
    chunks = (a.nz + zchunk - 1) / zchunk;
    const size_t smem = NSTAGE * sizeof(Plane<Real>);
    // the dynamic shared-memory opt-in is per device; remember it per ordinal
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
        e = cudaFuncSetAttribute(fused_kernel<Real, KAHAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    count_launch();
    fused_kernel<Real, KAHAN><<<dim3(bx, by, chunks), dim3(FX, FY), smem, s>>>(a, zchunk);
    return cudaGetLastError();
}

template <typename Real>
__global__ void to_halo_kernel(const FusedArgs a, double *halo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nx+1
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > a.nx + 1 || j > a.ny + 1) return;
    const H I{a.nx + 2, a.ny + 2};
    const Real *T = (const Real *)a.T_in;
    auto tv = [&](int ii, int jj, int kk) -> double {
        const int64_t q = (int64_t)ii + (int64_t)a.nx * ((int64_t)jj + (int64_t)a.ny * kk);
        double t = (double)T[q];
        if (a.Tc_in) t -= (double)a.Tc_in[q];
        return t;
    };
    const bool ix = i >= 1 && i <= a.nx, iy = j >= 1 && j <= a.ny, iz = k >= 1 && k <= a.nz;
    double val;
    if (ix && iy && iz) {
        val = tv(i - 1, j - 1, k - 1);
    } else {
        // ghost: the face value of the first out-of-range axis (z, then y, then x)
        int f;
        if (!iz) f = k == 0 ? 4 : 5;
        else if (!iy) f = j == 0 ? 2 : 3;
        else f = i == 0 ? 0 : 1;
        if (a.bc_type[f] == BC_ROBIN) {
            const int ci = min(max(i, 1), a.nx) - 1, cj = min(max(j, 1), a.ny) - 1, ck = min(max(k, 1), a.nz) - 1;
            const int64_t q = (int64_t)ci + (int64_t)a.nx * ((int64_t)cj + (int64_t)a.ny * ck);
            const double t0 = tv(ci, cj, ck);
            const double d = f < 2 ? a.dx : (f < 4 ? a.dy : a.dz);
            const double kv = (double)((const Real *)a.k)[q];
            val = t0 - (a.bc_h[f] * d / kv) * (t0 - a.bc_Tamb[f]);
        } else {
            val = a.bc_T[f];
        }
    }
    halo[I(i, j, k)] = val;
}

template <typename Real>
__global__ void from_halo_kernel(const FusedArgs a, const double *halo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= a.nx || j >= a.ny) return;
    const H I{a.nx + 2, a.ny + 2};
    const int64_t q = (int64_t)i + (int64_t)a.nx * ((int64_t)j + (int64_t)a.ny * k);
    ((Real *)a.T_out)[q] = (Real)halo[I(i + 1, j + 1, k + 1)];
    if (a.Tc_out) a.Tc_out[q] = 0.0f;
}

}  // namespace

cudaError_t launch_ref_stencil(const RefHeatArgs &a, cudaStream_t s)
{
    count_launch();
    const dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8, (a.nz + REF_ZC - 1) / REF_ZC);
    if (a.f32) ref_stencil_kernel<float><<<grid, dim3(32, 8), 0, s>>>(a);
    else ref_stencil_kernel<double><<<grid, dim3(32, 8), 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_ref_arrhenius(const RefArrheniusArgs &a, cudaStream_t s)
{
    count_launch();
    ref_arrhenius_kernel<<<ref_grid(a.nx, a.ny, a.nz), dim3(32, 8), 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_ref_props(const RefPropsArgs &a, cudaStream_t s)
{
    count_launch();
    ref_props_kernel<<<ref_grid(a.nx, a.ny, a.nz), dim3(32, 8), 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_ref_damage_props(const RefArrheniusArgs &d, const RefPropsArgs &a, cudaStream_t s)
{
    count_launch();
    ref_damage_props_kernel<<<ref_grid(a.nx, a.ny, a.nz), dim3(32, 8), 0, s>>>(d, a);
    return cudaGetLastError();
}

cudaError_t launch_ref_shadow(int64_t nh, const double *T, float *t32a, float *t32b, const double *kappa,
                              const double *density, const double *heatcap, const double *coeff, float *p32,
                              cudaStream_t s)
{
    if (nh <= 0) return cudaSuccess;
    int64_t b = (nh + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    count_launch();
    ref_shadow_kernel<<<(int)b, 256, 0, s>>>(nh, T, t32a, t32b, kappa, density, heatcap, coeff, p32);
    return cudaGetLastError();
}

cudaError_t launch_ref_finalize(int nx, int ny, int nz, const double *rhokap, double *tissue, cudaStream_t s)
{
    count_launch();
    ref_finalize_kernel<<<ref_grid(nx, ny, nz), dim3(32, 8), 0, s>>>(nx, ny, nz, rhokap, tissue);
    return cudaGetLastError();
}

cudaError_t launch_fused_step(const FusedArgs &a, bool fp64, cudaStream_t s)
{
    return fp64 ? launch_fused_t<double, false>(a, s) : launch_fused_t<float, true>(a, s);
}

cudaError_t launch_fused_to_halo(const FusedArgs &a, bool fp64, double *halo, cudaStream_t s)
{
    const dim3 g((a.nx + 2 + 31) / 32, (a.ny + 2 + 7) / 8, a.nz + 2);
    count_launch();
    if (fp64) to_halo_kernel<double><<<g, dim3(32, 8), 0, s>>>(a, halo);
    else to_halo_kernel<float><<<g, dim3(32, 8), 0, s>>>(a, halo);
    return cudaGetLastError();
}

cudaError_t launch_fused_from_halo(const FusedArgs &a, bool fp64, const double *halo, cudaStream_t s)
{
    const dim3 g((a.nx + 31) / 32, (a.ny + 7) / 8, a.nz);
    count_launch();
    if (fp64) from_halo_kernel<double><<<g, dim3(32, 8), 0, s>>>(a, halo);
    else from_halo_kernel<float><<<g, dim3(32, 8), 0, s>>>(a, halo);
    return cudaGetLastError();
}

}  // namespace tam
