// heat.cu -- explicit heat diffusion, Arrhenius damage and ablation on sm_103a.
//
// Two families of kernels:
//  * reference path (FP64, reference array layout with halos): the stencil of
//    src/3dFD.f90:113-187, Arrhenius of src/3dFD.f90:424-466 and the property
//    / ablation update of src/3dFD.f90:312-361, each evaluated with explicit
//    round-to-nearest operations in the reference's order of evaluation so
//    the result matches the Fortran arithmetic (no FMA contraction);
//  * fused config-mode step: stencil + latent-heat clamp + Arrhenius (FP64
//    exponent ln A - Ea/RT) + ablation in one pass, with FP32 storage and a
//    Kahan-compensated temperature, or plain FP64.  Each thread marches a
//    (x, y) column through a z-chunk keeping the z-neighbours in registers.
#include <cstdio>

#include "tam_device.cuh"
#include "tam_kernels.h"

namespace tam {

namespace {

// ------------------------------------------------------- reference path --
struct H {
    int64_t hx, hy;
    __device__ __forceinline__ int64_t operator()(int i, int j, int k) const
    {
        return (int64_t)i + hx * ((int64_t)j + hy * (int64_t)k);
    }
};

// Face term of src/3dFD.f90:119-132: a = 0.5*(kM/(dM*cM))*(1/d^2).
__device__ __forceinline__ double ref_face(double kc, double kn, double dc, double dn, double cc, double cn,
                                           double id2)
{
    const double kh = MUL(0.5, ADD(kc, kn));
    const double dh = MUL(0.5, ADD(dc, dn));
    const double ch = MUL(0.5, ADD(cc, cn));
    return MUL(MUL(0.5, DIV(kh, MUL(dh, ch))), id2);
}

// u = a*T- - 2b*T + d*T+ with b = 0.5(a+d)   (src/3dFD.f90:130-132)
__device__ __forceinline__ double ref_axis(double a, double d, double tm, double t, double tp)
{
    const double b = MUL(0.5, ADD(a, d));
    return ADD(SUB(MUL(a, tm), MUL(MUL(2.0, b), t)), MUL(d, tp));
}

__global__ void ref_stencil_kernel(const RefHeatArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > a.nx || j > a.ny) return;
    const H I{a.nx + 2, a.ny + 2};
    const int64_t c = I(i, j, k);
    const double *K = a.kappa, *D = a.density, *C = a.heatcap, *t0 = a.t0;
    const double kc = K[c], dc = D[c], cc = C[c], T = t0[c];

    int64_t m = I(i, j, k - 1), p = I(i, j, k + 1);
    double am = ref_face(kc, K[m], dc, D[m], cc, C[m], a.idz2);
    double ap = ref_face(kc, K[p], dc, D[p], cc, C[p], a.idz2);
    const double u_zz = ref_axis(am, ap, t0[m], T, t0[p]);
    m = I(i, j - 1, k);
    p = I(i, j + 1, k);
    am = ref_face(kc, K[m], dc, D[m], cc, C[m], a.idy2);
    ap = ref_face(kc, K[p], dc, D[p], cc, C[p], a.idy2);
    const double u_yy = ref_axis(am, ap, t0[m], T, t0[p]);
    m = I(i - 1, j, k);
    p = I(i + 1, j, k);
    am = ref_face(kc, K[m], dc, D[m], cc, C[m], a.idx2);
    ap = ref_face(kc, K[p], dc, D[p], cc, C[p], a.idx2);
    const double u_xx = ref_axis(am, ap, t0[m], T, t0[p]);

    // source and latent-heat clamp (src/3dFD.f90:166-183)
    const int64_t q = (int64_t)(i - 1) + (int64_t)a.nx * ((int64_t)(j - 1) + (int64_t)a.ny * (int64_t)(k - 1));
    const double J = a.J[q];
    const double tempIncrease = MUL(a.delt, ADD(ADD(u_xx, u_yy), u_zz));
    const double energyIncrease =
        ADD(MUL(MUL(MUL(a.laserOn, J), a.delt), a.vvox), MUL(MUL(cc, a.mvox), tempIncrease));
    const double heat = ADD(ADD(T, tempIncrease), MUL(MUL(a.laserOn, a.coeff[c]), J));
    double tn;
    const double Qv = a.Q[q];
    if (T >= 373.0 && Qv < a.qvapor) {
        if (energyIncrease > 0.0) {
            const double qn = ADD(Qv, energyIncrease);
            a.Q[q] = qn < a.qvapor ? qn : a.qvapor;
            tn = 373.0;
        } else {
            tn = heat;
        }
    } else {
        tn = heat;
        if (T < 0.0) atomicOr(a.err, DEVERR_NEG_T);
    }
    if (tn != tn) atomicOr(a.err, DEVERR_NAN);
    a.tn[c] = tn;
}

__global__ void ref_arrhenius_kernel(const RefArrheniusArgs a)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int z = blockIdx.z + 1;
    if (x > a.nx || y > a.ny) return;
    const H I{a.nx + 2, a.ny + 2};
    const int64_t ni = (int64_t)a.nx * a.ny * a.nz;
    const int64_t q = (int64_t)(x - 1) + (int64_t)a.nx * ((int64_t)(y - 1) + (int64_t)a.ny * (int64_t)(z - 1));
    const double T = a.temp[I(x, y, z)];
    double om = a.tissue[q];
    // src/3dFD.f90:450-452 with A=3.1d98, dE=6.3d5, R=8.314d0
    if (T >= 316.0 && T < 373.0 && a.rhokap[I(x, y, z)] >= 0.0) {
        om = ADD(om, MUL(MUL(a.delt, 3.1e98), exp(-DIV(6.3e5, MUL(8.314, T)))));
        a.tissue[q] = om;
    }
    // src/3dFD.f90:455-461
    double *t1 = a.thres + q, *t2 = a.thres + q + ni, *t3 = a.thres + q + 2 * ni;
    if (*t1 == 0.0 && om >= 0.53) *t1 = a.time;
    else if (*t2 == 0.0 && om >= 1.0) *t2 = a.time;
    else if (*t3 == 0.0 && om >= 10000.0) *t3 = a.time;
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
__global__ void ref_props_kernel(const RefPropsArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > a.nx || j > a.ny) return;
    const H I{a.nx + 2, a.ny + 2};
    const int64_t c = I(i, j, k);
    const int64_t q = (int64_t)(i - 1) + (int64_t)a.nx * ((int64_t)(j - 1) + (int64_t)a.ny * (int64_t)(k - 1));
    const double abl_T = ADD(a.ablate_temp, 273.0);
    const double T = a.temp[c];
    // WaterContent = getWaterContent(Q, watercontent)  (src/3dFD.f90:328)
    const double wa = SUB(0.75, MUL(0.75, DIV(a.Q[q], a.qvapor)));
    double w = wa < 0.75 ? wa : 0.75;
    const double wo = a.water[q];
    w = w < wo ? w : wo;
    w = w > 0.0 ? w : 0.0;
    a.water[q] = w;

    const double *rk = a.rk_old;
    const bool abl = T >= abl_T;
    bool zero = abl || !(rk[c] > 0.0);
    if (!zero) {
        // backward neighbours (already swept): zero if zero before or ablated now
        bool iso = true;
        if (i > 1) iso = iso && (rk[I(i - 1, j, k)] == 0.0 || a.temp[I(i - 1, j, k)] >= abl_T);
        else iso = iso && (rk[I(i - 1, j, k)] == 0.0);
        if (j > 1) iso = iso && (rk[I(i, j - 1, k)] == 0.0 || a.temp[I(i, j - 1, k)] >= abl_T);
        else iso = iso && (rk[I(i, j - 1, k)] == 0.0);
        if (k > 1) iso = iso && (rk[I(i, j, k - 1)] == 0.0 || a.temp[I(i, j, k - 1)] >= abl_T);
        else iso = iso && (rk[I(i, j, k - 1)] == 0.0);
        // forward neighbours (not yet swept): old values
        iso = iso && rk[I(i + 1, j, k)] == 0.0 && rk[I(i, j + 1, k)] == 0.0 && rk[I(i, j, k + 1)] == 0.0;
        zero = iso;
    }
    if (!zero) {
        const double dn = skin_dens(w);
        const double hc = skin_cap(w);
        a.density[c] = dn;
        a.rk_new[c] = ADD(MUL(w, a.mu_water), a.mu_protein);
        a.heatcap[c] = hc;
        a.kappa[c] = skin_cond(w, dn);
        a.coeff[c] = DIV(a.delt, MUL(dn, hc));
    } else {
        if (T < 0.0) atomicOr(a.err, DEVERR_NEG_T);
        const double dn = air_dens(T);
        const double hc = 1.006e3;
        const double kk = air_cond(T);
        a.density[c] = dn;
        a.heatcap[c] = hc;
        a.rk_new[c] = 0.0;
        a.kappa[c] = kk;
        a.alpha[c] = DIV(kk, MUL(dn, hc));
        a.coeff[c] = DIV(a.delt, MUL(air_dens(T), hc));
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
constexpr int FX = 32, FY = 8;

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

// (ghost - true centre) for a boundary face
template <typename Real>
__device__ __forceinline__ Real gdiff(const FusedArgs &a, int f, Real d, const Pt<Real> &c)
{
    if (a.bc_type[f] == BC_ROBIN) {
        const Real beta = (Real)a.bc_h[f] * d / c.k;
        return -beta * ((c.T - (Real)a.bc_Tamb[f]) - c.e);
    }
    return ((Real)a.bc_T[f] - c.T) + c.e;
}

template <typename Real, bool KAHAN>
__global__ void __launch_bounds__(FX *FY) fused_kernel(const FusedArgs a, int zchunk)
{
    const int x = blockIdx.x * FX + threadIdx.x, y = blockIdx.y * FY + threadIdx.y;
    if (x >= a.nx || y >= a.ny) return;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(a.nz, z0 + zchunk);
    if (z0 >= z1) return;
    const int64_t sy = a.nx, sz = (int64_t)a.nx * a.ny, ni = sz * a.nz;
    const Real *T = (const Real *)a.T_in, *K = (const Real *)a.k, *R = (const Real *)a.rho,
               *C = (const Real *)a.c;
    Real *To = (Real *)a.T_out;
    Real *J = (Real *)a.J, *Q = (Real *)a.Q;
    const float *E = a.Tc_in;
    float *Eo = a.Tc_out;
    const Real dx = (Real)a.dx, dy = (Real)a.dy, dz = (Real)a.dz;
    const Real cx = (Real)(a.opscale / (a.dx * a.dx)), cy = (Real)(a.opscale / (a.dy * a.dy)),
               cz = (Real)(a.opscale / (a.dz * a.dz));
    const Real dt = (Real)a.dt, P = (Real)a.P, vvox = (Real)a.vvox;
    const Real Tboil = (Real)a.T_boil, lw = (Real)a.lw;

    int64_t v = x + sy * y + sz * z0;
    Pt<Real> cur = ld<Real, KAHAN>(T, E, K, R, C, v);
    Pt<Real> prv;
    if (z0 > 0) prv = ld<Real, KAHAN>(T, E, K, R, C, v - sz);
    Real am_z = z0 > 0 ? falpha(cur, prv) : M<Real>::div(cur.k, cur.r * cur.h);
    unsigned errbits = 0;
    for (int z = z0; z < z1; ++z, v += sz) {
        Pt<Real> nxt;
        const bool has_n = z + 1 < a.nz;
        if (has_n) nxt = ld<Real, KAHAN>(T, E, K, R, C, v + sz);
        const Real aself = M<Real>::div(cur.k, cur.r * cur.h);
        // z axis
        const Real dzm = z > 0 ? tdiff(prv, cur) : gdiff<Real>(a, 4, dz, cur);
        const Real ap_z = has_n ? falpha(cur, nxt) : aself;
        const Real dzp = has_n ? tdiff(nxt, cur) : gdiff<Real>(a, 5, dz, cur);
        Real lap = cz * (am_z * dzm + ap_z * dzp);
        // y axis
        if (y > 0) {
            const Pt<Real> nb = ld<Real, KAHAN>(T, E, K, R, C, v - sy);
            lap += cy * falpha(cur, nb) * tdiff(nb, cur);
        } else {
            lap += cy * aself * gdiff<Real>(a, 2, dy, cur);
        }
        if (y < a.ny - 1) {
            const Pt<Real> nb = ld<Real, KAHAN>(T, E, K, R, C, v + sy);
            lap += cy * falpha(cur, nb) * tdiff(nb, cur);
        } else {
            lap += cy * aself * gdiff<Real>(a, 3, dy, cur);
        }
        // x axis
        if (x > 0) {
            const Pt<Real> nb = ld<Real, KAHAN>(T, E, K, R, C, v - 1);
            lap += cx * falpha(cur, nb) * tdiff(nb, cur);
        } else {
            lap += cx * aself * gdiff<Real>(a, 0, dx, cur);
        }
        if (x < a.nx - 1) {
            const Pt<Real> nb = ld<Real, KAHAN>(T, E, K, R, C, v + 1);
            lap += cx * falpha(cur, nb) * tdiff(nb, cur);
        } else {
            lap += cx * aself * gdiff<Real>(a, 1, dx, cur);
        }

        const Real dT = dt * lap;
        const Real Jv = P != (Real)0 ? J[v] : (Real)0;
        const Real rc = cur.r * cur.h;
        const Real src = M<Real>::div(P * Jv * dt, rc);
        Real Tn, En = (Real)0;
        bool clamped = false;
        if (a.boil && cur.T >= Tboil) {
            const Real qv = lw * cur.r * vvox;
            const Real Qv = Q[v];
            if (Qv < qv) {
                const Real Ein = (P * Jv * dt + rc * dT) * vvox;
                if (Ein > (Real)0) {
                    const Real qn = Qv + Ein;
                    Q[v] = qn < qv ? qn : qv;
                    Tn = Tboil;
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
        const double Tt = (double)Tn - (double)En;
        if (!(Tt == Tt)) errbits |= DEVERR_NAN;
        else if (Tt < 0.0) errbits |= DEVERR_NEG_T;
        if (a.arrhenius && Tt >= a.T_lo && Tt < a.T_hi) {
            const double o = a.omega[v];
            const double on = o + a.dt * exp(a.lnA - a.Ea / (a.Rgas * Tt));
            a.omega[v] = on;
#pragma unroll
            for (int t = 0; t < 3; ++t)
                if (o < a.thr[t] && on >= a.thr[t]) a.thres[v + t * ni] = a.t_new;
        }
        if (Tt >= a.T_abl && a.mat[v] != 0) {
            a.mat[v] = 0;  // optics -> air
            J[v] = (Real)0;
            atomicAdd(a.n_ablated, 1ull);
        }
        prv = cur;
        am_z = ap_z;
        if (has_n) cur = nxt;
    }
    if (errbits) atomicOr(a.err, errbits);
}

template <typename Real, bool KAHAN>
cudaError_t launch_fused_t(const FusedArgs &a, cudaStream_t s)
{
    const int bx = (a.nx + FX - 1) / FX, by = (a.ny + FY - 1) / FY;
    // enough z-chunks to fill every SM several times over
    int64_t want = 152 * 8;
    int chunks = (int)((want + (int64_t)bx * by - 1) / ((int64_t)bx * by));
    if (chunks < 1) chunks = 1;
    if (chunks > a.nz) chunks = a.nz;
    const int zchunk = (a.nz + chunks - 1) / chunks;
    chunks = (a.nz + zchunk - 1) / zchunk;
    count_launch();
    fused_kernel<Real, KAHAN><<<dim3(bx, by, chunks), dim3(FX, FY), 0, s>>>(a, zchunk);
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
    ref_stencil_kernel<<<ref_grid(a.nx, a.ny, a.nz), dim3(32, 8), 0, s>>>(a);
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
