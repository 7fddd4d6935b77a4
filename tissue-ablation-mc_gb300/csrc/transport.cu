// transport.cu -- photon-packet transport on sm_103a.
//
// One packet per thread, persistent warps that refill dead lanes from a
// global packet counter (warp-aggregated).  Each lane walks its packet
// through the voxel grid with a cell-relative DDA, scatters with the
// Henyey-Greenstein rotation of src/stokes.f90:6-153, applies Fresnel faces
// and Russian roulette, and deposits w*d*mua per voxel visit (the path-length
// absorption estimator of src/inttau2.f90:46,53) into the FP64 tally with one
// red.global.add.f64 per visit.
//
// Follows: src/sourceph.f90:7-49 (launch), src/inttau2.f90:7-121 (tau
// integration and wall distance), src/stokes.f90:6-153 (HG), src/ch_opt.f90
// (optical constants via the material table).  Random numbers come from
// Philox4x32-10 with counter {event, packet_lo, packet_hi, stream}.
#include <curand_philox4x32_x.h>

#include "tam_device.cuh"
#include "tam_kernels.h"

namespace tam {

namespace {

constexpr int TPB = 256;

template <typename Real> struct MatR {
    Real mut, mua, alb, g, g2, n;
};

// HG deflection with the arithmetic of src/stokes.f90:6-153 (PI/TWOPI are
// the truncated constants of src/constants.f90:13).  Leaves the direction
// unchanged when the sampled cosine is exactly +-1 (the `goto 100`).
template <typename Real>
__device__ __forceinline__ void stokes(Real hgg, Real g2, Real u0, Real u1, Real &cost, Real &sint, Real &phi,
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
        return;
    }
    const Real costp = cost, sintp = sint, phip = phi;
    const Real t = M<Real>::div(one - g2, one - hgg + (Real)2 * hgg * u0);
    Real bmu = M<Real>::div((one + g2) - t * t, (Real)2 * hgg);
    Real cosb2 = bmu * bmu;
    if (M<Real>::abs(bmu) > one) {
        bmu = bmu > one ? one : -one;
        cosb2 = one;
    }
    if (bmu == one || bmu == -one) return;
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

template <typename Real> __device__ __forceinline__ double warp_sum(Real v)
{
    double d = (double)v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    return d;
}

template <typename Real, int MED>
__device__ __forceinline__ void lookup(const TransportArgs &a, const MatR<Real> *lut, int ix, int iy, int iz,
                                       MatR<Real> &m)
{
    if (MED == MED_RHOKAP) {
        const int64_t hx = a.nx + 2, hy = a.ny + 2;
        const Real v = (Real)__ldg(a.rhokap + ((ix + 1) + hx * ((iy + 1) + hy * (int64_t)(iz + 1))));
        m.mut = v;
        m.mua = v;
        m.alb = (Real)0;
        m.g = (Real)0;
        m.g2 = (Real)0;
        m.n = (Real)a.rhokap_n;
    } else {
        int id = __ldg(a.mat + (ix + (int64_t)a.nx * (iy + (int64_t)a.ny * iz)));
        if (id >= a.nmat) id = 0;
        m = lut[id];
    }
}

template <typename Real, int MED> __global__ void __launch_bounds__(TPB) transport_kernel(const TransportArgs a)
{
    __shared__ MatR<Real> lut[MAX_MAT];
    if (MED == MED_MATERIAL) {
        for (int t = threadIdx.x; t < MAX_MAT; t += blockDim.x) {
            const OptMat &o = a.lut[t < a.nmat ? t : 0];
            MatR<Real> m;
            m.mut = (Real)(o.mua + o.mus);
            m.mua = (Real)o.mua;
            m.alb = (o.mua + o.mus) > 0.0 ? (Real)(o.mus / (o.mua + o.mus)) : (Real)0;
            m.g = (Real)o.g;
            m.g2 = (Real)(o.g * o.g);
            m.n = (Real)o.n;
            lut[t] = m;
        }
    }
    __syncthreads();

    const Real hx = (Real)(2.0 * a.xmax / a.nx), hy = (Real)(2.0 * a.ymax / a.ny), hz = (Real)(2.0 * a.zmax / a.nz);
    const Real BIG = (Real)1.0e30;
    const Real TWOPI = (Real)TWOPI_R;
    const Real nudge = (Real)a.nudge;
    const uint32_t k0 = (uint32_t)a.seed, k1 = (uint32_t)(a.seed >> 32);
    const unsigned lane = threadIdx.x & 31u;
    const Real wmin = (Real)a.roulette_w, rm = (Real)a.roulette_m, inv_rm = (Real)(1.0 / a.roulette_m);

    // packet state
    bool alive = false, exhausted = false;
    int ix = 0, iy = 0, iz = 0;
    Real fx = 0, fy = 0, fz = 0;
    Real cost = 0, sint = 0, phi = 0, cosp = 0, sinp = 0;
    Real nx = 0, ny = 0, nz = 0, inx = 0, iny = 0, inz = 0;
    Real w = 0, tau = 0, dep = 0;
    uint32_t ev = 0, plo = 0, phi32 = 0;
    int64_t nsteps = 0;
    MatR<Real> m;
    m.mut = m.mua = m.alb = m.g = m.g2 = m.n = (Real)0;
    // per-thread tallies
    Real tSpec = 0, tRefl = 0, tTran = 0, tSide = 0, tRN = 0, tMiss = 0;
    unsigned long long cSteps = 0, cScat = 0, cOvf = 0;
    unsigned errbits = 0;

    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !alive && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(a.work, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!alive && !exhausted) {
                const unsigned long long my = base + __popc(need & ((1u << lane) - 1u));
                if (my >= (unsigned long long)a.n) {
                    exhausted = true;
                } else {
                    // ---- launch (src/sourceph.f90:7-49 / Gaussian beam) ----
                    const uint64_t pid = (uint64_t)a.p0 + my;
                    plo = (uint32_t)pid;
                    phi32 = (uint32_t)(pid >> 32);
                    const U4 r = philox4x32_10(0u, plo, phi32, a.stream, k0, k1);
                    ev = 1;
                    const Real u0 = Uniform<Real>::from(r.x), u1 = Uniform<Real>::from(r.y);
                    const Real u2 = Uniform<Real>::from(r.z), u3 = Uniform<Real>::from(r.w);
                    const Real R = (Real)a.source_radius;
                    const Real rad = a.source == SRC_DISK ? M<Real>::sqrt(u0 * (R * R))
                                                          : R * M<Real>::sqrt((Real)-0.5 * M<Real>::log(u0));
                    Real st, ct;
                    M<Real>::sincos(u1 * TWOPI, &st, &ct);
                    const Real X = rad * ct + (Real)a.xmax, Y = rad * st + (Real)a.ymax;
                    phi = TWOPI * u2;
                    M<Real>::sincos(phi, &sinp, &cosp);
                    cost = (Real)-1;
                    sint = (Real)0;
                    if (!(X >= (Real)0 && X < (Real)(2.0 * a.xmax) && Y >= (Real)0 && Y < (Real)(2.0 * a.ymax))) {
                        tMiss += (Real)1;
                    } else {
                        ix = (int)((Real)a.nx * X / (Real)(2.0 * a.xmax));
                        iy = (int)((Real)a.ny * Y / (Real)(2.0 * a.ymax));
                        ix = ix > a.nx - 1 ? a.nx - 1 : ix;
                        iy = iy > a.ny - 1 ? a.ny - 1 : iy;
                        iz = a.nz - 1;
                        fx = X - (Real)ix * hx;
                        fy = Y - (Real)iy * hy;
                        fz = hz - (Real)1.e-8 * hz;
                        lookup<Real, MED>(a, lut, ix, iy, iz, m);
                        w = (Real)1;
                        if (a.fresnel) {
                            Real rsp = ((Real)a.n_ambient - m.n) / ((Real)a.n_ambient + m.n);
                            rsp = rsp * rsp;
                            tSpec += rsp;
                            w = (Real)1 - rsp;
                        }
                        tau = -M<Real>::log(u3);
                        nx = sint * cosp;
                        ny = sint * sinp;
                        nz = cost;
                        inx = (Real)1 / nx;
                        iny = (Real)1 / ny;
                        inz = (Real)1 / nz;
                        dep = (Real)0;
                        nsteps = 0;
                        alive = true;
                    }
                }
            }
        }
        if (__all_sync(0xffffffffu, exhausted && !alive)) break;
        if (!alive) continue;

        // ---- flight: cross voxels until the interaction point (src/inttau2.f90:37-63) ----
        bool interact = false;
        for (;;) {
            if (++nsteps > a.max_steps) {
                cOvf += 1;
                errbits |= DEVERR_STEP_CAP;
                alive = false;
                break;
            }
            Real ddx = nx > (Real)0 ? (hx - fx) * inx : (nx < (Real)0 ? -fx * inx : BIG);
            Real ddy = ny > (Real)0 ? (hy - fy) * iny : (ny < (Real)0 ? -fy * iny : BIG);
            Real ddz = nz > (Real)0 ? (hz - fz) * inz : (nz < (Real)0 ? -fz * inz : BIG);
            ddx = ddx < (Real)0 ? (Real)0 : ddx;
            ddy = ddy < (Real)0 ? (Real)0 : ddy;
            ddz = ddz < (Real)0 ? (Real)0 : ddz;
            // tie order of src/inttau2.f90:116-118 (z over y over x)
            int ax = 2;
            Real dw = ddz;
            if (ddy < dw) { dw = ddy; ax = 1; }
            if (ddx < dw) { dw = ddx; ax = 0; }
            const Real taucell = dw * m.mut;
            if (taucell < tau) {
                dep += w * dw * m.mua;
                tau -= taucell;
                int nxt;
                Real nc;
                if (ax == 0) {
                    fy = clamp0h(fy + ny * dw, hy);
                    fz = clamp0h(fz + nz * dw, hz);
                    nc = nx;
                    nxt = nx > (Real)0 ? ix + 1 : ix - 1;
                } else if (ax == 1) {
                    fx = clamp0h(fx + nx * dw, hx);
                    fz = clamp0h(fz + nz * dw, hz);
                    nc = ny;
                    nxt = ny > (Real)0 ? iy + 1 : iy - 1;
                } else {
                    fx = clamp0h(fx + nx * dw, hx);
                    fy = clamp0h(fy + ny * dw, hy);
                    nc = nz;
                    nxt = nz > (Real)0 ? iz + 1 : iz - 1;
                }
                const int nax = ax == 0 ? a.nx : (ax == 1 ? a.ny : a.nz);
                // flush the visit's deposit before leaving the cell
                if (dep != (Real)0) {
                    atomicAdd(a.jmean + (ix + (int64_t)a.nx * (iy + (int64_t)a.ny * iz)), (double)dep);
                    dep = (Real)0;
                }
                if (nxt < 0 || nxt >= nax) {
                    const Real hn = ax == 0 ? hx : (ax == 1 ? hy : hz);
                    const Real face = nc > (Real)0 ? hn : (Real)0;
                    if (ax == 0) fx = face;
                    else if (ax == 1) fy = face;
                    else fz = face;
                    if (a.fresnel) {
                        const U4 r = philox4x32_10(ev++, plo, phi32, a.stream, k0, k1);
                        const Real R = fresnel<Real>(m.n, (Real)a.n_ambient, M<Real>::abs(nc));
                        if (Uniform<Real>::from(r.x) < R) {
                            if (ax == 2) {
                                cost = -cost;
                            } else if (ax == 0) {
                                cosp = -cosp;
                                phi = (Real)PI_R - phi;
                                if (phi < (Real)0) phi += TWOPI;
                            } else {
                                sinp = -sinp;
                                phi = TWOPI - phi;
                            }
                            nx = sint * cosp;
                            ny = sint * sinp;
                            nz = cost;
                            inx = (Real)1 / nx;
                            iny = (Real)1 / ny;
                            inz = (Real)1 / nz;
                            continue;
                        }
                    }
                    if (ax == 2) {
                        if (nc > (Real)0) tRefl += w;
                        else tTran += w;
                    } else {
                        tSide += w;
                    }
                    alive = false;
                    break;
                }
                // the reference snaps a crossed coordinate to the face +- delta
                // (src/inttau2.f90:140-169); nudge carries that delta
                if (ax == 0) { ix = nxt; fx = nx > (Real)0 ? nudge : hx - nudge; }
                else if (ax == 1) { iy = nxt; fy = ny > (Real)0 ? nudge : hy - nudge; }
                else { iz = nxt; fz = nz > (Real)0 ? nudge : hz - nudge; }
                lookup<Real, MED>(a, lut, ix, iy, iz, m);
            } else {
                const Real dd = M<Real>::div(tau, m.mut);
                dep += w * dd * m.mua;
                fx = clamp0h(fx + nx * dd, hx);
                fy = clamp0h(fy + ny * dd, hy);
                fz = clamp0h(fz + nz * dd, hz);
                interact = true;
                break;
            }
        }
        if (!alive) {
            if (dep != (Real)0) {
                atomicAdd(a.jmean + (ix + (int64_t)a.nx * (iy + (int64_t)a.ny * iz)), (double)dep);
                dep = (Real)0;
            }
            cSteps += (unsigned long long)nsteps;
            continue;
        }
        if (interact) {
            // ---- interaction: implicit capture, HG scatter, roulette ----
            w *= m.alb;
            bool die = !(w > (Real)0);
            if (!die) {
                cScat += 1;
                const U4 r = philox4x32_10(ev++, plo, phi32, a.stream, k0, k1);
                stokes<Real>(m.g, m.g2, Uniform<Real>::from(r.x), Uniform<Real>::from(r.y), cost, sint, phi, cosp,
                             sinp);
                nx = sint * cosp;
                ny = sint * sinp;
                nz = cost;
                if (!(nz == nz) || !(nx == nx) || !(ny == ny)) {
                    errbits |= DEVERR_NAN;
                    die = true;
                } else {
                    inx = (Real)1 / nx;
                    iny = (Real)1 / ny;
                    inz = (Real)1 / nz;
                    if (a.roulette && w < wmin) {
                        if (Uniform<Real>::from(r.z) < inv_rm) {
                            tRN += w * (rm - (Real)1);
                            w *= rm;
                        } else {
                            tRN -= w;
                            die = true;
                        }
                    }
                    tau = -M<Real>::log(Uniform<Real>::from(r.w));
                }
            }
            if (die) {
                if (dep != (Real)0) {
                    atomicAdd(a.jmean + (ix + (int64_t)a.nx * (iy + (int64_t)a.ny * iz)), (double)dep);
                    dep = (Real)0;
                }
                cSteps += (unsigned long long)nsteps;
                alive = false;
            }
        }
    }

    // ---- block reduction of the escape tallies ----
    double v[7] = {warp_sum(tSpec), warp_sum(tRefl), warp_sum(tTran), warp_sum(tSide),
                   warp_sum(tRN), warp_sum(tMiss), 0.0};
    unsigned long long c3[3] = {cSteps, cScat, cOvf};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c3[i] += __shfl_xor_sync(0xffffffffu, c3[i], o);
    errbits = __reduce_or_sync(0xffffffffu, errbits);
    if (lane == 0) {
        atomicAdd(a.tally + T_SPECULAR, v[0]);
        atomicAdd(a.tally + T_REFLECTED, v[1]);
        atomicAdd(a.tally + T_TRANSMITTED, v[2]);
        atomicAdd(a.tally + T_SIDE, v[3]);
        atomicAdd(a.tally + T_ROULETTE_NET, v[4]);
        atomicAdd(a.tally + T_MISSED, v[5]);
        atomicAdd(a.tally + T_STEPS, (double)c3[0]);
        atomicAdd(a.tally + T_SCATTERS, (double)c3[1]);
        atomicAdd(a.tally + T_OVERFLOW, (double)c3[2]);
        if (errbits) atomicOr(a.err, errbits);
    }
}

__global__ void scale_f64_kernel(double *out, double *in, double f, int64_t n, int zero_in)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        out[q] = in[q] * f;
        if (zero_in) in[q] = 0.0;
    }
}

__global__ void scale_f32_kernel(float *out, double *in, double f, int64_t n, int zero_in)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        out[q] = (float)(in[q] * f);
        if (zero_in) in[q] = 0.0;
    }
}

__global__ void philox_selftest_kernel(const uint32_t *in, uint32_t *mine, uint32_t *ref, int64_t n)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t *p = in + 6 * q;
        const U4 r = philox4x32_10(p[0], p[1], p[2], p[3], p[4], p[5]);
        mine[4 * q + 0] = r.x;
        mine[4 * q + 1] = r.y;
        mine[4 * q + 2] = r.z;
        mine[4 * q + 3] = r.w;
        const uint4 c = make_uint4(p[0], p[1], p[2], p[3]);
        const uint2 k = make_uint2(p[4], p[5]);
        const uint4 o = curand_Philox4x32_10(c, k);
        ref[4 * q + 0] = o.x;
        ref[4 * q + 1] = o.y;
        ref[4 * q + 2] = o.z;
        ref[4 * q + 3] = o.w;
    }
}

int grid_for(int64_t n, int tpb)
{
    int64_t b = (n + tpb - 1) / tpb;
    if (b > 152 * 32) b = 152 * 32;
    return (int)(b > 0 ? b : 1);
}

template <typename Real, int MED> cudaError_t launch_t(const TransportArgs &a, int sm_count, cudaStream_t s)
{
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_kernel<Real, MED>, TPB, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = (int64_t)sm_count * per_sm;
    const int64_t need = (a.n + TPB - 1) / TPB;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    count_launch();
    transport_kernel<Real, MED><<<(unsigned)blocks, TPB, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_transport(const TransportArgs &a, bool fp64, int sm_count, cudaStream_t s)
{
    if (a.n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if (fp64) {
        return a.medium == MED_RHOKAP ? launch_t<double, MED_RHOKAP>(a, sm_count, s)
                                      : launch_t<double, MED_MATERIAL>(a, sm_count, s);
    }
    return a.medium == MED_RHOKAP ? launch_t<float, MED_RHOKAP>(a, sm_count, s)
                                  : launch_t<float, MED_MATERIAL>(a, sm_count, s);
}

cudaError_t launch_scale_f64(double *out, double *in, double f, int64_t n, bool zero_in, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    scale_f64_kernel<<<grid_for(n, 256), 256, 0, s>>>(out, in, f, n, zero_in ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_scale_to_f32(float *out, double *in, double f, int64_t n, bool zero_in, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    scale_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(out, in, f, n, zero_in ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_philox_selftest(const uint32_t *in, uint32_t *mine, uint32_t *ref, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    philox_selftest_kernel<<<grid_for(n, 256), 256, 0, s>>>(in, mine, ref, n);
    return cudaGetLastError();
}

}  // namespace tam
