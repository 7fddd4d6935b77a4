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

#include <algorithm>

#include "tam_device.cuh"
#include "tam_kernels.h"
#include "transport_common.cuh"

namespace tam {

namespace {

constexpr int TPB = 256;
// Resident blocks per SM requested for the FP32 transport kernel (register cap).
#ifndef TAM_TR_MINB
#define TAM_TR_MINB 4
#endif

// Tally update of one voxel visit: an FP64 reduction into jmean (L2-resident
// for grids up to ~16 M voxels), or -- for grids whose FP64 tally is far
// larger than L2 -- an FP32 reduction into a box-sized tally around the
// beam's entry, which stays L2-resident and which the host flushes into
// jmean every few million packets; the rare deposits outside the box go to
// jmean directly.
template <bool T32, typename Real>
__device__ __forceinline__ void deposit(const TransportArgs &a, int cidx, int ix, int iy, int iz, Real dep)
{
    if constexpr (T32) {
        const unsigned bx = (unsigned)(ix - a.bx0), by = (unsigned)(iy - a.by0), bz = (unsigned)(iz - a.bz0);
        if (bx < (unsigned)a.bnx && by < (unsigned)a.bny && bz < (unsigned)a.bnz) {
            atomicAdd(a.jmean32 + (bx + (unsigned)a.bnx * (by + (unsigned)a.bny * bz)), (float)dep);
            return;
        }
    }
    atomicAdd(a.jmean + cidx, (double)dep);
}

// Optical properties of the current cell: extinction and absorption for the
// DDA, the material id for the albedo / HG / index lookups at events.  A
// uniform medium (every voxel the same material) needs no per-cell fetch.
template <typename Real, int MED>
__device__ __forceinline__ void fetch(const TransportArgs &a, const MatR<Real> *lut, int ix, int iy, int iz,
                                      int cidx, Real &mut, Real &mua, int &mid)
{
    if (MED == MED_RHOKAP) {
        const int64_t hx = a.nx + 2, hy = a.ny + 2;
        const Real v = (Real)__ldg(a.rhokap + ((ix + 1) + hx * ((iy + 1) + hy * (int64_t)(iz + 1))));
        mut = v;
        mua = v;
        mid = 0;
    } else if (MED == MED_MATERIAL) {
        // large grids: most cells lie in bricks of one material, whose id the
        // small (L2- and mostly L1-resident) brick table holds; the material
        // grid itself is read only inside mixed bricks
        int id;
        if (a.btab) {
            id = __ldg(a.btab + ((ix >> 3) + a.bbx * ((iy >> 3) + a.bby * (iz >> 3))));
            if (id == 0xFF) id = __ldg(a.mat + cidx);
        } else {
            id = __ldg(a.mat + cidx);
        }
        id = id < a.nmat ? id : 0;
        mid = id;
        mut = lut[id].mut;
        mua = lut[id].mua;
    } else {
        mid = a.uniform_id;
        mut = lut[mid].mut;
        mua = lut[mid].mua;
    }
}

// Event loop per lane: DEAD (needs a packet) -> FLY (one voxel step per
// iteration: cross a face, reach an outer face, or reach the interaction
// point) -> SCAT (waits at the interaction point) or FACE (waits on an outer
// face for its Fresnel draw) -> FLY ...  The events (Philox block, HG
// rotation, roulette, new optical depth; Fresnel reflect-or-escape) are the
// expensive part; the event batch runs once at least scat_min lanes of the
// warp wait, or when no lane is flying, so it executes with most lanes
// active.  Every packet sees the same sequence of events and random numbers
// as a straight loop.
//
// The DDA is incremental (Amanatides & Woo): per flight, the distance tm to
// the next face of each axis and the cell width td along the ray; a crossing
// moves tm of the crossed axis by td.  In-cell positions are reconstructed
// only at events (interaction, outer face).
template <typename Real> __device__ __forceinline__ const TrConst<Real> &consts(const TransportArgs &a)
{
    if constexpr (sizeof(Real) == 4) return a.cf;
    else return a.cd;
}

template <typename Real, int MED, bool T32>
__global__ void __launch_bounds__(TPB, sizeof(Real) == 4 ? TAM_TR_MINB : 2) transport_kernel(const __grid_constant__ TransportArgs a, int scat_min)
{
    __shared__ MatR<Real> lut[MAX_MAT];
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
    // per-packet (rare) tallies accumulate in shared memory, not registers
    __shared__ double s_tal[5];  // specular, reflected, transmitted, side, roulette net
    __shared__ unsigned long long s_cnt[2];  // voxel steps, scatters
    __shared__ unsigned s_err;
    if (threadIdx.x < 5) s_tal[threadIdx.x] = 0.0;
    if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0ull;
    if (threadIdx.x == 0) s_err = 0u;
    __syncthreads();

    const unsigned FULL = 0xffffffffu;
    const TrConst<Real> &K = consts<Real>(a);
    const Real hx = K.hx, hy = K.hy, hz = K.hz;
    const Real BIG = (Real)1.0e30;
    const Real TWOPI = (Real)TWOPI_R;
    // after a crossing the next face along the crossed axis is (h - nudge)
    // away along the axis: tm advances by td * (1 - nudge / h)
    const Real knx = K.knx, kny = K.kny, knz = K.knz;
    const uint32_t strm = a.stream_dev ? *a.stream_dev : a.stream;
    const unsigned lane = threadIdx.x & 31u;
    const Real wmin = K.wmin, rm = K.rm, inv_rm = K.inv_rm;
    const int NX = a.nx, NY = a.ny, NZ = a.nz, SY = a.nx, SZ = a.nx * a.ny;
    const uint32_t max_steps = a.max_steps > 0xfffffff0ll ? 0xfffffff0u : (uint32_t)a.max_steps;
    const Real namb = K.namb;
    // FP32 in a uniform medium: the flight is tracked by distance (tau / mut
    // once per flight) instead of optical depth per voxel step
    constexpr bool DIST = sizeof(Real) == 4 && MED == MED_UNIFORM;
    const Real inv_mut = DIST ? (Real)1 / lut[a.uniform_id >= 0 ? a.uniform_id : 0].mut : (Real)0;
    // a uniform medium's properties stay in registers (no fetch per crossing)
    const int mid_u = MED == MED_UNIFORM ? (a.uniform_id >= 0 ? a.uniform_id : 0) : 0;
    const Real mut_u = lut[mid_u].mut, mua_u = lut[mid_u].mua;
    // only the reference medium nudges a crossed coordinate past the face
    // (config mode's factor is exactly 1)
    constexpr bool NUDGE = MED == MED_RHOKAP;

    int mode = M_DEAD;
    bool exhausted = false;
    int ix = 0, iy = 0, iz = 0, cidx = 0, mid = 0, sgx = 1, sgy = 1, sgz = 1, fax = 0;
    Real fx = 0, fy = 0, fz = 0, nx = 0, ny = 0, nz = 0, sint = 0, phi = 0;
    Real cpv = 1, spv = 0;  // FP32 path: (cos phi, sin phi) in place of phi
    Real tdx = 0, tdy = 0, tdz = 0, tmx = 0, tmy = 0, tmz = 0, t = 0;
    Real w = 0, tau = 0, dep = 0, mut = 0, mua = 0;
    uint32_t ev = 0, plo = 0, phi32 = 0, nsteps = 0;
    uint32_t cScat = 0;
    uint64_t cSteps = 0;  // voxel steps of this thread's finished packets (reduced once at the end)
    auto props = [&]() {
        if constexpr (MED == MED_UNIFORM) {
            mid = mid_u;
            mut = mut_u;
            mua = mua_u;
        } else {
            fetch<Real, MED>(a, lut, ix, iy, iz, cidx, mut, mua, mid);
        }
    };

    for (;;) {
        // ---------------------------------------------- refill dead lanes --
        // (exhausted is warp-uniform: set once the counter has passed n)
        const unsigned need = exhausted ? 0u : __ballot_sync(FULL, mode == M_DEAD);
        if (need && (__popc(need) >= TAM_REFILL_MIN || need == FULL)) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(a.work, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            exhausted = base + (unsigned long long)__popc(need) >= (unsigned long long)a.n;
            if (mode == M_DEAD) {
                const unsigned long long my = base + __popc(need & ((1u << lane) - 1u));
                if (my < (unsigned long long)a.n) {
                    // launch (src/sourceph.f90:7-49; Gaussian beam in config mode)
                    const uint64_t pid = (uint64_t)a.p0 + my;
                    plo = (uint32_t)pid;
                    phi32 = (uint32_t)(pid >> 32);
                    const U4 r = philox4x32_10_rk(0u, plo, phi32, strm, a.rk);
                    ev = 1;
                    const Real u0 = Uniform<Real>::from(r.x), u1 = Uniform<Real>::from(r.y);
                    const Real u2 = Uniform<Real>::from(r.z), u3 = Uniform<Real>::from(r.w);
                    const Real R = K.src_r;
                    const Real rad = a.source == SRC_DISK ? M<Real>::sqrt(u0 * (R * R))
                                                          : R * M<Real>::sqrt((Real)0.5 * M<Real>::neglog(u0));
                    Real st, ct, sp, cp;
                    M<Real>::sincos(u1 * TWOPI, &st, &ct);
                    const Real X = rad * ct + K.xmax, Y = rad * st + K.ymax;
                    phi = TWOPI * u2;
                    if constexpr (MED == MED_RHOKAP) {
                        // reference medium: a pure absorber (any interaction
                        // ends the packet) launched straight down, so the
                        // azimuth only enters nx = ny = sint * (cos, sin) phi
                        // = +-0, which the walk treats alike; its sincos (an
                        // FP64 one in the parity form) is skipped
                        cp = (Real)1;
                        sp = (Real)0;
                    } else {
                        M<Real>::sincos(phi, &sp, &cp);
                    }
                    cpv = cp;
                    spv = sp;
                    sint = (Real)0;
                    if (!(X >= (Real)0 && X < K.w2x && Y >= (Real)0 && Y < K.w2y)) {
                        atomicAdd(a.tally + T_MISSED, 1.0);
                    } else {
                        ix = (int)((Real)NX * X / K.w2x);
                        iy = (int)((Real)NY * Y / K.w2y);
                        ix = ix > NX - 1 ? NX - 1 : ix;
                        iy = iy > NY - 1 ? NY - 1 : iy;
                        iz = NZ - 1;
                        cidx = ix + SY * iy + SZ * iz;
                        fx = X - (Real)ix * hx;
                        fy = Y - (Real)iy * hy;
                        fz = hz - (Real)1.e-8 * hz;
                        props();
                        w = (Real)1;
                        if (a.fresnel) {
                            const Real nt = MED == MED_RHOKAP ? K.rhokap_n : lut[mid].n;
                            Real rsp = (namb - nt) / (namb + nt);
                            rsp = rsp * rsp;
                            atomicAdd(&s_tal[0], (double)rsp);
                            w = (Real)1 - rsp;
                        }
                        tau = M<Real>::neglog(u3);
                        if constexpr (DIST) tau *= inv_mut;
                        nx = sint * cp;  // direction (0, 0, -1): +-0 in x and y
                        ny = sint * sp;
                        nz = (Real)-1;
                        axis_setup(nx, fx, hx, BIG, tdx, tmx, sgx);
                        axis_setup(ny, fy, hy, BIG, tdy, tmy, sgy);
                        axis_setup(nz, fz, hz, BIG, tdz, tmz, sgz);
                        t = (Real)0;
                        dep = (Real)0;
                        nsteps = 0;
                        mode = M_FLY;
                    }
                }
            }
        }
        // ------------------------------------------------- flight phase --
        // voxel steps of the flying lanes until enough lanes wait to scatter,
        // no lane flies, or a lane needs a new packet
        unsigned sc, fl;
        // -------------------------- one voxel step (src/inttau2.f90:37-63) --
        auto vstep = [&]() {
        if (mode == M_FLY) {
            if (++nsteps > max_steps) {
                if (dep != (Real)0) deposit<T32>(a, cidx, ix, iy, iz, dep);
                dep = (Real)0;
                atomicAdd(a.tally + T_OVERFLOW, 1.0);
                atomicOr(&s_err, (unsigned)DEVERR_STEP_CAP);
                cSteps += nsteps;
                mode = M_DEAD;
            } else {
                // nearest face; ties go z over y over x (src/inttau2.f90:116-118)
                int ax = 2;
                Real tmin = tmz;
                if (tmy < tmin) { tmin = tmy; ax = 1; }
                if (tmx < tmin) { tmin = tmx; ax = 0; }
                Real dw;
                bool cross;
                if constexpr (DIST) {
                    // tau holds the flight distance of the interaction point
                    cross = tmin < tau;
                    const Real tend = cross ? tmin : tau;
                    dw = tend - t;
                    dw = dw < (Real)0 ? (Real)0 : dw;
                    dep += w * dw * mua;
                    t = tend;
                } else {
                    dw = tmin - t;
                    dw = dw < (Real)0 ? (Real)0 : dw;
                    const Real taucell = dw * mut;
                    cross = taucell < tau;
                    if (cross) {
                        dep += w * dw * mua;
                        tau -= taucell;
                        t = tmin;
                    }
                }
                if (cross) {
                    const bool cx = ax == 0, cy = ax == 1, cz = ax == 2;
                    const int sg = cx ? sgx : (cy ? sgy : sgz);
                    const int j = (cx ? ix : (cy ? iy : iz)) + sg;
                    const int N = cx ? NX : (cy ? NY : NZ);
                    deposit<T32>(a, cidx, ix, iy, iz, dep);
                    dep = (Real)0;
                    if ((unsigned)j < (unsigned)N) {
                        // step into the next cell (branch-free over the axis); the
                        // reference snaps the crossed coordinate to the face +- delta
                        // (src/inttau2.f90:140-169), which knx/kny/knz carry
                        ix = cx ? j : ix;
                        iy = cy ? j : iy;
                        iz = cz ? j : iz;
                        cidx += cx ? sg : (cy ? sg * SY : sg * SZ);
                        tmx = cx ? tmx + (NUDGE ? tdx * knx : tdx) : tmx;
                        tmy = cy ? tmy + (NUDGE ? tdy * kny : tdy) : tmy;
                        tmz = cz ? tmz + (NUDGE ? tdz * knz : tdz) : tmz;
                        props();
                    } else if (a.fresnel) {
                        // outer face: the packet sits on it; the Fresnel draw
                        // waits for the event batch
                        fax = ax;
                        mode = M_FACE;
                    } else {
                        // outer face without Fresnel: escape
                        atomicAdd(&s_tal[cz ? (sgz > 0 ? 1 : 2) : 3], (double)w);
                        cSteps += nsteps;
                        mode = M_DEAD;
                    }
                } else {
                    // interaction point inside this cell; the in-cell position
                    // is reconstructed in the event batch
                    if constexpr (!DIST) {
                        const Real dd = M<Real>::div(tau, mut);
                        dep += w * dd * mua;
                        t += dd;
                    }
                    mode = M_SCAT;
                }
            }
        }
        };
        for (;;) {
            // TAM_VSTEPS voxel steps per vote (transport_common.cuh)
#pragma unroll
            for (int q = 0; q < TAM_VSTEPS; ++q) vstep();
            sc = __ballot_sync(FULL, mode >= M_SCAT);
            fl = __ballot_sync(FULL, mode == M_FLY);
            if (fl == 0 || __popc(sc) >= scat_min || (!exhausted && __popc(~(sc | fl)) >= TAM_REFILL_MIN)) break;
        }
        if ((sc | fl) == 0) {
            if (exhausted) break;
            continue;
        }

        // ------------------------------------------------- event batch --
        // interactions (implicit capture, HG scatter, roulette) and Fresnel
        // faces, handled together once enough lanes wait; both kinds draw
        // their uniforms from one Philox block per lane
        if (sc && (__popc(sc) >= scat_min || fl == 0)) {
            if (mode >= M_SCAT) {
                const bool face = mode == M_FACE;
                if (!face) w *= MED == MED_RHOKAP ? (Real)0 : lut[mid].alb;
                bool die = !face && !(w > (Real)0);
                U4 r{0u, 0u, 0u, 0u};
                if (!die) r = philox4x32_10_rk(ev++, plo, phi32, strm, a.rk);
                if (face) {
                    const bool cx = fax == 0, cy = fax == 1;
                    const Real nc = cx ? nx : (cy ? ny : nz);
                    const Real nt = MED == MED_RHOKAP ? K.rhokap_n : lut[mid].n;
                    if (Uniform<Real>::from(r.x) < fresnel<Real>(nt, namb, M<Real>::abs(nc))) {
                        // reflect: mirror the crossed direction component; the
                        // next face along it is one cell width back
                        if (cx) {
                            fy = axis_pos(ny, fy, hy, tmy, t);
                            fz = axis_pos(nz, fz, hz, tmz, t);
                            fx = sgx > 0 ? hx : (Real)0;
                            nx = -nx;
                            sgx = -sgx;
                            tmx = t + tdx;
                            if constexpr (sizeof(Real) == 4) {
                                cpv = -cpv;  // phi -> PI - phi
                            } else {
                                phi = (Real)PI_R - phi;
                                if (phi < (Real)0) phi += TWOPI;
                            }
                        } else if (cy) {
                            fx = axis_pos(nx, fx, hx, tmx, t);
                            fz = axis_pos(nz, fz, hz, tmz, t);
                            fy = sgy > 0 ? hy : (Real)0;
                            ny = -ny;
                            sgy = -sgy;
                            tmy = t + tdy;
                            if constexpr (sizeof(Real) == 4) {
                                spv = -spv;  // phi -> TWOPI - phi
                            } else {
                                phi = TWOPI - phi;
                            }
                        } else {
                            fx = axis_pos(nx, fx, hx, tmx, t);
                            fy = axis_pos(ny, fy, hy, tmy, t);
                            fz = sgz > 0 ? hz : (Real)0;
                            nz = -nz;
                            sgz = -sgz;
                            tmz = t + tdz;
                        }
                        mode = M_FLY;
                    } else {
                        atomicAdd(&s_tal[(!cx && !cy) ? (sgz > 0 ? 1 : 2) : 3], (double)w);
                        cSteps += nsteps;
                        mode = M_DEAD;
                    }
                } else if (!die) {
                    cScat += 1;
                    fx = axis_pos(nx, fx, hx, tmx, t);
                    fy = axis_pos(ny, fy, hy, tmy, t);
                    fz = axis_pos(nz, fz, hz, tmz, t);
                    Real cost = nz;
                    if constexpr (sizeof(Real) == 4) {
                        if (stokes_f32(lut[mid].g, lut[mid].g2, Uniform<Real>::from(r.x), Uniform<Real>::from(r.y), cost,
                                       sint, cpv, spv)) {
                            nx = sint * cpv;
                            ny = sint * spv;
                            nz = cost;
                        }
                    } else {
                        Real cp, sp;
                        if (stokes<Real>(lut[mid].g, lut[mid].g2, Uniform<Real>::from(r.x), Uniform<Real>::from(r.y),
                                         cost, sint, phi, cp, sp)) {
                            nx = sint * cp;
                            ny = sint * sp;
                            nz = cost;
                        }
                    }
                    if (!(nz == nz) || !(nx == nx) || !(ny == ny)) {
                        atomicOr(&s_err, (unsigned)DEVERR_NAN);
                        die = true;
                    } else {
                        axis_setup(nx, fx, hx, BIG, tdx, tmx, sgx);
                        axis_setup(ny, fy, hy, BIG, tdy, tmy, sgy);
                        axis_setup(nz, fz, hz, BIG, tdz, tmz, sgz);
                        t = (Real)0;
                        if (a.roulette && w < wmin) {
                            if (Uniform<Real>::from(r.z) < inv_rm) {
                                atomicAdd(&s_tal[4], (double)(w * (rm - (Real)1)));
                                w *= rm;
                            } else {
                                atomicAdd(&s_tal[4], -(double)w);
                                die = true;
                            }
                        }
                        tau = M<Real>::neglog(Uniform<Real>::from(r.w));
                        if constexpr (DIST) tau *= inv_mut;
                    }
                    if (!die) mode = M_FLY;
                }
                if (die) {
                    if (dep != (Real)0) deposit<T32>(a, cidx, ix, iy, iz, dep);
                    dep = (Real)0;
                    cSteps += nsteps;
                    mode = M_DEAD;
                }
            }
        }
    }

    // ---- block reduction of the tallies ----
    const unsigned c1 = __reduce_add_sync(FULL, cScat);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cSteps += __shfl_xor_sync(FULL, cSteps, o);
    if (lane == 0) {
        atomicAdd(&s_cnt[1], (unsigned long long)c1);
        atomicAdd(&s_cnt[0], (unsigned long long)cSteps);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(a.tally + T_SPECULAR, s_tal[0]);
        atomicAdd(a.tally + T_REFLECTED, s_tal[1]);
        atomicAdd(a.tally + T_TRANSMITTED, s_tal[2]);
        atomicAdd(a.tally + T_SIDE, s_tal[3]);
        atomicAdd(a.tally + T_ROULETTE_NET, s_tal[4]);
        atomicAdd(a.tally + T_STEPS, (double)s_cnt[0]);
        atomicAdd(a.tally + T_SCATTERS, (double)s_cnt[1]);
        if (s_err) atomicOr(a.err, s_err);
    }
}

// One warp per 8^3 brick: lane l takes the brick's x-rows l and l + 32 (of
// 64: y fastest, then z), the warp compares its smallest and largest id.
__global__ void brick_table_kernel(const uint8_t *mat, int nx, int ny, int nz, int bbx, int bby, int64_t nb,
                                   uint8_t *btab)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < nb; b += nw) {
        const int bx = (int)(b % bbx);
        const int64_t rest = b / bbx;
        const int by = (int)(rest % bby), bz = (int)(rest / bby);
        int lo = 256, hi = -1;
        for (int row = lane; row < 64; row += 32) {
            const int y = by * 8 + (row & 7), z = bz * 8 + (row >> 3);
            if (y >= ny || z >= nz) continue;
            const uint8_t *p = mat + (int64_t)nx * (y + (int64_t)ny * z);
            for (int x = bx * 8; x < bx * 8 + 8 && x < nx; ++x) {
                const int v = p[x];
                lo = min(lo, v);
                hi = max(hi, v);
            }
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (lane == 0) btab[b] = (uint8_t)(lo == hi ? lo : 0xFF);
    }
}

// out = in * f (normalisation of the tally), and with `sum` the total of
// `in` added to *sum: one FP64 atomic per block, so the grid is kept to a few
// thousand blocks
template <typename Out>
__global__ void scale_kernel(Out *out, double *in, double f, int64_t n, int zero_in, double *sum,
                             const double *f_dev)
{
    if (f_dev) f = *f_dev;
    double acc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double v = in[q];
        out[q] = (Out)(v * f);
        acc += v;
        if (zero_in) in[q] = 0.0;
    }
    if (!sum) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double ws[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) ws[wid] = acc;
    __syncthreads();
    if (wid == 0) {
        acc = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) atomicAdd(sum, acc);
    }
}

__global__ void flush_f32_kernel(double *acc, float *part, int nx, int ny, int bx0, int by0, int bz0, int bnx, int bny,
                                 int64_t n)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const float v = part[q];
        if (v != 0.f) {
            const int64_t x = bx0 + q % bnx, y = by0 + (q / bnx) % bny, z = bz0 + q / ((int64_t)bnx * bny);
            acc[x + (int64_t)nx * (y + (int64_t)ny * z)] += (double)v;
            part[q] = 0.f;
        }
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

template <typename Real, int MED, bool T32 = false>
cudaError_t launch_t(const TransportArgs &a, int sm_count, cudaStream_t s)
{
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_kernel<Real, MED, T32>, TPB, 0);
    const int scat_min = a.scat_min > 0 ? a.scat_min : 20;
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = (int64_t)sm_count * per_sm;
    const int64_t need = (a.n + TPB - 1) / TPB;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    count_launch();
    transport_kernel<Real, MED, T32><<<(unsigned)blocks, TPB, 0, s>>>(a, scat_min);
    return cudaGetLastError();
}

}  // namespace

// The per-launch constants, in the order of operations a thread used to
// evaluate them in FP64 (so the FP64 form's values are unchanged), and their
// FP32 roundings.
static void fill_consts(TransportArgs &a)
{
    TrConst<double> &d = a.cd;
    d.hx = 2.0 * a.xmax / a.nx;
    d.hy = 2.0 * a.ymax / a.ny;
    d.hz = 2.0 * a.zmax / a.nz;
    d.knx = 1.0 - a.nudge / (2.0 * a.xmax / a.nx);
    d.kny = 1.0 - a.nudge / (2.0 * a.ymax / a.ny);
    d.knz = 1.0 - a.nudge / (2.0 * a.zmax / a.nz);
    d.w2x = 2.0 * a.xmax;
    d.w2y = 2.0 * a.ymax;
    d.xmax = a.xmax;
    d.ymax = a.ymax;
    d.wmin = a.roulette_w;
    d.rm = a.roulette_m;
    d.inv_rm = 1.0 / a.roulette_m;
    d.namb = a.n_ambient;
    d.rhokap_n = a.rhokap_n;
    d.src_r = a.source_radius;
    TrConst<float> &f = a.cf;
    f.hx = (float)d.hx, f.hy = (float)d.hy, f.hz = (float)d.hz;
    f.knx = (float)d.knx, f.kny = (float)d.kny, f.knz = (float)d.knz;
    f.w2x = (float)d.w2x, f.w2y = (float)d.w2y, f.xmax = (float)d.xmax, f.ymax = (float)d.ymax;
    f.wmin = (float)d.wmin, f.rm = (float)d.rm, f.inv_rm = (float)d.inv_rm;
    f.namb = (float)d.namb, f.rhokap_n = (float)d.rhokap_n, f.src_r = (float)d.src_r;
}

void fill_batch_inst(const TransportArgs &args, BatchTrInst &b)
{
    TransportArgs a = args;
    fill_consts(a);
    const TrConst<float> &f = a.cf;
    b.nx = a.nx, b.ny = a.ny, b.nz = a.nz;
    b.source = a.source, b.fresnel = a.fresnel, b.roulette = a.roulette;
    b.hx = f.hx, b.hy = f.hy, b.hz = f.hz, b.w2x = f.w2x, b.w2y = f.w2y, b.xmax = f.xmax, b.ymax = f.ymax;
    b.src_r = f.src_r, b.namb = f.namb, b.wmin = f.wmin, b.rm = f.rm, b.inv_rm = f.inv_rm;
    // the material's FP32 properties as the single pass's shared table holds them
    const OptMat &o = a.lut[a.uniform_id >= 0 && a.uniform_id < a.nmat ? a.uniform_id : 0];
    b.mut = (float)(o.mua + o.mus);
    b.mua = (float)o.mua;
    b.alb = (o.mua + o.mus) > 0.0 ? (float)(o.mus / (o.mua + o.mus)) : 0.f;
    b.g = (float)o.g;
    b.g2 = (float)(o.g * o.g);
    b.n = (float)o.n;
    b.inv_mut = 1.0f / b.mut;  // IEEE single division: the bits of the single pass's 1 / mut
    b.seed = a.seed;
    b.stream = a.stream;
    b.max_steps = a.max_steps > 0xfffffff0ll ? 0xfffffff0u : (uint32_t)a.max_steps;
    b.first = 0;
    b.count = a.n;
    b.jmean = a.jmean;
    b.tally = a.tally;
}

cudaError_t launch_transport(const TransportArgs &args, bool fp64, int sm_count, cudaStream_t s)
{
    if (args.n <= 0) return cudaSuccess;
    TransportArgs a = args;
    fill_consts(a);
    philox_round_keys(a.seed, a.rk);
    cudaError_t e = cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if (fp64) {
        // the FP32 box tally is a config-mode form; on the FP64 transport it
        // serves its checks against the FP64 oracle on the same streams
        if (a.medium == MED_RHOKAP) {
            if (a.jmean32) return cudaErrorInvalidValue;
            return launch_t<double, MED_RHOKAP>(a, sm_count, s);
        }
        if (a.uniform_id >= 0)
            return a.jmean32 ? launch_t<double, MED_UNIFORM, true>(a, sm_count, s) : launch_t<double, MED_UNIFORM>(a, sm_count, s);
        return a.jmean32 ? launch_t<double, MED_MATERIAL, true>(a, sm_count, s) : launch_t<double, MED_MATERIAL>(a, sm_count, s);
    }
    if (a.medium == MED_RHOKAP) {
        if (a.jmean32) return cudaErrorInvalidValue;  // the FP32 tally is a config-mode form
        return launch_t<float, MED_RHOKAP>(a, sm_count, s);
    }
    // the tally's precision is a template parameter: no per-deposit branch
    if (a.uniform_id >= 0)
        return a.jmean32 ? launch_t<float, MED_UNIFORM, true>(a, sm_count, s) : launch_t<float, MED_UNIFORM>(a, sm_count, s);
    return a.jmean32 ? launch_t<float, MED_MATERIAL, true>(a, sm_count, s) : launch_t<float, MED_MATERIAL>(a, sm_count, s);
}

// at least four elements per thread, at most 152 x 16 blocks (atomics on *sum)
static int scale_grid(int64_t n)
{
    int64_t b = (n + 1023) / 1024;
    if (b > 152 * 16) b = 152 * 16;
    return (int)(b > 0 ? b : 1);
}

cudaError_t launch_scale_f64(double *out, double *in, double f, int64_t n, bool zero_in, cudaStream_t s, double *sum,
                             const double *f_dev)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    scale_kernel<double><<<scale_grid(n), 256, 0, s>>>(out, in, f, n, zero_in ? 1 : 0, sum, f_dev);
    return cudaGetLastError();
}

int64_t brick_table_size(int nx, int ny, int nz)
{
    return (int64_t)((nx + 7) / 8) * ((ny + 7) / 8) * ((nz + 7) / 8);
}

cudaError_t launch_brick_table(const uint8_t *mat, int nx, int ny, int nz, uint8_t *btab, cudaStream_t s)
{
    const int64_t nb = brick_table_size(nx, ny, nz);
    const int64_t blocks = std::min<int64_t>((nb + 7) / 8, 152 * 32);
    count_launch();
    brick_table_kernel<<<(unsigned)blocks, 256, 0, s>>>(mat, nx, ny, nz, (nx + 7) / 8, (ny + 7) / 8, nb, btab);
    return cudaGetLastError();
}

cudaError_t launch_flush_f32(double *acc, float *part, int nx, int ny, int bx0, int by0, int bz0, int bnx, int bny,
                             int bnz, cudaStream_t s)
{
    const int64_t n = (int64_t)bnx * bny * bnz;
    if (n <= 0) return cudaSuccess;
    count_launch();
    flush_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(acc, part, nx, ny, bx0, by0, bz0, bnx, bny, n);
    return cudaGetLastError();
}

cudaError_t launch_scale_to_f32(float *out, double *in, double f, int64_t n, bool zero_in, cudaStream_t s, double *sum)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    scale_kernel<float><<<scale_grid(n), 256, 0, s>>>(out, in, f, n, zero_in ? 1 : 0, sum, nullptr);
    return cudaGetLastError();
}

namespace {
// Ceiling of the tally updates: `per_thread` fire-and-forget atomic adds per
// thread (red.global.add, the result unused, as the transport's deposits) at
// cells drawn from Philox inside the kernel, so no index stream is read; four
// cells per Philox block, mapped to [0, cells) by a 32 x 32 high product.
template <typename Real>
__global__ void __launch_bounds__(256) atomic_peak_kernel(Real *acc, uint32_t cells, int per_thread, uint32_t seed)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = 0; i < per_thread; i += 4) {
        const U4 r = philox4x32_10((uint32_t)i, t, 0x7a11u, 0u, seed, 0x5eedu);
        atomicAdd(acc + __umulhi(r.x, cells), (Real)1);
        atomicAdd(acc + __umulhi(r.y, cells), (Real)1);
        atomicAdd(acc + __umulhi(r.z, cells), (Real)1);
        atomicAdd(acc + __umulhi(r.w, cells), (Real)1);
    }
}
}  // namespace

cudaError_t launch_atomic_peak(void *acc, bool fp32, uint32_t cells, int blocks, int per_thread, uint32_t seed,
                               cudaStream_t s)
{
    count_launch();
    if (fp32) atomic_peak_kernel<float><<<blocks, 256, 0, s>>>((float *)acc, cells, per_thread, seed);
    else atomic_peak_kernel<double><<<blocks, 256, 0, s>>>((double *)acc, cells, per_thread, seed);
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
