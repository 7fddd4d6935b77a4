// transport_batch.cu -- MC passes of many instances in one launch.
//
// The batched form of the FP32 uniform-medium transport (transport.cu,
// transport_kernel<float, MED_UNIFORM>): src/sourceph.f90:7-49 with the
// Gaussian beam, the tau integration of src/inttau2.f90:37-63 as an
// incremental DDA tracked by distance, the HG rotation of src/stokes.f90,
// Fresnel faces and Russian roulette.  The instances' packets form one
// range; persistent warps draw packets from it with one counter, and each
// lane finds its packet's instance by a binary search of the instances'
// first packets, so instances of every size and cost share the GPU without a
// tail per instance.  Each lane keeps its instance's grid size and
// absorption in registers and reads the rest of its constants from a
// shared-memory table of the instances.  A packet uses its instance's Philox
// key and stream and its index within the instance, so it walks exactly as
// in that instance's own pass; escape weights and step / scatter counts
// accumulate per instance in shared memory and go to each instance's tally
// at the end.
#include "tam_device.cuh"
#include "tam_kernels.h"
#include "transport_common.cuh"

namespace tam {

namespace {

constexpr int BTPB = 256;

__global__ void __launch_bounds__(BTPB, 4)
    batch_transport_kernel(const BatchTrInst *__restrict__ insts, int ninst, int64_t total,
                           unsigned long long *work, int scat_min)
{
    __shared__ BatchTrInst s_in[MAX_BATCH_TR];
    __shared__ int64_t s_first[MAX_BATCH_TR];
    __shared__ double s_tal[MAX_BATCH_TR][5];  // specular, reflected, transmitted, side, roulette net
    __shared__ unsigned long long s_cnt[MAX_BATCH_TR][2];  // voxel steps, scatters
    for (int t = threadIdx.x; t < ninst; t += blockDim.x) {
        s_in[t] = insts[t];
        s_first[t] = insts[t].first;
        for (int k = 0; k < 5; ++k) s_tal[t][k] = 0.0;
        s_cnt[t][0] = s_cnt[t][1] = 0ull;
    }
    __syncthreads();

    const unsigned FULL = 0xffffffffu;
    const float BIG = 1.0e30f;
    const float TWOPI = (float)TWOPI_R;
    const unsigned lane = threadIdx.x & 31u;

    int mode = M_DEAD;
    bool exhausted = false;
    int inst = 0;
    int NX = 1, NY = 1, NZ = 1, SZ = 1;  // the lane's instance: grid
    float mua = 0.f;                     // ... and absorption
    int ix = 0, iy = 0, iz = 0, cidx = 0, sgx = 1, sgy = 1, sgz = 1, fax = 0;
    float fx = 0, fy = 0, fz = 0, nx = 0, ny = 0, nz = 0, sint = 0;
    float cpv = 1, spv = 0;
    float tdx = 0, tdy = 0, tdz = 0, tmx = 0, tmy = 0, tmz = 0, t = 0;
    float w = 0, tau = 0, dep = 0;
    double *jm = nullptr;  // the lane's instance's tally
    // voxel steps the packet may still take (its instance's cap counts down,
    // so the per-step test needs no table lookup; steps taken = cap - left)
    uint32_t ev = 0, plo = 0, phi32 = 0, left = 0, nscat = 0;

    // the packet's end: its counts go to its instance
    auto retire = [&]() {
        atomicAdd(&s_cnt[inst][0], (unsigned long long)(uint32_t)(s_in[inst].max_steps - left));
        atomicAdd(&s_cnt[inst][1], (unsigned long long)nscat);
        mode = M_DEAD;
    };

    for (;;) {
        // ---------------------------------------------- refill dead lanes --
        const unsigned need = exhausted ? 0u : __ballot_sync(FULL, mode == M_DEAD);
        if (need && (__popc(need) >= TAM_REFILL_MIN || need == FULL)) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(work, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            exhausted = base + (unsigned long long)__popc(need) >= (unsigned long long)total;
            if (mode == M_DEAD) {
                const unsigned long long my = base + __popc(need & ((1u << lane) - 1u));
                if (my < (unsigned long long)total) {
                    // the packet's instance: the last whose first packet is <= my
                    int lo = 0, hi = ninst - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (s_first[mid] <= (int64_t)my) lo = mid;
                        else hi = mid - 1;
                    }
                    inst = lo;
                    const BatchTrInst &I = s_in[inst];
                    NX = I.nx;
                    NY = I.ny;
                    NZ = I.nz;
                    SZ = I.nx * I.ny;
                    mua = I.mua;
                    // launch (src/sourceph.f90:7-49 with the Gaussian beam)
                    const uint64_t pid = (uint64_t)((int64_t)my - I.first);
                    plo = (uint32_t)pid;
                    phi32 = (uint32_t)(pid >> 32);
                    const U4 r = philox4x32_10(0u, plo, phi32, I.stream, (uint32_t)I.seed, (uint32_t)(I.seed >> 32));
                    ev = 1;
                    const float u0 = Uniform<float>::from(r.x), u1 = Uniform<float>::from(r.y);
                    const float u2 = Uniform<float>::from(r.z), u3 = Uniform<float>::from(r.w);
                    const float R = I.src_r;
                    const float rad = I.source == SRC_DISK ? M<float>::sqrt(u0 * (R * R))
                                                           : R * M<float>::sqrt(0.5f * M<float>::neglog(u0));
                    float st, ct, sp, cp;
                    M<float>::sincos(u1 * TWOPI, &st, &ct);
                    const float X = rad * ct + I.xmax, Y = rad * st + I.ymax;
                    M<float>::sincos(TWOPI * u2, &sp, &cp);
                    cpv = cp;
                    spv = sp;
                    sint = 0.f;
                    left = I.max_steps;
                    jm = I.jmean;
                    nscat = 0;
                    if (!(X >= 0.f && X < I.w2x && Y >= 0.f && Y < I.w2y)) {
                        atomicAdd(I.tally + T_MISSED, 1.0);
                        retire();
                    } else {
                        ix = (int)((float)NX * X / I.w2x);
                        iy = (int)((float)NY * Y / I.w2y);
                        ix = ix > NX - 1 ? NX - 1 : ix;
                        iy = iy > NY - 1 ? NY - 1 : iy;
                        iz = NZ - 1;
                        cidx = ix + NX * iy + SZ * iz;
                        fx = X - (float)ix * I.hx;
                        fy = Y - (float)iy * I.hy;
                        fz = I.hz - 1.e-8f * I.hz;
                        w = 1.f;
                        if (I.fresnel) {
                            float rsp = (I.namb - I.n) / (I.namb + I.n);
                            rsp = rsp * rsp;
                            atomicAdd(&s_tal[inst][0], (double)rsp);
                            w = 1.f - rsp;
                        }
                        // the flight by distance: tau / mut once per flight
                        tau = M<float>::neglog(u3) * I.inv_mut;
                        nx = sint * cp;
                        ny = sint * sp;
                        nz = -1.f;
                        axis_setup(nx, fx, I.hx, BIG, tdx, tmx, sgx);
                        axis_setup(ny, fy, I.hy, BIG, tdy, tmy, sgy);
                        axis_setup(nz, fz, I.hz, BIG, tdz, tmz, sgz);
                        t = 0.f;
                        dep = 0.f;
                        mode = M_FLY;
                    }
                }
            }
        }
        // ------------------------------------------------- flight phase --
        unsigned sc, fl;
        auto vstep = [&]() {
            if (mode != M_FLY) return;
            if (left-- == 0u) {
                // past the cap (left wraps: cap - left = cap + 1 steps, as the single pass counts)
                if (dep != 0.f) atomicAdd(jm + cidx, (double)dep);
                dep = 0.f;
                atomicAdd(s_in[inst].tally + T_OVERFLOW, 1.0);
                atomicOr(s_in[inst].err, (unsigned)DEVERR_STEP_CAP);
                retire();
                return;
            }
            // nearest face; ties go z over y over x (src/inttau2.f90:116-118)
            int ax = 2;
            float tmin = tmz;
            if (tmy < tmin) { tmin = tmy; ax = 1; }
            if (tmx < tmin) { tmin = tmx; ax = 0; }
            const bool cross = tmin < tau;
            const float tend = cross ? tmin : tau;
            float dw = tend - t;
            dw = dw < 0.f ? 0.f : dw;
            dep += w * dw * mua;
            t = tend;
            if (!cross) {
                mode = M_SCAT;  // the interaction point lies in this cell
                return;
            }
            const bool cx = ax == 0, cy = ax == 1, cz = ax == 2;
            const int sg = cx ? sgx : (cy ? sgy : sgz);
            const int j = (cx ? ix : (cy ? iy : iz)) + sg;
            const int N = cx ? NX : (cy ? NY : NZ);
            atomicAdd(jm + cidx, (double)dep);
            dep = 0.f;
            if ((unsigned)j < (unsigned)N) {
                ix = cx ? j : ix;
                iy = cy ? j : iy;
                iz = cz ? j : iz;
                cidx += cx ? sg : (cy ? sg * NX : sg * SZ);
                tmx = cx ? tmx + tdx : tmx;
                tmy = cy ? tmy + tdy : tmy;
                tmz = cz ? tmz + tdz : tmz;
            } else if (s_in[inst].fresnel) {
                fax = ax;
                mode = M_FACE;  // on an outer face: the Fresnel draw waits for the event batch
            } else {
                atomicAdd(&s_tal[inst][cz ? (sgz > 0 ? 1 : 2) : 3], (double)w);
                retire();
            }
        };
        for (;;) {
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
        if (sc && (__popc(sc) >= scat_min || fl == 0)) {
            if (mode >= M_SCAT) {
                const BatchTrInst &I = s_in[inst];
                const bool face = mode == M_FACE;
                if (!face) w *= I.alb;
                bool die = !face && !(w > 0.f);
                U4 r{0u, 0u, 0u, 0u};
                if (!die) r = philox4x32_10(ev++, plo, phi32, I.stream, (uint32_t)I.seed, (uint32_t)(I.seed >> 32));
                if (face) {
                    const bool cx = fax == 0, cy = fax == 1;
                    const float nc = cx ? nx : (cy ? ny : nz);
                    if (Uniform<float>::from(r.x) < fresnel<float>(I.n, I.namb, M<float>::abs(nc))) {
                        // reflect: mirror the crossed component; the next face along it is a cell width back
                        if (cx) {
                            fy = axis_pos(ny, fy, I.hy, tmy, t);
                            fz = axis_pos(nz, fz, I.hz, tmz, t);
                            fx = sgx > 0 ? I.hx : 0.f;
                            nx = -nx;
                            sgx = -sgx;
                            tmx = t + tdx;
                            cpv = -cpv;
                        } else if (cy) {
                            fx = axis_pos(nx, fx, I.hx, tmx, t);
                            fz = axis_pos(nz, fz, I.hz, tmz, t);
                            fy = sgy > 0 ? I.hy : 0.f;
                            ny = -ny;
                            sgy = -sgy;
                            tmy = t + tdy;
                            spv = -spv;
                        } else {
                            fx = axis_pos(nx, fx, I.hx, tmx, t);
                            fy = axis_pos(ny, fy, I.hy, tmy, t);
                            fz = sgz > 0 ? I.hz : 0.f;
                            nz = -nz;
                            sgz = -sgz;
                            tmz = t + tdz;
                        }
                        mode = M_FLY;
                    } else {
                        atomicAdd(&s_tal[inst][(!cx && !cy) ? (sgz > 0 ? 1 : 2) : 3], (double)w);
                        retire();
                    }
                } else if (!die) {
                    nscat += 1;
                    fx = axis_pos(nx, fx, I.hx, tmx, t);
                    fy = axis_pos(ny, fy, I.hy, tmy, t);
                    fz = axis_pos(nz, fz, I.hz, tmz, t);
                    float cost = nz;
                    if (stokes_f32(I.g, I.g2, Uniform<float>::from(r.x), Uniform<float>::from(r.y), cost, sint, cpv,
                                   spv)) {
                        nx = sint * cpv;
                        ny = sint * spv;
                        nz = cost;
                    }
                    if (!(nz == nz) || !(nx == nx) || !(ny == ny)) {
                        atomicOr(I.err, (unsigned)DEVERR_NAN);
                        die = true;
                    } else {
                        axis_setup(nx, fx, I.hx, BIG, tdx, tmx, sgx);
                        axis_setup(ny, fy, I.hy, BIG, tdy, tmy, sgy);
                        axis_setup(nz, fz, I.hz, BIG, tdz, tmz, sgz);
                        t = 0.f;
                        if (I.roulette && w < I.wmin) {
                            if (Uniform<float>::from(r.z) < I.inv_rm) {
                                atomicAdd(&s_tal[inst][4], (double)(w * (I.rm - 1.f)));
                                w *= I.rm;
                            } else {
                                atomicAdd(&s_tal[inst][4], -(double)w);
                                die = true;
                            }
                        }
                        tau = M<float>::neglog(Uniform<float>::from(r.w)) * I.inv_mut;
                    }
                    if (!die) mode = M_FLY;
                }
                if (die) {
                    if (dep != 0.f) atomicAdd(jm + cidx, (double)dep);
                    dep = 0.f;
                    retire();
                }
            }
        }
    }

    // ---- the instances' tallies ----
    __syncthreads();
    for (int q = threadIdx.x; q < ninst; q += blockDim.x) {
        double *tl = s_in[q].tally;
        if (s_tal[q][0] != 0.0) atomicAdd(tl + T_SPECULAR, s_tal[q][0]);
        if (s_tal[q][1] != 0.0) atomicAdd(tl + T_REFLECTED, s_tal[q][1]);
        if (s_tal[q][2] != 0.0) atomicAdd(tl + T_TRANSMITTED, s_tal[q][2]);
        if (s_tal[q][3] != 0.0) atomicAdd(tl + T_SIDE, s_tal[q][3]);
        if (s_tal[q][4] != 0.0) atomicAdd(tl + T_ROULETTE_NET, s_tal[q][4]);
        if (s_cnt[q][0]) atomicAdd(tl + T_STEPS, (double)s_cnt[q][0]);
        if (s_cnt[q][1]) atomicAdd(tl + T_SCATTERS, (double)s_cnt[q][1]);
    }
}

}  // namespace

cudaError_t launch_batch_transport(const BatchTrInst *insts, int n, int64_t total, unsigned long long *work,
                                   int scat_min, int sm_count, cudaStream_t s)
{
    if (n < 1 || n > MAX_BATCH_TR || total <= 0) return n < 1 || total <= 0 ? cudaSuccess : cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_transport_kernel, BTPB, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = (int64_t)sm_count * per_sm;
    const int64_t need = (total + BTPB - 1) / BTPB;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    count_launch();
    batch_transport_kernel<<<(unsigned)blocks, BTPB, 0, s>>>(insts, n, total, work, scat_min > 0 ? scat_min : 20);
    return cudaGetLastError();
}

}  // namespace tam
