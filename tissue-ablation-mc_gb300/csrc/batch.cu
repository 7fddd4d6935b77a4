// batch.cu -- the FP32 heat step of many independent instances in one
// persistent launch.
//
// The batched workload runs tens of tissue instances of uneven sizes; their
// individual heat steps are too short to keep the device busy one launch at a
// time.  Here one cooperative launch (one resident block per slot, every block
// co-resident) advances every instance by K steps: for each step the blocks
// share out the tile columns of all instances, and a software grid barrier
// separates the steps.  The barrier's wait is bounded; a block that gives up
// records DEVERR_SYNC_TIMEOUT and every block leaves at its next barrier.
//
// The per-voxel arithmetic is that of the class-table FP32 step: thermal
// properties by material class, face coefficients k_f/(rho_f c_f) from the
// per-instance class table, Kahan-compensated temperature, latent-heat clamp,
// Arrhenius damage and ablation (rare_update_f32).  Neighbours are read with
// cached global loads (any row pitch: the instances' edges need not be
// multiples of four), the z column stays in registers.
#include <cstdint>

#include "heat_common.cuh"

namespace tam {

namespace {

constexpr long long BARRIER_CYCLES = 4000000000ll;  // ~2 s at 2 GHz

// Bounded grid-wide barrier for co-resident blocks.  Returns false (for the
// whole block) once any block has flagged a time-out.
__device__ bool grid_barrier(BatchSync *g, unsigned nblocks, unsigned *err)
{
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        volatile unsigned *gen = &g->gen;
        volatile unsigned *abort_flag = &g->abort;
        const unsigned my = *gen;
        __threadfence();
        if (atomicAdd(&g->count, 1u) == nblocks - 1) {
            g->count = 0;
            __threadfence();
            atomicAdd(&g->gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*gen == my) {
                if (*abort_flag) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > BARRIER_CYCLES) {
                    atomicOr(err, (unsigned)DEVERR_SYNC_TIMEOUT);
                    atomicExch(&g->abort, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*abort_flag) ok = 0;
    }
    return __syncthreads_and(ok) != 0;
}

// Laplacian of a voxel with a face on the grid boundary: ghost faces carry
// the voxel's own properties (kept out of line: boundary voxels are few).
__device__ __noinline__ float boundary_lap(const BatchInst &I, const float *row, const float *T, const float *E,
                                           int v, int cv, int x, int y, int z, int kc, int kp, int kn,
                                           float Tc, float ec, float tzm, float tzp)
{
    const FusedArgs &a = I.a;
    const int nx = a.nx, ny = a.ny, nz = a.nz, cp = I.cls_pitch;
    const int sy = nx;
    const float cx = a.fc[FC_CX], cy = a.fc[FC_CY], cz = a.fc[FC_CZ];
    const float kk = I.L.k[kc], rr = I.L.rho[kc], hh = I.L.c[kc];
    float lap = z > 0 ? cz * row[kp] * tzm : ghost_term<float>(a, 4, Tc, ec, kk, rr, hh);
    lap += z + 1 < nz ? cz * row[kn] * tzp : ghost_term<float>(a, 5, Tc, ec, kk, rr, hh);
    if (y > 0) lap += cy * row[__ldg(I.cls + cv - cp) & (MAX_MAT - 1)] * ((__ldg(T + v - sy) - Tc) - (__ldg(E + v - sy) - ec));
    else lap += ghost_term<float>(a, 2, Tc, ec, kk, rr, hh);
    if (y < ny - 1) lap += cy * row[__ldg(I.cls + cv + cp) & (MAX_MAT - 1)] * ((__ldg(T + v + sy) - Tc) - (__ldg(E + v + sy) - ec));
    else lap += ghost_term<float>(a, 3, Tc, ec, kk, rr, hh);
    if (x > 0) lap += cx * row[__ldg(I.cls + cv - 1) & (MAX_MAT - 1)] * ((__ldg(T + v - 1) - Tc) - (__ldg(E + v - 1) - ec));
    else lap += ghost_term<float>(a, 0, Tc, ec, kk, rr, hh);
    if (x < nx - 1) lap += cx * row[__ldg(I.cls + cv + 1) & (MAX_MAT - 1)] * ((__ldg(T + v + 1) - Tc) - (__ldg(E + v + 1) - ec));
    else lap += ghost_term<float>(a, 1, Tc, ec, kk, rr, hh);
    return lap;
}

// Latent-heat clamp of a voxel at or above the boiling temperature
// (src/3dFD.f90:169-175): true when the voxel absorbed the step's energy.
__device__ __noinline__ bool boil_clamp(const FusedArgs &a, const ClassLut &L, int kc, int v, float sPJ, float dT)
{
    float *Q = (float *)a.Q;
    const float rr = L.rho[kc], rc = rr * L.c[kc];
    const float qv = a.fc[FC_LW] * rr * a.fc[FC_VVOX];
    const float Qv = Q[v];
    if (Qv < qv) {
        const float Ein = (sPJ + rc * dT) * a.fc[FC_VVOX];
        if (Ein > 0.f) {
            const float qn = Qv + Ein;
            Q[v] = qn < qv ? qn : qv;
            return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(FX *FY, 4)
    batch_heat_kernel(const BatchInst *__restrict__ insts, int n, const int *__restrict__ prefix,
                      const BatchStep *__restrict__ steps, int K, BatchSync *sync, unsigned *err)
{
    __shared__ float s_fa[MAX_MAT * MAX_MAT];
    __shared__ int s_inst;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int total = prefix[n];
    int loaded = -1;
    for (int k = 0; k < K; ++k) {
        for (int item = blockIdx.x; item < total; item += gridDim.x) {
            // instance of this work item: last i with prefix[i] <= item
            if (tx == 0 && ty == 0) {
                int lo = 0, hi = n - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (prefix[mid] <= item) lo = mid;
                    else hi = mid - 1;
                }
                s_inst = lo;
            }
            __syncthreads();
            const int i = s_inst;
            const BatchInst &I = insts[i];
            const BatchStep st = steps[(int64_t)k * n + i];
            if (i != loaded) {
                for (int t = ty * FX + tx; t < MAX_MAT * MAX_MAT; t += FX * FY) s_fa[t] = I.L.fa[t];
                loaded = i;
            }
            __syncthreads();
            if (!st.active) continue;  // block-uniform
            const FusedArgs &a = I.a;
            const int local = item - prefix[i];
            const int bx = local % I.tiles_x, by = (local / I.tiles_x) % I.tiles_y, bz = local / (I.tiles_x * I.tiles_y);
            const int nx = a.nx, ny = a.ny, nz = a.nz;
            const int x = bx * FX + tx, y = by * FY + ty;
            if (x >= nx || y >= ny) continue;
            const int z0 = bz * I.zchunk, z1 = min(nz, z0 + I.zchunk);
            const int src = (I.fcur + k) & 1;
            const float *T = I.T[src], *E = I.E[src];
            float *To = I.T[src ^ 1], *Eo = I.E[src ^ 1];
            const float *J = (const float *)a.J;
            // instances hold fewer than 2^31 voxels (checked on the host)
            const int sy = nx, sz = nx * ny, ni = sz * nz;
            const int cp = I.cls_pitch;
            const int csz = cp * ny;
            const float cx = a.fc[FC_CX], cy = a.fc[FC_CY], cz = a.fc[FC_CZ], dt = a.fc[FC_DT];
            const float Pdt = st.pdt;
            const bool xy_inner = x > 0 && x < nx - 1 && y > 0 && y < ny - 1;
            int v = x + sy * y + sz * z0;
            int cv = x + cp * y + csz * z0;
            float Tp = 0.f, ep = 0.f;
            int kp = 0;
            if (z0 > 0) {
                Tp = __ldg(T + v - sz);
                ep = __ldg(E + v - sz);
                kp = __ldg(I.cls + cv - csz) & (MAX_MAT - 1);
            }
            float Tc = __ldg(T + v), ec = __ldg(E + v);
            int kc = __ldg(I.cls + cv) & (MAX_MAT - 1);
            // the plane above is loaded one iteration ahead, so its latency
            // overlaps the update of the current plane
            float Tn_ = 0.f, en_ = 0.f;
            int kn = 0;
            if (z0 + 1 < nz) {
                Tn_ = __ldg(T + v + sz);
                en_ = __ldg(E + v + sz);
                kn = __ldg(I.cls + cv + csz) & (MAX_MAT - 1);
            }
            unsigned errbits = 0;
            for (int z = z0; z < z1; ++z, v += sz, cv += csz) {
                const bool has_n = z + 1 < nz;
                float Tn2 = 0.f, en2 = 0.f;
                int kn2 = 0;
                if (z + 2 < nz) {
                    Tn2 = __ldg(T + v + 2 * sz);
                    en2 = __ldg(E + v + 2 * sz);
                    kn2 = __ldg(I.cls + cv + 2 * csz) & (MAX_MAT - 1);
                }
                const float *row = s_fa + kc * MAX_MAT;
                const float tzm = (Tp - Tc) - (ep - ec), tzp = (Tn_ - Tc) - (en_ - ec);
                float lap;
                if (xy_inner && z > 0 && has_n) {
                    const float txm = (__ldg(T + v - 1) - Tc) - (__ldg(E + v - 1) - ec);
                    const float txp = (__ldg(T + v + 1) - Tc) - (__ldg(E + v + 1) - ec);
                    const float tym = (__ldg(T + v - sy) - Tc) - (__ldg(E + v - sy) - ec);
                    const float typ = (__ldg(T + v + sy) - Tc) - (__ldg(E + v + sy) - ec);
                    lap = cz * (row[kp] * tzm + row[kn] * tzp) +
                          cy * (row[__ldg(I.cls + cv - cp) & (MAX_MAT - 1)] * tym +
                                row[__ldg(I.cls + cv + cp) & (MAX_MAT - 1)] * typ) +
                          cx * (row[__ldg(I.cls + cv - 1) & (MAX_MAT - 1)] * txm +
                                row[__ldg(I.cls + cv + 1) & (MAX_MAT - 1)] * txp);
                } else {
                    lap = boundary_lap(I, row, T, E, v, cv, x, y, z, kc, kp, kn, Tc, ec, tzm, tzp);
                }
                const float dT = dt * lap;
                const float sPJ = Pdt != 0.f ? Pdt * __ldg(J + v) : 0.f;
                const float srcT = sPJ * I.L.irc[kc];
                float Tnew = a.fc[FC_TBOIL], Enew = 0.f;
                const bool clamped = a.boil && Tc >= a.fc[FC_TBOIL] && boil_clamp(a, I.L, kc, v, sPJ, dT);
                if (!clamped) {
                    const float inc = dT + srcT;
                    const float yk = inc - ec;
                    const float t = Tc + yk;
                    Enew = (t - Tc) - yk;
                    Tnew = t;
                }
                To[v] = Tnew;
                Eo[v] = Enew;
                const float Ts = Tnew - Enew;
                if (!(Ts == Ts)) errbits |= DEVERR_NAN;
                else if (Ts < 0.f) errbits |= DEVERR_NEG_T;
                if (Ts >= a.fc[FC_SCREEN]) rare_update_f32(a, v, ni, Tnew, Enew, st.t_new);
                Tp = Tc;
                ep = ec;
                kp = kc;
                Tc = Tn_;
                ec = en_;
                kc = kn;
                Tn_ = Tn2;
                en_ = en2;
                kn = kn2;
            }
            if (errbits) atomicOr(a.err, errbits);
        }
        if (!grid_barrier(sync, gridDim.x, err)) return;
    }
}

}  // namespace

cudaError_t batch_heat_blocks(int *blocks)
{
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_heat_kernel, FX * FY, 0);
    if (e != cudaSuccess) return e;
    *blocks = sms * (per > 0 ? per : 1);
    return cudaSuccess;
}

cudaError_t launch_batch_heat(const BatchInst *insts, int n, const int *prefix, const BatchStep *steps, int K,
                              BatchSync *sync, unsigned *err, int blocks, cudaStream_t s)
{
    if (n <= 0 || K <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(sync, 0, sizeof(BatchSync), s);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&insts, (void *)&n, (void *)&prefix, (void *)&steps, (void *)&K, (void *)&sync,
                    (void *)&err};
    count_launch();
    return cudaLaunchCooperativeKernel((const void *)batch_heat_kernel, dim3(blocks), dim3(FX, FY), args, 0, s);
}

}  // namespace tam
