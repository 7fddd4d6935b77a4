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
// Arrhenius damage and ablation (rare_update_f32).  Three forms, chosen by
// "batch.staged": the default stages each tile's planes in shared memory with
// 4-byte cp.async copies (any row pitch: the instances' edges need not be
// multiples of four) and updates two x-adjacent voxels per thread
// (batch_pairs_kernel, whose one-step form also serves single contexts with
// such rows); batch_staged_kernel does the same with one voxel per thread;
// batch_heat_kernel reads neighbours with cached global loads.
#include <cstdint>

#include "grid_sync.cuh"
#include "heat_common.cuh"

namespace tam {

namespace {

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

// ------------------------------------------------ staged class-table step --
// The same per-voxel update with the tile's planes staged in shared memory by
// cp.async (LDGSTS, 4-byte copies: instance rows need not be 16-byte aligned)
// through a ring of AS stages, AD planes ahead of the plane being updated.
// The block's work items are tile columns of a z-chunk, across instances.
// Per voxel: T, the Kahan term, J and the class id read once
// from HBM (tile halos from L2), T and the Kahan term written once.
__device__ __forceinline__ void async4(void *s, const void *g)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(g)
                 : "memory");
}
__device__ __forceinline__ void async16(void *s, const void *g)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(s)),
                 "l"(g)
                 : "memory");
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int AS = 6;                  // ring stages
constexpr int AD = AS - 1;             // planes in flight: plane i + AD is issued at the update of plane i
constexpr int AP = 40;                 // floats per staged T / E row: x0 - 4 .. x0 + 35
constexpr int AR = FY + 2;             // staged rows y0 - 1 .. y0 + 8
constexpr int ACP = 64;                // class bytes per staged row: x0 - 16 .. x0 + 47
constexpr int A_T = 0, A_E = AR * AP * 4, A_J = 2 * AR * AP * 4, A_C = A_J + FX * FY * 4;
constexpr int A_STAGE = ((A_C + AR * ACP + 127) / 128) * 128;  // 4864 bytes
constexpr int A_SMEM = AS * A_STAGE + 128;                     // + alignment slack

// Tile column of one instance: voxels x0..x0+31, y0..y0+7, z0..z1-1.
struct Item {
    int inst, x0, y0, z0, z1;
};

__device__ __forceinline__ Item item_at(const BatchInst *insts, int n, const int *prefix, int item)
{
    int lo = 0, hi = n - 1;  // last i with prefix[i] <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= item) lo = mid;
        else hi = mid - 1;
    }
    const BatchInst &I = insts[lo];
    const int local = item - __ldg(prefix + lo), tx = I.tiles_x, ty = I.tiles_y;
    Item it;
    it.inst = lo;
    it.x0 = (local % tx) * FX;
    it.y0 = ((local / tx) % ty) * FY;
    it.z0 = (local / (tx * ty)) * I.zchunk;
    it.z1 = min(I.a.nz, it.z0 + I.zchunk);
    return it;
}

// Per-thread copies of every plane of an item (offsets within a plane; -1:
// no copy): own voxel, one halo element (rows y0-1 / y0+8 by the first two
// warps, columns x0-1 / x0+32 by lanes 1-8 of the next two) and one 16-byte
// chunk of class ids (warps 4-5, four chunks per staged row).
struct Offs {
    int own, ext, c;
    int sx;  // shared offsets: halo element (floats) in the low 16 bits, class chunk (bytes) in the high
};

__device__ __forceinline__ Offs offsets_for(int nx, int ny, int cp, bool uni, const Item &it, int tx, int ty)
{
    Offs o;
    const int x = it.x0 + tx, y = it.y0 + ty;
    int s_ext = 0, s_c = 0;
    o.own = (x < nx && y < ny) ? x + nx * y : -1;
    o.ext = -1;
    if (ty == 0) {
        if (it.y0 > 0 && x < nx) o.ext = x + nx * (it.y0 - 1), s_ext = tx + 4;
    } else if (ty == 1) {
        if (it.y0 + FY < ny && x < nx) o.ext = x + nx * (it.y0 + FY), s_ext = (FY + 1) * AP + tx + 4;
    } else if ((ty == 2 || ty == 3) && tx >= 1 && tx <= FY) {
        const int yy = it.y0 - 1 + tx;
        if (ty == 2 && it.x0 > 0 && yy < ny) o.ext = it.x0 - 1 + nx * yy, s_ext = tx * AP + 3;
        if (ty == 3 && it.x0 + FX < nx && yy < ny) o.ext = it.x0 + FX + nx * yy, s_ext = tx * AP + FX + 4;
    }
    o.c = -1;
    const int q = (ty - 4) * FX + tx;
    if (!uni && q >= 0 && q < AR * 4) {
        const int r = q >> 2, ch = q & 3;
        const int yy = it.y0 - 1 + r, xb = it.x0 - 16 + 16 * ch;
        if (yy >= 0 && yy < ny && xb >= 0 && xb + 16 <= cp) o.c = xb + cp * yy, s_c = r * ACP + 16 * ch;
    }
    o.sx = s_ext | s_c << 16;
    return o;
}

// Block-uniform description of the item being updated, in shared memory
// (written by one thread, read after a barrier) so that it holds no
// registers: where its planes come from and go to, and the step's source.
struct __align__(16) Src {
    const float *T, *E;
    const float *J;
    const uint8_t *C;
    float *To, *Eo;
    double t_new;
    int sz, csz, nz, z0;
    int np, jon, nx, ny;
    float pdt;
};

// Issue the copies of plane p (z = z0 - 1 + p, nothing past z1 or outside
// the grid) into stage b; every call commits one group.
__device__ __forceinline__ void issue_plane(const Src &d, const Offs &o, int p, unsigned char *b, int tx, int ty)
{
    const int zz = d.z0 - 1 + p;
    if (p <= d.np + 1 && zz >= 0 && zz < d.nz) {
        const int po = d.sz * zz;
        float *bT = (float *)(b + A_T), *bE = (float *)(b + A_E);
        if (o.own >= 0) {
            const int so = (ty + 1) * AP + tx + 4;
            async4(bT + so, d.T + po + o.own);
            async4(bE + so, d.E + po + o.own);
            if (d.jon && p >= 1 && p <= d.np) async4((float *)(b + A_J) + ty * FX + tx, d.J + po + o.own);
        }
        if (o.ext >= 0) {
            const int se = o.sx & 0xffff;
            async4(bT + se, d.T + po + o.ext);
            async4(bE + se, d.E + po + o.ext);
        }
        if (o.c >= 0) async16(b + A_C + (o.sx >> 16), d.C + d.csz * zz + o.c);
    }
    async_commit();
}

// Sum of the ghost terms of the boundary faces in mask gm (bit f = face f).
__device__ __forceinline__ float ghost_sum(const FusedArgs &a, const ClassLut &L, unsigned gm, int kc, float Tc,
                                           float ec)
{
    return ghost_faces(a, gm, Tc, ec, L.k[kc], L.rho[kc], L.c[kc]);
}

constexpr int ARGS_WORDS = (int)(sizeof(FusedArgs) / 4), LUT_WORDS = (int)(sizeof(ClassLut) / 4);
static_assert(sizeof(FusedArgs) % 4 == 0 && sizeof(ClassLut) % 4 == 0, "word copies");

// K steps of every instance (GRID: persistent cooperative launch, items
// strided over the grid, a bounded grid barrier between steps) or one step
// with one item per block (!GRID, K == 1).  Each item streams its planes
// z0-1 .. z1 through the ring, AD - 2 planes ahead of the next one needed;
// the instance's constants and class table sit in shared memory.
#ifndef TAM_STAGED_MINB
#define TAM_STAGED_MINB 3
#endif
template <bool GRID>
__global__ void __launch_bounds__(FX *FY, TAM_STAGED_MINB)
    batch_staged_kernel(const BatchInst *__restrict__ insts, int n, const int *__restrict__ prefix,
                        const BatchStep *__restrict__ steps, int K, BatchSync *sync, unsigned *err)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(16) unsigned char s_args_raw[sizeof(FusedArgs)];
    __shared__ __align__(16) unsigned char s_lut_raw[sizeof(ClassLut)];
    __shared__ Src d;
    const FusedArgs &A = *reinterpret_cast<const FusedArgs *>(s_args_raw);
    const ClassLut &L = *reinterpret_cast<const ClassLut *>(s_lut_raw);
    unsigned char *sm = smem_raw + ((128 - ((unsigned)__cvta_generic_to_shared(smem_raw) & 127)) & 127);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * FX + tx;
    const int total = __ldg(prefix + n);
    const int stride = GRID ? (int)gridDim.x : total;
    int loaded = -1;
    for (int k = 0; k < K; ++k) {
        for (int item = blockIdx.x; item < total; item += stride) {
            const Item it = item_at(insts, n, prefix, item);
            const BatchStep st = steps[(int64_t)k * n + it.inst];
            if (!st.active) continue;  // block-uniform
            const BatchInst &I = insts[it.inst];
            // every thread finished the previous item (its last barrier)
            if (it.inst != loaded) {
                for (int w = tid; w < ARGS_WORDS; w += FX * FY)
                    ((uint32_t *)s_args_raw)[w] = ((const uint32_t *)&I.a)[w];
                for (int w = tid; w < LUT_WORDS; w += FX * FY)
                    ((uint32_t *)s_lut_raw)[w] = ((const uint32_t *)&I.L)[w];
                loaded = it.inst;
            }
            if (tid == 0) {
                const int fc = (I.fcur + k) & 1;
                d.T = I.T[fc];
                d.E = I.E[fc];
                d.To = I.T[fc ^ 1];
                d.Eo = I.E[fc ^ 1];
                d.J = (const float *)I.a.J;
                d.C = I.cls;
                d.nx = I.a.nx;
                d.ny = I.a.ny;
                d.sz = I.a.nx * I.a.ny;
                d.csz = I.cls_pitch * I.a.ny;
                d.nz = I.a.nz;
                d.z0 = it.z0;
                d.np = it.z1 - it.z0;
                d.jon = st.pdt != 0.f;
                d.pdt = st.pdt;
                d.t_new = st.t_new;
            }
            const int uc = I.L.uniform;
            const Offs o = offsets_for(I.a.nx, I.a.ny, I.cls_pitch, uc >= 0, it, tx, ty);
            __syncthreads();  // the item's description is visible
            // planes 0 .. AD-1 (z0-1 .. z0+AD-2) in flight
#pragma unroll
            for (int p = 0; p < AD; ++p) issue_plane(d, o, p, sm + p * A_STAGE, tx, ty);
            async_wait<AD - 2>();
            __syncthreads();  // planes 0 and 1 (and the instance's tables) are visible to the block
            const int x = it.x0 + tx, y = it.y0 + ty;
            const bool own = o.own >= 0;
            const bool xy_inner = x > 0 && x < d.nx - 1 && y > 0 && y < d.ny - 1;
            const int so = (ty + 1) * AP + tx + 4, co = (ty + 1) * ACP + tx + 16;
            float Tp = 0.f, ep = 0.f, Tc = 0.f, ec = 0.f;
            int kp = uc, kc = uc;
            if (own) {
                if (it.z0 > 0) {
                    Tp = ((const float *)(sm + A_T))[so];
                    ep = ((const float *)(sm + A_E))[so];
                    if (uc < 0) kp = (sm + A_C)[co] & (MAX_MAT - 1);
                }
                Tc = ((const float *)(sm + A_STAGE + A_T))[so];
                ec = ((const float *)(sm + A_STAGE + A_E))[so];
                if (uc < 0) kc = (sm + A_STAGE + A_C)[co] & (MAX_MAT - 1);
            }
            int v = x + d.nx * y + d.sz * it.z0;
            unsigned errbits = 0;
            int si = AD % AS, sc = 1, sn = 2;  // stages: next issue, plane z, plane z+1
            for (int i = 0; i < d.np; ++i, v += d.sz) {
                issue_plane(d, o, i + AD, sm + si * A_STAGE, tx, ty);
                async_wait<AD - 2>();
                __syncthreads();  // plane z+1 has landed for the whole block
                const unsigned char *P = sm + sc * A_STAGE, *N = sm + sn * A_STAGE;
                const int z = it.z0 + i;
                const bool has_n = z + 1 < d.nz;
                float Tn_ = 0.f, en_ = 0.f;
                int kn = uc;
                if (own && has_n) {
                    Tn_ = ((const float *)(N + A_T))[so];
                    en_ = ((const float *)(N + A_E))[so];
                    if (uc < 0) kn = (N + A_C)[co] & (MAX_MAT - 1);
                }
                if (own) {
                    const float *PT = (const float *)(P + A_T), *PE = (const float *)(P + A_E);
                    const float *row = L.fa + kc * MAX_MAT;
                    const float Jv = d.jon ? ((const float *)(P + A_J))[ty * FX + tx] : 0.f;
                    const bool near = Tc >= A.fc[FC_SCREEN];
                    double o_pre = 0.0;
                    if (near) o_pre = A.omega[v];
                    const float tzm = (Tp - Tc) - (ep - ec), tzp = (Tn_ - Tc) - (en_ - ec);
                    const float txm = (PT[so - 1] - Tc) - (PE[so - 1] - ec), txp = (PT[so + 1] - Tc) - (PE[so + 1] - ec);
                    const float tym = (PT[so - AP] - Tc) - (PE[so - AP] - ec),
                                typ = (PT[so + AP] - Tc) - (PE[so + AP] - ec);
                    float axm, axp, aym, ayp;
                    if (uc >= 0) {
                        axm = axp = aym = ayp = row[uc];
                    } else {
                        const unsigned char *PC = P + A_C;
                        axm = row[PC[co - 1] & (MAX_MAT - 1)];
                        axp = row[PC[co + 1] & (MAX_MAT - 1)];
                        aym = row[PC[co - ACP] & (MAX_MAT - 1)];
                        ayp = row[PC[co + ACP] & (MAX_MAT - 1)];
                    }
                    const float azm = row[kp], azp = row[kn];
                    const float cx = A.fc[FC_CX], cy = A.fc[FC_CY], cz = A.fc[FC_CZ];
                    float lap;
                    if (xy_inner && z > 0 && has_n) {
                        lap = (cz * (azm * tzm + azp * tzp) + cy * (aym * tym + ayp * typ)) + cx * (axm * txm + axp * txp);
                    } else {
                        // faces on the grid boundary (bit f: x-, x+, y-, y+, z-, z+)
                        // take the ghost term instead of the neighbour's
                        const unsigned gm = (unsigned)(x == 0) | (unsigned)(x == d.nx - 1) << 1 | (unsigned)(y == 0) << 2 |
                                            (unsigned)(y == d.ny - 1) << 3 | (unsigned)(z == 0) << 4 |
                                            (unsigned)(!has_n) << 5;
                        lap = (cz * ((gm & 16 ? 0.f : azm * tzm) + (gm & 32 ? 0.f : azp * tzp)) +
                               cy * ((gm & 4 ? 0.f : aym * tym) + (gm & 8 ? 0.f : ayp * typ))) +
                              cx * ((gm & 1 ? 0.f : axm * txm) + (gm & 2 ? 0.f : axp * txp));
                        lap += ghost_sum(A, L, gm, kc, Tc, ec);
                    }
                    const float dT = A.fc[FC_DT] * lap;
                    const float sPJ = d.pdt * Jv;
                    const float srcT = sPJ * L.irc[kc];
                    float Tnew = A.fc[FC_TBOIL], Enew = A.fc[FC_TBOIL_E];
                    const bool clamped = A.boil && Tc >= Tnew && boil_clamp(A, L, kc, v, sPJ, dT);
                    if (!clamped) {
                        const float inc = dT + srcT;
                        const float yk = inc - ec;
                        const float t = Tc + yk;
                        Enew = (t - Tc) - yk;
                        Tnew = t;
                    }
                    d.To[v] = Tnew;
                    d.Eo[v] = Enew;
                    const float Ts = Tnew - Enew;
                    errbits |= (Ts == Ts) ? (Ts < 0.f ? (unsigned)DEVERR_NEG_T : 0u) : (unsigned)DEVERR_NAN;
                    if (Ts >= A.fc[FC_SCREEN])
                        rare_update_f32(A, v, (int64_t)d.sz * d.nz, Tnew, Enew, d.t_new, near, o_pre);
                }
                Tp = Tc;
                ep = ec;
                kp = kc;
                Tc = Tn_;
                ec = en_;
                kc = kn;
                si = si + 1 == AS ? 0 : si + 1;
                sc = sn;
                sn = sn + 1 == AS ? 0 : sn + 1;
                // no barrier here: the issue of the next iteration overwrites the
                // stage of plane z-1, last read one iteration ago, before the
                // barrier every thread has passed
            }
            async_wait<0>();
            __syncthreads();  // the next item rewrites the stages and the instance's tables
            if (errbits) atomicOr(I.a.err, errbits);  // (the shared copy may already hold the next instance)
        }
        if (GRID && k + 1 < K && !grid_barrier(sync, gridDim.x, err)) return;
    }
}

// ------------------------------------------- staged step, voxel pairs --
// The staged step with 128 threads per 32 x 8 tile, each updating two
// x-adjacent voxels: 64-bit shared-memory loads of a pair's own, y- and
// z-neighbour values and J, its inner x-neighbours from registers.  The
// stage layout and the ring are those of the one-voxel form.
struct Offs2 {
    int own, ext, c;
    int sx;  // halo (floats) in bits 0-15, class chunk (bytes) in bits 16-30
    int next, n1;  // halo elements (0, 1 or 2); second own voxel present
};

__device__ __forceinline__ Offs2 offsets2_for(int nx, int ny, int cp, bool uni, const Item &it, int tp, int ty)
{
    Offs2 o;
    const int tx = 2 * tp, x = it.x0 + tx, y = it.y0 + ty;
    int s_ext = 0, s_c = 0;
    o.own = (x < nx && y < ny) ? x + nx * y : -1;
    o.n1 = x + 1 < nx;
    o.ext = -1;
    o.next = 0;
    if (ty == 0 || ty == 1) {
        const int yy = ty == 0 ? it.y0 - 1 : it.y0 + FY;
        if (yy >= 0 && yy < ny && x < nx) {
            o.ext = x + nx * yy;
            o.next = x + 1 < nx ? 2 : 1;
            s_ext = (ty == 0 ? 0 : (FY + 1) * AP) + tx + 4;
        }
    } else if ((ty == 2 || ty == 3) && tp >= 1 && tp <= FY) {
        const int yy = it.y0 - 1 + tp;
        if (ty == 2 && it.x0 > 0 && yy < ny) o.ext = it.x0 - 1 + nx * yy, o.next = 1, s_ext = tp * AP + 3;
        if (ty == 3 && it.x0 + FX < nx && yy < ny) o.ext = it.x0 + FX + nx * yy, o.next = 1, s_ext = tp * AP + FX + 4;
    }
    o.c = -1;
    const int q = (ty - 4) * (FX / 2) + tp;
    if (!uni && q >= 0 && q < AR * 4) {
        const int r = q >> 2, ch = q & 3;
        const int yy = it.y0 - 1 + r, xb = it.x0 - 16 + 16 * ch;
        if (yy >= 0 && yy < ny && xb >= 0 && xb + 16 <= cp) o.c = xb + cp * yy, s_c = r * ACP + 16 * ch;
    }
    o.sx = s_ext | s_c << 16;
    return o;
}

__device__ __forceinline__ void issue_plane2(const Src &d, const Offs2 &o, int p, unsigned char *b, int tp, int ty)
{
    const int zz = d.z0 - 1 + p;
    if (p <= d.np + 1 && zz >= 0 && zz < d.nz) {
        const int po = d.sz * zz;
        float *bT = (float *)(b + A_T), *bE = (float *)(b + A_E);
        if (o.own >= 0) {
            const int so = (ty + 1) * AP + 2 * tp + 4;
            const float *gT = d.T + po + o.own, *gE = d.E + po + o.own;
            async4(bT + so, gT);
            async4(bE + so, gE);
            if (o.n1) {
                async4(bT + so + 1, gT + 1);
                async4(bE + so + 1, gE + 1);
            }
            if (d.jon && p >= 1 && p <= d.np) {
                float *bJ = (float *)(b + A_J) + ty * FX + 2 * tp;
                const float *gJ = d.J + po + o.own;
                async4(bJ, gJ);
                if (o.n1) async4(bJ + 1, gJ + 1);
            }
        }
        if (o.next) {
            const int se = o.sx & 0xffff;
            const float *gT = d.T + po + o.ext, *gE = d.E + po + o.ext;
            async4(bT + se, gT);
            async4(bE + se, gE);
            if (o.next == 2) {
                async4(bT + se + 1, gT + 1);
                async4(bE + se + 1, gE + 1);
            }
        }
        if (o.c >= 0) async16(b + A_C + (o.sx >> 16), d.C + d.csz * zz + o.c);
    }
    async_commit();
}

#ifndef TAM_PAIRS_MINB
#define TAM_PAIRS_MINB 5  // 96 registers without spills; 6 blocks spill and run 25 % slower
#endif
// GRID: K steps of every instance (persistent cooperative launch).  !GRID:
// one step of one instance, one block per item; the step (`one`) and the
// buffer pair it reads (`one_fcur`) come as parameters.
template <bool GRID>
__global__ void __launch_bounds__(FX / 2 * FY, TAM_PAIRS_MINB)
    batch_pairs_kernel(const BatchInst *__restrict__ insts, int n, const int *__restrict__ prefix,
                       const BatchStep *__restrict__ steps, int K, BatchSync *sync, unsigned *err, BatchStep one,
                       int one_fcur)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(16) unsigned char s_args_raw[sizeof(FusedArgs)];
    __shared__ __align__(16) unsigned char s_lut_raw[sizeof(ClassLut)];
    __shared__ Src d;
    const FusedArgs &A = *reinterpret_cast<const FusedArgs *>(s_args_raw);
    const ClassLut &L = *reinterpret_cast<const ClassLut *>(s_lut_raw);
    unsigned char *sm = smem_raw + ((128 - ((unsigned)__cvta_generic_to_shared(smem_raw) & 127)) & 127);
    const int tp = threadIdx.x, ty = threadIdx.y, tid = ty * (FX / 2) + tp;
    const int total = __ldg(prefix + n);
    const int stride = GRID ? (int)gridDim.x : total;
    int loaded = -1;
    for (int k = 0; k < K; ++k) {
        for (int item = blockIdx.x; item < total; item += stride) {
            const Item it = item_at(insts, n, prefix, item);
            const BatchStep st = GRID ? steps[(int64_t)k * n + it.inst] : one;
            if (!st.active) continue;  // block-uniform
            const BatchInst &I = insts[it.inst];
            // every thread finished the previous item (its last barrier)
            if (it.inst != loaded) {
                for (int w = tid; w < ARGS_WORDS; w += FX / 2 * FY)
                    ((uint32_t *)s_args_raw)[w] = ((const uint32_t *)&I.a)[w];
                for (int w = tid; w < LUT_WORDS; w += FX / 2 * FY)
                    ((uint32_t *)s_lut_raw)[w] = ((const uint32_t *)&I.L)[w];
                loaded = it.inst;
            }
            if (tid == 0) {
                const int fc = ((GRID ? I.fcur : one_fcur) + k) & 1;
                d.T = I.T[fc];
                d.E = I.E[fc];
                d.To = I.T[fc ^ 1];
                d.Eo = I.E[fc ^ 1];
                d.J = (const float *)I.a.J;
                d.C = I.cls;
                d.nx = I.a.nx;
                d.ny = I.a.ny;
                d.sz = I.a.nx * I.a.ny;
                d.csz = I.cls_pitch * I.a.ny;
                d.nz = I.a.nz;
                d.z0 = it.z0;
                d.np = it.z1 - it.z0;
                d.jon = st.pdt != 0.f;
                d.pdt = st.pdt;
                d.t_new = st.t_new;
            }
            const int uc = I.L.uniform;
            const Offs2 o = offsets2_for(I.a.nx, I.a.ny, I.cls_pitch, uc >= 0, it, tp, ty);
            __syncthreads();  // the item's description is visible
#pragma unroll 1
            for (int p = 0; p < AD; ++p) issue_plane2(d, o, p, sm + p * A_STAGE, tp, ty);
            async_wait<AD - 2>();
            __syncthreads();  // planes 0 and 1 (and the instance's tables) are visible to the block
            const int tx = 2 * tp, x = it.x0 + tx, y = it.y0 + ty;
            const bool in0 = o.own >= 0, in1 = in0 && o.n1;
            const int q = (ty + 1) * AP + tx + 4, qc = (ty + 1) * ACP + tx + 16, oj = ty * FX + tx;
            auto cls2 = [&](const unsigned char *b, int &k0, int &k1) {
                const unsigned short w = *reinterpret_cast<const unsigned short *>(b + A_C + qc);
                k0 = w & (MAX_MAT - 1);
                k1 = (w >> 8) & (MAX_MAT - 1);
            };
            float2 Tp = {0.f, 0.f}, ep = {0.f, 0.f}, Tc = {0.f, 0.f}, ec = {0.f, 0.f};
            int kp0 = uc, kp1 = uc, kc0 = uc, kc1 = uc;
            if (in0) {
                if (it.z0 > 0) {
                    Tp = *reinterpret_cast<const float2 *>((const float *)(sm + A_T) + q);
                    ep = *reinterpret_cast<const float2 *>((const float *)(sm + A_E) + q);
                    if (uc < 0) cls2(sm, kp0, kp1);
                }
                Tc = *reinterpret_cast<const float2 *>((const float *)(sm + A_STAGE + A_T) + q);
                ec = *reinterpret_cast<const float2 *>((const float *)(sm + A_STAGE + A_E) + q);
                if (uc < 0) cls2(sm + A_STAGE, kc0, kc1);
            }
            int v = x + d.nx * y + d.sz * it.z0;
            unsigned errbits = 0;
            int si = AD % AS, sc = 1, sn = 2;  // stages: next issue, plane z, plane z+1
            for (int i = 0; i < d.np; ++i, v += d.sz) {
                issue_plane2(d, o, i + AD, sm + si * A_STAGE, tp, ty);
                async_wait<AD - 2>();
                __syncthreads();  // plane z+1 has landed for the whole block
                const unsigned char *P = sm + sc * A_STAGE, *N = sm + sn * A_STAGE;
                const int z = it.z0 + i;
                const bool has_n = z + 1 < d.nz;
                float2 Tn = {0.f, 0.f}, en = {0.f, 0.f};
                int kn0 = uc, kn1 = uc;
                if (in0 && has_n) {
                    Tn = *reinterpret_cast<const float2 *>((const float *)(N + A_T) + q);
                    en = *reinterpret_cast<const float2 *>((const float *)(N + A_E) + q);
                    if (uc < 0) cls2(N, kn0, kn1);
                }
                if (in0) {
                    const float *PT = (const float *)(P + A_T), *PE = (const float *)(P + A_E);
                    const float2 Ty0 = *reinterpret_cast<const float2 *>(PT + q - AP),
                                 Ty1 = *reinterpret_cast<const float2 *>(PT + q + AP);
                    const float2 Ey0 = *reinterpret_cast<const float2 *>(PE + q - AP),
                                 Ey1 = *reinterpret_cast<const float2 *>(PE + q + AP);
                    const float Txl = PT[q - 1], Txr = PT[q + 2], Exl = PE[q - 1], Exr = PE[q + 2];
                    const float2 Jv = d.jon ? *reinterpret_cast<const float2 *>((const float *)(P + A_J) + oj)
                                            : make_float2(0.f, 0.f);
                    const float screen = A.fc[FC_SCREEN];
                    const bool near0 = Tc.x >= screen, near1 = in1 && Tc.y >= screen;
                    double o_pre[2] = {0.0, 0.0};
                    if (near0) o_pre[0] = A.omega[v];
                    if (near1) o_pre[1] = A.omega[v + 1];
                    const float cx = A.fc[FC_CX], cy = A.fc[FC_CY], cz = A.fc[FC_CZ];
                    const bool yz_inner = y > 0 && y < d.ny - 1 && z > 0 && has_n;
                    // the pair's Laplacians; boundary faces, the latent-heat clamp and
                    // the damage update are rare and go through one call site each
                    float lap[2], tcs[2] = {Tc.x, Tc.y}, e0s[2] = {ec.x, ec.y};
                    int kks[2] = {kc0, kc1};
                    unsigned gms = 0;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int xx = x + h;
                        const float tc = tcs[h], e0 = e0s[h];
                        const float tzm = ((h ? Tp.y : Tp.x) - tc) - ((h ? ep.y : ep.x) - e0);
                        const float tzp = ((h ? Tn.y : Tn.x) - tc) - ((h ? en.y : en.x) - e0);
                        const float txm = ((h ? Tc.x : Txl) - tc) - ((h ? ec.x : Exl) - e0);
                        const float txp = ((h ? Txr : Tc.y) - tc) - ((h ? Exr : ec.y) - e0);
                        const float tym = ((h ? Ty0.y : Ty0.x) - tc) - ((h ? Ey0.y : Ey0.x) - e0);
                        const float typ = ((h ? Ty1.y : Ty1.x) - tc) - ((h ? Ey1.y : Ey1.x) - e0);
                        const float *row = L.fa + kks[h] * MAX_MAT;
                        float axm, axp, aym, ayp;
                        if (uc >= 0) {
                            axm = axp = aym = ayp = row[uc];
                        } else {
                            const unsigned char *PC = P + A_C;
                            axm = row[h ? kc0 : (PC[qc - 1] & (MAX_MAT - 1))];
                            axp = row[h ? (PC[qc + 2] & (MAX_MAT - 1)) : kc1];
                            aym = row[PC[qc + h - ACP] & (MAX_MAT - 1)];
                            ayp = row[PC[qc + h + ACP] & (MAX_MAT - 1)];
                        }
                        const float azm = row[h ? kp1 : kp0], azp = row[h ? kn1 : kn0];
                        if (yz_inner && xx > 0 && xx < d.nx - 1) {
                            lap[h] = (cz * (azm * tzm + azp * tzp) + cy * (aym * tym + ayp * typ)) +
                                     cx * (axm * txm + axp * txp);
                        } else {
                            const unsigned gm = (unsigned)(xx == 0) | (unsigned)(xx >= d.nx - 1) << 1 |
                                                (unsigned)(y == 0) << 2 | (unsigned)(y == d.ny - 1) << 3 |
                                                (unsigned)(z == 0) << 4 | (unsigned)(!has_n) << 5;
                            lap[h] = (cz * ((gm & 16 ? 0.f : azm * tzm) + (gm & 32 ? 0.f : azp * tzp)) +
                                      cy * ((gm & 4 ? 0.f : aym * tym) + (gm & 8 ? 0.f : ayp * typ))) +
                                     cx * ((gm & 1 ? 0.f : axm * txm) + (gm & 2 ? 0.f : axp * txp));
                            if (h == 0 || in1) gms |= gm << (8 * h);
                        }
                    }
#pragma unroll 1
                    for (int h = 0; h < 2; ++h)
                        if ((gms >> (8 * h)) & 0xffu)
                            (h ? lap[1] : lap[0]) += ghost_sum(A, L, (gms >> (8 * h)) & 0xffu, h ? kc1 : kc0,
                                                               h ? Tc.y : Tc.x, h ? ec.y : ec.x);
                    const float dt = A.fc[FC_DT], tboil = A.fc[FC_TBOIL];
                    float Tnew[2], Enew[2];
                    unsigned boil = 0, hot = 0;
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        if ((h == 0 || in1) && A.boil && tcs[h] >= tboil) boil |= 1u << h;
                    unsigned clamped = 0;
#pragma unroll 1
                    for (unsigned m = boil; m; m &= m - 1) {
                        const int h = __ffs(m) - 1;
                        if (boil_clamp(A, L, h ? kc1 : kc0, v + h, d.pdt * (h ? Jv.y : Jv.x), dt * (h ? lap[1] : lap[0])))
                            clamped |= 1u << h;
                    }
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const float tc = tcs[h], e0 = e0s[h];
                        const float sPJ = d.pdt * (h ? Jv.y : Jv.x);
                        float tn = tboil, en_ = A.fc[FC_TBOIL_E];
                        if (!(clamped >> h & 1u)) {
                            const float inc = dt * lap[h] + sPJ * L.irc[kks[h]];
                            const float yk = inc - e0;
                            const float t = tc + yk;
                            en_ = (t - tc) - yk;
                            tn = t;
                        }
                        Tnew[h] = tn;
                        Enew[h] = en_;
                        const float Ts = tn - en_;
                        if (h == 0 || in1) {
                            errbits |= (Ts == Ts) ? (Ts < 0.f ? (unsigned)DEVERR_NEG_T : 0u) : (unsigned)DEVERR_NAN;
                            if (Ts >= screen) hot |= 1u << h;
                        }
                    }
                    // damage and ablation of the pair's voxels in the window, from one call site
#pragma unroll 1
                    for (unsigned m = hot; m; m &= m - 1) {
                        const int h = __ffs(m) - 1;
                        rare_update_f32(A, v + h, (int64_t)d.sz * d.nz, h ? Tnew[1] : Tnew[0], h ? Enew[1] : Enew[0],
                                        d.t_new, h ? near1 : near0, h ? o_pre[1] : o_pre[0]);
                    }
                    float *To = d.To, *Eo = d.Eo;
                    if (in1 && !(v & 1)) {  // 8-byte aligned pair
                        *reinterpret_cast<float2 *>(To + v) = make_float2(Tnew[0], Tnew[1]);
                        *reinterpret_cast<float2 *>(Eo + v) = make_float2(Enew[0], Enew[1]);
                    } else {
                        To[v] = Tnew[0];
                        Eo[v] = Enew[0];
                        if (in1) {
                            To[v + 1] = Tnew[1];
                            Eo[v + 1] = Enew[1];
                        }
                    }
                }
                Tp = Tc;
                ep = ec;
                Tc = Tn;
                ec = en;
                kp0 = kc0;
                kp1 = kc1;
                kc0 = kn0;
                kc1 = kn1;
                si = si + 1 == AS ? 0 : si + 1;
                sc = sn;
                sn = sn + 1 == AS ? 0 : sn + 1;
                // no barrier here (as in the one-voxel form)
            }
            async_wait<0>();
            __syncthreads();  // the next item rewrites the stages and the instance's tables
            if (errbits) atomicOr(I.a.err, errbits);
        }
        if (GRID && k + 1 < K && !grid_barrier(sync, gridDim.x, err)) return;
    }
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
                float Tnew = a.fc[FC_TBOIL], Enew = a.fc[FC_TBOIL_E];
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

cudaError_t batch_heat_blocks(int *blocks, int staged)
{
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = staged == 2   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_pairs_kernel<true>, FX / 2 * FY,
                                                                          A_SMEM)
            : staged == 1 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_staged_kernel<true>, FX * FY,
                                                                          A_SMEM)
                          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_heat_kernel, FX * FY, 0);
    if (e != cudaSuccess) return e;
    *blocks = sms * (per > 0 ? per : 1);
    return cudaSuccess;
}

cudaError_t launch_batch_heat(const BatchInst *insts, int n, const int *prefix, const BatchStep *steps, int K,
                              BatchSync *sync, unsigned *err, int blocks, int staged, cudaStream_t s)
{
    if (n <= 0 || K <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(sync, 0, sizeof(BatchSync), s);
    if (e != cudaSuccess) return e;
    BatchStep one{};
    int one_fcur = 0;
    void *args[] = {(void *)&insts, (void *)&n, (void *)&prefix, (void *)&steps, (void *)&K, (void *)&sync,
                    (void *)&err};
    void *args2[] = {(void *)&insts, (void *)&n,    (void *)&prefix, (void *)&steps,   (void *)&K,
                     (void *)&sync,  (void *)&err,  (void *)&one,    (void *)&one_fcur};
    count_launch();
    if (staged == 2)
        return cudaLaunchCooperativeKernel((const void *)batch_pairs_kernel<true>, dim3(blocks), dim3(FX / 2, FY),
                                           args2, A_SMEM, s);
    if (staged == 1)
        return cudaLaunchCooperativeKernel((const void *)batch_staged_kernel<true>, dim3(blocks), dim3(FX, FY), args,
                                           A_SMEM, s);
    return cudaLaunchCooperativeKernel((const void *)batch_heat_kernel, dim3(blocks), dim3(FX, FY), args, 0, s);
}

cudaError_t launch_staged_step(const BatchInst *inst, const int *prefix, int items, const BatchStep &step, int fcur,
                               cudaStream_t s)
{
    if (items <= 0) return cudaSuccess;
    count_launch();
    batch_pairs_kernel<false><<<items, dim3(FX / 2, FY), A_SMEM, s>>>(inst, 1, prefix, nullptr, 1, nullptr, nullptr,
                                                                       step, fcur);
    return cudaGetLastError();
}

}  // namespace tam
