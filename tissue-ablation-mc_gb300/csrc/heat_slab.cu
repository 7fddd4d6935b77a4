// heat_slab.cu -- the FP32 + Kahan fused heat step, slab form.
//
// The physics of the class-table step (heat_tma.cu, fused_cls2_kernel):
// src/3dFD.f90:113-187 with the config-mode operator, Robin / Dirichlet
// ghost faces, the latent-heat clamp, Arrhenius damage and ablation, in FP32
// with a Kahan-compensated temperature (true T = T - e), arranged so that
// the loop over the planes does nothing but the interior update:
//
//  * a block owns a tile of 32 x 8 voxels and marches it through a slab of
//    z planes; every thread updates two x-adjacent voxels (64-bit shared
//    loads and global stores), and the z neighbours travel in registers;
//  * one elected thread streams each plane into a ring of 5-6
//    shared-memory stages with cp.async.bulk.tensor (TMA): T and the Kahan
//    term with a one-voxel x / y halo, J of the tile's own voxels, and for
//    heterogeneous grids the u8 class ids with halo.  One block barrier and
//    one bounded mbarrier wait per plane;
//  * every voxel takes the interior formula, each face difference formed
//    from the true values (T_n - T_c) - (e_n - e_c), with dt folded into the
//    face coefficients.  A boundary face becomes a ghost neighbour: before
//    the loads of a plane, the thread owning a boundary voxel writes into
//    that voxel's own halo cell of the staged plane (only that thread reads
//    it) the value pair that makes the interior term equal the face's ghost
//    term -- the Dirichlet temperature with a zero Kahan term, or for a
//    convective face the voxel's own pair shifted by the Robin difference
//    with its rounding error carried in the Kahan term -- and the z faces
//    swap the register neighbours the same way;
//  * voxels whose old temperature has reached boiling, whose old or new
//    temperature reaches the damage / ablation screen, or whose new
//    temperature is negative or NaN are only listed (in shared memory, by
//    local index); once the block has written all its planes it takes the
//    list again: latent-heat clamp (the stencil redone from global memory),
//    Arrhenius damage, ablation and the error word.  No call stays in the
//    plane loop, so its registers hold only the interior update (an
//    out-of-line call there cost ~40 % of the step);
//  * the slabs are launched from the top face down: the beam enters there,
//    so the blocks with the longest lists start first instead of forming the
//    launch's tail.
#include <algorithm>
#include <atomic>
#include <vector>

#include "heat_common.cuh"
#include "slab_common.cuh"
#include "tma_common.cuh"

namespace tam {

struct FusedSlab {
    CUtensorMap T[2], E[2], J, cls;
    const uint8_t *cls_grid;  // the class grid (rows of cls_pitch bytes) for the fix-up pass
    int cls_pitch;
    int nx, ny, nz;
    // heterogeneous grids: per (tile, plane) the one class of the tile and its
    // x / y rim, or 0xFF; per block of the launch at z-chunk list_zc its class
    // (or 0xFF); the blocks of one class (item | class << 24) and the others
    uint8_t *tflag, *bclass;
    unsigned *one_items, *mixed_items;
    int n_one, n_mixed, list_zc;
    bool mixed_first;         // mixed blocks make up a quarter or more of the top three z-chunks
    unsigned gen;             // lists rebuilt so many times
};

namespace {

constexpr int SP = 16;          // voxel pairs per tile row
constexpr int SW = 2 * SP;      // voxels per tile row
constexpr int SR = 8;           // voxel rows per tile
// (5 or 4 stages with 8 blocks per SM, and 5 stages with 7, measured within
// 1 % of 6 stages with 7 blocks on the 200^3 step)
#ifndef TAM_SLAB_STAGES
#define TAM_SLAB_STAGES 6
#endif
constexpr int SLAB_STAGES = TAM_SLAB_STAGES;  // ring stages of the one-class kernel (prefetch depth stages - 2 planes)
constexpr int SLAB_ZMAX = 8;    // planes per block at most (the list holds every voxel of a slab)

// The class-grid kernel (80 registers at 6 blocks per SM, its stages 640 B
// larger) runs 5 stages at 7 blocks per SM: 679 against 710 us per step on
// the 512^3 vessel grid, 4.0 % less at 256^3; 4 stages at 8 blocks, 682 us.
#ifndef TAM_SLAB_STAGES_CLS
#define TAM_SLAB_STAGES_CLS 5
#endif
template <bool UNIFORM> struct SlabLayout {
    static constexpr int NST = UNIFORM ? SLAB_STAGES : TAM_SLAB_STAGES_CLS;  // ring stages
    static constexpr int TP = SW + 8;                        // staged T / Kahan row: x from the tile origin - 4
    static constexpr int CP = 64;                            // staged class row (u8) from the tile origin - 16
    static constexpr int H_BYTES = (((SR + 2) * TP * 4 + 127) / 128) * 128;  // T or Kahan term with halo
    static constexpr int J_BYTES = SR * SW * 4;              // own voxels
    static constexpr int C_BYTES = (((SR + 2) * CP + 127) / 128) * 128;
    static constexpr int T_OFF = 0, E_OFF = H_BYTES, J_OFF = 2 * H_BYTES, C_OFF = 2 * H_BYTES + J_BYTES;
    static constexpr int STAGE = ((C_OFF + (UNIFORM ? 0 : C_BYTES) + 127) / 128) * 128;
    static constexpr uint32_t TX_H = 2 * (SR + 2) * TP * 4, TX_J = J_BYTES, TX_C = (SR + 2) * CP;
    static constexpr int LIST = SW * SR * SLAB_ZMAX;         // list entries (u16 local indices)
    static constexpr int SMEM = NST * STAGE + NST * 8 + LIST * 2 + 16 + 128;
    static_assert(J_BYTES % 128 == 0, "own-voxel array keeps 128-byte stage alignment");
    static_assert(LIST <= 65536, "local indices fit 16 bits");
};

#ifndef TAM_SLAB_MINB
#define TAM_SLAB_MINB 7
#endif
#ifndef TAM_SLAB_MINB_CLS
#define TAM_SLAB_MINB_CLS 7
#endif
constexpr int slab_minb(bool uniform) { return uniform ? TAM_SLAB_MINB : TAM_SLAB_MINB_CLS; }

struct SlabMaps {
    CUtensorMap T, E, J, cls;
};

__device__ __forceinline__ float2 lds2(const float *p) { return *reinterpret_cast<const float2 *>(p); }

template <bool UNIFORM>
__global__ void __launch_bounds__(SP *SR, slab_minb(UNIFORM))
    slab_step_kernel(const __grid_constant__ FusedArgs a, const __grid_constant__ SlabMaps m,
                     const __grid_constant__ ClassLut L, const uint8_t *cls, int cpitch, int zchunk, float rare_thr,
                     const unsigned *items, int early)
{
    using Lay = SlabLayout<UNIFORM>;
    // early: the launch behind this one (the other list's blocks, which
    // touch other voxels) may start as soon as this one's blocks are placed
    if (early) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    constexpr int TP = Lay::TP, CP = Lay::CP, NST = Lay::NST;
    extern __shared__ unsigned char smem_raw[];
    __shared__ float s_fa[UNIFORM ? 1 : MAX_MAT * MAX_MAT];
    unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + NST * Lay::STAGE);
    unsigned short *list = reinterpret_cast<unsigned short *>(sm + NST * Lay::STAGE + NST * 8);
    int *s_cnt = reinterpret_cast<int *>(sm + NST * Lay::STAGE + NST * 8 + Lay::LIST * 2);
    const int tid = threadIdx.x;
    const int r = tid / SP, p = tid % SP;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    // the block's tile and z-chunk: its place in the launch, or on a
    // heterogeneous grid the item of a list (one list per kernel: the
    // one-class kernel takes the blocks whose tile, rim and planes hold one
    // class, with that class in the item's top byte; the class kernel the rest)
    int bx = (int)blockIdx.x, by = (int)blockIdx.y, bz = (int)blockIdx.z, nzc = (int)gridDim.z;
    unsigned item_cls = 0xFFu;
    if (items) {
        const unsigned it = items[blockIdx.x], u = it & 0xFFFFFFu;
        const unsigned gx = (unsigned)(nx + SW - 1) / SW, gy = (unsigned)(ny + SR - 1) / SR;
        item_cls = it >> 24;
        bx = (int)(u % gx);
        by = (int)((u / gx) % gy);
        bz = (int)(u / (gx * gy));
        nzc = (nz + zchunk - 1) / zchunk;
    }
    const int bxW = bx * SW, byR = by * SR;
    const int x = bxW + 2 * p, y = byR + r;
    // slabs from the top face down (see the file comment)
    const int z0 = (nzc - 1 - bz) * zchunk;
    const int z1 = min(nz, z0 + zchunk);
    const int nplanes = z1 - z0, last = nplanes + 1;
    const bool act = x < nx && y < ny;  // nx is even: the pair's second voxel is inside too
    const int sz = nx * ny;             // the launcher keeps nx * ny * nz below 2^31
    const int gxT = bxW - 4, gy = byR - 1, gxO = bxW, gyO = byR;
    const int gxC = bxW - 16;           // 16-byte aligned origin of the class rows
    const bool leader = tid == 0;
    const float Pdt = step_pdt<float>(a);
    // face coefficients with dt folded in
    const float cxd = a.fc[FC_DT] * a.fc[FC_CX], cyd = a.fc[FC_DT] * a.fc[FC_CY], czd = a.fc[FC_DT] * a.fc[FC_CZ];
    const int uc = UNIFORM && item_cls != 0xFFu ? (int)item_cls : (L.uniform >= 0 ? L.uniform : 0);
    const float au = L.fa[uc * MAX_MAT + uc];
    const float Cx = cxd * au, Cy = cyd * au, Cz = czd * au, C6 = 2.f * ((Cx + Cy) + Cz);
    const float Ku = Pdt * L.irc[uc];
    // boundary faces of the pair in x / y: x- of the first voxel, x+ of the
    // second, y- and y+ of both
    const unsigned exy = (unsigned)(x == 0) | (unsigned)(x + 1 == nx - 1) << 1 | (unsigned)(y == 0) << 2 |
                         (unsigned)(y == ny - 1) << 3;
    const float lo = 0.5f * rare_thr;  // new temperatures outside (0, rare_thr) are listed
    if (!UNIFORM)
        for (int t = tid; t < MAX_MAT * MAX_MAT; t += SP * SR) s_fa[t] = L.fa[t];

    auto issue = [&](int idx) {
        unsigned char *b = sm + (idx % NST) * Lay::STAGE;
        uint64_t *br = bar + (idx % NST);
        const int zz = z0 - 1 + idx;
        const bool own = idx >= 1 && idx <= nplanes;  // the halo planes need no J
        fence_proxy_async();
        mbar_expect_tx(br, Lay::TX_H + (own ? Lay::TX_J : 0u) + (UNIFORM ? 0u : Lay::TX_C));
        tma_load_3d(b + Lay::T_OFF, &m.T, gxT, gy, zz, br);
        tma_load_3d(b + Lay::E_OFF, &m.E, gxT, gy, zz, br);
        if (own) tma_load_3d(b + Lay::J_OFF, &m.J, gxO, gyO, zz, br);
        if (!UNIFORM) tma_load_3d(b + Lay::C_OFF, &m.cls, gxC, gy, zz, br);
    };

    if (leader) {
        for (int s = 0; s < NST; ++s) mbar_init(bar + s, 1);
        *s_cnt = 0;
        fence_mbar_init();
        fence_proxy_async();
    }
    __syncthreads();
    if (leader)
        for (int idx = 0; idx < NST && idx <= last; ++idx) issue(idx);
    int issued = NST < last + 1 ? NST : last + 1;
    bool ok = mbar_wait(bar, 0) && mbar_wait(bar + 1, 0);
    const int qT = (r + 1) * TP + 4 + 2 * p;   // the pair in the staged T / Kahan rows (even: 8-byte aligned)
    const int qO = r * SW + 2 * p;             // ... in the own-voxel J
    const int qC = (r + 1) * CP + 16 + 2 * p;  // ... in the class rows (even)
    float2 Tp = {0.f, 0.f}, Tc = {0.f, 0.f}, Ep = {0.f, 0.f}, Ec = {0.f, 0.f};
    int kp0 = uc, kp1 = uc, kc0 = uc, kc1 = uc;
    auto cls2 = [&](const unsigned char *b, int i, int &k0, int &k1) {
        const unsigned short w = *reinterpret_cast<const unsigned short *>(b + Lay::C_OFF + i);
        k0 = w & (MAX_MAT - 1);
        k1 = (w >> 8) & (MAX_MAT - 1);
    };
    if (ok && act) {
        Tc = lds2((const float *)(sm + Lay::STAGE + Lay::T_OFF) + qT);
        Ec = lds2((const float *)(sm + Lay::STAGE + Lay::E_OFF) + qT);
        if (!UNIFORM) cls2(sm + Lay::STAGE, qC, kc0, kc1);
        if (z0 > 0) {
            Tp = lds2((const float *)(sm + Lay::T_OFF) + qT);
            Ep = lds2((const float *)(sm + Lay::E_OFF) + qT);
            if (!UNIFORM) cls2(sm, qC, kp0, kp1);
        }
    }
    float *To = (float *)a.T_out + (x + nx * y + sz * z0), *Eo = a.Tc_out + (x + nx * y + sz * z0);
    int s1 = 1, s2 = 2;  // stages of the plane being updated and of the next plane
    uint32_t ph2 = 0;    // phase of stage s2's barrier
    for (int i = 0; i < nplanes; ++i, To += sz, Eo += sz) {
        // every thread is done with the stages of plane i - 1: stage i is free
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        if (i + NST <= last) {
            if (leader) issue(i + NST);
            issued = i + NST + 1;
        }
        ok = mbar_wait(bar + s2, ph2);
        const unsigned char *S = sm + s1 * Lay::STAGE, *N = sm + s2 * Lay::STAGE;
        s1 = s2;
        if (++s2 == NST) {
            s2 = 0;
            ph2 ^= 1u;
        }
        if (!(ok && act)) continue;
        const int z = z0 + i;
        const float *ST = (const float *)(S + Lay::T_OFF), *SE = (const float *)(S + Lay::E_OFF);
        if (exy) {
            // ghost neighbours of this thread's boundary faces, in its own halo cells
            float *WT = (float *)(S + Lay::T_OFF), *WE = (float *)(S + Lay::E_OFF);
            unsigned char *WC = (unsigned char *)(S + Lay::C_OFF);
            if (exy & 1u) {
                const float2 g = ghost_pair(a, 0, Tc.x, Ec.x, L.k[kc0]);
                WT[qT - 1] = g.x;
                WE[qT - 1] = g.y;
                if (!UNIFORM) WC[qC - 1] = (unsigned char)kc0;
            }
            if (exy & 2u) {
                const float2 g = ghost_pair(a, 1, Tc.y, Ec.y, L.k[kc1]);
                WT[qT + 2] = g.x;
                WE[qT + 2] = g.y;
                if (!UNIFORM) WC[qC + 2] = (unsigned char)kc1;
            }
            if (exy & 12u) {
                const int f = (exy & 4u) ? 2 : 3, o = (exy & 4u) ? -TP : TP, oc = (exy & 4u) ? -CP : CP;
                const float2 g0 = ghost_pair(a, f, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(a, f, Tc.y, Ec.y, L.k[kc1]);
                *reinterpret_cast<float2 *>(WT + qT + o) = make_float2(g0.x, g1.x);
                *reinterpret_cast<float2 *>(WE + qT + o) = make_float2(g0.y, g1.y);
                if (!UNIFORM) {
                    WC[qC + oc] = (unsigned char)kc0;
                    WC[qC + 1 + oc] = (unsigned char)kc1;
                }
            }
        }
        const float2 Tn = lds2((const float *)(N + Lay::T_OFF) + qT);
        const float2 En = lds2((const float *)(N + Lay::E_OFF) + qT);
        const float2 tym = lds2(ST + qT - TP), typ = lds2(ST + qT + TP);
        const float2 eym = lds2(SE + qT - TP), eyp = lds2(SE + qT + TP);
        const float txl = ST[qT - 1], txr = ST[qT + 2], exl = SE[qT - 1], exr = SE[qT + 2];
        const float2 j2 = lds2((const float *)(S + Lay::J_OFF) + qO);
        int kn0 = uc, kn1 = uc;
        if (!UNIFORM) cls2(N, qC, kn0, kn1);
        // ghost neighbours of the z boundary planes (registers only)
        float2 Tpz = Tp, Epz = Ep;
        int kpz0 = kp0, kpz1 = kp1;
        if (z == 0) {
            const float2 g0 = ghost_pair(a, 4, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(a, 4, Tc.y, Ec.y, L.k[kc1]);
            Tpz = make_float2(g0.x, g1.x);
            Epz = make_float2(g0.y, g1.y);
            kpz0 = kc0;
            kpz1 = kc1;
        }
        float2 Tnz = Tn, Enz = En;
        int knz0 = kn0, knz1 = kn1;
        if (z == nz - 1) {
            const float2 g0 = ghost_pair(a, 5, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(a, 5, Tc.y, Ec.y, L.k[kc1]);
            Tnz = make_float2(g0.x, g1.x);
            Enz = make_float2(g0.y, g1.y);
            knz0 = kc0;
            knz1 = kc1;
        }
        unsigned fix = 0;
        float tn[2], en[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float tc = h ? Tc.y : Tc.x, e0 = h ? Ec.y : Ec.x;
            const float txm = h ? Tc.x : txl, txp = h ? txr : Tc.y, exm = h ? Ec.x : exl, exp_ = h ? exr : Ec.y;
            const float tyM = h ? tym.y : tym.x, tyP = h ? typ.y : typ.x;
            const float eyM = h ? eym.y : eym.x, eyP = h ? eyp.y : eyp.x;
            const float tzM = h ? Tpz.y : Tpz.x, tzP = h ? Tnz.y : Tnz.x, ezM = h ? Epz.y : Epz.x, ezP = h ? Enz.y : Enz.x;
            float dT;
            if (UNIFORM) {
                // sum over the faces of C_f [(T_f - T_c) - (e_f - e_c)]
                const float sx = ((txm - tc) + (txp - tc)) - (exm + exp_);
                const float sy = ((tyM - tc) + (tyP - tc)) - (eyM + eyP);
                const float sz_ = ((tzM - tc) + (tzP - tc)) - (ezM + ezP);
                dT = __fmaf_rn(Cz, sz_, __fmaf_rn(Cy, sy, __fmaf_rn(Cx, sx, C6 * e0)));
            } else {
                const int k = h ? kc1 : kc0;
                const unsigned char *SC = S + Lay::C_OFF;
                const float *frow = s_fa + k * MAX_MAT;
                const float axm = cxd * frow[h ? kc0 : (SC[qC - 1] & (MAX_MAT - 1))];
                const float axp = cxd * frow[h ? (SC[qC + 2] & (MAX_MAT - 1)) : kc1];
                const float aym = cyd * frow[SC[qC + h - CP] & (MAX_MAT - 1)];
                const float ayp = cyd * frow[SC[qC + h + CP] & (MAX_MAT - 1)];
                const float azm = czd * frow[h ? kpz1 : kpz0];
                const float azp = czd * frow[h ? knz1 : knz0];
                dT = ((azm * ((tzM - tc) - (ezM - e0)) + azp * ((tzP - tc) - (ezP - e0))) +
                      (aym * ((tyM - tc) - (eyM - e0)) + ayp * ((tyP - tc) - (eyP - e0)))) +
                     (axm * ((txm - tc) - (exm - e0)) + axp * ((txp - tc) - (exp_ - e0)));
            }
            const float Kk = UNIFORM ? Ku : Pdt * L.irc[h ? kc1 : kc0];
            const float inc = __fmaf_rn(Kk, h ? j2.y : j2.x, dT);
            const float yk = inc - e0;
            const float t = tc + yk;
            const float e = (t - tc) - yk;
            // listed: old or new temperature at the screen, or a new one negative or NaN
            const float tm = tc > t ? tc : t;
            if (!(fabsf(tm - lo) < lo)) fix |= 1u << h;
            tn[h] = t;
            en[h] = e;
        }
        *reinterpret_cast<float2 *>(To) = make_float2(tn[0], tn[1]);
        *reinterpret_cast<float2 *>(Eo) = make_float2(en[0], en[1]);
        if (fix) {
            const int n = __popc(fix);
            const int at = atomicAdd(s_cnt, n);
            const int l = (i * SR + r) * SW + 2 * p;
            if (fix & 1u) list[at] = (unsigned short)l;
            if (fix & 2u) list[at + n - 1] = (unsigned short)(l + 1);
        }
        Tp = Tc;
        Tc = Tn;
        Ep = Ec;
        Ec = En;
        if (!UNIFORM) {
            kp0 = kc0;
            kp1 = kc1;
            kc0 = kn0;
            kc1 = kn1;
        }
    }
    // the last plane's wait may have failed in some threads only: agree first
    ok = __syncthreads_and(ok) != 0;
    unsigned errbits = 0;
    if (!ok) {
        errbits |= DEVERR_SYNC_TIMEOUT;
        for (int idx = issued > NST ? issued - NST : 0; idx < issued; ++idx)
            (void)mbar_wait(bar + (idx % NST), (uint32_t)((idx / NST) & 1));
    } else {
        // the listed voxels; this block's own plane stores come first.  Most
        // of them are in the damage window only: their pairs and damage
        // integrals are loaded four entries at a time, so the loads of the
        // four overlap, and the damage is added without further reads; the
        // others (boiling, ablation, NaN / negative) go through slab_fix.
        __syncthreads();
        const int cnt = *s_cnt;
        const double t_new = step_tnew(a);
        const int64_t ni = (int64_t)sz * nz;
        const float *Ti = (const float *)a.T_in;
        const float *Tw = (const float *)a.T_out, *Ew = a.Tc_out;
        constexpr int NT = SP * SR, B = 4;
        for (int q = tid; q < cnt; q += B * NT) {
            int vv[B], xx[B], yy[B], zz[B];
            float tt[B], ee[B], tcv[B];
            double oo[B];
#pragma unroll
            for (int j = 0; j < B; ++j) {
                const int qq = q + j * NT;
                vv[j] = -1;
                if (qq < cnt) {
                    const int l = list[qq];
                    xx[j] = bxW + l % SW;
                    yy[j] = byR + (l / SW) % SR;
                    zz[j] = z0 + l / (SW * SR);
                    vv[j] = xx[j] + nx * yy[j] + sz * zz[j];
                    tt[j] = Tw[vv[j]];
                    ee[j] = Ew[vv[j]];
                    tcv[j] = Ti[vv[j]];
                    oo[j] = a.omega[vv[j]];
                }
            }
#pragma unroll
            for (int j = 0; j < B; ++j) {
                if (vv[j] < 0) continue;
                const float Ts = tt[j] - ee[j];
                const bool general = (a.boil && tcv[j] >= a.fc[FC_TBOIL]) || !(Ts >= 0.f) ||
                                     ge_ff(tt[j], ee[j], a.fc[FC_TABL], a.fc[FC_TABL_LO]);
                if (general)
                    slab_fix<UNIFORM>(a, L, cls, cpitch, xx[j], yy[j], zz[j], Pdt, t_new, errbits, (const float *)a.T_in,
                                      a.Tc_in, (float *)a.T_out, a.Tc_out, uc);
                else if (Ts >= a.fc[FC_SCREEN]) rare_update_f32(a, vv[j], ni, tt[j], ee[j], t_new, true, oo[j]);
            }
        }
    }
    if (errbits) atomicOr(a.err, errbits);
}

// The z-chunk of a launch: measured fastest at 200^3 (37.7 us against 38.4
// at 5, 40.6 at 8).
int eff_zchunk(int requested, int nz)
{
    int zchunk = requested > 0 ? requested : 6;
    if (zchunk > SLAB_ZMAX) zchunk = SLAB_ZMAX;
    if (zchunk > nz) zchunk = nz;
    return zchunk;
}

// items == nullptr: every block of the grid; else `n` listed blocks
template <bool UNIFORM>
cudaError_t launch_slab_t(const FusedArgs &a, const SlabMaps &m, const ClassLut &L, const uint8_t *cls, int cpitch,
                          float rare_thr, const unsigned *items, int n, int early, bool overlap, cudaStream_t s)
{
    const int bx = (a.nx + SW - 1) / SW, by = (a.ny + SR - 1) / SR;
    const int zchunk = eff_zchunk(a.zchunk, a.nz);
    const int chunks = (a.nz + zchunk - 1) / zchunk;
    const int smem = SlabLayout<UNIFORM>::SMEM;
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
        e = cudaFuncSetAttribute(slab_step_kernel<UNIFORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    count_launch();
    const dim3 grid = items ? dim3((unsigned)n, 1, 1) : dim3(bx, by, chunks);
    if (!overlap) {
        slab_step_kernel<UNIFORM><<<grid, SP * SR, smem, s>>>(a, m, L, cls, cpitch, zchunk, rare_thr, items, early);
        return cudaGetLastError();
    }
    // programmatic dependent launch: may begin while the launch before it
    // (which signals early) is still running
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(SP * SR);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, slab_step_kernel<UNIFORM>, a, m, L, cls, cpitch, zchunk, rare_thr, items, 0);
}

// The slab kernel's tile flags: for every (tile, plane), the class that all
// voxels of the 32 x 8 tile and of its one-voxel x / y rim (inside the grid)
// hold, or 0xFF when they differ.  One warp per (tile, plane): each lane
// takes one x column of the rim rows and of the tile rows, lanes 0 and 1 the
// rim columns, and the warp compares its lanes' smallest and largest class.
__global__ void slab_tile_flags_kernel(const uint8_t *cls, int pitch, int nx, int ny, int nz, uint8_t *flags)
{
    const int tx = (nx + SW - 1) / SW, ty = (ny + SR - 1) / SR;
    const int64_t items = (int64_t)tx * ty * nz;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < items; it += nw) {
        // it = (z * ty + tile row) * tx + tile column: neighbouring warps read neighbouring tiles
        const int txi = (int)(it % tx);
        const int64_t rest = it / tx;
        const int tyi = (int)(rest % ty), z = (int)(rest / ty);
        const int bx = txi * SW, by = tyi * SR;
        const uint8_t *pl = cls + (int64_t)pitch * ny * z;
        int cmin = 255, cmax = -1;
        auto take = [&](int xx, int yy) {
            if (xx < 0 || xx >= nx || yy < 0 || yy >= ny) return;
            const int c = pl[(int64_t)pitch * yy + xx] & (MAX_MAT - 1);
            cmin = min(cmin, c);
            cmax = max(cmax, c);
        };
        for (int yy = by - 1; yy <= by + SR; ++yy) take(bx + lane, yy);
        if (lane < 2)
            for (int yy = by; yy < by + SR; ++yy) take(lane ? bx + SW : bx - 1, yy);
        cmin = __reduce_min_sync(0xffffffffu, cmin);
        cmax = __reduce_max_sync(0xffffffffu, cmax);
        if (lane == 0) flags[((int64_t)tyi * tx + txi) * nz + z] = (uint8_t)(cmin == cmax ? cmin : 0xFF);
    }
}

// Per block of the slab launch at z-chunk zc (launch order: x tiles fastest,
// then y tiles, then z-chunks from the top face down): the class that the
// tile flags of all its planes z0 - 1 .. z1 (inside the grid) agree on, or 0xFF.
__global__ void slab_block_class_kernel(const uint8_t *flags, int tx, int ty, int nz, int zc, uint8_t *bclass)
{
    const int nzc = (nz + zc - 1) / zc;
    const int64_t items = (int64_t)tx * ty * nzc;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < items; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tile = u % ((int64_t)tx * ty);
        const int bz = (int)(u / ((int64_t)tx * ty));
        const int z0 = (nzc - 1 - bz) * zc, z1 = min(nz, z0 + zc);
        const int za = max(z0 - 1, 0), zb = min(z1, nz - 1);
        const uint8_t *f = flags + tile * nz;
        int c = f[za];
        for (int z = za + 1; z <= zb && c != 0xFF; ++z)
            if (f[z] != c) c = 0xFF;
        bclass[u] = (uint8_t)c;
    }
}

}  // namespace

cudaError_t fused_slab_tile_flags(FusedSlab *m, int zchunk, cudaStream_t s)
{
    const int tx = (m->nx + SW - 1) / SW, ty = (m->ny + SR - 1) / SR;
    const int zc = eff_zchunk(zchunk, m->nz), nzc = (m->nz + zc - 1) / zc;
    const int64_t tiles = (int64_t)tx * ty * m->nz, items = (int64_t)tx * ty * nzc;
    // until the new lists are complete the class kernel takes every block
    // (so a failure below leaves a correct step)
    m->n_one = m->n_mixed = 0;
    m->list_zc = 0;
    ++m->gen;
    if (items >= (int64_t)1 << 24) return cudaSuccess;  // list entries hold the block's index in 24 bits
    count_launch(2);
    slab_tile_flags_kernel<<<(unsigned)std::min<int64_t>((tiles + 7) / 8, 152 * 32), 256, 0, s>>>(
        m->cls_grid, m->cls_pitch, m->nx, m->ny, m->nz, m->tflag);
    slab_block_class_kernel<<<(unsigned)std::min<int64_t>((items + 255) / 256, 152 * 16), 256, 0, s>>>(
        m->tflag, tx, ty, m->nz, zc, m->bclass);
    // the two lists, in launch order, built on the host (a rare call: after a
    // change of the class grid or of the z-chunk)
    std::vector<uint8_t> bc((size_t)items);
    cudaError_t e = cudaMemcpyAsync(bc.data(), m->bclass, (size_t)items, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    std::vector<unsigned> one, mixed;
    int64_t top_mixed = 0;
    for (int64_t u = 0; u < items; ++u) {
        if (bc[u] < MAX_MAT) {
            one.push_back((unsigned)u | (unsigned)bc[u] << 24);
        } else {
            mixed.push_back((unsigned)u);
            if (u < 3 * (int64_t)tx * ty) ++top_mixed;  // the top z-chunks come first in launch order
        }
    }
    if (!one.empty()) e = cudaMemcpyAsync(m->one_items, one.data(), one.size() * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !mixed.empty())
        e = cudaMemcpyAsync(m->mixed_items, mixed.data(), mixed.size() * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    m->n_one = (int)one.size();
    m->n_mixed = (int)mixed.size();
    m->mixed_first = 4 * top_mixed >= std::min<int64_t>(items, 3 * (int64_t)tx * ty);
    m->list_zc = zc;
    ++m->gen;
    return cudaSuccess;
}

unsigned fused_slab_generation(const FusedSlab *m) { return m ? m->gen : 0u; }

bool fused_slab_supported(int nx, int ny, int nz)
{
    return nx > 0 && nx % 4 == 0 && (int64_t)nx * ny * nz < ((int64_t)1 << 31) - 64;
}

cudaError_t fused_slab_create(FusedSlab **out, int nx, int ny, int nz, float *const T[2], float *const Tc[2],
                              const float *J, const uint8_t *cls, int pitch)
{
    *out = nullptr;
    if (!fused_slab_supported(nx, ny, nz) || pitch % 16 != 0 || pitch < nx) return cudaErrorNotSupported;
    cudaError_t e = encoder();
    if (e != cudaSuccess) return e;
    FusedSlab *m = new FusedSlab();
    m->cls_grid = cls;
    m->cls_pitch = pitch;
    m->nx = nx;
    m->ny = ny;
    m->nz = nz;
    m->tflag = m->bclass = nullptr;
    m->one_items = m->mixed_items = nullptr;
    m->n_one = m->n_mixed = 0;
    m->list_zc = 0;  // no lists: the class kernel takes every block
    m->mixed_first = false;
    m->gen = 0;
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = encode(&m->T[b], T[b], nx, ny, nz, SW + 8, SR + 2);
        if (e == cudaSuccess) e = encode(&m->E[b], Tc[b], nx, ny, nz, SW + 8, SR + 2);
    }
    if (e == cudaSuccess) e = encode(&m->J, J, nx, ny, nz, SW, SR);
    if (e == cudaSuccess) e = encode_u8(&m->cls, cls, pitch, ny, nz, SlabLayout<false>::CP, SR + 2);
    // tile flags and lists, sized for the smallest z-chunk (the most blocks)
    const int64_t tiles = (int64_t)((nx + SW - 1) / SW) * ((ny + SR - 1) / SR);
    if (e == cudaSuccess) e = cudaMalloc(&m->tflag, (size_t)(tiles * nz));
    if (e == cudaSuccess) e = cudaMalloc(&m->bclass, (size_t)(tiles * nz));
    if (e == cudaSuccess) e = cudaMalloc(&m->one_items, (size_t)(tiles * nz) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&m->mixed_items, (size_t)(tiles * nz) * 4);
    if (e != cudaSuccess) {
        fused_slab_destroy(m);
        return e;
    }
    *out = m;
    return cudaSuccess;
}

void fused_slab_destroy(FusedSlab *m)
{
    if (!m) return;
    for (void *p : {(void *)m->tflag, (void *)m->bclass, (void *)m->one_items, (void *)m->mixed_items})
        if (p) cudaFree(p);
    delete m;
}

cudaError_t launch_fused_slab(const FusedArgs &a0, const FusedSlab *sm, int which, const ClassLut &L, cudaStream_t s)
{
    FusedArgs a = a0;
    fill_fused_consts(a);
    SlabMaps m;
    m.T = sm->T[which];
    m.E = sm->E[which];
    m.J = sm->J;
    m.cls = sm->cls;
    // one screen for the listed rare work: damage / ablation, and boiling
    float rare_thr = a.fc[FC_SCREEN];
    if (a.boil && a.fc[FC_TBOIL] < rare_thr) rare_thr = a.fc[FC_TBOIL];
    if (L.uniform >= 0)
        return launch_slab_t<true>(a, m, L, sm->cls_grid, sm->cls_pitch, rare_thr, nullptr, 0, 0, false, s);
    if (sm->list_zc != eff_zchunk(a.zchunk, a.nz))  // no lists for this z-chunk: the class kernel everywhere
        return launch_slab_t<false>(a, m, L, sm->cls_grid, sm->cls_pitch, rare_thr, nullptr, 0, 0, false, s);
    // two launches over disjoint blocks: the second may start as soon as the
    // first one's blocks are placed (programmatic dependent launch), and the
    // next step's launch waits for both.  The beam enters at the top face, so
    // the top blocks carry the longest lists: the mixed blocks go first when
    // they make up a quarter or more of the top three z-chunks (a layered
    // grid whose thin top layers meet there: 50 against 62 us per
    // 256 x 256 x 128 step), else the one-class blocks (a grid of scattered
    // vessels: 78 against 84 us at 256^3)
    cudaError_t e = cudaSuccess;
    const bool both = sm->n_one > 0 && sm->n_mixed > 0;
    auto mixed = [&](int early, bool overlap) {
        return sm->n_mixed > 0 ? launch_slab_t<false>(a, m, L, sm->cls_grid, sm->cls_pitch, rare_thr, sm->mixed_items,
                                                      sm->n_mixed, early, overlap, s)
                               : cudaSuccess;
    };
    auto one = [&](int early, bool overlap) {
        return sm->n_one > 0 ? launch_slab_t<true>(a, m, L, sm->cls_grid, sm->cls_pitch, rare_thr, sm->one_items,
                                                   sm->n_one, early, overlap, s)
                             : cudaSuccess;
    };
    if (sm->mixed_first) {
        e = mixed(both ? 1 : 0, false);
        if (e == cudaSuccess) e = one(0, both);
    } else {
        e = one(both ? 1 : 0, false);
        if (e == cudaSuccess) e = mixed(0, both);
    }
    return e;
}

}  // namespace tam
