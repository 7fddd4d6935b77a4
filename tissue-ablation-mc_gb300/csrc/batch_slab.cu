// batch_slab.cu -- the batched FP32 heat step in the slab form.
//
// All instances of a batch advance K steps in one cooperative launch, as in
// batch.cu: per step the resident blocks share out the work items (instance,
// 32 x 8 tile, z-chunk) of every instance, and a
// bounded software grid barrier separates the steps.  Each item is updated
// with the scheme of the single-instance slab kernel (heat_slab.cu): two
// x-adjacent voxels per thread, z neighbours in registers, the ghost
// neighbour of a boundary face written into the thread's own halo cell,
// voxels needing rare work (boiling, damage window, ablation, negative or NaN)
// listed and handled after the item's planes.  The list holds every voxel of
// an item of up to BATCH_SLAB_ZMAX planes, so that an item's z-chunk can be
// long and the ring's start-up latency is paid once per long item.
//
// The instances' grid edges are arbitrary, so their rows are generally not
// 16-byte aligned and TMA tensor copies cannot stage them.  A staged row is
// instead the run of 16-byte chunks that covers it, copied chunk by chunk
// with 16-byte cp.async by all threads of the block (each thread then
// arrives on the stage's mbarrier, which completes once every thread's
// copies have landed); where the row starts inside its first chunk,
// (index & 3), is applied when it is read.  The context arrays carry 256
// bytes of slack at both ends, so a chunk never leaves its allocation.  Rows
// and planes outside the grid are not copied; their cells are read only
// after the thread that owns the boundary voxel has written its ghost value
// there.
#include "grid_sync.cuh"
#include "heat_common.cuh"
#include "slab_common.cuh"
#include "tma_common.cuh"

namespace tam {

namespace {

constexpr int BP = 16;       // voxel pairs per tile row
constexpr int BW = 2 * BP;   // voxels per tile row
constexpr int BR = 8;        // voxel rows per tile
// ring stages (with 8 blocks of the per-step kernel per SM: 6 stages and
// 7 blocks ran 5 % slower, 8 stages and 5 blocks 11 %, 4 stages 4 %)
#ifndef TAM_BSLAB_STAGES
#define TAM_BSLAB_STAGES 5
#endif
constexpr int BS = TAM_BSLAB_STAGES;
constexpr int RT = 44;       // floats per staged T / Kahan row: the chunks covering x0 - 4 .. x0 + 35
constexpr int RJ = 36;       // floats per staged J row: the chunks covering x0 .. x0 + 31
constexpr int RC = 64;       // bytes per staged class row: x0 - 16 .. x0 + 47 (the class grid's rows are aligned)
static_assert(BATCH_SLAB_ZMAX * BW * BR <= 65536, "local indices fit 16 bits");

template <bool UNIFORM> struct BLay {
    static constexpr int T_OFF = 0, E_OFF = (BR + 2) * RT * 4, J_OFF = 2 * (BR + 2) * RT * 4;
    static constexpr int C_OFF = J_OFF + BR * RJ * 4;
    static constexpr int STAGE = ((C_OFF + (UNIFORM ? 0 : (BR + 2) * RC) + 127) / 128) * 128;
    static constexpr int LIST = BW * BR * BATCH_SLAB_ZMAX;   // u16 local indices: every voxel of an item
    static constexpr int SMEM = BS * STAGE + BS * 8 + LIST * 2 + 16 + 128;
    static_assert(E_OFF % 16 == 0 && J_OFF % 16 == 0 && C_OFF % 16 == 0, "16-byte aligned copy targets");
};
#ifndef TAM_BSLAB_MINB
#define TAM_BSLAB_MINB 4  // 128 registers without spills; 5 blocks spill
#endif
constexpr int bslab_minb(bool uniform) { return uniform ? TAM_BSLAB_MINB : 4; }

// Block-uniform description of the item (written by one thread).
struct __align__(16) BItem {
    const float *T, *E, *J;
    const uint8_t *C;
    float *To, *Eo;
    double t_new;
    float pdt;
    int inst, x0, y0, z0, z1, cpitch;
};

// The listed voxels of an item whose tile starts at (bxW, byR, zb) (the
// block's own plane stores come first), as in the single-instance slab
// kernel: the damage-window voxels' pairs and damage integrals loaded four
// entries at a time, the others through slab_fix; returns error bits.  The
// whole block shares the list out, so a hot region's many entries do not
// wait on the few threads that own them.
template <bool UNIFORM>
__device__ __noinline__ unsigned list_pass(const FusedArgs &A, const ClassLut &L, const unsigned short *list, int cnt,
                                           int bxW, int byR, int zb, const float *Ti, const float *Ei, float *Tw,
                                           float *Ew, const uint8_t *cls, int cpitch, float Pdt, double t_new)
{
    unsigned errbits = 0;
    const int nx = A.nx, sz = A.nx * A.ny;
    const int64_t ni = (int64_t)sz * A.nz;
    constexpr int NT = BP * BR, B = 4;
    for (int q = (int)threadIdx.x; q < cnt; q += B * NT) {
        int vv[B], xx[B], yy[B], zz[B];
        float tt[B], ee[B], tcv[B];
        double oo[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const int qq = q + j * NT;
            vv[j] = -1;
            if (qq < cnt) {
                const int l = list[qq];
                xx[j] = bxW + l % BW;
                yy[j] = byR + (l / BW) % BR;
                zz[j] = zb + l / (BW * BR);
                vv[j] = xx[j] + nx * yy[j] + sz * zz[j];
                tt[j] = Tw[vv[j]];
                ee[j] = Ew[vv[j]];
                tcv[j] = Ti[vv[j]];
                oo[j] = A.omega[vv[j]];
            }
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if (vv[j] < 0) continue;
            const float Ts = tt[j] - ee[j];
            const bool general = (A.boil && tcv[j] >= A.fc[FC_TBOIL]) || !(Ts >= 0.f) ||
                                 ge_ff(tt[j], ee[j], A.fc[FC_TABL], A.fc[FC_TABL_LO]);
            if (general) slab_fix<UNIFORM>(A, L, cls, cpitch, xx[j], yy[j], zz[j], Pdt, t_new, errbits, Ti, Ei, Tw, Ew);
            else if (Ts >= A.fc[FC_SCREEN]) rare_update_f32(A, vv[j], ni, tt[j], ee[j], t_new, true, oo[j]);
        }
    }
    return errbits;
}

template <bool UNIFORM>
__global__ void __launch_bounds__(BP *BR, bslab_minb(UNIFORM))
    batch_slab_kernel(const BatchInst *__restrict__ insts, int n, const int *__restrict__ prefix,
                      const BatchStep *__restrict__ steps, int K, BatchSync *sync, unsigned *err)
{
    using Lay = BLay<UNIFORM>;
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(16) unsigned char s_args_raw[sizeof(FusedArgs)];
    __shared__ __align__(16) unsigned char s_lut_raw[sizeof(ClassLut)];
    __shared__ BItem d;
    FusedArgs &A = *reinterpret_cast<FusedArgs *>(s_args_raw);
    const ClassLut &L = *reinterpret_cast<const ClassLut *>(s_lut_raw);
    unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + BS * Lay::STAGE);
    unsigned short *list = reinterpret_cast<unsigned short *>(sm + BS * Lay::STAGE + BS * 8);
    int *s_cnt = reinterpret_cast<int *>(sm + BS * Lay::STAGE + BS * 8 + Lay::LIST * 2);
    const int tid = threadIdx.x, r = tid / BP, p = tid % BP;
    constexpr int ARGS_W = (int)(sizeof(FusedArgs) / 4), LUT_W = (int)(sizeof(ClassLut) / 4);
    static_assert(sizeof(FusedArgs) % 4 == 0 && sizeof(ClassLut) % 4 == 0, "word copies");

    if (tid == 0) {
        for (int s = 0; s < BS; ++s) mbar_init(bar + s, BP * BR);  // every thread arrives on each phase
        fence_mbar_init();
    }
    __syncthreads();
    const int total = __ldg(prefix + n);
    int loaded = -1;
    uint32_t G = 0;  // planes this block has issued: plane g sits in stage g % BS, phase (g / BS) & 1
    for (int k = 0; k < K; ++k) {
        for (int item = blockIdx.x; item < total; item += gridDim.x) {
            // the item's instance: the last i with prefix[i] <= item
            int lo = 0, hi = n - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(prefix + mid) <= item) lo = mid;
                else hi = mid - 1;
            }
            const int inst = lo;
            const BatchStep st = steps[(int64_t)k * n + inst];
            if (!st.active) continue;  // block-uniform
            const BatchInst &I = insts[inst];
            // every thread has finished the previous item (its closing barrier)
            if (inst != loaded) {
                for (int w = tid; w < ARGS_W; w += BP * BR) ((uint32_t *)s_args_raw)[w] = ((const uint32_t *)&I.a)[w];
                for (int w = tid; w < LUT_W; w += BP * BR) ((uint32_t *)s_lut_raw)[w] = ((const uint32_t *)&I.L)[w];
                loaded = inst;
                __syncthreads();
            }
            if (tid == 0) {
                const int fc = (I.fcur + k) & 1;
                const int local = item - __ldg(prefix + inst), tx = I.tiles_x, ty = I.tiles_y;
                d.T = I.T[fc];
                d.E = I.E[fc];
                d.To = I.T[fc ^ 1];
                d.Eo = I.E[fc ^ 1];
                d.J = (const float *)I.a.J;
                d.C = I.cls;
                d.cpitch = I.cls_pitch;
                d.pdt = st.pdt;
                d.t_new = st.t_new;
                d.inst = inst;
                d.x0 = (local % tx) * BW;
                d.y0 = ((local / tx) % ty) * BR;
                d.z0 = (local / (tx * ty)) * I.zchunk;
                d.z1 = min(I.a.nz, d.z0 + I.zchunk);
                *s_cnt = 0;
            }
            __syncthreads();

            const int nx = A.nx, ny = A.ny, nz = A.nz, sz = nx * ny;  // instances hold < 2^31 voxels
            const int bxW = d.x0, byR = d.y0, z0 = d.z0, np = d.z1 - d.z0, last = np + 1;
            const int x = bxW + 2 * p, y = byR + r;
            const bool act = x < nx && y < ny;
            const bool half = act && x + 1 >= nx;  // the pair's second voxel lies outside the grid
            const float Pdt = d.pdt;
            const float cxd = A.fc[FC_DT] * A.fc[FC_CX], cyd = A.fc[FC_DT] * A.fc[FC_CY], czd = A.fc[FC_DT] * A.fc[FC_CZ];
            const int uc = L.uniform >= 0 ? L.uniform : 0;
            const float au = L.fa[uc * MAX_MAT + uc];
            const float Cx = cxd * au, Cy = cyd * au, Cz = czd * au, C6 = 2.f * ((Cx + Cy) + Cz);
            const float Ku = Pdt * L.irc[uc];
            const unsigned exy = (unsigned)(x == 0) | (unsigned)(x + 1 == nx - 1) << 1 | (unsigned)(y == 0) << 2 |
                                 (unsigned)(y == ny - 1) << 3;
            float rare_thr = A.fc[FC_SCREEN];
            if (A.boil && A.fc[FC_TBOIL] < rare_thr) rare_thr = A.fc[FC_TBOIL];
            const float lo_t = 0.5f * rare_thr;  // new temperatures outside (0, rare_thr) are listed

            // planes idx = 0 .. last (z = z0 - 1 .. z1): rows y0 - 1 .. y0 + 8 of T and
            // the Kahan term (11 chunks each), rows y0 .. y0 + 7 of J for the item's
            // own planes (9 chunks each) and the class rows (4 chunks each).  Every
            // thread copies one or two units of 16 bytes per array with cp.async
            // and then arrives on the stage's barrier, which completes once every
            // thread's copies have landed.  Units 0..109: T and Kahan-term chunk
            // (row u / 11, chunk u % 11); 110..181: J (row (u - 110) / 9);
            // 182..221: class rows (row (u - 182) / 4).  Thread t takes units t and
            // t + 128.  Per unit: its row's first index plus 4 x chunk (the plane's
            // offset is added, then the sum rounded down to a chunk), its shared
            // offset, and its kind (0: none, the row is outside the grid).
            int rbA = 0, rbB = 0, dA = 0, dB = 0, kA = 0, kB = 0;
            {
                auto unit = [&](int u, int &rb, int &dst, int &kind) {
                    if (u < 110) {
                        const int q = u / 11, c = u % 11, yy = byR - 1 + q;
                        if (yy >= 0 && yy < ny) kind = 1, rb = bxW - 4 + nx * yy + 4 * c, dst = Lay::T_OFF + q * RT * 4 + 16 * c;
                    } else if (u < 182) {
                        const int q = (u - 110) / 9, c = (u - 110) % 9, yy = byR + q;
                        if (yy < ny) kind = 2, rb = bxW + nx * yy + 4 * c, dst = Lay::J_OFF + q * RJ * 4 + 16 * c;
                    } else if (!UNIFORM && u < 222) {
                        const int q = (u - 182) / 4, c = (u - 182) % 4, yy = byR - 1 + q;
                        if (yy >= 0 && yy < ny) kind = 3, rb = d.cpitch * yy + bxW - 16 + 16 * c, dst = Lay::C_OFF + q * RC + 16 * c;
                    }
                };
                unit(tid, rbA, dA, kA);
                unit(tid + BP * BR, rbB, dB, kB);
            }
            auto issue = [&](int idx) {
                const uint32_t g = G + (uint32_t)idx;
                unsigned char *b = sm + (g % BS) * Lay::STAGE;
                const int zz = z0 - 1 + idx;
                if (zz >= 0 && zz < nz) {
                    const bool own = idx >= 1 && idx <= np;
                    const int pz = sz * zz;
                    if (kA == 1) {
                        const int q = (rbA + pz) & ~3;  // >= -4: inside the slack before the array
                        cp_async16(b + dA, d.T + q);
                        cp_async16(b + dA + (Lay::E_OFF - Lay::T_OFF), d.E + q);
                    } else if (kA == 2 && own) {
                        cp_async16(b + dA, d.J + ((rbA + pz) & ~3));
                    }
                    if (kB == 2 && own) cp_async16(b + dB, d.J + ((rbB + pz) & ~3));
                    else if (!UNIFORM && kB == 3) cp_async16(b + dB, d.C + (d.cpitch * ny * zz + rbB));
                }
                cp_async_arrive(bar + g % BS);
            };
            auto stage = [&](int idx) { return sm + ((G + (uint32_t)idx) % BS) * Lay::STAGE; };
            auto wait = [&](int idx) {
                const uint32_t g = G + (uint32_t)idx;
                return mbar_wait(bar + g % BS, (g / BS) & 1u);
            };

            for (int idx = 0; idx < BS && idx <= last; ++idx) issue(idx);
            int issued = BS < last + 1 ? BS : last + 1;
            bool ok = wait(0) && wait(1);
            // where a row starts inside its first chunk: (index of x0 - 4) & 3,
            // the same for the row's J (x0) and for both arrays
            const int dnx = nx & 3, dsz = sz & 3;
            int mc = (bxW + nx * y + sz * z0) & 3;  // row y of plane z (the one being updated)
            const int qC = (r + 1) * RC + 16 + 2 * p;
            float2 Tp = {0.f, 0.f}, Tc = {0.f, 0.f}, Ep = {0.f, 0.f}, Ec = {0.f, 0.f};
            int kp0 = uc, kp1 = uc, kc0 = uc, kc1 = uc;
            auto cls2 = [&](const unsigned char *b, int &k0, int &k1) {
                const unsigned short w = *reinterpret_cast<const unsigned short *>(b + Lay::C_OFF + qC);
                k0 = w & (MAX_MAT - 1);
                k1 = (w >> 8) & (MAX_MAT - 1);
            };
            auto ld2 = [](const unsigned char *b, int i) {
                const float *f = reinterpret_cast<const float *>(b);
                return make_float2(f[i], f[i + 1]);
            };
            if (ok && act) {
                const unsigned char *S1 = stage(1), *S0 = stage(0);
                const int o = (r + 1) * RT + mc + 4 + 2 * p;
                Tc = ld2(S1 + Lay::T_OFF, o);
                Ec = ld2(S1 + Lay::E_OFF, o);
                if (!UNIFORM) cls2(S1, kc0, kc1);
                if (z0 > 0) {
                    const int op = (r + 1) * RT + ((mc - dsz) & 3) + 4 + 2 * p;
                    Tp = ld2(S0 + Lay::T_OFF, op);
                    Ep = ld2(S0 + Lay::E_OFF, op);
                    if (!UNIFORM) cls2(S0, kp0, kp1);
                }
            }
            int v = x + nx * y + sz * z0;
            for (int i = 0; i < np; ++i, v += sz, mc = (mc + dsz) & 3) {
                // every thread is done with the stages of plane i - 1: its stage is free
                ok = __syncthreads_and(ok) != 0;
                if (!ok) break;
                if (i + BS <= last) {
                    issue(i + BS);
                    issued = i + BS + 1;
                }
                ok = wait(i + 2);
                if (!(ok && act)) continue;
                unsigned char *S = stage(i + 1);
                const unsigned char *N = stage(i + 2);
                const int z = z0 + i;
                const int mn = (mc + dsz) & 3, mym = (mc - dnx) & 3, myp = (mc + dnx) & 3;
                const int oS = (r + 1) * RT + mc + 4 + 2 * p;  // the pair in its row
                const int oM = r * RT + mym + 4 + 2 * p;       // ... in the row below (y - 1)
                const int oP = (r + 2) * RT + myp + 4 + 2 * p; // ... in the row above (y + 1)
                const int oN = (r + 1) * RT + mn + 4 + 2 * p;  // ... in the next plane
                const int oJ = r * RJ + mc + 2 * p;
                if (exy) {
                    // ghost neighbours of this thread's boundary faces, in its own halo cells
                    float *WT = reinterpret_cast<float *>(S + Lay::T_OFF), *WE = reinterpret_cast<float *>(S + Lay::E_OFF);
                    unsigned char *WC = S + Lay::C_OFF;
                    if (exy & 1u) {
                        const float2 g = ghost_pair(A, 0, Tc.x, Ec.x, L.k[kc0]);
                        WT[oS - 1] = g.x;
                        WE[oS - 1] = g.y;
                        if (!UNIFORM) WC[qC - 1] = (unsigned char)kc0;
                    }
                    if (exy & 2u) {
                        const float2 g = ghost_pair(A, 1, Tc.y, Ec.y, L.k[kc1]);
                        WT[oS + 2] = g.x;
                        WE[oS + 2] = g.y;
                        if (!UNIFORM) WC[qC + 2] = (unsigned char)kc1;
                    }
                    if (exy & 12u) {
                        const int f = (exy & 4u) ? 2 : 3, o = (exy & 4u) ? oM : oP, oc = (exy & 4u) ? -RC : RC;
                        const float2 g0 = ghost_pair(A, f, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(A, f, Tc.y, Ec.y, L.k[kc1]);
                        WT[o] = g0.x;
                        WT[o + 1] = g1.x;
                        WE[o] = g0.y;
                        WE[o + 1] = g1.y;
                        if (!UNIFORM) {
                            WC[qC + oc] = (unsigned char)kc0;
                            WC[qC + 1 + oc] = (unsigned char)kc1;
                        }
                    }
                }
                if (half) {
                    // the first voxel's x+ face is the grid boundary: its ghost takes the
                    // place of the (absent) second voxel, which is neither stored nor listed
                    const float2 g = ghost_pair(A, 1, Tc.x, Ec.x, L.k[kc0]);
                    Tc.y = g.x;
                    Ec.y = g.y;
                    kc1 = kc0;
                }
                const float2 Tn = ld2(N + Lay::T_OFF, oN), En = ld2(N + Lay::E_OFF, oN);
                const float2 tym = ld2(S + Lay::T_OFF, oM), typ = ld2(S + Lay::T_OFF, oP);
                const float2 eym = ld2(S + Lay::E_OFF, oM), eyp = ld2(S + Lay::E_OFF, oP);
                const float *ST = reinterpret_cast<const float *>(S + Lay::T_OFF);
                const float *SE = reinterpret_cast<const float *>(S + Lay::E_OFF);
                const float txl = ST[oS - 1], txr = ST[oS + 2], exl = SE[oS - 1], exr = SE[oS + 2];
                const float2 j2 = ld2(S + Lay::J_OFF, oJ);
                int kn0 = uc, kn1 = uc;
                if (!UNIFORM) cls2(N, kn0, kn1);
                // ghost neighbours of the z boundary planes (registers only)
                float2 Tpz = Tp, Epz = Ep;
                int kpz0 = kp0, kpz1 = kp1;
                if (z == 0) {
                    const float2 g0 = ghost_pair(A, 4, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(A, 4, Tc.y, Ec.y, L.k[kc1]);
                    Tpz = make_float2(g0.x, g1.x);
                    Epz = make_float2(g0.y, g1.y);
                    kpz0 = kc0;
                    kpz1 = kc1;
                }
                float2 Tnz = Tn, Enz = En;
                int knz0 = kn0, knz1 = kn1;
                if (z == nz - 1) {
                    const float2 g0 = ghost_pair(A, 5, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(A, 5, Tc.y, Ec.y, L.k[kc1]);
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
                    const float tzM = h ? Tpz.y : Tpz.x, tzP = h ? Tnz.y : Tnz.x, ezM = h ? Epz.y : Epz.x,
                                ezP = h ? Enz.y : Enz.x;
                    float dT;
                    if (UNIFORM) {
                        const float sx = ((txm - tc) + (txp - tc)) - (exm + exp_);
                        const float sy = ((tyM - tc) + (tyP - tc)) - (eyM + eyP);
                        const float sz_ = ((tzM - tc) + (tzP - tc)) - (ezM + ezP);
                        dT = __fmaf_rn(Cz, sz_, __fmaf_rn(Cy, sy, __fmaf_rn(Cx, sx, C6 * e0)));
                    } else {
                        const int kk = h ? kc1 : kc0;
                        const unsigned char *SC = S + Lay::C_OFF;
                        const float *frow = L.fa + kk * MAX_MAT;
                        const float axm = cxd * frow[h ? kc0 : (SC[qC - 1] & (MAX_MAT - 1))];
                        const float axp = cxd * frow[h ? (SC[qC + 2] & (MAX_MAT - 1)) : kc1];
                        const float aym = cyd * frow[SC[qC + h - RC] & (MAX_MAT - 1)];
                        const float ayp = cyd * frow[SC[qC + h + RC] & (MAX_MAT - 1)];
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
                    const float tm = tc > t ? tc : t;
                    if (!(fabsf(tm - lo_t) < lo_t)) fix |= 1u << h;
                    tn[h] = t;
                    en[h] = e;
                }
                // rows are not 8-byte aligned in general: scalar stores
                float *To = d.To + v, *Eo = d.Eo + v;
                To[0] = tn[0];
                Eo[0] = en[0];
                if (!half) {
                    To[1] = tn[1];
                    Eo[1] = en[1];
                } else {
                    fix &= 1u;
                }
                if (fix) {
                    const int nf = __popc(fix);
                    const int at = atomicAdd(s_cnt, nf);
                    const int l = (i * BR + r) * BW + 2 * p;
                    if (fix & 1u) list[at] = (unsigned short)l;
                    if (fix & 2u) list[at + nf - 1] = (unsigned short)(l + 1);
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
            if (!ok) {
                // wait (bounded) for this block's copies in flight, then leave;
                // the other blocks leave at their next grid barrier
                for (int idx = issued > BS ? issued - BS : 0; idx < issued; ++idx) (void)wait(idx);
                if (tid == 0) {
                    atomicOr(err, (unsigned)DEVERR_SYNC_TIMEOUT);
                    atomicOr(A.err, (unsigned)DEVERR_SYNC_TIMEOUT);
                    atomicExch(&sync->abort, 1u);
                }
                return;
            }
            // (the barrier above also made the block's plane stores and list visible)
            const unsigned errbits =
                list_pass<UNIFORM>(A, L, list, *s_cnt, bxW, byR, z0, d.T, d.E, d.To, d.Eo, d.C, d.cpitch, Pdt, d.t_new);
            if (errbits) atomicOr(A.err, errbits);
            G += (uint32_t)issued;
            __syncthreads();  // the next item rewrites the stages, the list and the instance's tables
        }
        if (k + 1 < K && !grid_barrier(sync, gridDim.x, err)) return;
    }
}

// ------------------------------------------- one step per launch, rare pass apart --
// The same item update with one block per item and one launch per step
// (batch.staged 4).  The voxels needing rare work are not handled by the
// block: each warp marks them per plane (one ballot word per voxel of the
// pair), and the block appends them to the step's list of rare voxels
// (indices into the batch's voxels) with one global atomic per item; a
// second kernel then works through that list for the whole GPU.  With the
// latent-heat fix-up and the damage update out of this kernel, the plane
// loop's registers set its occupancy.
#ifndef TAM_BSTEP_MINB
#define TAM_BSTEP_MINB 8  // 63 registers without spills; 8 blocks also fill the shared memory
#endif
template <bool UNIFORM> struct SLay {
    // + the marks: 8 words per plane of the longest item (dynamic)
    static constexpr int SMEM = BS * BLay<UNIFORM>::STAGE + BS * 8 + 128;
};

template <bool UNIFORM>
__global__ void __launch_bounds__(BP *BR, UNIFORM ? TAM_BSTEP_MINB : 5)
    batch_slab_step_kernel(const BatchInst *__restrict__ insts, int n, const int *__restrict__ prefix,
                           const int *__restrict__ vox0, const BatchStep *__restrict__ steps, int k, unsigned *rare,
                           unsigned *rare_cnt, unsigned *err)
{
    using Lay = BLay<UNIFORM>;
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(16) unsigned char s_args_raw[sizeof(FusedArgs)];
    __shared__ __align__(16) unsigned char s_lut_raw[sizeof(ClassLut)];
    __shared__ BItem d;
    __shared__ unsigned s_wsum[4], s_base;
    FusedArgs &A = *reinterpret_cast<FusedArgs *>(s_args_raw);
    const ClassLut &L = *reinterpret_cast<const ClassLut *>(s_lut_raw);
    unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + BS * Lay::STAGE);
    // per plane: 4 warps x 2 voxels of the pair, one word each (bit = lane)
    unsigned *s_mask = reinterpret_cast<unsigned *>(sm + BS * Lay::STAGE + BS * 8);
    const int tid = threadIdx.x, r = tid / BP, p = tid % BP;
    constexpr int ARGS_W = (int)(sizeof(FusedArgs) / 4), LUT_W = (int)(sizeof(ClassLut) / 4);
    const unsigned FULL = 0xffffffffu;

    const int item = blockIdx.x;
    int lo = 0, hi = n - 1;  // the item's instance: the last i with prefix[i] <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= item) lo = mid;
        else hi = mid - 1;
    }
    const int inst = lo;
    const BatchStep st = steps[(int64_t)k * n + inst];
    if (!st.active) return;  // block-uniform
    const BatchInst &I = insts[inst];
    if (tid == 0) {
        for (int s = 0; s < BS; ++s) mbar_init(bar + s, BP * BR);  // every thread arrives on each phase
        fence_mbar_init();
    }
    for (int w = tid; w < ARGS_W; w += BP * BR) ((uint32_t *)s_args_raw)[w] = ((const uint32_t *)&I.a)[w];
    for (int w = tid; w < LUT_W; w += BP * BR) ((uint32_t *)s_lut_raw)[w] = ((const uint32_t *)&I.L)[w];
    if (tid == 0) {
        const int fc = (I.fcur + k) & 1;
        const int local = item - __ldg(prefix + inst), tx = I.tiles_x, ty = I.tiles_y;
        d.T = I.T[fc];
        d.E = I.E[fc];
        d.To = I.T[fc ^ 1];
        d.Eo = I.E[fc ^ 1];
        d.J = (const float *)I.a.J;
        d.C = I.cls;
        d.cpitch = I.cls_pitch;
        d.pdt = st.pdt;
        d.t_new = st.t_new;
        d.inst = inst;
        d.x0 = (local % tx) * BW;
        d.y0 = ((local / tx) % ty) * BR;
        d.z0 = (local / (tx * ty)) * I.zchunk;
        d.z1 = min(I.a.nz, d.z0 + I.zchunk);
    }
    __syncthreads();
    const uint32_t G = 0;  // planes issued before this item (one item per block)

            const int nx = A.nx, ny = A.ny, nz = A.nz, sz = nx * ny;  // instances hold < 2^31 voxels
            const int bxW = d.x0, byR = d.y0, z0 = d.z0, np = d.z1 - d.z0, last = np + 1;
            const int x = bxW + 2 * p, y = byR + r;
            const bool act = x < nx && y < ny;
            const bool half = act && x + 1 >= nx;  // the pair's second voxel lies outside the grid
            const float Pdt = d.pdt;
            const float cxd = A.fc[FC_DT] * A.fc[FC_CX], cyd = A.fc[FC_DT] * A.fc[FC_CY], czd = A.fc[FC_DT] * A.fc[FC_CZ];
            const int uc = L.uniform >= 0 ? L.uniform : 0;
            const float au = L.fa[uc * MAX_MAT + uc];
            const float Cx = cxd * au, Cy = cyd * au, Cz = czd * au, C6 = 2.f * ((Cx + Cy) + Cz);
            const float Ku = Pdt * L.irc[uc];
            const unsigned exy = (unsigned)(x == 0) | (unsigned)(x + 1 == nx - 1) << 1 | (unsigned)(y == 0) << 2 |
                                 (unsigned)(y == ny - 1) << 3;
            float rare_thr = A.fc[FC_SCREEN];
            if (A.boil && A.fc[FC_TBOIL] < rare_thr) rare_thr = A.fc[FC_TBOIL];
            const float lo_t = 0.5f * rare_thr;  // new temperatures outside (0, rare_thr) are marked

            // planes idx = 0 .. last (z = z0 - 1 .. z1): rows y0 - 1 .. y0 + 8 of T and
            // the Kahan term (11 chunks each), rows y0 .. y0 + 7 of J for the item's
            // own planes (9 chunks each) and the class rows (4 chunks each).  Every
            // thread copies one or two units of 16 bytes per array with cp.async
            // and then arrives on the stage's barrier, which completes once every
            // thread's copies have landed.  Units 0..109: T and Kahan-term chunk
            // (row u / 11, chunk u % 11); 110..181: J (row (u - 110) / 9);
            // 182..221: class rows (row (u - 182) / 4).  Thread t takes units t and
            // t + 128.  Per unit: its row's first index plus 4 x chunk (the plane's
            // offset is added, then the sum rounded down to a chunk), its shared
            // offset, and its kind (0: none, the row is outside the grid).
            int rbA = 0, rbB = 0, dA = 0, dB = 0, kA = 0, kB = 0;
            {
                auto unit = [&](int u, int &rb, int &dst, int &kind) {
                    if (u < 110) {
                        const int q = u / 11, c = u % 11, yy = byR - 1 + q;
                        if (yy >= 0 && yy < ny) kind = 1, rb = bxW - 4 + nx * yy + 4 * c, dst = Lay::T_OFF + q * RT * 4 + 16 * c;
                    } else if (u < 182) {
                        const int q = (u - 110) / 9, c = (u - 110) % 9, yy = byR + q;
                        if (yy < ny) kind = 2, rb = bxW + nx * yy + 4 * c, dst = Lay::J_OFF + q * RJ * 4 + 16 * c;
                    } else if (!UNIFORM && u < 222) {
                        const int q = (u - 182) / 4, c = (u - 182) % 4, yy = byR - 1 + q;
                        if (yy >= 0 && yy < ny) kind = 3, rb = d.cpitch * yy + bxW - 16 + 16 * c, dst = Lay::C_OFF + q * RC + 16 * c;
                    }
                };
                unit(tid, rbA, dA, kA);
                unit(tid + BP * BR, rbB, dB, kB);
            }
            auto issue = [&](int idx) {
                const uint32_t g = G + (uint32_t)idx;
                unsigned char *b = sm + (g % BS) * Lay::STAGE;
                const int zz = z0 - 1 + idx;
                if (zz >= 0 && zz < nz) {
                    const bool own = idx >= 1 && idx <= np;
                    const int pz = sz * zz;
                    if (kA == 1) {
                        const int q = (rbA + pz) & ~3;  // >= -4: inside the slack before the array
                        cp_async16(b + dA, d.T + q);
                        cp_async16(b + dA + (Lay::E_OFF - Lay::T_OFF), d.E + q);
                    } else if (kA == 2 && own) {
                        cp_async16(b + dA, d.J + ((rbA + pz) & ~3));
                    }
                    if (kB == 2 && own) cp_async16(b + dB, d.J + ((rbB + pz) & ~3));
                    else if (!UNIFORM && kB == 3) cp_async16(b + dB, d.C + (d.cpitch * ny * zz + rbB));
                }
                cp_async_arrive(bar + g % BS);
            };
            auto stage = [&](int idx) { return sm + ((G + (uint32_t)idx) % BS) * Lay::STAGE; };
            auto wait = [&](int idx) {
                const uint32_t g = G + (uint32_t)idx;
                return mbar_wait(bar + g % BS, (g / BS) & 1u);
            };

            for (int idx = 0; idx < BS && idx <= last; ++idx) issue(idx);
            int issued = BS < last + 1 ? BS : last + 1;
            bool ok = wait(0) && wait(1);
            // where a row starts inside its first chunk: (index of x0 - 4) & 3,
            // the same for the row's J (x0) and for both arrays
            const int dnx = nx & 3, dsz = sz & 3;
            int mc = (bxW + nx * y + sz * z0) & 3;  // row y of plane z (the one being updated)
            const int qC = (r + 1) * RC + 16 + 2 * p;
            float2 Tp = {0.f, 0.f}, Tc = {0.f, 0.f}, Ep = {0.f, 0.f}, Ec = {0.f, 0.f};
            int kp0 = uc, kp1 = uc, kc0 = uc, kc1 = uc;
            auto cls2 = [&](const unsigned char *b, int &k0, int &k1) {
                const unsigned short w = *reinterpret_cast<const unsigned short *>(b + Lay::C_OFF + qC);
                k0 = w & (MAX_MAT - 1);
                k1 = (w >> 8) & (MAX_MAT - 1);
            };
            auto ld2 = [](const unsigned char *b, int i) {
                const float *f = reinterpret_cast<const float *>(b);
                return make_float2(f[i], f[i + 1]);
            };
            if (ok && act) {
                const unsigned char *S1 = stage(1), *S0 = stage(0);
                const int o = (r + 1) * RT + mc + 4 + 2 * p;
                Tc = ld2(S1 + Lay::T_OFF, o);
                Ec = ld2(S1 + Lay::E_OFF, o);
                if (!UNIFORM) cls2(S1, kc0, kc1);
                if (z0 > 0) {
                    const int op = (r + 1) * RT + ((mc - dsz) & 3) + 4 + 2 * p;
                    Tp = ld2(S0 + Lay::T_OFF, op);
                    Ep = ld2(S0 + Lay::E_OFF, op);
                    if (!UNIFORM) cls2(S0, kp0, kp1);
                }
            }
            int v = x + nx * y + sz * z0;
            for (int i = 0; i < np; ++i, v += sz, mc = (mc + dsz) & 3) {
                // every thread is done with the stages of plane i - 1: its stage is free
                ok = __syncthreads_and(ok) != 0;
                if (!ok) break;
                if (i + BS <= last) {
                    issue(i + BS);
                    issued = i + BS + 1;
                }
                ok = wait(i + 2);
                unsigned fix = 0;
                float2 Tn = {0.f, 0.f}, En = {0.f, 0.f};
                int kn0 = uc, kn1 = uc;
                if (ok && act) {
                unsigned char *S = stage(i + 1);
                const unsigned char *N = stage(i + 2);
                const int z = z0 + i;
                const int mn = (mc + dsz) & 3, mym = (mc - dnx) & 3, myp = (mc + dnx) & 3;
                const int oS = (r + 1) * RT + mc + 4 + 2 * p;  // the pair in its row
                const int oM = r * RT + mym + 4 + 2 * p;       // ... in the row below (y - 1)
                const int oP = (r + 2) * RT + myp + 4 + 2 * p; // ... in the row above (y + 1)
                const int oN = (r + 1) * RT + mn + 4 + 2 * p;  // ... in the next plane
                const int oJ = r * RJ + mc + 2 * p;
                if (exy) {
                    // ghost neighbours of this thread's boundary faces, in its own halo cells
                    float *WT = reinterpret_cast<float *>(S + Lay::T_OFF), *WE = reinterpret_cast<float *>(S + Lay::E_OFF);
                    unsigned char *WC = S + Lay::C_OFF;
                    if (exy & 1u) {
                        const float2 g = ghost_pair(A, 0, Tc.x, Ec.x, L.k[kc0]);
                        WT[oS - 1] = g.x;
                        WE[oS - 1] = g.y;
                        if (!UNIFORM) WC[qC - 1] = (unsigned char)kc0;
                    }
                    if (exy & 2u) {
                        const float2 g = ghost_pair(A, 1, Tc.y, Ec.y, L.k[kc1]);
                        WT[oS + 2] = g.x;
                        WE[oS + 2] = g.y;
                        if (!UNIFORM) WC[qC + 2] = (unsigned char)kc1;
                    }
                    if (exy & 12u) {
                        const int f = (exy & 4u) ? 2 : 3, o = (exy & 4u) ? oM : oP, oc = (exy & 4u) ? -RC : RC;
                        const float2 g0 = ghost_pair(A, f, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(A, f, Tc.y, Ec.y, L.k[kc1]);
                        WT[o] = g0.x;
                        WT[o + 1] = g1.x;
                        WE[o] = g0.y;
                        WE[o + 1] = g1.y;
                        if (!UNIFORM) {
                            WC[qC + oc] = (unsigned char)kc0;
                            WC[qC + 1 + oc] = (unsigned char)kc1;
                        }
                    }
                }
                if (half) {
                    // the first voxel's x+ face is the grid boundary: its ghost takes the
                    // place of the (absent) second voxel, which is neither stored nor listed
                    const float2 g = ghost_pair(A, 1, Tc.x, Ec.x, L.k[kc0]);
                    Tc.y = g.x;
                    Ec.y = g.y;
                    kc1 = kc0;
                }
                Tn = ld2(N + Lay::T_OFF, oN);
                En = ld2(N + Lay::E_OFF, oN);
                const float2 tym = ld2(S + Lay::T_OFF, oM), typ = ld2(S + Lay::T_OFF, oP);
                const float2 eym = ld2(S + Lay::E_OFF, oM), eyp = ld2(S + Lay::E_OFF, oP);
                const float *ST = reinterpret_cast<const float *>(S + Lay::T_OFF);
                const float *SE = reinterpret_cast<const float *>(S + Lay::E_OFF);
                const float txl = ST[oS - 1], txr = ST[oS + 2], exl = SE[oS - 1], exr = SE[oS + 2];
                const float2 j2 = ld2(S + Lay::J_OFF, oJ);
                if (!UNIFORM) cls2(N, kn0, kn1);
                // ghost neighbours of the z boundary planes (registers only)
                float2 Tpz = Tp, Epz = Ep;
                int kpz0 = kp0, kpz1 = kp1;
                if (z == 0) {
                    const float2 g0 = ghost_pair(A, 4, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(A, 4, Tc.y, Ec.y, L.k[kc1]);
                    Tpz = make_float2(g0.x, g1.x);
                    Epz = make_float2(g0.y, g1.y);
                    kpz0 = kc0;
                    kpz1 = kc1;
                }
                float2 Tnz = Tn, Enz = En;
                int knz0 = kn0, knz1 = kn1;
                if (z == nz - 1) {
                    const float2 g0 = ghost_pair(A, 5, Tc.x, Ec.x, L.k[kc0]), g1 = ghost_pair(A, 5, Tc.y, Ec.y, L.k[kc1]);
                    Tnz = make_float2(g0.x, g1.x);
                    Enz = make_float2(g0.y, g1.y);
                    knz0 = kc0;
                    knz1 = kc1;
                }
                float tn[2], en[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float tc = h ? Tc.y : Tc.x, e0 = h ? Ec.y : Ec.x;
                    const float txm = h ? Tc.x : txl, txp = h ? txr : Tc.y, exm = h ? Ec.x : exl, exp_ = h ? exr : Ec.y;
                    const float tyM = h ? tym.y : tym.x, tyP = h ? typ.y : typ.x;
                    const float eyM = h ? eym.y : eym.x, eyP = h ? eyp.y : eyp.x;
                    const float tzM = h ? Tpz.y : Tpz.x, tzP = h ? Tnz.y : Tnz.x, ezM = h ? Epz.y : Epz.x,
                                ezP = h ? Enz.y : Enz.x;
                    float dT;
                    if (UNIFORM) {
                        const float sx = ((txm - tc) + (txp - tc)) - (exm + exp_);
                        const float sy = ((tyM - tc) + (tyP - tc)) - (eyM + eyP);
                        const float sz_ = ((tzM - tc) + (tzP - tc)) - (ezM + ezP);
                        dT = __fmaf_rn(Cz, sz_, __fmaf_rn(Cy, sy, __fmaf_rn(Cx, sx, C6 * e0)));
                    } else {
                        const int kk = h ? kc1 : kc0;
                        const unsigned char *SC = S + Lay::C_OFF;
                        const float *frow = L.fa + kk * MAX_MAT;
                        const float axm = cxd * frow[h ? kc0 : (SC[qC - 1] & (MAX_MAT - 1))];
                        const float axp = cxd * frow[h ? (SC[qC + 2] & (MAX_MAT - 1)) : kc1];
                        const float aym = cyd * frow[SC[qC + h - RC] & (MAX_MAT - 1)];
                        const float ayp = cyd * frow[SC[qC + h + RC] & (MAX_MAT - 1)];
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
                    const float tm = tc > t ? tc : t;
                    if (!(fabsf(tm - lo_t) < lo_t)) fix |= 1u << h;
                    tn[h] = t;
                    en[h] = e;
                }
                // rows are not 8-byte aligned in general: scalar stores
                float *To = d.To + v, *Eo = d.Eo + v;
                To[0] = tn[0];
                Eo[0] = en[0];
                if (!half) {
                    To[1] = tn[1];
                    Eo[1] = en[1];
                } else {
                    fix &= 1u;
                }
                }
                // the plane's marks: per warp, one word per voxel of the pair (bit = lane)
                {
                    const unsigned b0 = __ballot_sync(0xffffffffu, (fix & 1u) != 0u);
                    const unsigned b1 = __ballot_sync(0xffffffffu, (fix & 2u) != 0u);
                    if ((tid & 31) == 0) {
                        s_mask[(i * 4 + (tid >> 5)) * 2] = b0;
                        s_mask[(i * 4 + (tid >> 5)) * 2 + 1] = b1;
                    }
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
            // the last plane's wait may have failed in some threads only: agree
            // (the barrier also makes every warp's marks visible)
            ok = __syncthreads_and(ok) != 0;
            if (!ok) {
                for (int idx = issued > BS ? issued - BS : 0; idx < issued; ++idx) (void)wait(idx);
                if (tid == 0) {
                    atomicOr(err, (unsigned)DEVERR_SYNC_TIMEOUT);
                    atomicOr(A.err, (unsigned)DEVERR_SYNC_TIMEOUT);
                }
                return;
            }
            // the marked voxels join the step's list: a block-wide prefix sum of the
            // marks' counts, one global atomic for the item's share of the list
            // thread t takes words t, t + 128, ... (BATCH_STEP_ZMAX planes: at most 8)
            const int nw = np * 8;
            unsigned c = 0;
            for (int wi = tid; wi < nw; wi += BP * BR) c += __popc(s_mask[wi]);
            unsigned incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned t = __shfl_up_sync(FULL, incl, o);
                if ((tid & 31) >= o) incl += t;
            }
            if ((tid & 31) == 31) s_wsum[tid >> 5] = incl;
            __syncthreads();
            unsigned wofs = 0, tot = 0;
#pragma unroll
            for (int wp = 0; wp < BP * BR / 32; ++wp) {
                const unsigned t = s_wsum[wp];
                if (wp < (tid >> 5)) wofs += t;
                tot += t;
            }
            if (tid == 0) s_base = tot ? atomicAdd(rare_cnt, tot) : 0u;
            __syncthreads();
            if (c) {
                unsigned at = s_base + wofs + incl - c;
                const int vb = __ldg(vox0 + inst);
                auto emit = [&](unsigned word, int wi) {
                    const int i = wi >> 3, wp = (wi >> 1) & 3, h = wi & 1;
                    while (word) {
                        const int l = __ffs(word) - 1;
                        word &= word - 1;
                        const int xx = bxW + 2 * (l & 15) + h, yy = byR + 2 * wp + (l >> 4);
                        rare[at++] = (unsigned)(vb + xx + nx * yy + sz * (z0 + i));
                    }
                };
                for (int wi = tid; wi < nw; wi += BP * BR) emit(s_mask[wi], wi);
            }
}

// The step's list of rare voxels, for the whole GPU: each entry's instance
// (by the batch's voxel offsets), its latent-heat fix-up when it was boiling,
// is ablating or went negative / NaN, else its damage update.
template <bool UNIFORM>
__global__ void __launch_bounds__(256)
    batch_rare_kernel(const BatchInst *__restrict__ insts, int n, const int *__restrict__ vox0,
                      const BatchStep *__restrict__ steps, int k, const unsigned *__restrict__ rare,
                      const unsigned *rare_cnt)
{
    const unsigned cnt = *rare_cnt;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += gridDim.x * blockDim.x) {
        const int g = (int)rare[q];
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(vox0 + mid) <= g) lo = mid;
            else hi = mid - 1;
        }
        const BatchInst &I = insts[lo];
        const FusedArgs &a = I.a;
        const BatchStep st = steps[(int64_t)k * n + lo];
        const int fc = (I.fcur + k) & 1;
        const float *Ti = I.T[fc], *Ei = I.E[fc];
        float *To = I.T[fc ^ 1], *Eo = I.E[fc ^ 1];
        const int nx = a.nx, ny = a.ny, v = g - __ldg(vox0 + lo);
        const int x = v % nx, y = (v / nx) % ny, z = v / (nx * ny);
        const float t = To[v], e = Eo[v], tc = Ti[v];
        const float Ts = t - e;
        unsigned bits = 0;
        const bool general = (a.boil && tc >= a.fc[FC_TBOIL]) || !(Ts >= 0.f) ||
                             ge_ff(t, e, a.fc[FC_TABL], a.fc[FC_TABL_LO]);
        if (general) slab_fix<UNIFORM>(a, I.L, I.cls, I.cls_pitch, x, y, z, st.pdt, st.t_new, bits, Ti, Ei, To, Eo);
        else if (Ts >= a.fc[FC_SCREEN]) rare_update_f32(a, v, (int64_t)nx * ny * a.nz, t, e, st.t_new);
        if (bits) atomicOr(a.err, bits);
    }
}

template <bool UNIFORM> cudaError_t prepare()
{
    static bool done[64] = {false};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 64 && done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(batch_slab_kernel<UNIFORM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             BLay<UNIFORM>::SMEM);
    if (e == cudaSuccess && dev < 64) done[dev] = true;
    return e;
}

}  // namespace

cudaError_t batch_slab_blocks(int *blocks, bool uniform)
{
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = uniform ? prepare<true>() : prepare<false>();
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = uniform ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_slab_kernel<true>, BP * BR,
                                                                    BLay<true>::SMEM)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_slab_kernel<false>, BP * BR,
                                                                    BLay<false>::SMEM);
    if (e != cudaSuccess) return e;
    *blocks = sms * (per > 0 ? per : 1);
    return cudaSuccess;
}

cudaError_t launch_batch_slab(const BatchInst *insts, int n, const int *prefix, const BatchStep *steps, int K,
                              BatchSync *sync, unsigned *err, int blocks, bool uniform, cudaStream_t s)
{
    if (n <= 0 || K <= 0) return cudaSuccess;
    cudaError_t e = uniform ? prepare<true>() : prepare<false>();
    if (e == cudaSuccess) e = cudaMemsetAsync(sync, 0, sizeof(BatchSync), s);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&insts, (void *)&n, (void *)&prefix, (void *)&steps, (void *)&K, (void *)&sync,
                    (void *)&err};
    count_launch();
    if (uniform)
        return cudaLaunchCooperativeKernel((const void *)batch_slab_kernel<true>, dim3(blocks), dim3(BP * BR), args,
                                           BLay<true>::SMEM, s);
    return cudaLaunchCooperativeKernel((const void *)batch_slab_kernel<false>, dim3(blocks), dim3(BP * BR), args,
                                       BLay<false>::SMEM, s);
}

cudaError_t launch_batch_slab_steps(const BatchInst *insts, int n, const int *prefix, int items, int zmax,
                                    const int *vox0, const BatchStep *steps, int K, unsigned *rare,
                                    unsigned *rare_cnt, unsigned *err, bool uniform, int sm_count, cudaStream_t s)
{
    if (n <= 0 || K <= 0 || items <= 0) return cudaSuccess;
    if (zmax < 1 || zmax > BATCH_STEP_ZMAX) return cudaErrorInvalidValue;
    const int mask = 8 * 4 * zmax;
    for (int k = 0; k < K; ++k) {
        cudaError_t e = cudaMemsetAsync(rare_cnt, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
        count_launch(2);
        if (uniform) {
            batch_slab_step_kernel<true><<<items, BP * BR, SLay<true>::SMEM + mask, s>>>(insts, n, prefix, vox0, steps,
                                                                                      k, rare, rare_cnt, err);
            batch_rare_kernel<true><<<sm_count * 8, 256, 0, s>>>(insts, n, vox0, steps, k, rare, rare_cnt);
        } else {
            batch_slab_step_kernel<false><<<items, BP * BR, SLay<false>::SMEM + mask, s>>>(insts, n, prefix, vox0,
                                                                                        steps, k, rare, rare_cnt,
                                                                                        err);
            batch_rare_kernel<false><<<sm_count * 8, 256, 0, s>>>(insts, n, vox0, steps, k, rare, rare_cnt);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace tam
