// heat_tma.cu -- the FP32 + Kahan fused heat step with TMA plane staging.
//
// The physics of fused_kernel<float, true> (heat.cu) in two TMA forms:
//  * fused_tma_kernel: the face diffusivities k_f/(rho_f c_f) and 1/(rho c)
//    are precomputed per voxel (face_coeff_kernel) and staged with the planes;
//    used once k, rho or c have been uploaded per voxel;
//  * fused_cls_kernel: thermal properties by material class, face
//    coefficients from a class-pair table in shared memory; only T, the Kahan
//    term, J and (for heterogeneous grids) the class ids are staged.
// One elected thread streams each z-plane of the block's tile into a ring of
// shared-memory stages with cp.async.bulk.tensor, several planes ahead of the
// plane being updated; completion is tracked by one mbarrier per stage
// (transaction bytes), and every wait is bounded.  The x origin of a tile is
// rounded down to a 16-byte boundary (bx*32 - 4 for FP32, bx*32 - 16 for u8),
// so the FP32 x halo sits in columns 3 and 36 of a 40-wide row; out-of-range
// rows, columns and planes read as zeros and are never used (those faces take
// the boundary path).
#include <cuda.h>

#include <atomic>

#include "heat_common.cuh"
#include "tma_common.cuh"

namespace tam {

struct FusedTma {
    CUtensorMap T[2], E[2], ax, ay, az, irc, J;
};
struct FusedCls {  // tensor maps for 1 and 2 rows of voxels per thread
    CUtensorMap T[2][2], E[2][2], J[2], cls[2];
};

namespace {

constexpr int TS = 4;                                  // shared-memory stages
constexpr int TPITCH = FX + 8;                         // 40 floats per staged row
constexpr int TROWS = FY + 2;                          // 10 rows
constexpr int ARR_BYTES = ((TROWS * TPITCH * 4 + 127) / 128) * 128;  // 1664: T, E, Ax, Ay (with halo)
constexpr int OWN_BYTES = FY * FX * 4;                 // 1024: Az, 1/(rho c), J (own voxels)
constexpr int STAGE_BYTES = 4 * ARR_BYTES + 3 * OWN_BYTES;  // 9728
constexpr uint32_t TX_BYTES = 4u * TROWS * TPITCH * 4 + 3u * FY * FX * 4;  // bytes landed per plane
constexpr int SMEM_BYTES = TS * STAGE_BYTES + TS * 8 + 128;

static_assert(STAGE_BYTES % 128 == 0, "stage alignment");

struct Maps {  // the seven maps of one launch
    CUtensorMap T, E, ax, ay, az, irc, J;
};


struct View {  // one staged plane
    const float *T, *E, *ax, *ay, *az, *irc, *J;
};

__global__ void __launch_bounds__(FX *FY, 4)
    fused_tma_kernel(const __grid_constant__ FusedArgs a, const __grid_constant__ Maps m, int zchunk)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + TS * STAGE_BYTES);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = blockIdx.x * FX + tx, y = blockIdx.y * FY + ty;
    const bool in = x < a.nx && y < a.ny;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(a.nz, z0 + zchunk);
    const int nplanes = z1 - z0;
    const int64_t sy = a.nx, sz = (int64_t)a.nx * a.ny, ni = sz * a.nz;
    float *To = (float *)a.T_out, *Q = (float *)a.Q;
    float *Eo = a.Tc_out;
    const float dt = a.fc[FC_DT], Pdt = step_pdt<float>(a);
    const double t_new = step_tnew(a);
    const bool src_on = Pdt != 0.f;
    const bool xy_inner = x > 0 && x < a.nx - 1 && y > 0 && y < a.ny - 1;
    const bool leader = tx == 0 && ty == 0;
    const int gx = blockIdx.x * FX - 4, gy = blockIdx.y * FY - 1;
    unsigned errbits = 0;

    auto view = [&](int idx) {
        const unsigned char *b = sm + (idx % TS) * STAGE_BYTES;
        View v;
        v.T = (const float *)(b + 0 * ARR_BYTES);
        v.E = (const float *)(b + 1 * ARR_BYTES);
        v.ax = (const float *)(b + 2 * ARR_BYTES);
        v.ay = (const float *)(b + 3 * ARR_BYTES);
        v.az = (const float *)(b + 4 * ARR_BYTES);
        v.irc = (const float *)(b + 4 * ARR_BYTES + OWN_BYTES);
        v.J = (const float *)(b + 4 * ARR_BYTES + 2 * OWN_BYTES);
        return v;
    };
    // plane z0 - 1 + idx into stage idx % TS
    auto issue = [&](int idx) {
        unsigned char *b = sm + (idx % TS) * STAGE_BYTES;
        uint64_t *br = bar + (idx % TS);
        const int zz = z0 - 1 + idx;
        fence_proxy_async();
        mbar_expect_tx(br, TX_BYTES);
        tma_load_3d(b + 0 * ARR_BYTES, &m.T, gx, gy, zz, br);
        tma_load_3d(b + 1 * ARR_BYTES, &m.E, gx, gy, zz, br);
        tma_load_3d(b + 2 * ARR_BYTES, &m.ax, gx, gy, zz, br);
        tma_load_3d(b + 3 * ARR_BYTES, &m.ay, gx, gy, zz, br);
        tma_load_3d(b + 4 * ARR_BYTES, &m.az, gx + 4, gy + 1, zz, br);
        tma_load_3d(b + 4 * ARR_BYTES + OWN_BYTES, &m.irc, gx + 4, gy + 1, zz, br);
        tma_load_3d(b + 4 * ARR_BYTES + 2 * OWN_BYTES, &m.J, gx + 4, gy + 1, zz, br);
    };
    auto wait = [&](int idx) { return mbar_wait(bar + (idx % TS), (uint32_t)((idx / TS) & 1)); };

    if (leader) {
        for (int s = 0; s < TS; ++s) mbar_init(bar + s, 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    __syncthreads();
    if (leader) {
        issue(0);
        issue(1);
        if (nplanes >= 1) issue(2);
    }
    // every wait decision is made block-uniform before anyone acts on it
    bool ok = __syncthreads_and(wait(0) && wait(1)) != 0;
    const int q = (ty + 1) * TPITCH + tx + 4;  // own voxel in the halo'd arrays
    const int o = ty * FX + tx;                // own voxel in the own-only arrays
    // z column in registers: temperature, Kahan term, and the +z face coefficient
    float Tp = 0.f, ep = 0.f, azp = 0.f, Tc = 0.f, ec = 0.f, azc = 0.f;
    if (in && ok) {
        const View C0 = view(1);
        Tc = C0.T[q];
        ec = C0.E[q];
        azc = C0.az[o];
        if (z0 > 0) {
            const View Pm = view(0);
            Tp = Pm.T[q];
            ep = Pm.E[q];
            azp = Pm.az[o];
        }
    }
    int issued = nplanes >= 1 ? 3 : 2;  // planes idx < issued are (or were) in flight
    for (int i = 0; i < nplanes && ok; ++i) {
        const int z = z0 + i;
        const int64_t v = (int64_t)x + sy * y + sz * z;
        const bool has_n = z + 1 < a.nz;
        if (leader && i + 3 <= nplanes + 1) issue(i + 3);
        issued = i + 3 <= nplanes + 1 ? i + 4 : issued;
        ok = __syncthreads_and(wait(i + 2)) != 0;  // plane z+1 has landed for the whole block
        if (!ok) break;
        const View P = view(i + 1), N = view(i + 2);
        float Tn_ = 0.f, en_ = 0.f, azn = 0.f;
        if (in && has_n) {
            Tn_ = N.T[q];
            en_ = N.E[q];
            azn = N.az[o];
        }
        if (in) {
            const float Jv = src_on ? P.J[o] : 0.f;
            const float tzm = (Tp - Tc) - (ep - ec), tzp = (Tn_ - Tc) - (en_ - ec);
            const float txm = (P.T[q - 1] - Tc) - (P.E[q - 1] - ec), txp = (P.T[q + 1] - Tc) - (P.E[q + 1] - ec);
            const float tym = (P.T[q - TPITCH] - Tc) - (P.E[q - TPITCH] - ec),
                        typ = (P.T[q + TPITCH] - Tc) - (P.E[q + TPITCH] - ec);
            float lap;
            if (xy_inner && z > 0 && has_n) {
                lap = azp * tzm + azc * tzp + P.ay[q - TPITCH] * tym + P.ay[q] * typ + P.ax[q - 1] * txm +
                      P.ax[q] * txp;
            } else {
                // a face of this voxel lies on the grid boundary: ghost faces
                // use the voxel's own properties
                const float kk = ((const float *)a.k)[v], rr = ((const float *)a.rho)[v],
                            hh = ((const float *)a.c)[v];
                lap = z > 0 ? azp * tzm : ghost_term<float>(a, 4, Tc, ec, kk, rr, hh);
                lap += has_n ? azc * tzp : ghost_term<float>(a, 5, Tc, ec, kk, rr, hh);
                lap += y > 0 ? P.ay[q - TPITCH] * tym : ghost_term<float>(a, 2, Tc, ec, kk, rr, hh);
                lap += y < a.ny - 1 ? P.ay[q] * typ : ghost_term<float>(a, 3, Tc, ec, kk, rr, hh);
                lap += x > 0 ? P.ax[q - 1] * txm : ghost_term<float>(a, 0, Tc, ec, kk, rr, hh);
                lap += x < a.nx - 1 ? P.ax[q] * txp : ghost_term<float>(a, 1, Tc, ec, kk, rr, hh);
            }
            const float dT = dt * lap;
            const float sPJ = Pdt * Jv;
            const float src = sPJ * P.irc[o];
            float Tnew, Enew = 0.f;
            bool clamped = false;
            if (a.boil && Tc >= a.fc[FC_TBOIL]) {
                const float rr = ((const float *)a.rho)[v], rc = rr * ((const float *)a.c)[v];
                const float qv = a.fc[FC_LW] * rr * a.fc[FC_VVOX];
                const float Qv = Q[v];
                if (Qv < qv) {
                    const float Ein = (sPJ + rc * dT) * a.fc[FC_VVOX];
                    if (Ein > 0.f) {
                        const float qn = Qv + Ein;
                        Q[v] = qn < qv ? qn : qv;
                        Tnew = a.fc[FC_TBOIL];
                        Enew = a.fc[FC_TBOIL_E];
                        clamped = true;
                    }
                }
            }
            if (!clamped) {
                const float inc = dT + src;
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
            if (Ts >= a.fc[FC_SCREEN]) rare_update_f32(a, v, ni, Tnew, Enew, t_new);
        }
        __syncthreads();  // every thread is done with the stage the next issue overwrites
        Tp = Tc;
        ep = ec;
        azp = azc;
        Tc = Tn_;
        ec = en_;
        azc = azn;
    }
    if (!ok) {
        // a stage never completed: record it and drain what may still be in
        // flight (the last phase of each stage)
        errbits |= DEVERR_SYNC_TIMEOUT;
        for (int idx = issued > TS ? issued - TS : 0; idx < issued; ++idx) (void)wait(idx);
    }
    if (errbits) atomicOr(a.err, errbits);
}

// ------------------------------------------------------------------------
// Class-table form.  When the thermal properties are those of a material
// table indexed by a per-voxel class id (u8), the face coefficients need no
// arrays: k_f/(rho_f c_f) for a pair of classes comes from a 16 x 16 table in
// shared memory and 1/(rho c), k, rho, c from per-class tables.  Per plane the
// ring then stages T and the Kahan term (with halo), J (own voxels) and the
// class ids (with halo) -- 13 bytes read and 8 written per voxel instead of
// 28 + 8.  A uniform grid (one class everywhere) stages no class ids at all.
constexpr int CTS = 6;                          // stages of the class-table ring
constexpr int CPITCH = 64;                      // class row: x from bx*32 - 16, 64 bytes

// Stage layout of the class-table ring for RY rows of voxels per thread (the
// block covers 32 x 8*RY voxels per plane).
template <bool UNIFORM, int RY> struct ClsLayout {
    static constexpr int ROWS = FY * RY + 2;                                  // staged rows with halo
    static constexpr int TE_BYTES = ((ROWS * TPITCH * 4 + 127) / 128) * 128;  // T or Kahan term
    static constexpr int J_BYTES = FY * RY * FX * 4;                          // own voxels only
    static constexpr int C_BYTES = ((ROWS * CPITCH + 127) / 128) * 128;       // class ids with halo
    static constexpr int T_OFF = 0, E_OFF = TE_BYTES, J_OFF = 2 * TE_BYTES, C_OFF = 2 * TE_BYTES + J_BYTES;
    static constexpr int STAGE = ((C_OFF + (UNIFORM ? 0 : C_BYTES) + 127) / 128) * 128;
    static constexpr uint32_t TX =
        2u * ROWS * TPITCH * 4 + (uint32_t)J_BYTES + (UNIFORM ? 0u : (uint32_t)(ROWS * CPITCH));
    static constexpr int SMEM = CTS * STAGE + CTS * 8 + 128;
};

struct ClsMaps {  // the maps of one launch
    CUtensorMap T, E, J, cls;
};

template <bool UNIFORM, int RY>
__global__ void __launch_bounds__(FX *FY, RY == 1 ? 4 : 3)
    fused_cls_kernel(const __grid_constant__ FusedArgs a, const __grid_constant__ ClsMaps m,
                     const __grid_constant__ ClassLut L, int zchunk)
{
    using Lay = ClsLayout<UNIFORM, RY>;
    extern __shared__ unsigned char smem_raw[];
    __shared__ float s_fa[MAX_MAT * MAX_MAT];
    unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + CTS * Lay::STAGE);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = blockIdx.x * FX + tx, ybase = blockIdx.y * FY * RY + ty;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(a.nz, z0 + zchunk);
    const int nplanes = z1 - z0;
    const int last = nplanes + 1;  // plane indices 0 .. last (z0 - 1 .. z1)
    const int64_t sy = a.nx, sz = (int64_t)a.nx * a.ny, ni = sz * a.nz;
    float *To = (float *)a.T_out, *Q = (float *)a.Q;
    float *Eo = a.Tc_out;
    const float dt = a.fc[FC_DT], Pdt = step_pdt<float>(a);
    const double t_new = step_tnew(a);
    const float cx = a.fc[FC_CX], cy = a.fc[FC_CY], cz = a.fc[FC_CZ];
    const bool leader = tx == 0 && ty == 0;
    const int gx = blockIdx.x * FX - 4, gy = blockIdx.y * FY * RY - 1, gx8 = blockIdx.x * FX - 16;
    const int uc = L.uniform >= 0 ? L.uniform : 0;
    const float au = L.fa[uc * MAX_MAT + uc];
    const float Cx = cx * au, Cy = cy * au, Cz = cz * au;
    const float irc_u = L.irc[uc];
    unsigned errbits = 0;
    if (!UNIFORM)
        for (int t = ty * FX + tx; t < MAX_MAT * MAX_MAT; t += FX * FY) s_fa[t] = L.fa[t];

    auto stage = [&](int idx) { return sm + (idx % CTS) * Lay::STAGE; };
    auto issue = [&](int idx) {
        unsigned char *b = stage(idx);
        uint64_t *br = bar + (idx % CTS);
        const int zz = z0 - 1 + idx;
        fence_proxy_async();
        mbar_expect_tx(br, Lay::TX);
        tma_load_3d(b + Lay::T_OFF, &m.T, gx, gy, zz, br);
        tma_load_3d(b + Lay::E_OFF, &m.E, gx, gy, zz, br);
        tma_load_3d(b + Lay::J_OFF, &m.J, gx + 4, gy + 1, zz, br);
        if (!UNIFORM) tma_load_3d(b + Lay::C_OFF, &m.cls, gx8, gy, zz, br);
    };
    auto wait = [&](int idx) { return mbar_wait(bar + (idx % CTS), (uint32_t)((idx / CTS) & 1)); };

    if (leader) {
        for (int s = 0; s < CTS; ++s) mbar_init(bar + s, 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    __syncthreads();
    int issued = 0;  // planes 0 .. issued-1 have been issued
    if (leader)
        for (int idx = 0; idx <= CTS - 2 && idx <= last; ++idx) issue(idx);
    issued = (CTS - 1 < last + 1) ? CTS - 1 : last + 1;
    bool ok = __syncthreads_and(wait(0) && wait(1)) != 0;
    // z columns of this thread's RY voxels in registers
    float Tp[RY], ep[RY], Tc[RY], ec[RY];
    int kp[RY], kc[RY];
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const int row = ty + r * FY + 1;
        const int q = row * TPITCH + tx + 4, qc = row * CPITCH + tx + 16;
        Tp[r] = ep[r] = Tc[r] = ec[r] = 0.f;
        kp[r] = kc[r] = 0;
        if (ok) {
            const unsigned char *C0 = stage(1);
            Tc[r] = ((const float *)(C0 + Lay::T_OFF))[q];
            ec[r] = ((const float *)(C0 + Lay::E_OFF))[q];
            if (!UNIFORM) kc[r] = (C0 + Lay::C_OFF)[qc] & (MAX_MAT - 1);
            if (z0 > 0) {
                const unsigned char *Pm = stage(0);
                Tp[r] = ((const float *)(Pm + Lay::T_OFF))[q];
                ep[r] = ((const float *)(Pm + Lay::E_OFF))[q];
                if (!UNIFORM) kp[r] = (Pm + Lay::C_OFF)[qc] & (MAX_MAT - 1);
            }
        }
    }
    for (int i = 0; i < nplanes && ok; ++i) {
        const int z = z0 + i;
        const bool has_n = z + 1 < a.nz;
        if (i + CTS - 1 <= last) {
            if (leader) issue(i + CTS - 1);
            issued = i + CTS;
        }
        ok = __syncthreads_and(wait(i + 2)) != 0;  // plane z+1 has landed for the whole block
        if (!ok) break;
        const unsigned char *P = stage(i + 1), *N = stage(i + 2);
        const float *PT = (const float *)(P + Lay::T_OFF), *PE = (const float *)(P + Lay::E_OFF);
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            const int y = ybase + r * FY;
            const int row = ty + r * FY + 1;
            const int q = row * TPITCH + tx + 4, qc = row * CPITCH + tx + 16, o = (ty + r * FY) * FX + tx;
            float Tn_ = 0.f, en_ = 0.f;
            int kn = 0;
            if (has_n) {
                Tn_ = ((const float *)(N + Lay::T_OFF))[q];
                en_ = ((const float *)(N + Lay::E_OFF))[q];
                if (!UNIFORM) kn = (N + Lay::C_OFF)[qc] & (MAX_MAT - 1);
            }
            if (x < a.nx && y < a.ny) {
                const float tc = Tc[r], e0 = ec[r];
                const int k = UNIFORM ? uc : kc[r];
                const int64_t v = (int64_t)x + sy * y + sz * z;
                const float Jv = ((const float *)(P + Lay::J_OFF))[o];  // Pdt is 0 while the source is off
                // a voxel near the damage window: load its damage integral now so
                // the load overlaps the update below
                const bool near = tc >= a.fc[FC_SCREEN];
                double o_pre = 0.0;
                if (near) o_pre = a.omega[v];
                const float tzm = (Tp[r] - tc) - (ep[r] - e0), tzp = (Tn_ - tc) - (en_ - e0);
                const float txm = (PT[q - 1] - tc) - (PE[q - 1] - e0), txp = (PT[q + 1] - tc) - (PE[q + 1] - e0);
                const float tym = (PT[q - TPITCH] - tc) - (PE[q - TPITCH] - e0),
                            typ = (PT[q + TPITCH] - tc) - (PE[q + TPITCH] - e0);
                // face coefficients of the six faces (uniform: one value per axis)
                float axm = Cx, axp = Cx, aym = Cy, ayp = Cy, azm = Cz, azp = Cz;
                if (!UNIFORM) {
                    const unsigned char *PC = P + Lay::C_OFF;
                    const float *frow = s_fa + k * MAX_MAT;
                    axm = cx * frow[PC[qc - 1] & (MAX_MAT - 1)];
                    axp = cx * frow[PC[qc + 1] & (MAX_MAT - 1)];
                    aym = cy * frow[PC[qc - CPITCH] & (MAX_MAT - 1)];
                    ayp = cy * frow[PC[qc + CPITCH] & (MAX_MAT - 1)];
                    azm = cz * frow[kp[r]];
                    azp = cz * frow[kn];
                }
                float lap;
                if (x > 0 && x < a.nx - 1 && y > 0 && y < a.ny - 1 && z > 0 && has_n) {
                    // three independent two-term chains (short dependency depth)
                    lap = ((azm * tzm + azp * tzp) + (aym * tym + ayp * typ)) + (axm * txm + axp * txp);
                } else {
                    // a face of this voxel lies on the grid boundary: ghost faces
                    // use the voxel's own properties
                    const float kk = L.k[k], rr = L.rho[k], hh = L.c[k];
                    lap = z > 0 ? azm * tzm : ghost_term<float>(a, 4, tc, e0, kk, rr, hh);
                    lap += has_n ? azp * tzp : ghost_term<float>(a, 5, tc, e0, kk, rr, hh);
                    lap += y > 0 ? aym * tym : ghost_term<float>(a, 2, tc, e0, kk, rr, hh);
                    lap += y < a.ny - 1 ? ayp * typ : ghost_term<float>(a, 3, tc, e0, kk, rr, hh);
                    lap += x > 0 ? axm * txm : ghost_term<float>(a, 0, tc, e0, kk, rr, hh);
                    lap += x < a.nx - 1 ? axp * txp : ghost_term<float>(a, 1, tc, e0, kk, rr, hh);
                }
                const float dT = dt * lap;
                const float sPJ = Pdt * Jv;
                const float src = sPJ * (UNIFORM ? irc_u : L.irc[k]);
                float Tnew, Enew = 0.f;
                bool clamped = false;
                if (a.boil && tc >= a.fc[FC_TBOIL]) {
                    const float rr = L.rho[k], rc = rr * L.c[k];
                    const float qv = a.fc[FC_LW] * rr * a.fc[FC_VVOX];
                    const float Qv = Q[v];
                    if (Qv < qv) {
                        const float Ein = (sPJ + rc * dT) * a.fc[FC_VVOX];
                        if (Ein > 0.f) {
                            const float qn = Qv + Ein;
                            Q[v] = qn < qv ? qn : qv;
                            Tnew = a.fc[FC_TBOIL];
                            Enew = a.fc[FC_TBOIL_E];
                            clamped = true;
                        }
                    }
                }
                if (!clamped) {
                    const float inc = dT + src;
                    const float yk = inc - e0;
                    const float t = tc + yk;
                    Enew = (t - tc) - yk;
                    Tnew = t;
                }
                To[v] = Tnew;
                Eo[v] = Enew;
                const float Ts = Tnew - Enew;
                errbits |= (Ts == Ts) ? (Ts < 0.f ? (unsigned)DEVERR_NEG_T : 0u) : (unsigned)DEVERR_NAN;
                if (Ts >= a.fc[FC_SCREEN]) rare_update_f32(a, v, ni, Tnew, Enew, t_new, near, o_pre);
            }
            Tp[r] = Tc[r];
            ep[r] = ec[r];
            Tc[r] = Tn_;
            ec[r] = en_;
            kp[r] = kc[r];
            kc[r] = kn;
        }
        __syncthreads();  // every thread is done with the stage the next issue overwrites
    }
    if (!ok) {
        errbits |= DEVERR_SYNC_TIMEOUT;
        for (int idx = issued > CTS ? issued - CTS : 0; idx < issued; ++idx) (void)wait(idx);
    }
    if (errbits) atomicOr(a.err, errbits);
}

// Paired form of the class-table step: the same ring and stage layout, 128
// threads per 32 x 8 tile, each updating two x-adjacent voxels with 64-bit
// shared-memory loads and global stores (the staged rows start 16 bytes
// before the tile, so a pair sits at an even offset).  Per voxel it issues
// half the shared-memory loads, stores and per-plane work of the one-voxel
// form.  Needs nx even (the pair never straddles a row end).
// 7 resident blocks of 128 threads per SM (72 registers) measured fastest;
// the boundary faces' ghost terms and the pair's damage updates each go
// through one out-of-line call site, which keeps the spill at 8 bytes
#ifndef TAM_CLS2_MINB
#define TAM_CLS2_MINB 7
#endif
template <bool UNIFORM>
__global__ void __launch_bounds__(FX / 2 * FY, TAM_CLS2_MINB)
    fused_cls2_kernel(const __grid_constant__ FusedArgs a, const __grid_constant__ ClsMaps m,
                      const __grid_constant__ ClassLut L, int zchunk)
{
    using Lay = ClsLayout<UNIFORM, 1>;
    extern __shared__ unsigned char smem_raw[];
    __shared__ float s_fa[MAX_MAT * MAX_MAT];
    unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + CTS * Lay::STAGE);
    const int tp = threadIdx.x, ty = threadIdx.y;  // pair index 0..15, row 0..7
    const int tx = 2 * tp;                          // first voxel of the pair within the tile
    const int x = blockIdx.x * FX + tx, y = blockIdx.y * FY + ty;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(a.nz, z0 + zchunk);
    const int nplanes = z1 - z0;
    const int last = nplanes + 1;
    const int64_t sy = a.nx, sz = (int64_t)a.nx * a.ny, ni = sz * a.nz;
    float *To = (float *)a.T_out, *Q = (float *)a.Q;
    float *Eo = a.Tc_out;
    const float dt = a.fc[FC_DT], Pdt = step_pdt<float>(a);
    const double t_new = step_tnew(a);
    const float cx = a.fc[FC_CX], cy = a.fc[FC_CY], cz = a.fc[FC_CZ];
    const bool leader = tp == 0 && ty == 0;
    const int gx = blockIdx.x * FX - 4, gy = blockIdx.y * FY - 1, gx8 = blockIdx.x * FX - 16;
    const int uc = L.uniform >= 0 ? L.uniform : 0;
    const float au = L.fa[uc * MAX_MAT + uc];
    const float Cx = cx * au, Cy = cy * au, Cz = cz * au;
    const float irc_u = L.irc[uc];
    unsigned errbits = 0;
    if (!UNIFORM)
        for (int t = ty * (FX / 2) + tp; t < MAX_MAT * MAX_MAT; t += FX / 2 * FY) s_fa[t] = L.fa[t];

    auto stage = [&](int idx) { return sm + (idx % CTS) * Lay::STAGE; };
    auto issue = [&](int idx) {
        unsigned char *b = stage(idx);
        uint64_t *br = bar + (idx % CTS);
        const int zz = z0 - 1 + idx;
        fence_proxy_async();
        mbar_expect_tx(br, Lay::TX);
        tma_load_3d(b + Lay::T_OFF, &m.T, gx, gy, zz, br);
        tma_load_3d(b + Lay::E_OFF, &m.E, gx, gy, zz, br);
        tma_load_3d(b + Lay::J_OFF, &m.J, gx + 4, gy + 1, zz, br);
        if (!UNIFORM) tma_load_3d(b + Lay::C_OFF, &m.cls, gx8, gy, zz, br);
    };
    auto wait = [&](int idx) { return mbar_wait(bar + (idx % CTS), (uint32_t)((idx / CTS) & 1)); };

    if (leader) {
        for (int s = 0; s < CTS; ++s) mbar_init(bar + s, 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    __syncthreads();
    int issued = 0;
    if (leader)
        for (int idx = 0; idx <= CTS - 2 && idx <= last; ++idx) issue(idx);
    issued = (CTS - 1 < last + 1) ? CTS - 1 : last + 1;
    bool ok = __syncthreads_and(wait(0) && wait(1)) != 0;
    const int q = (ty + 1) * TPITCH + tx + 4;     // first voxel of the pair in the T / E rows (even)
    const int qc = (ty + 1) * CPITCH + tx + 16;   // ... in the class rows (even)
    const int o = ty * FX + tx;                   // ... in J (even)
    const bool in0 = x < a.nx && y < a.ny, in1 = x + 1 < a.nx && y < a.ny;
    float2 Tp = {0.f, 0.f}, ep = {0.f, 0.f}, Tc = {0.f, 0.f}, ec = {0.f, 0.f};
    int kp0 = 0, kp1 = 0, kc0 = 0, kc1 = 0;
    auto cls2 = [&](const unsigned char *b, int i, int &k0, int &k1) {
        const unsigned short w = *reinterpret_cast<const unsigned short *>(b + Lay::C_OFF + i);
        k0 = w & (MAX_MAT - 1);
        k1 = (w >> 8) & (MAX_MAT - 1);
    };
    if (ok) {
        const unsigned char *C0 = stage(1);
        Tc = *reinterpret_cast<const float2 *>((const float *)(C0 + Lay::T_OFF) + q);
        ec = *reinterpret_cast<const float2 *>((const float *)(C0 + Lay::E_OFF) + q);
        if (!UNIFORM) cls2(C0, qc, kc0, kc1);
        if (z0 > 0) {
            const unsigned char *Pm = stage(0);
            Tp = *reinterpret_cast<const float2 *>((const float *)(Pm + Lay::T_OFF) + q);
            ep = *reinterpret_cast<const float2 *>((const float *)(Pm + Lay::E_OFF) + q);
            if (!UNIFORM) cls2(Pm, qc, kp0, kp1);
        }
    }
    for (int i = 0; i < nplanes && ok; ++i) {
        const int z = z0 + i;
        const bool has_n = z + 1 < a.nz;
        if (i + CTS - 1 <= last) {
            if (leader) issue(i + CTS - 1);
            issued = i + CTS;
        }
        ok = __syncthreads_and(wait(i + 2)) != 0;
        if (!ok) break;
        const unsigned char *P = stage(i + 1), *N = stage(i + 2);
        const float *PT = (const float *)(P + Lay::T_OFF), *PE = (const float *)(P + Lay::E_OFF);
        float2 Tn = {0.f, 0.f}, en = {0.f, 0.f};
        int kn0 = 0, kn1 = 0;
        if (has_n) {
            Tn = *reinterpret_cast<const float2 *>((const float *)(N + Lay::T_OFF) + q);
            en = *reinterpret_cast<const float2 *>((const float *)(N + Lay::E_OFF) + q);
            if (!UNIFORM) cls2(N, qc, kn0, kn1);
        }
        if (in0) {
            const float2 Ty0 = *reinterpret_cast<const float2 *>(PT + q - TPITCH),
                         Ty1 = *reinterpret_cast<const float2 *>(PT + q + TPITCH);
            const float2 Ey0 = *reinterpret_cast<const float2 *>(PE + q - TPITCH),
                         Ey1 = *reinterpret_cast<const float2 *>(PE + q + TPITCH);
            const float Txl = PT[q - 1], Txr = PT[q + 2], Exl = PE[q - 1], Exr = PE[q + 2];
            const float2 Jv = *reinterpret_cast<const float2 *>((const float *)(P + Lay::J_OFF) + o);
            const int64_t v = (int64_t)x + sy * y + sz * z;
            float Tnew[2], Enew[2];
            unsigned hot = 0;
            // voxels near the damage window: load their damage integrals now so
            // the loads overlap the update below
            const bool near0 = Tc.x >= a.fc[FC_SCREEN], near1 = Tc.y >= a.fc[FC_SCREEN];
            double o_pre[2] = {0.0, 0.0};
            if (near0) o_pre[0] = a.omega[v];
            if (near1) o_pre[1] = a.omega[v + 1];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const bool inh = h == 0 || in1;
                const int xx = x + h;
                const float tc = h ? Tc.y : Tc.x, e0 = h ? ec.y : ec.x;
                const float tpz = h ? Tp.y : Tp.x, epz = h ? ep.y : ep.x;
                const float tnz = h ? Tn.y : Tn.x, enz = h ? en.y : en.x;
                const float txmT = h ? Tc.x : Txl, txmE = h ? ec.x : Exl;  // x- neighbour
                const float txpT = h ? Txr : Tc.y, txpE = h ? Exr : ec.y;  // x+ neighbour
                const float tymT = h ? Ty0.y : Ty0.x, tymE = h ? Ey0.y : Ey0.x;
                const float typT = h ? Ty1.y : Ty1.x, typE = h ? Ey1.y : Ey1.x;
                const int k = UNIFORM ? uc : (h ? kc1 : kc0);
                const float tzm = (tpz - tc) - (epz - e0), tzp = (tnz - tc) - (enz - e0);
                const float txm = (txmT - tc) - (txmE - e0), txp = (txpT - tc) - (txpE - e0);
                const float tym = (tymT - tc) - (tymE - e0), typ = (typT - tc) - (typE - e0);
                float axm = Cx, axp = Cx, aym = Cy, ayp = Cy, azm = Cz, azp = Cz;
                if (!UNIFORM) {
                    const unsigned char *PC = P + Lay::C_OFF;
                    const float *frow = s_fa + k * MAX_MAT;
                    const int cxm = h ? kc0 : (PC[qc - 1] & (MAX_MAT - 1));
                    const int cxp = h ? (PC[qc + 2] & (MAX_MAT - 1)) : kc1;
                    axm = cx * frow[cxm];
                    axp = cx * frow[cxp];
                    aym = cy * frow[PC[qc + h - CPITCH] & (MAX_MAT - 1)];
                    ayp = cy * frow[PC[qc + h + CPITCH] & (MAX_MAT - 1)];
                    azm = cz * frow[h ? kp1 : kp0];
                    azp = cz * frow[h ? kn1 : kn0];
                }
                float lap;
                if (xx > 0 && xx < a.nx - 1 && y > 0 && y < a.ny - 1 && z > 0 && has_n) {
                    lap = ((azm * tzm + azp * tzp) + (aym * tym + ayp * typ)) + (axm * txm + axp * txp);
                } else {
                    // boundary faces (bit f: x-, x+, y-, y+, z-, z+) take the ghost
                    // term, summed by one out-of-line call
                    const unsigned gm = (unsigned)(xx == 0) | (unsigned)(xx >= a.nx - 1) << 1 | (unsigned)(y == 0) << 2 |
                                        (unsigned)(y == a.ny - 1) << 3 | (unsigned)(z == 0) << 4 |
                                        (unsigned)(!has_n) << 5;
                    lap = ((gm & 16 ? 0.f : azm * tzm) + (gm & 32 ? 0.f : azp * tzp)) +
                          ((gm & 4 ? 0.f : aym * tym) + (gm & 8 ? 0.f : ayp * typ)) +
                          ((gm & 1 ? 0.f : axm * txm) + (gm & 2 ? 0.f : axp * txp));
                    if (inh) lap += ghost_faces(a, gm, tc, e0, L.k[k], L.rho[k], L.c[k]);
                }
                const float dT = dt * lap;
                const float sPJ = Pdt * (h ? Jv.y : Jv.x);
                const float src = sPJ * (UNIFORM ? irc_u : L.irc[k]);
                float tn = a.fc[FC_TBOIL], en_ = a.fc[FC_TBOIL_E];
                bool clamped = false;
                if (inh && a.boil && tc >= a.fc[FC_TBOIL]) {
                    const float rr = L.rho[k], rc = rr * L.c[k];
                    const float qv = a.fc[FC_LW] * rr * a.fc[FC_VVOX];
                    const float Qv = Q[v + h];
                    if (Qv < qv) {
                        const float Ein = (sPJ + rc * dT) * a.fc[FC_VVOX];
                        if (Ein > 0.f) {
                            const float qn = Qv + Ein;
                            Q[v + h] = qn < qv ? qn : qv;
                            clamped = true;
                        }
                    }
                }
                if (!clamped) {
                    const float inc = dT + src;
                    const float yk = inc - e0;
                    const float t = tc + yk;
                    en_ = (t - tc) - yk;
                    tn = t;
                }
                Tnew[h] = tn;
                Enew[h] = en_;
                const float Ts = tn - en_;
                if (inh) {
                    errbits |= (Ts == Ts) ? (Ts < 0.f ? (unsigned)DEVERR_NEG_T : 0u) : (unsigned)DEVERR_NAN;
                    if (Ts >= a.fc[FC_SCREEN]) hot |= 1u << h;
                }
            }
            // damage and ablation of the pair's voxels in the window, from one call site
#pragma unroll 1
            for (unsigned m = hot; m; m &= m - 1) {
                const int h = __ffs(m) - 1;
                rare_update_f32(a, v + h, ni, h ? Tnew[1] : Tnew[0], h ? Enew[1] : Enew[0], t_new,
                                h ? near1 : near0, h ? o_pre[1] : o_pre[0]);
            }
            if (in1) {
                *reinterpret_cast<float2 *>(To + v) = make_float2(Tnew[0], Tnew[1]);
                *reinterpret_cast<float2 *>(Eo + v) = make_float2(Enew[0], Enew[1]);
            } else {
                To[v] = Tnew[0];
                Eo[v] = Enew[0];
            }
        }
        __syncthreads();
        Tp = Tc;
        ep = ec;
        Tc = Tn;
        ec = en;
        kp0 = kc0;
        kp1 = kc1;
        kc0 = kn0;
        kc1 = kn1;
    }
    if (!ok) {
        errbits |= DEVERR_SYNC_TIMEOUT;
        for (int idx = issued > CTS ? issued - CTS : 0; idx < issued; ++idx) (void)wait(idx);
    }
    if (errbits) atomicOr(a.err, errbits);
}


// Class grid (row pitch `pitch`) from the material ids; ids beyond the table
// map to 0 as in the property fill.
__global__ void cls_from_mat_kernel(const uint8_t *mat, int nmat, uint8_t *cls, int nx, int ny, int nz, int pitch)
{
    const int64_t n = (int64_t)pitch * ny * nz;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(u % pitch);
        const int64_t row = u / pitch;
        uint8_t c = 0;
        if (x < nx) {
            const int m = mat[row * nx + x];
            c = (uint8_t)(m < nmat ? m : 0);
        }
        cls[u] = c;
    }
}

// Forward face coefficients of the FP32 step: A_x(v) = opscale/dx^2 *
// k_f/(rho_f c_f) on the face between v and v+x (arithmetic face means, as
// in the stencil of src/3dFD.f90:119-164), likewise A_y, A_z; and 1/(rho c).
__global__ void face_coeff_kernel(const float *k, const float *r, const float *c, float cx, float cy, float cz,
                                  int nx, int ny, int nz, float *ax, float *ay, float *az, float *irc)
{
    const int64_t n = (int64_t)nx * ny * nz, sy = nx, sz = (int64_t)nx * ny;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / sz);
        Pt<float> self;
        self.k = k[v];
        self.r = r[v];
        self.h = c[v];
        auto nb = [&](int64_t u) {
            Pt<float> p;
            p.k = k[u];
            p.r = r[u];
            p.h = c[u];
            return p;
        };
        ax[v] = x + 1 < nx ? cx * falpha(self, nb(v + 1)) : 0.f;
        ay[v] = y + 1 < ny ? cy * falpha(self, nb(v + sy)) : 0.f;
        az[v] = z + 1 < nz ? cz * falpha(self, nb(v + sz)) : 0.f;
        irc[v] = 1.f / (self.r * self.h);
    }
}

}  // namespace

cudaError_t launch_face_coeffs(const FusedArgs &a0, float *ax, float *ay, float *az, float *irc, cudaStream_t s)
{
    FusedArgs a = a0;
    fill_fused_consts(a);
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    count_launch();
    face_coeff_kernel<<<(unsigned)blocks, 256, 0, s>>>((const float *)a.k, (const float *)a.rho, (const float *)a.c,
                                                       a.fc[FC_CX], a.fc[FC_CY], a.fc[FC_CZ], a.nx, a.ny, a.nz, ax,
                                                       ay, az, irc);
    return cudaGetLastError();
}

bool fused_tma_supported(int nx) { return nx >= 1 && (nx * 4) % 16 == 0; }

cudaError_t fused_tma_create(FusedTma **out, int nx, int ny, int nz, float *const T[2], float *const Tc[2],
                             const float *ax, const float *ay, const float *az, const float *irc, const float *J)
{
    *out = nullptr;
    if (!fused_tma_supported(nx)) return cudaErrorNotSupported;
    cudaError_t e = encoder();
    if (e != cudaSuccess) return e;
    FusedTma *m = new FusedTma();
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = encode(&m->T[b], T[b], nx, ny, nz, TPITCH, TROWS);
        if (e == cudaSuccess) e = encode(&m->E[b], Tc[b], nx, ny, nz, TPITCH, TROWS);
    }
    if (e == cudaSuccess) e = encode(&m->ax, ax, nx, ny, nz, TPITCH, TROWS);
    if (e == cudaSuccess) e = encode(&m->ay, ay, nx, ny, nz, TPITCH, TROWS);
    if (e == cudaSuccess) e = encode(&m->az, az, nx, ny, nz, FX, FY);
    if (e == cudaSuccess) e = encode(&m->irc, irc, nx, ny, nz, FX, FY);
    if (e == cudaSuccess) e = encode(&m->J, J, nx, ny, nz, FX, FY);
    if (e != cudaSuccess) {
        delete m;
        return e;
    }
    *out = m;
    return cudaSuccess;
}

void fused_tma_destroy(FusedTma *m) { delete m; }

int cls_pitch_for(int nx) { return (nx + 15) / 16 * 16; }

cudaError_t launch_cls_from_mat(const uint8_t *mat, int nmat, uint8_t *cls, int nx, int ny, int nz, int pitch,
                                cudaStream_t s)
{
    const int64_t n = (int64_t)pitch * ny * nz;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) return cudaSuccess;
    count_launch();
    cls_from_mat_kernel<<<(unsigned)blocks, 256, 0, s>>>(mat, nmat, cls, nx, ny, nz, pitch);
    return cudaGetLastError();
}

cudaError_t fused_cls_create(FusedCls **out, int nx, int ny, int nz, float *const T[2], float *const Tc[2],
                             const float *J, const uint8_t *cls, int pitch)
{
    *out = nullptr;
    if (!fused_tma_supported(nx) || pitch % 16 != 0 || pitch < nx) return cudaErrorNotSupported;
    cudaError_t e = encoder();
    if (e != cudaSuccess) return e;
    FusedCls *m = new FusedCls();
    for (int ry = 1; ry <= 2 && e == cudaSuccess; ++ry) {
        const int rows = FY * ry + 2;
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
            e = encode(&m->T[ry - 1][b], T[b], nx, ny, nz, TPITCH, rows);
            if (e == cudaSuccess) e = encode(&m->E[ry - 1][b], Tc[b], nx, ny, nz, TPITCH, rows);
        }
        if (e == cudaSuccess) e = encode(&m->J[ry - 1], J, nx, ny, nz, FX, FY * ry);
        if (e == cudaSuccess) e = encode_u8(&m->cls[ry - 1], cls, pitch, ny, nz, CPITCH, rows);
    }
    if (e != cudaSuccess) {
        delete m;
        return e;
    }
    *out = m;
    return cudaSuccess;
}

void fused_cls_destroy(FusedCls *m) { delete m; }

namespace {
template <bool UNIFORM, int RY>
cudaError_t launch_cls_t(const FusedArgs &a, const ClsMaps &m, const ClassLut &L, cudaStream_t s)
{
    const int bx = (a.nx + FX - 1) / FX, by = (a.ny + FY * RY - 1) / (FY * RY);
    int zchunk = a.zchunk > 0 ? a.zchunk : 8;  // 8 planes per block measured fastest at 200^3
    if (zchunk > a.nz) zchunk = a.nz;
    const int chunks = (a.nz + zchunk - 1) / zchunk;
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
        e = cudaFuncSetAttribute(fused_cls_kernel<UNIFORM, RY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 ClsLayout<UNIFORM, RY>::SMEM);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    count_launch();
    fused_cls_kernel<UNIFORM, RY><<<dim3(bx, by, chunks), dim3(FX, FY), ClsLayout<UNIFORM, RY>::SMEM, s>>>(a, m, L,
                                                                                                     zchunk);
    return cudaGetLastError();
}
}  // namespace

namespace {
template <bool UNIFORM>
cudaError_t launch_cls2_t(const FusedArgs &a, const ClsMaps &m, const ClassLut &L, cudaStream_t s)
{
    const int bx = (a.nx + FX - 1) / FX, by = (a.ny + FY - 1) / FY;
    int zchunk = a.zchunk > 0 ? a.zchunk : 3;  // short columns, many blocks: measured fastest at 200^3
    if (zchunk > a.nz) zchunk = a.nz;
    const int chunks = (a.nz + zchunk - 1) / zchunk;
    const int smem = ClsLayout<UNIFORM, 1>::SMEM;
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
        e = cudaFuncSetAttribute(fused_cls2_kernel<UNIFORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    count_launch();
    fused_cls2_kernel<UNIFORM><<<dim3(bx, by, chunks), dim3(FX / 2, FY), smem, s>>>(a, m, L, zchunk);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_fused_cls(const FusedArgs &a0, const FusedCls *cm, int which, const ClassLut &L, int rows,
                             cudaStream_t s)
{
    FusedArgs a = a0;
    fill_fused_consts(a);
    if (rows == 0 && a.nx % 2 == 0) {  // paired form
        ClsMaps m;
        m.T = cm->T[0][which];
        m.E = cm->E[0][which];
        m.J = cm->J[0];
        m.cls = cm->cls[0];
        return L.uniform >= 0 ? launch_cls2_t<true>(a, m, L, s) : launch_cls2_t<false>(a, m, L, s);
    }
    const int ry = rows == 2 ? 2 : 1;
    ClsMaps m;
    m.T = cm->T[ry - 1][which];
    m.E = cm->E[ry - 1][which];
    m.J = cm->J[ry - 1];
    m.cls = cm->cls[ry - 1];
    if (ry == 1) return L.uniform >= 0 ? launch_cls_t<true, 1>(a, m, L, s) : launch_cls_t<false, 1>(a, m, L, s);
    return L.uniform >= 0 ? launch_cls_t<true, 2>(a, m, L, s) : launch_cls_t<false, 2>(a, m, L, s);
}

cudaError_t launch_fused_tma(const FusedArgs &a0, const FusedTma *tm, int which, cudaStream_t s)
{
    FusedArgs a = a0;
    fill_fused_consts(a);
    Maps m;
    m.T = tm->T[which];
    m.E = tm->E[which];
    m.ax = tm->ax;
    m.ay = tm->ay;
    m.az = tm->az;
    m.irc = tm->irc;
    m.J = tm->J;
    const int bx = (a.nx + FX - 1) / FX, by = (a.ny + FY - 1) / FY;
    int zchunk = a.zchunk > 0 ? a.zchunk : 8;  // 8 planes per block measured fastest at 200^3
    if (zchunk > a.nz) zchunk = a.nz;
    const int chunks = (a.nz + zchunk - 1) / zchunk;
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
        e = cudaFuncSetAttribute(fused_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    count_launch();
    fused_tma_kernel<<<dim3(bx, by, chunks), dim3(FX, FY), SMEM_BYTES, s>>>(a, m, zchunk);
    return cudaGetLastError();
}

}  // namespace tam
