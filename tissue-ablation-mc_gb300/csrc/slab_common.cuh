// slab_common.cuh -- per-voxel pieces of the slab-form FP32 heat step shared
// by the single-instance kernel (heat_slab.cu) and the batched one
// (batch_slab.cu): the fix-up of a listed voxel and the ghost neighbour of a
// boundary face.
#pragma once

#include "heat_common.cuh"

namespace tam {
namespace {

// One listed voxel: the latent-heat clamp (src/3dFD.f90:169-175 in the
// config-mode form; the stencil redone from global memory with its ghost
// faces), the error word, then damage and ablation of the new temperature.
// Ti / Ei: the step's input temperature and Kahan term; To / Eo: its output.
// UNIFORM: every voxel around holds class `ucls` (default: the grid's one class).
template <bool UNIFORM>
__device__ __noinline__ void slab_fix(const FusedArgs &a, const ClassLut &L, const uint8_t *cls, int cpitch, int x,
                                      int y, int z, float Pdt, double t_new, unsigned &errbits, const float *Ti,
                                      const float *Ei, float *To, float *Eo, int ucls = -1)
{
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int64_t sy = nx, sz = (int64_t)nx * ny, ni = sz * nz, v = x + sy * y + sz * z;
    const float tc = Ti[v], e0 = Ei[v];
    float t = To[v], e = Eo[v];
    const int64_t cs = (int64_t)cpitch * ny;
    auto klass = [&](int xx, int yy, int zz) -> int {
        return UNIFORM ? (ucls >= 0 ? ucls : L.uniform) : (cls[xx + (int64_t)cpitch * yy + cs * zz] & (MAX_MAT - 1));
    };
    const int k = klass(x, y, z);
    if (a.boil && tc >= a.fc[FC_TBOIL]) {
        const float rr = L.rho[k], rc = rr * L.c[k];
        const float qv = a.fc[FC_LW] * rr * a.fc[FC_VVOX];
        float *Q = (float *)a.Q;
        const float Qv = Q[v];
        if (Qv < qv) {
            // dT of this step
            const unsigned gm = (unsigned)(x == 0) | (unsigned)(x == nx - 1) << 1 | (unsigned)(y == 0) << 2 |
                                (unsigned)(y == ny - 1) << 3 | (unsigned)(z == 0) << 4 | (unsigned)(z == nz - 1) << 5;
            const float dt = a.fc[FC_DT];
            const float cf[3] = {dt * a.fc[FC_CX], dt * a.fc[FC_CY], dt * a.fc[FC_CZ]};
            const int64_t st[3] = {1, sy, sz};
            float dT = 0.f;
#pragma unroll
            for (int f = 0; f < 6; ++f) {
                if (gm >> f & 1u) continue;
                const int ax = f >> 1, sg = (f & 1) ? 1 : -1;
                const int kn = klass(x + (ax == 0 ? sg : 0), y + (ax == 1 ? sg : 0), z + (ax == 2 ? sg : 0));
                const int64_t n = v + sg * st[ax];
                dT += cf[ax] * L.fa[k * MAX_MAT + kn] * ((Ti[n] - tc) - (Ei[n] - e0));
            }
            if (gm) dT += dt * ghost_faces(a, gm, tc, e0, L.k[k], L.rho[k], L.c[k]);
            const float Ein = (Pdt * ((const float *)a.J)[v] + rc * dT) * a.fc[FC_VVOX];
            if (Ein > 0.f) {
                const float qn = Qv + Ein;
                Q[v] = qn < qv ? qn : qv;
                t = a.fc[FC_TBOIL];
                e = a.fc[FC_TBOIL_E];
                To[v] = t;
                Eo[v] = e;
            }
        }
    }
    const float Ts = t - e;
    errbits |= (Ts == Ts) ? (Ts < 0.f ? (unsigned)DEVERR_NEG_T : 0u) : (unsigned)DEVERR_NAN;
    if (Ts >= a.fc[FC_SCREEN]) rare_update_f32(a, v, ni, t, e, t_new);
}

// The value pair (T, e) of a ghost neighbour across boundary face f of a
// voxel with pair (tc, e0) and conductivity k: the interior term
// (T - tc) - (e - e0) then equals the face's ghost difference
// (ghost_term in heat_common.cuh).  Dirichlet: (T_bc, 0).  Robin: the
// difference D = -(h d / k)((tc - T_amb) - e0) added to tc, with the
// rounding of tc + D carried in the Kahan term.
__device__ __forceinline__ float2 ghost_pair(const FusedArgs &a, int f, float tc, float e0, float k)
{
    if (a.bc_type[f] == BC_ROBIN) {
        const float D = -(a.fc[FC_BCHD + f] / k) * ((tc - a.fc[FC_BCTA + f]) - e0);
        const float tg = tc + D;
        return make_float2(tg, e0 + ((tg - tc) - D));
    }
    return make_float2(a.fc[FC_BCT + f], 0.f);
}

}  // namespace
}  // namespace tam
