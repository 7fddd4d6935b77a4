// tam_api.cpp -- the C ABI of include/tam.h.
//
// Host side of the drop-in boundary: context and device memory, the
// reference's set-up (src/mcpolar.f90:55-140, src/ch_opt.f90:7-25,
// src/gridset.f90:6-46, src/3dFD.f90:233-309), its outer driver loop and
// pulse state machine (src/mcpolar.f90:148-186, src/3dFD.f90:199-214), the
// res/input.params reader (src/mcpolar.f90:79-94) and the writer
// (src/writer.f90:6-81).  All grid work runs in the sm_103a kernels; there
// is no CPU fallback.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/tam.h"
#include "tam_kernels.h"
#include "tam_util.h"

#define TAM_VERSION_STRING "tam-gb300 0.1.0 (sm_103a)"

namespace {

thread_local std::string g_thread_err;

// Reference constants (src/constants.f90:12-13, src/thermalConst_mod.f90:5-6).
constexpr double WATER_INIT = 0.75;
constexpr double PROTEIN = 1.0 - WATER_INIT;
constexpr double AIR_HEAT_CAP = 1.006e3;
constexpr double LW = 2256.e3;
constexpr int SPOTS = 9 * 9;

double air_cond(double T) { return -0.188521 * std::exp(-(0.000367259 * (T - 273.15))) + 0.212453; }
double air_dens(double T) { return 101.325e3 / (287.058 * T); }
double skin_dens(double w) { return 1000.0 / (w + 0.649 * PROTEIN); }
double skin_cap(double w) { return 1000.0 * (4.2 * w + 1.09 * PROTEIN); }
double skin_cond(double w, double rho) { return rho * (6.28e-4 * w + 1.17e-4 * PROTEIN); }

}  // namespace

struct tam_ctx {
    tam_params p{};
    tam_config cfg{};
    bool config = false;
    bool fp64 = true;  // precision of transport and of the fused heat step
    int device = 0;
    int sm_count = 152;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;

    int nx = 0, ny = 0, nz = 0;
    int64_t ni = 0, nh = 0;

    // module scalars (opt_prop, Heat)
    double hgg = 0, g2 = 0, mua = 0, mus = 0, kappa_opt = 0, albedo = 0, mu_water = 0, mu_protein = 0, delta = 0;
    double delt = 0, dx = 0, dy = 0, dz = 0, volumeVoxel = 0, massVoxel = 0, QVapor = 0;
    double pulseLength = 0, realPulseLength = 0, total_time = 0;
    double time = 0, pulseCount = 0, repetitionCount = 0, laserOn = 1;
    int laser_flag = 1, pulseFlag = 0, pulsesDone = 0, loops_left = 0, counter = 0;

    // device buffers
    std::vector<void *> allocs;
    unsigned *d_err = nullptr;
    double *d_tally = nullptr;
    unsigned long long *d_work = nullptr, *d_nabl = nullptr, *d_cnt = nullptr;
    double *d_jmean = nullptr, *d_jglob = nullptr, *d_sum = nullptr;
    // reference mode
    double *d_T[2] = {nullptr, nullptr};
    int tcur = 0;
    double *d_rk[2] = {nullptr, nullptr};
    int rcur = 0;
    double *d_kappa = nullptr, *d_density = nullptr, *d_heatcap = nullptr, *d_coeff = nullptr, *d_alpha = nullptr;
    double *d_Q = nullptr, *d_water = nullptr, *d_tissue = nullptr, *d_thres = nullptr;
    // config mode
    void *d_Tf[2] = {nullptr, nullptr};
    float *d_Tc[2] = {nullptr, nullptr};
    int fcur = 0;
    void *d_k = nullptr, *d_rho = nullptr, *d_c = nullptr, *d_J = nullptr, *d_Qf = nullptr;
    uint8_t *d_mat = nullptr;
    double *d_halo = nullptr;  // scratch in the reference halo layout
    tam::MatThermal lut{};
    double cdt = 0;            // config-mode step
    bool need_trace = true;
    long long nabl_at_trace = 0;
    int32_t since_check = 0;   // heat steps since the last re-trace check (config mode)
    double props_delt = -1.0;  // delt of the last property update whose results are intact (<0: none)
    // reference mode, FP32 form: FP32 copies of the temperatures (ping-pong
    // with d_T) and of kappa, density, heatcap and coeff (4 x nh, in that
    // order), kept by the heat step and the property update; rebuilt from the
    // FP64 fields when anything else has written those (shadow_ok false)
    float *d_t32[2] = {nullptr, nullptr};
    float *d_p32 = nullptr;
    bool shadow_ok = false;

    // tuning knobs
    int scat_min = 20;
    int tally32 = -1;                // FP32 transport: -1 auto (FP32 tally when the FP64 one exceeds 256 MB), 0 off, 1 on
    int bricks = -1;                 // material lookups through the brick table: -1 auto (grids of 2^25 voxels
                                     // and more), 0 off, 1 on
    int64_t tally32_chunk = (int64_t)1 << 24;  // packets per flush of the FP32 tally (each launch ends in a tail)
    int64_t tally32_box = (int64_t)24 << 20;   // cells of the FP32 box tally at most (96 MB: L2-resident)
    int64_t j32_cells = 0;                     // cells allocated for the FP32 box tally
    float *d_j32 = nullptr;
    uint8_t *d_btab = nullptr;       // brick table of the material grid (transport on large grids)
    int zchunk = 0;
    bool use_tma = true;
    tam::FusedTma *tma = nullptr;  // tensor maps of the FP32 fused step
    float *d_ax = nullptr, *d_ay = nullptr, *d_az = nullptr, *d_irc = nullptr;  // its face coefficients
    bool coeff_dirty = true;
    // class-table form of the FP32 fused step: thermal properties by material
    // class (valid until k, rho or c are uploaded per voxel)
    bool use_cls = true;
    int cls_rows = 0;                // class-table step: 0 = voxel pairs (measured fastest), 1 or 2 rows
    bool arr_fp64 = false;           // FP32 form: FP64 Arrhenius exponent instead of float-float
    // heat steps replayed from CUDA graphs (single context, TMA and cp.async
    // fused forms): chunks of GRAPH_STEPS steps whose P dt and end times come
    // from a device table refreshed before each replay
    bool use_graph = true;
    bool heat_warm = false;                  // a step ran as an ordinary launch (kernel attributes set)
    cudaStream_t cap_stream = nullptr;       // capture stream (replays run on `stream`)
    tam::StepVals *d_sv = nullptr;           // the table
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // by the buffer pair the chunk reads first
    int glaunches[2] = {0, 0};                       // kernels in each graph
    std::vector<unsigned char> gkey[2];      // what the graphs were captured with
    // reference-mode outer iterations replayed from CUDA graphs: chunks of
    // REF_GRAPH_ITERS iterations whose changing values come from a device table
    bool ref_warm = false;                   // an iteration ran as ordinary launches
    tam::RefIterVals *d_iv = nullptr;
    cudaGraphExec_t rexec[4] = {nullptr, nullptr, nullptr, nullptr};  // by (temperature, rhokap) buffers read first
    std::vector<unsigned char> rkey[4];
    int batch_staged = 4;            // batched steps: slab form one launch per step (4) or persistent (3),
                                     // staged voxel pairs (2), staged voxels (1), cached loads (0)
    int batch_streams = 0;           // 1: batched steps as each instance's own steps on its stream, overlapped
    int batch_transport = 1;         // batched loops: the instances' uniform-medium passes in one launch
    int batch_zchunk = 0;            // batched steps: z planes per work item (0: heat.zchunk, else the default)
    // staged class-table step of this context alone (rows not aligned for TMA)
    tam::BatchInst *d_sinst = nullptr;
    int *d_sprefix = nullptr;
    tam::BatchInst h_sinst{};
    int s_items = 0;
    tam::FusedCls *fcls = nullptr;
    tam::FusedSlab *fslab = nullptr;
    bool use_slab = true;            // class-table step: the slab form where the grid allows it
    uint8_t *d_cls = nullptr;
    int cls_pitch = 0;
    bool thermal_by_class = false;
    int cls_uniform = -1;            // >= 0 while every voxel has this thermal class
    tam::ClassLut clut{};
    int uniform_id = -1;             // >= 0 while every voxel holds this material
    long long nabl_at_uniform = 0;

    // CUDA events around the transport kernel and the heat loop
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool have_mc_time = false, have_heat_time = false;
    int64_t heat_launches = 0;

    // last pass
    double tally[tam::N_TALLY] = {0};
    bool tally_stale = false;  // the host copy lags the device tallies (read back on demand)
    int64_t last_n = 0;
    int64_t mc_passes = 0;
    unsigned errbits_seen = 0;
};

namespace {
// The fields were written by something other than the heat step and the
// property update (set-up, an upload, a checkpoint load, new constants): the
// property update recomputes every voxel next time and the FP32 copies are
// rebuilt before the next heat step.
void fields_changed(tam_ctx *ctx)
{
    ctx->props_delt = -1.0;
    ctx->shadow_ok = false;
}
}  // namespace

namespace {

}  // namespace

void tam::set_thread_error(const std::string &msg) { g_thread_err = msg; }

namespace {

int fail(tam_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    g_thread_err = msg;
    return code;
}

#define CK(expr)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess) return fail(ctx, TAM_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define RC(expr)                      \
    do {                              \
        int r_ = (expr);              \
        if (r_ != TAM_OK) return r_;  \
    } while (0)

// Every context array has DPAD bytes of slack before and after it (the
// pointer stays 256-byte aligned): the batched heat step copies whole
// 16-byte-aligned chunks around a row, which may reach up to 16 bytes before
// an array and a row's length past its end.
constexpr size_t DPAD = 256;
int dalloc(tam_ctx *ctx, void **p, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    void *base = nullptr;
    cudaError_t e = cudaMalloc(&base, bytes + 2 * DPAD);
    if (e != cudaSuccess) {
        *p = nullptr;
        (void)cudaGetLastError();
        return fail(ctx, TAM_E_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                           cudaGetErrorString(e));
    }
    ctx->allocs.push_back(base);
    *p = (char *)base + DPAD;
    return TAM_OK;
}
// Free one array allocated by dalloc before the context ends.
void dfree(tam_ctx *ctx, void *p)
{
    if (!p) return;
    void *base = (char *)p - DPAD;
    ctx->allocs.erase(std::remove(ctx->allocs.begin(), ctx->allocs.end(), base), ctx->allocs.end());
    cudaFree(base);
}

template <typename T> int dalloc_t(tam_ctx *ctx, T **p, int64_t n)
{
    void *v = nullptr;
    int r = dalloc(ctx, &v, (size_t)n * sizeof(T));
    *p = (T *)v;
    return r;
}

// Wait for the stream, then fold the device error word into the status.
int finish(tam_ctx *ctx, const char *what)
{
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    unsigned bits = 0;
    CK(cudaMemcpy(&bits, ctx->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    const unsigned fresh = bits & ~ctx->errbits_seen;
    ctx->errbits_seen |= bits;
    if (fresh) {
        std::string m = std::string(what) + ": device error word 0x";
        char buf[16];
        std::snprintf(buf, sizeof buf, "%x", fresh);
        m += buf;
        if (fresh & TAM_DEVERR_STEP_CAP) m += " (packet step cap reached)";
        if (fresh & TAM_DEVERR_NAN) m += " (NaN)";
        if (fresh & TAM_DEVERR_NEG_T) m += " (negative temperature in kelvin)";
        return fail(ctx, TAM_E_DEVICE, m);
    }
    return TAM_OK;
}

// ----------------------------------------------------- pulse / getPwr --
// src/3dFD.f90:365-421 (procedure pointer selected in initThermalCoeff)
double get_pwr(tam_ctx *c)
{
    const double P = c->p.power;
    switch (c->p.pulse_type) {
    case TAM_PULSE_GAUSSIAN: {
        const double fact = 2. * std::sqrt(2. * std::log(2.));
        const double mu = fact * c->pulseLength, sig = c->pulseLength / fact;
        const double tm = c->time - mu;
        return P * std::exp(-((tm * tm) / (2.0 * (sig * sig))));
    }
    case TAM_PULSE_TOPHAT: return c->laser_flag ? P : 0.0;
    default: {
        const double m = P / c->pulseLength, cc = 2.0 * P;
        if (!c->laser_flag) return 0.0;
        double v;
        if (c->pulseFlag) {
            v = -m * c->time + cc;
        } else if (c->time >= c->pulseLength) {
            c->pulseFlag = 1;
            v = -m * c->time + cc;
        } else {
            return m * c->time;
        }
        return v < 0.0 ? 0.0 : v;
    }
    }
}

// src/3dFD.f90:199-214; returns true when this update switched the laser on
bool pulse_update(tam_ctx *c, double dt)
{
    bool on = false;
    if (c->pulseCount >= c->realPulseLength && c->laser_flag) {
        c->laser_flag = 0;
        c->laserOn = 0.;
        c->pulseCount = 0.;
        c->pulsesDone += 1;
        c->repetitionCount = 0.;
    } else if (c->repetitionCount >= c->p.repetition_rate_1 && !c->laser_flag && c->pulsesDone < c->p.pulses_to_do) {
        c->laser_flag = 1;
        c->laserOn = 1.;
        c->pulseCount = 0.;
        c->repetitionCount = 0.;
        on = true;
    }
    c->pulseCount += dt;
    c->repetitionCount += dt;
    c->time += dt;
    return on;
}

int validate_params(const tam_params *p, std::string &why)
{
    if (p->nxg < 1 || p->nyg < 1 || p->nzg < 1) { why = "grid sizes must be >= 1"; return 0; }
    if ((int64_t)p->nxg * p->nyg * p->nzg > (int64_t)1 << 34) { why = "grid too large"; return 0; }
    if (!(p->xmax > 0) || !(p->ymax > 0) || !(p->zmax > 0)) { why = "xmax, ymax, zmax must be > 0"; return 0; }
    if (p->nphotons < 0) { why = "nphotons must be >= 0"; return 0; }
    if (p->loops < 1) { why = "loops must be >= 1"; return 0; }
    if (p->numproc < 1) { why = "numproc must be >= 1"; return 0; }
    if (!(p->power > 0)) { why = "power must be > 0"; return 0; }
    if (p->pulse_type < 0 || p->pulse_type > 2) { why = "no pulse type"; return 0; }
    if (p->mode != TAM_MODE_REFERENCE && p->mode != TAM_MODE_CONFIG) { why = "bad mode"; return 0; }
    if (p->precision != TAM_FP64 && p->precision != TAM_FP32) { why = "bad precision"; return 0; }
    return 1;
}

// module Heat initial scalars (src/mcpolar.f90:66-73)
void reset_scalars(tam_ctx *ctx)
{
    ctx->time = 0.;
    ctx->pulseCount = 0.;
    ctx->repetitionCount = 0.;
    ctx->laserOn = 1.;
    ctx->laser_flag = 1;
    ctx->pulseFlag = 0;
    ctx->pulsesDone = 0;
    ctx->counter = 0;
}

// ---------------------------------------------------- reference set-up --
int ref_setup(tam_ctx *ctx)
{
    reset_scalars(ctx);
    fields_changed(ctx);  // properties set here, not by the update kernel
    const tam_params &p = ctx->p;
    const int nx = ctx->nx, ny = ctx->ny, nz = ctx->nz;
    cudaStream_t s = ctx->stream;
    // init_opt1 (src/ch_opt.f90:15-22)
    ctx->hgg = 0.9;
    ctx->g2 = ctx->hgg * ctx->hgg;
    ctx->mu_water = 510.0;
    ctx->mu_protein = 170.0;
    ctx->mua = ctx->mu_water + ctx->mu_protein;
    ctx->mus = 0.;
    ctx->kappa_opt = ctx->mus + ctx->mua;
    ctx->albedo = ctx->mus / ctx->kappa_opt;
    // gridset: rhokap = kappa inside, 0 on the halo (src/gridset.f90:34-45)
    for (int b = 0; b < 2; ++b) CK(tam::launch_fill_halo(ctx->d_rk[b], nx, ny, nz, ctx->kappa_opt, 0.0, 0.0, false, s));
    ctx->rcur = 0;
    ctx->delta = 1.e-8 * (2. * p.zmax / nz);  // src/mcpolar.f90:112
    // temperature (src/mcpolar.f90:123-129)
    for (int b = 0; b < 2; ++b) CK(tam::launch_ref_init_temp(ctx->d_T[b], nx, ny, nz, s));
    ctx->tcur = 0;
    // initThermalCoeff (src/3dFD.f90:249-307)
    ctx->dx = (2.0 * p.xmax * 1.e-2) / (nx + 2.0);
    ctx->dy = (2.0 * p.ymax * 1.e-2) / (ny + 2.0);
    ctx->dz = (2.0 * p.zmax * 1.e-2) / (nz + 2.0);
    const double heatCaptmp = skin_cap(WATER_INIT);
    const double densitytmp = skin_dens(WATER_INIT);
    const double kappatmp = skin_cond(WATER_INIT, densitytmp);
    const double alphatmp = kappatmp / (densitytmp * skin_cap(WATER_INIT));
    const double alpha_air = air_cond(25.0 + 273.0) / (air_dens(25.0 + 273.0) * AIR_HEAT_CAP);
    CK(cudaMemsetAsync(ctx->d_Q, 0, ctx->ni * sizeof(double), s));
    CK(tam::launch_fill_f64(ctx->d_water, WATER_INIT, ctx->ni, s));
    CK(tam::launch_fill_halo(ctx->d_alpha, nx, ny, nz, alphatmp, alphatmp, alpha_air, true, s));
    CK(tam::launch_fill_halo(ctx->d_kappa, nx, ny, nz, skin_cond(WATER_INIT, densitytmp), air_cond(25. + 273.), 0.0,
                             false, s));
    CK(tam::launch_fill_f64(ctx->d_density, densitytmp, ctx->nh, s));
    CK(tam::launch_fill_f64(ctx->d_heatcap, heatCaptmp, ctx->nh, s));
    const double constd = (1.0 / (ctx->dx * ctx->dx)) + (1.0 / (ctx->dy * ctx->dy)) + (1.0 / (ctx->dz * ctx->dz));
    ctx->delt = 1.0 / (1.0 * alphatmp * constd);
    CK(tam::launch_fill_halo(ctx->d_coeff, nx, ny, nz, alphatmp * ctx->delt / kappatmp, 0.0, 0.0, false, s));
    ctx->pulseLength = (p.energy_per_pixel * 1.e-3 * (double)SPOTS) / p.power;
    ctx->volumeVoxel = (2.0 * p.xmax * 1.e-2 / nx) * (2.0 * p.ymax * 1.e-2 / ny) * (2.0 * p.zmax * 1.e-2 / nz);
    ctx->massVoxel = densitytmp * ctx->volumeVoxel;
    ctx->QVapor = LW * ctx->massVoxel;
    switch (p.pulse_type) {
    case TAM_PULSE_TOPHAT: ctx->realPulseLength = ctx->pulseLength; break;
    case TAM_PULSE_GAUSSIAN: ctx->realPulseLength = 20000.0 * ctx->pulseLength; break;
    default: ctx->realPulseLength = 2.0 * ctx->pulseLength; break;
    }
    // total_time override (src/mcpolar.f90:134-140)
    ctx->total_time = p.total_time;
    if (p.pulse_type == TAM_PULSE_GAUSSIAN) {
        ctx->total_time = 2. * ctx->pulseLength * (2. * std::sqrt(2. * std::log(2.)));
        ctx->realPulseLength = ctx->total_time;
    } else if ((int64_t)(ctx->total_time / ctx->delt) <= (int64_t)(ctx->realPulseLength / ctx->delt)) {
        ctx->total_time = ctx->delt * (ctx->realPulseLength / ctx->delt + 2000.);
    }
    return TAM_OK;
}

// -------------------------------------------------------- config set-up --
// Thermal properties by material class: the class grid (a pitched copy of the
// material ids) and the per-class tables of the class-table heat step.  `u` is
// the material every voxel holds, or -1.
int set_thermal_classes(tam_ctx *ctx, int u)
{
    tam::ClassLut &L = ctx->clut;
    const int nm = ctx->cfg.nmat;
    for (int i = 0; i < tam::MAX_MAT; ++i) {
        const int a = i < nm ? i : 0;
        const double ki = ctx->lut.k[a], ri = ctx->lut.rho[a], ci = ctx->lut.c[a];
        L.k[i] = (float)ki;
        L.rho[i] = (float)ri;
        L.c[i] = (float)ci;
        L.irc[i] = (float)(1.0 / (ri * ci));
        for (int j = 0; j < tam::MAX_MAT; ++j) {
            const int b = j < nm ? j : 0;
            const double kf = 0.5 * (ki + ctx->lut.k[b]), rf = 0.5 * (ri + ctx->lut.rho[b]),
                         cf = 0.5 * (ci + ctx->lut.c[b]);
            L.fa[i * tam::MAX_MAT + j] = (float)(kf / (rf * cf));
        }
    }
    ctx->cls_uniform = u;
    L.uniform = u;
    ctx->thermal_by_class = true;
    if (ctx->d_cls)
        CK(tam::launch_cls_from_mat(ctx->d_mat, nm, ctx->d_cls, ctx->nx, ctx->ny, ctx->nz, ctx->cls_pitch, ctx->stream));
    if (ctx->d_cls && ctx->fslab && u < 0) CK(tam::fused_slab_tile_flags(ctx->fslab, ctx->zchunk, ctx->stream));
    return TAM_OK;
}

int cfg_setup(tam_ctx *ctx)
{
    reset_scalars(ctx);
    const tam_params &p = ctx->p;
    const tam_config &c = ctx->cfg;
    const int nx = ctx->nx, ny = ctx->ny, nz = ctx->nz;
    cudaStream_t s = ctx->stream;
    for (int m = 0; m < TAM_MAX_MATERIALS; ++m) {
        const tam_material &mm = c.mat[m < c.nmat ? m : 0];
        ctx->lut.k[m] = mm.k;
        ctx->lut.rho[m] = mm.rho;
        ctx->lut.c[m] = mm.c;
        ctx->lut.mut[m] = mm.mua + mm.mus;
    }
    ctx->dx = 2.0 * p.xmax * 1.e-2 / nx;
    ctx->dy = 2.0 * p.ymax * 1.e-2 / ny;
    ctx->dz = 2.0 * p.zmax * 1.e-2 / nz;
    ctx->volumeVoxel = ctx->dx * ctx->dy * ctx->dz;
    double amax = 0.0;
    for (int m = 1; m < c.nmat; ++m) {
        const double a = c.mat[m].k / (c.mat[m].rho * c.mat[m].c);
        if (a > amax) amax = a;
    }
    if (c.nmat == 1) amax = c.mat[0].k / (c.mat[0].rho * c.mat[0].c);
    if (c.dt > 0) {
        ctx->cdt = c.dt;
    } else {
        const double sum = 1.0 / (ctx->dx * ctx->dx) + 1.0 / (ctx->dy * ctx->dy) + 1.0 / (ctx->dz * ctx->dz);
        ctx->cdt = c.dt_factor / (2.0 * c.opscale * amax * sum);
    }
    ctx->delt = ctx->cdt;
    // pulse: energy (mJ) over power (no 81-spot factor in config mode)
    ctx->pulseLength = p.energy_per_pixel * 1.e-3 / p.power;
    switch (p.pulse_type) {
    case TAM_PULSE_TOPHAT: ctx->realPulseLength = ctx->pulseLength; break;
    case TAM_PULSE_GAUSSIAN: ctx->realPulseLength = 2. * ctx->pulseLength * (2. * std::sqrt(2. * std::log(2.))); break;
    default: ctx->realPulseLength = 2.0 * ctx->pulseLength; break;
    }
    ctx->total_time = p.total_time;
    const uint8_t m0 = (uint8_t)(c.nmat > 1 ? 1 : 0);
    CK(tam::launch_fill_u8(ctx->d_mat, m0, ctx->ni, s));
    ctx->uniform_id = m0;
    ctx->nabl_at_uniform = 0;
    CK(tam::launch_props_from_mat(ctx->d_mat, c.nmat, ctx->lut, ctx->d_k, ctx->d_rho, ctx->d_c, ctx->fp64, ctx->ni, s));
    ctx->coeff_dirty = true;
    RC(set_thermal_classes(ctx, m0));
    for (int b = 0; b < 2; ++b) {
        CK(tam::launch_fill_real(ctx->d_Tf[b], ctx->fp64, c.T0, ctx->ni, s));
        if (!ctx->fp64) CK(cudaMemsetAsync(ctx->d_Tc[b], 0, ctx->ni * sizeof(float), s));
    }
    ctx->fcur = 0;
    CK(cudaMemsetAsync(ctx->d_J, 0, ctx->ni * (ctx->fp64 ? 8 : 4), s));
    CK(cudaMemsetAsync(ctx->d_Qf, 0, ctx->ni * (ctx->fp64 ? 8 : 4), s));
    CK(cudaMemsetAsync(ctx->d_tissue, 0, ctx->ni * sizeof(double), s));
    CK(cudaMemsetAsync(ctx->d_thres, 0, 3 * ctx->ni * sizeof(double), s));
    CK(cudaMemsetAsync(ctx->d_nabl, 0, sizeof(unsigned long long), s));
    ctx->need_trace = true;
    ctx->nabl_at_trace = 0;
    return TAM_OK;
}

tam::FusedArgs fused_args(tam_ctx *ctx)
{
    const tam_config &c = ctx->cfg;
    tam::FusedArgs a{};
    a.nx = ctx->nx;
    a.ny = ctx->ny;
    a.nz = ctx->nz;
    a.dx = ctx->dx;
    a.dy = ctx->dy;
    a.dz = ctx->dz;
    a.opscale = c.opscale;
    a.dt = ctx->cdt;
    a.arr_fp64 = ctx->arr_fp64 ? 1 : 0;
    a.vvox = ctx->volumeVoxel;
    a.boil = c.boil;
    a.T_boil = c.T_boil;
    a.lw = c.lw;
    a.T_abl = c.T_abl;
    a.arrhenius = c.arrhenius;
    a.lnA = std::log(c.A);
    a.Ea = c.Ea;
    a.Rgas = c.Rgas;
    a.T_lo = c.T_lo;
    a.T_hi = c.T_hi;
    for (int t = 0; t < 3; ++t) a.thr[t] = c.thr[t];
    for (int f = 0; f < 6; ++f) {
        a.bc_type[f] = c.bc_type[f];
        a.bc_T[f] = c.bc_T[f];
        a.bc_h[f] = c.bc_h[f];
        a.bc_Tamb[f] = c.bc_Tamb[f];
    }
    a.T_in = ctx->d_Tf[ctx->fcur];
    a.T_out = ctx->d_Tf[1 - ctx->fcur];
    a.Tc_in = ctx->fp64 ? nullptr : ctx->d_Tc[ctx->fcur];
    a.Tc_out = ctx->fp64 ? nullptr : ctx->d_Tc[1 - ctx->fcur];
    a.k = ctx->d_k;
    a.rho = ctx->d_rho;
    a.c = ctx->d_c;
    a.J = ctx->d_J;
    a.Q = ctx->d_Qf;
    a.omega = ctx->d_tissue;
    a.thres = ctx->d_thres;
    a.mat = ctx->d_mat;
    a.n_ablated = ctx->d_nabl;
    a.err = ctx->d_err;
    a.zchunk = ctx->zchunk;
    return a;
}

// ------------------------------------------------------------ MC pass --
// One MC pass.  sync: wait for it and read its tallies back (API calls);
// the driver loops do not, so the host runs ahead of the device, and the
// tallies are read back when asked for.
// The arguments of one pass (t32: the pass deposits into the FP32 box
// tally, which is allocated here when it first grows).
int pass_args(tam_ctx *ctx, int64_t n, uint64_t seed, uint32_t stream, tam::TransportArgs &a, bool &t32)
{
    cudaStream_t s = ctx->stream;
    a = tam::TransportArgs{};
    a.nx = ctx->nx;
    a.ny = ctx->ny;
    a.nz = ctx->nz;
    a.xmax = ctx->p.xmax;
    a.ymax = ctx->p.ymax;
    a.zmax = ctx->p.zmax;
    if (ctx->config) {
        const tam_config &c = ctx->cfg;
        a.medium = tam::MED_MATERIAL;
        a.mat = ctx->d_mat;
        a.nmat = c.nmat;
        for (int m = 0; m < tam::MAX_MAT; ++m) {
            const tam_material &mm = c.mat[m < c.nmat ? m : 0];
            a.lut[m] = tam::OptMat{mm.mua, mm.mus, mm.g, mm.n};
        }
        a.n_ambient = c.n_ambient;
        a.source = c.source;
        a.source_radius = c.source_radius;
        a.fresnel = c.fresnel;
        a.roulette = c.roulette;
        a.roulette_w = c.roulette_w;
        a.roulette_m = c.roulette_m;
        a.max_steps = c.max_steps;
        a.nudge = 0.0;
    } else {
        // sourcephCO2: uniform disk of diameter 250 um, no Fresnel, no roulette
        a.medium = tam::MED_RHOKAP;
        a.rhokap = ctx->d_rk[ctx->rcur];
        a.rhokap_n = ctx->p.n2;
        a.n_ambient = ctx->p.n1;
        a.source = tam::SRC_DISK;
        a.source_radius = 250e-4 / 2.;
        a.fresnel = 0;
        a.roulette = 0;
        a.roulette_w = 0.0;
        a.roulette_m = 1.0;
        a.max_steps = (int64_t)1 << 40;
        a.nudge = ctx->delta;  // src/mcpolar.f90:112
    }
    a.scat_min = ctx->scat_min;
    a.uniform_id = -1;
    if (ctx->config && ctx->uniform_id >= 0) {
        // ablation turns voxels into material 0: the medium is no longer uniform
        unsigned long long nab = 0;
        CK(cudaMemcpyAsync(&nab, ctx->d_nabl, sizeof nab, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if ((long long)nab != ctx->nabl_at_uniform) ctx->uniform_id = -1;
        a.uniform_id = ctx->uniform_id;
    }
    // a heterogeneous grid too large for L2 next to its tally: the cells'
    // material ids come from the brick table where a brick holds one material
    // (rebuilt here, since heat steps may have ablated voxels since the last pass)
    if (ctx->config && a.uniform_id < 0 &&
        (ctx->bricks > 0 || (ctx->bricks < 0 && ctx->ni >= ((int64_t)1 << 25)))) {
        if (!ctx->d_btab) RC(dalloc_t(ctx, &ctx->d_btab, tam::brick_table_size(ctx->nx, ctx->ny, ctx->nz)));
        CK(tam::launch_brick_table(ctx->d_mat, ctx->nx, ctx->ny, ctx->nz, ctx->d_btab, s));
        a.btab = ctx->d_btab;
        a.bbx = (ctx->nx + 7) / 8;
        a.bby = (ctx->ny + 7) / 8;
    }
    a.seed = seed;
    a.stream = stream;
    a.p0 = 0;
    a.n = n;
    a.jmean = ctx->d_jmean;
    a.tally = ctx->d_tally;
    a.work = ctx->d_work;
    a.err = ctx->d_err;
    // FP32 tally for grids whose FP64 tally is far larger than L2: deposits in
    // FP32, flushed into the FP64 jmean after every chunk of packets, so each
    // voxel's FP32 partial sum stays short
    // (FP64 contexts use it only when asked, for checks on the same streams)
    t32 = ctx->config && (ctx->tally32 > 0 || (!ctx->fp64 && ctx->tally32 < 0 && ctx->ni * 8 > ((int64_t)256 << 20)));
    if (t32) {
        // the box: the whole grid if it fits the cap, else a block centred on
        // the beam axis (the source is centred on the top face) reaching down
        // from the top face, as near a cube as the grid allows
        const int64_t cap = ctx->tally32_box;
        int bn[3] = {ctx->nx, ctx->ny, ctx->nz};
        if (ctx->ni > cap) {
            const int side = std::max(1, (int)std::floor(std::cbrt((double)cap)));
            bn[0] = std::min(ctx->nx, side);
            bn[1] = std::min(ctx->ny, side);
            bn[2] = (int)std::max<int64_t>(1, std::min<int64_t>(ctx->nz, cap / ((int64_t)bn[0] * bn[1])));
        }
        a.bnx = bn[0];
        a.bny = bn[1];
        a.bnz = bn[2];
        a.bx0 = (ctx->nx - bn[0]) / 2;
        a.by0 = (ctx->ny - bn[1]) / 2;
        a.bz0 = ctx->nz - bn[2];
        const int64_t cells = (int64_t)bn[0] * bn[1] * bn[2];
        if (cells > ctx->j32_cells) {
            dfree(ctx, ctx->d_j32);
            ctx->d_j32 = nullptr;
            ctx->j32_cells = 0;
            RC(dalloc_t(ctx, &ctx->d_j32, cells));
            CK(cudaMemsetAsync(ctx->d_j32, 0, cells * sizeof(float), s));
            ctx->j32_cells = cells;
        }
    }
    a.jmean32 = t32 ? ctx->d_j32 : nullptr;
    return TAM_OK;
}

// Bookkeeping and normalisation (src/mcpolar.f90:174) after a pass's
// launches on stream s.
int pass_normalise(tam_ctx *ctx, int64_t n, cudaStream_t s)
{
    ctx->have_mc_time = true;
    ctx->last_n = n;
    ctx->mc_passes += 1;
    if (ctx->config) {
        const double f = n > 0 ? 1.0 / ((double)n * ctx->volumeVoxel) : 0.0;
        // the total absorbed weight (zeroed with the tallies) is summed in the same pass
        double *absorbed = ctx->d_tally + tam::T_ABSORBED;
        if (ctx->fp64) CK(tam::launch_scale_f64((double *)ctx->d_J, ctx->d_jmean, f, ctx->ni, false, s, absorbed));
        else CK(tam::launch_scale_to_f32((float *)ctx->d_J, ctx->d_jmean, f, ctx->ni, false, s, absorbed));
    } else {
        const tam_params &p = ctx->p;
        const double pw = get_pwr(ctx);
        const double den = (double)n * (2. * p.xmax * 1.e-2 / p.nxg) * (2. * p.ymax * 1.e-2 / p.nyg) *
                           (2. * p.zmax * 1.e-2 / p.nzg);
        const double f = n > 0 ? (pw / 81.0) / den : 0.0;
        CK(tam::launch_scale_f64(ctx->d_jglob, ctx->d_jmean, f, ctx->ni, false, s, ctx->d_tally + tam::T_ABSORBED));
    }
    ctx->tally_stale = true;
    return TAM_OK;
}

int mc_pass(tam_ctx *ctx, int64_t n, uint64_t seed, uint32_t stream, bool sync = true)
{
    cudaStream_t s = ctx->stream;
    tam::TransportArgs a;
    bool t32 = false;
    RC(pass_args(ctx, n, seed, stream, a, t32));
    CK(cudaMemsetAsync(ctx->d_jmean, 0, ctx->ni * sizeof(double), s));
    CK(cudaMemsetAsync(ctx->d_tally, 0, tam::N_TALLY * sizeof(double), s));
    CK(cudaEventRecord(ctx->ev[0], s));
    if (t32) {
        // chunks of packets with their global ids: the same Philox streams as one launch
        for (int64_t p0 = 0; p0 < n; p0 += ctx->tally32_chunk) {
            a.p0 = p0;
            a.n = std::min(ctx->tally32_chunk, n - p0);
            CK(tam::launch_transport(a, ctx->fp64, ctx->sm_count, s));
            CK(tam::launch_flush_f32(ctx->d_jmean, ctx->d_j32, ctx->nx, ctx->ny, a.bx0, a.by0, a.bz0, a.bnx, a.bny,
                                     a.bnz, s));
        }
    } else {
        CK(tam::launch_transport(a, ctx->fp64, ctx->sm_count, s));
    }
    CK(cudaEventRecord(ctx->ev[1], s));
    RC(pass_normalise(ctx, n, s));
    if (!sync) {
        CK(cudaGetLastError());
        return TAM_OK;
    }
    CK(cudaMemcpyAsync(ctx->tally, ctx->d_tally, sizeof(ctx->tally), cudaMemcpyDeviceToHost, s));
    ctx->tally_stale = false;
    return finish(ctx, "tam_mc_pass");
}

// Bring the host copy of the last pass's tallies up to date.
int refresh_tallies(tam_ctx *ctx)
{
    if (!ctx->tally_stale) return TAM_OK;
    CK(cudaMemcpyAsync(ctx->tally, ctx->d_tally, sizeof(ctx->tally), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->tally_stale = false;
    return TAM_OK;
}

// ------------------------------------------------------ heat (reference) --
int ref_heat(tam_ctx *ctx, int32_t loops)
{
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    if (ctx->pulseLength < ctx->delt) ctx->delt = ctx->pulseLength / 100.;  // src/3dFD.f90:102-105
    ctx->loops_left = (int)(ctx->total_time / ((double)loops * ctx->delt)) - ctx->counter;
    tam::RefHeatArgs a{};
    a.nx = ctx->nx;
    a.ny = ctx->ny;
    a.nz = ctx->nz;
    a.idx2 = 1.0 / (ctx->dx * ctx->dx);
    a.idy2 = 1.0 / (ctx->dy * ctx->dy);
    a.idz2 = 1.0 / (ctx->dz * ctx->dz);
    a.vvox = ctx->volumeVoxel;
    a.mvox = ctx->massVoxel;
    a.qvapor = ctx->QVapor;
    a.kappa = ctx->d_kappa;
    a.density = ctx->d_density;
    a.heatcap = ctx->d_heatcap;
    a.coeff = ctx->d_coeff;
    a.J = ctx->d_jglob;
    a.Q = ctx->d_Q;
    a.err = ctx->d_err;
    // the precision form: FP32 stencil arithmetic on FP32 copies of the
    // temperatures and properties, the update added to the FP64 temperatures
    a.f32 = ctx->fp64 ? 0 : 1;
    if (a.f32) {
        if (!ctx->shadow_ok) {
            CK(tam::launch_ref_shadow(ctx->nh, ctx->d_T[ctx->tcur], ctx->d_t32[0], ctx->d_t32[1], ctx->d_kappa,
                                      ctx->d_density, ctx->d_heatcap, ctx->d_coeff, ctx->d_p32, ctx->stream));
            ctx->shadow_ok = true;
        }
        a.p32 = ctx->d_p32;
        a.nh = ctx->nh;
    }
    for (int32_t it = 0; it < loops; ++it) {
        a.delt = ctx->delt;
        a.laserOn = ctx->laserOn;
        a.t0 = ctx->d_T[ctx->tcur];
        a.tn = ctx->d_T[1 - ctx->tcur];
        a.s0 = ctx->d_t32[ctx->tcur];
        a.sn = ctx->d_t32[1 - ctx->tcur];
        CK(tam::launch_ref_stencil(a, ctx->stream));
        ctx->tcur = 1 - ctx->tcur;  // t0 = tn (src/3dFD.f90:187)
        pulse_update(ctx, ctx->delt);
    }
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    ctx->have_heat_time = true;
    ctx->heat_launches = loops;
    return TAM_OK;
}

tam::RefArrheniusArgs arrhenius_args(const tam_ctx *ctx)
{
    tam::RefArrheniusArgs a{};
    a.nx = ctx->nx;
    a.ny = ctx->ny;
    a.nz = ctx->nz;
    a.delt = ctx->delt;
    a.time = ctx->time;
    a.temp = ctx->d_T[ctx->tcur];
    a.rhokap = ctx->d_rk[ctx->rcur];
    a.tissue = ctx->d_tissue;
    a.thres = ctx->d_thres;
    return a;
}

tam::RefPropsArgs props_args(const tam_ctx *ctx, double ablate_temp)
{
    tam::RefPropsArgs a{};
    a.nx = ctx->nx;
    a.ny = ctx->ny;
    a.nz = ctx->nz;
    a.abl_T = ablate_temp + 273.0;  // src/3dFD.f90: ablateTemp + 273 (one IEEE add, as on the device)
    a.delt = ctx->delt;
    a.qvapor = ctx->QVapor;
    a.mu_water = ctx->mu_water;
    a.mu_protein = ctx->mu_protein;
    a.temp = ctx->d_T[ctx->tcur];
    a.rk_old = ctx->d_rk[ctx->rcur];
    a.rk_new = ctx->d_rk[1 - ctx->rcur];
    a.kappa = ctx->d_kappa;
    a.density = ctx->d_density;
    a.heatcap = ctx->d_heatcap;
    a.coeff = ctx->d_coeff;
    a.alpha = ctx->d_alpha;
    a.Q = ctx->d_Q;
    a.water = ctx->d_water;
    a.err = ctx->d_err;
    a.reuse = ctx->props_delt == ctx->delt ? 1 : 0;
    a.p32 = ctx->fp64 ? nullptr : ctx->d_p32;  // FP32 copies written beside the FP64 properties
    a.nh = ctx->nh;
    return a;
}

// rhokap ping-pong and the delt whose skin properties are now in place
void props_done(tam_ctx *ctx)
{
    ctx->rcur = 1 - ctx->rcur;
    ctx->props_delt = ctx->delt;
}

int ref_arrhenius(tam_ctx *ctx)
{
    CK(tam::launch_ref_arrhenius(arrhenius_args(ctx), ctx->stream));
    return TAM_OK;
}

int ref_props(tam_ctx *ctx, double ablate_temp)
{
    CK(tam::launch_ref_props(props_args(ctx, ablate_temp), ctx->stream));
    props_done(ctx);
    return TAM_OK;
}

// Arrhenius followed by the property update, as the coupled loop calls them
// (src/mcpolar.f90:149-185), in one pass over the voxels
int ref_damage_props(tam_ctx *ctx, double ablate_temp)
{
    CK(tam::launch_ref_damage_props(arrhenius_args(ctx), props_args(ctx, ablate_temp), ctx->stream));
    props_done(ctx);
    return TAM_OK;
}

// --------------------------------------------------------- heat (config) --
// Default z planes per work item of the staged step: long columns for the
// batched launch (fewer halo planes; the batch's items fill the device) and
// shorter ones for one context alone (enough items for every SM).
constexpr int BATCH_ZCHUNK = 32, SINGLE_ZCHUNK = 8, BATCH_SLAB_ZCHUNK = 32;

// The batched-step description of one context; returns its work items.
// z planes per item: zforce if positive, else the context's heat.zchunk if
// set, else zdefault.
int batch_inst(tam_ctx *c, tam::BatchInst &I, int zdefault, int zforce = 0)
{
    I.a = fused_args(c);
    tam::fill_fused_consts(I.a);
    I.L = c->clut;
    I.cls = c->d_cls;
    I.cls_pitch = c->cls_pitch;
    for (int q = 0; q < 2; ++q) {
        I.T[q] = (float *)c->d_Tf[q];
        I.E[q] = c->d_Tc[q];
    }
    I.fcur = c->fcur;
    I.tiles_x = (c->nx + tam::FX_TILE - 1) / tam::FX_TILE;
    I.tiles_y = (c->ny + tam::FY_TILE - 1) / tam::FY_TILE;
    I.zchunk = zforce > 0 ? zforce : (c->zchunk > 0 ? c->zchunk : zdefault);
    if (I.zchunk > c->nz) I.zchunk = c->nz;
    return I.tiles_x * I.tiles_y * ((c->nz + I.zchunk - 1) / I.zchunk);
}

// Device description of this context for the staged class-table step (its
// rows are not 16-byte aligned for TMA, or TMA is off), rebuilt before each
// run of steps and copied only when it changed (classes, constants, tuning).
// The per-step source, time and buffer pair travel as kernel parameters.
int staged_setup(tam_ctx *ctx)
{
    if (!ctx->d_sinst) {
        RC(dalloc_t(ctx, &ctx->d_sinst, 1));
        RC(dalloc_t(ctx, &ctx->d_sprefix, 2));
    }
    tam::BatchInst I{};
    const int items = batch_inst(ctx, I, SINGLE_ZCHUNK);
    I.a.P = 0.0;
    I.a.t_new = 0.0;
    I.fcur = 0;
    if (items != ctx->s_items || std::memcmp(&I, &ctx->h_sinst, sizeof I) != 0) {
        // pageable sources: the copies take the bytes before they return
        ctx->h_sinst = I;
        ctx->s_items = items;
        const int pre[2] = {0, items};
        CK(cudaMemcpyAsync(ctx->d_sinst, &ctx->h_sinst, sizeof I, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_sprefix, pre, sizeof pre, cudaMemcpyHostToDevice, ctx->stream));
    }
    return TAM_OK;
}

// The slab form's per-block lists of a heterogeneous grid, for the context's
// z-chunk (after a change of the z-chunk; synchronises the stream).
int slab_lists(tam_ctx *ctx)
{
    if (!ctx->config || !ctx->d_cls || !ctx->fslab || ctx->cls_uniform >= 0) return TAM_OK;
    CK(tam::fused_slab_tile_flags(ctx->fslab, ctx->zchunk, ctx->stream));
    return TAM_OK;
}

// Forms of the config-mode heat step, by what the context's state allows.
enum HeatForm { HF_CLS = 0, HF_STAGED, HF_TMA, HF_CPASYNC, HF_SLAB };

HeatForm heat_form(const tam_ctx *ctx)
{
    if (ctx->fslab && ctx->use_slab && ctx->use_tma && ctx->use_cls && ctx->thermal_by_class) return HF_SLAB;
    if (ctx->fcls && ctx->use_tma && ctx->use_cls && ctx->thermal_by_class) return HF_CLS;
    if (!ctx->fp64 && ctx->use_cls && ctx->thermal_by_class && ctx->d_cls) return HF_STAGED;
    if (ctx->tma && ctx->use_tma) return HF_TMA;
    return HF_CPASYNC;
}

// Launch one heat step reading buffer pair `which` (a's buffers set here).
int launch_heat(tam_ctx *ctx, tam::FusedArgs &a, HeatForm form, int which, cudaStream_t s)
{
    a.T_in = ctx->d_Tf[which];
    a.T_out = ctx->d_Tf[1 - which];
    a.Tc_in = ctx->fp64 ? nullptr : ctx->d_Tc[which];
    a.Tc_out = ctx->fp64 ? nullptr : ctx->d_Tc[1 - which];
    switch (form) {
    case HF_SLAB: CK(tam::launch_fused_slab(a, ctx->fslab, which, ctx->clut, s)); break;
    case HF_CLS: CK(tam::launch_fused_cls(a, ctx->fcls, which, ctx->clut, ctx->cls_rows, s)); break;
    case HF_STAGED: {
        tam::BatchStep st{};
        st.t_new = a.t_new;
        st.pdt = (float)(a.P * ctx->cdt);
        st.active = 1;
        CK(tam::launch_staged_step(ctx->d_sinst, ctx->d_sprefix, ctx->s_items, st, which, s));
        break;
    }
    case HF_TMA: CK(tam::launch_fused_tma(a, ctx->tma, which, s)); break;
    default: CK(tam::launch_fused_step(a, ctx->fp64, s)); break;
    }
    // tissue left with six air neighbours turns to air (src/3dFD.f90:347-349)
    if (ctx->cfg.isolation)
        CK(tam::launch_isolate(ctx->d_mat, ctx->d_J, ctx->fp64, ctx->nx, ctx->ny, ctx->nz, ctx->d_nabl, s));
    return TAM_OK;
}

constexpr int GRAPH_STEPS = 16;  // heat steps per graph replay (even: a replay keeps the buffer pair)

// What a graph depends on besides the per-step values: the launch arguments
// (step values and buffer pointers masked), the class table and the knobs.
std::vector<unsigned char> graph_key(const tam_ctx *ctx, const tam::FusedArgs &a0, HeatForm form)
{
    tam::FusedArgs a = a0;
    a.P = 0.0;
    a.t_new = 0.0;
    a.sv = nullptr;
    a.T_in = a.T_out = nullptr;
    a.Tc_in = nullptr;
    a.Tc_out = nullptr;
    const int knobs[5] = {(int)form, ctx->cls_rows, ctx->zchunk, ctx->arr_fp64 ? 1 : 0,
                          (int)tam::fused_slab_generation(ctx->fslab)};  // the slab form's block lists
    std::vector<unsigned char> k(sizeof a + sizeof ctx->clut + sizeof knobs + 2 * sizeof(void *));
    unsigned char *p = k.data();
    std::memcpy(p, &a, sizeof a);
    p += sizeof a;
    std::memcpy(p, &ctx->clut, sizeof ctx->clut);
    p += sizeof ctx->clut;
    std::memcpy(p, knobs, sizeof knobs);
    p += sizeof knobs;
    const void *maps = form == HF_SLAB ? (const void *)ctx->fslab : (const void *)ctx->fcls;
    std::memcpy(p, &maps, sizeof(void *));
    std::memcpy(p + sizeof(void *), &ctx->tma, sizeof(void *));
    return k;
}

// Capture GRAPH_STEPS steps starting on buffer pair `which`, step j reading
// its values from d_sv[j].  False (and graphs off for this context) when the
// capture fails: the steps then run as ordinary launches.
bool graph_capture(tam_ctx *ctx, const tam::FusedArgs &a0, HeatForm form, int which)
{
    if (!ctx->cap_stream && cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if (!ctx->d_sv && dalloc_t(ctx, &ctx->d_sv, GRAPH_STEPS) != TAM_OK) return false;
    if (ctx->gexec[which]) {
        cudaGraphExecDestroy(ctx->gexec[which]);
        ctx->gexec[which] = nullptr;
    }
    if (cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    bool ok = true;
    const int64_t l0 = tam::launch_count();
    for (int j = 0; j < GRAPH_STEPS && ok; ++j) {
        tam::FusedArgs a = a0;
        a.sv = ctx->d_sv + j;
        ok = launch_heat(ctx, a, form, (which + j) & 1, ctx->cap_stream) == TAM_OK;
    }
    ctx->glaunches[which] = (int)(tam::launch_count() - l0);
    tam::count_launch(-ctx->glaunches[which]);  // captured, not launched; counted when replayed
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &g);
    ok = ok && e == cudaSuccess && g;
    if (ok) ok = cudaGraphInstantiate(&ctx->gexec[which], g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        (void)cudaGetLastError();
        ctx->gexec[which] = nullptr;
        ctx->err.clear();
    }
    return ok;
}

// nsteps config-mode heat steps.  With stop_on_trace the call returns as
// soon as a re-trace check has asked for a new MC pass (the driver loop then
// runs it before the next step), and a retrace_check of 0 (a check at the end
// of every call) means a check after every step, as the driver's
// one-step-per-iteration calls make it; *done receives the steps taken.
int cfg_heat(tam_ctx *ctx, int32_t nsteps, int32_t *done = nullptr, bool stop_on_trace = false)
{
    tam::FusedArgs a = fused_args(ctx);
    const int check = ctx->cfg.retrace_check > 0 ? ctx->cfg.retrace_check : (stop_on_trace ? 1 : 0);
    const HeatForm form = heat_form(ctx);
    if (form == HF_STAGED && nsteps > 0) RC(staged_setup(ctx));
    if (form == HF_TMA && ctx->coeff_dirty && nsteps > 0) {
        CK(tam::launch_face_coeffs(a, ctx->d_ax, ctx->d_ay, ctx->d_az, ctx->d_irc, ctx->stream));
        ctx->coeff_dirty = false;
    }
    const bool graphs = ctx->use_graph && form != HF_STAGED && nsteps >= GRAPH_STEPS;
    std::vector<unsigned char> key;
    if (graphs) key = graph_key(ctx, a, form);
    // re-trace check after a step: every `check` heat steps, counted across
    // calls (so a loop of one-step calls does not read the counter back every
    // step), or at the end of each call when no interval is set; and whenever
    // the source switches on
    auto retrace_check = [&](bool on) -> int {
        ctx->since_check = 0;
        unsigned long long n = 0;
        CK(cudaMemcpyAsync(&n, ctx->d_nabl, sizeof n, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        const long long fresh = (long long)n - ctx->nabl_at_trace;
        if ((double)fresh > ctx->cfg.retrace_fraction * (double)ctx->ni || (on && fresh > 0)) ctx->need_trace = true;
        return TAM_OK;
    };
    const bool retrace = ctx->cfg.retrace_fraction > 0;
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    int32_t it = 0;
    while (it < nsteps) {
        // a chunk replays a graph when none of its steps but the last needs
        // the host; the pulse machine is run ahead for the chunk and rolled
        // back when it does
        if (graphs && ctx->heat_warm && ctx->use_graph && nsteps - it >= GRAPH_STEPS) {
            const double t0 = ctx->time, pc0 = ctx->pulseCount, rc0 = ctx->repetitionCount, lo0 = ctx->laserOn;
            const int lf0 = ctx->laser_flag, pd0 = ctx->pulsesDone, sc0 = ctx->since_check;
            tam::StepVals tab[GRAPH_STEPS];
            bool fits = true, due = false, on = false;
            for (int j = 0; j < GRAPH_STEPS && fits; ++j) {
                tab[j].pdt = ctx->laserOn * get_pwr(ctx) * ctx->cdt;
                tab[j].t_new = ctx->time + ctx->cdt;
                on = pulse_update(ctx, ctx->cdt);
                due = false;
                if (retrace) due = (check ? ++ctx->since_check >= check : it + j + 1 == nsteps) || on;
                if (due && j + 1 < GRAPH_STEPS) fits = false;
            }
            const int which = ctx->fcur;
            if (fits && (ctx->gexec[which] == nullptr || ctx->gkey[which] != key)) {
                fits = graph_capture(ctx, a, form, which);
                if (fits) ctx->gkey[which] = key;
                else ctx->use_graph = false;
            }
            if (fits) {
                CK(cudaMemcpyAsync(ctx->d_sv, tab, sizeof tab, cudaMemcpyHostToDevice, ctx->stream));  // pageable: copied now
                CK(cudaGraphLaunch(ctx->gexec[which], ctx->stream));
                tam::count_launch(ctx->glaunches[which]);
                ctx->fcur = (ctx->fcur + GRAPH_STEPS) & 1;
                it += GRAPH_STEPS;
                if (due) RC(retrace_check(on));
                if (stop_on_trace && ctx->need_trace) break;
                continue;
            }
            ctx->time = t0;
            ctx->pulseCount = pc0;
            ctx->repetitionCount = rc0;
            ctx->laserOn = lo0;
            ctx->laser_flag = lf0;
            ctx->pulsesDone = pd0;
            ctx->since_check = sc0;
        }
        a.P = ctx->laserOn * get_pwr(ctx);
        a.t_new = ctx->time + ctx->cdt;
        RC(launch_heat(ctx, a, form, ctx->fcur, ctx->stream));
        ctx->heat_warm = true;
        ctx->fcur = 1 - ctx->fcur;
        const bool on = pulse_update(ctx, ctx->cdt);
        bool due = false;
        if (retrace) due = (check ? ++ctx->since_check >= check : it + 1 == nsteps) || on;
        if (due) RC(retrace_check(on));
        ++it;
        if (stop_on_trace && ctx->need_trace) break;
    }
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    ctx->have_heat_time = true;
    ctx->heat_launches = it;
    if (done) *done = it;
    return TAM_OK;
}

constexpr int ERR_EVERY = 64;  // iterations between device-error checks of the driver loops

// One outer iteration of the driver loop (src/mcpolar.f90:148-186).  sync:
// wait for the stream and fold the device error word into the status (loops
// do so every ERR_EVERY iterations and at their end).
int outer_iteration(tam_ctx *ctx, uint64_t seed, bool sync = true)
{
    const int64_t n = ctx->p.nphotons * (int64_t)ctx->p.numproc;
    if (ctx->config) {
        if (ctx->need_trace) {
            RC(mc_pass(ctx, n, seed, (uint32_t)ctx->mc_passes, false));
            unsigned long long nab = 0;
            CK(cudaMemcpy(&nab, ctx->d_nabl, sizeof nab, cudaMemcpyDeviceToHost));
            ctx->nabl_at_trace = (long long)nab;
            ctx->need_trace = false;
        }
        RC(cfg_heat(ctx, ctx->p.loops));
    } else {
        // src/mcpolar.f90:149-185
        if (ctx->laser_flag) RC(mc_pass(ctx, n, seed, (uint32_t)ctx->counter, false));
        RC(ref_heat(ctx, ctx->p.loops));
        RC(ref_damage_props(ctx, ctx->p.ablate_temp));
        ctx->ref_warm = true;
    }
    ctx->counter += 1;
    if (!sync) {
        CK(cudaGetLastError());
        return TAM_OK;
    }
    return finish(ctx, "tam_step_coupled");
}

// ------------------------------------------------------ field exchange --
struct FieldInfo {
    int64_t count;
    int esize;
    bool ok;
};

FieldInfo field_info(const tam_ctx *ctx, int f)
{
    const int64_t nh = ctx->nh, ni = ctx->ni;
    switch (f) {
    case TAM_F_TEMP:
    case TAM_F_RHOKAP:
    case TAM_F_KAPPA:
    case TAM_F_DENSITY:
    case TAM_F_HEATCAP: return {nh, 8, true};
    case TAM_F_COEFF:
    case TAM_F_ALPHA: return {nh, 8, !ctx->config};
    case TAM_F_JMEAN:
    case TAM_F_JMEAN_GLOBAL:
    case TAM_F_TISSUE:
    case TAM_F_Q: return {ni, 8, true};
    case TAM_F_WATER: return {ni, 8, !ctx->config};
    case TAM_F_THRESTIME: return {3 * ni, 8, true};
    case TAM_F_MATERIAL: return {ni, 1, ctx->config};
    default: return {0, 0, false};
    }
}

int halo_scratch(tam_ctx *ctx)
{
    if (!ctx->d_halo) RC(dalloc_t(ctx, &ctx->d_halo, ctx->nh));
    return TAM_OK;
}

}  // namespace

// =====================================================================
extern "C" {

const char *tam_version(void) { return TAM_VERSION_STRING; }
int tam_abi_version(void) { return TAM_ABI_VERSION; }

int64_t tam_struct_size(int32_t which)
{
    switch (which) {
    case 0: return (int64_t)sizeof(tam_params);
    case 1: return (int64_t)sizeof(tam_config);
    case 2: return (int64_t)sizeof(tam_state);
    case 3: return (int64_t)sizeof(tam_material);
    default: return -1;
    }
}

int tam_params_default(tam_params *p)
{
    if (!p) return fail(nullptr, TAM_E_INVALID, "null params");
    std::memset(p, 0, sizeof *p);
    // res/input.params as shipped
    p->nphotons = 125000;
    p->xmax = 0.03;
    p->ymax = 0.03;
    p->zmax = 0.06;
    p->n1 = 1.0;
    p->n2 = 1.38;
    p->total_time = 2.;
    p->loops = 1;
    p->repetition_rate_1 = 10000000.;
    p->power = 70;
    p->energy_per_pixel = 400;
    p->ablate_temp = 500;
    p->pulses_to_do = 1;
    p->pulse_type = TAM_PULSE_GAUSSIAN;
    p->nxg = p->nyg = p->nzg = 80;  // src/constants.f90:12
    p->numproc = 1;
    p->mode = TAM_MODE_REFERENCE;
    p->precision = TAM_FP64;
    p->device = 0;
    return TAM_OK;
}

int tam_config_default(tam_config *c)
{
    if (!c) return fail(nullptr, TAM_E_INVALID, "null config");
    std::memset(c, 0, sizeof *c);
    c->nmat = 2;
    c->mat[0] = tam_material{0.0, 0.0, 0.0, 1.0, 0.56, 1070.0, 3400.0};   // ablated: optics of air
    c->mat[1] = tam_material{0.3, 100.0, 0.9, 1.38, 0.56, 1070.0, 3400.0};
    c->n_ambient = 1.0;
    c->source = TAM_SRC_GAUSSIAN;
    c->source_radius = 0.1;
    c->fresnel = 1;
    c->roulette = 1;
    c->roulette_w = 1e-4;
    c->roulette_m = 10.0;
    c->T0 = 310.15;
    for (int f = 0; f < 6; ++f) {
        c->bc_type[f] = TAM_BC_DIRICHLET;
        c->bc_T[f] = 310.15;
        c->bc_h[f] = 0.0;
        c->bc_Tamb[f] = 298.15;
    }
    c->bc_type[5] = TAM_BC_ROBIN;  // beam face: convective, h = 10 W/m^2/K
    c->bc_h[5] = 10.0;
    c->dt_factor = 0.9;
    c->dt = 0.0;
    c->opscale = 1.0;
    c->boil = 1;
    c->T_boil = 373.15;
    c->lw = LW;
    c->T_abl = 373.15;
    c->arrhenius = 1;
    c->A = 3.1e98;
    c->Ea = 6.28e5;
    c->Rgas = 8.314;
    c->T_lo = 43.0 + 273.15;
    c->T_hi = 100.0 + 273.15;
    c->thr[0] = 0.53;
    c->thr[1] = 1.0;
    c->thr[2] = 1.0e4;
    c->retrace_fraction = 1e-3;
    c->retrace_check = 50;
    c->max_steps = 10000000;
    c->isolation = 0;
    return TAM_OK;
}

int tam_read_config(const char *path, tam_config *c)
{
    if (!path || !c) return fail(nullptr, TAM_E_INVALID, "null argument");
    std::ifstream in(path);
    if (!in) return fail(nullptr, TAM_E_IO, std::string("cannot open ") + path);
    tam_config q = *c;
    std::string line;
    int lineno = 0;
    auto bad = [&](const std::string &what) {
        return fail(nullptr, TAM_E_PARSE, std::string(path) + ":" + std::to_string(lineno) + ": " + what);
    };
    auto num = [](const std::string &t, double &v) -> bool {
        char *end = nullptr;
        const double x = std::strtod(t.c_str(), &end);
        if (t.empty() || *end != '\0' || !std::isfinite(x)) return false;
        v = x;
        return true;
    };
    auto inum = [](const std::string &t, long long &v) -> bool {
        char *end = nullptr;
        const long long x = std::strtoll(t.c_str(), &end, 10);
        if (t.empty() || *end != '\0') return false;
        v = x;
        return true;
    };
    while (std::getline(in, line)) {
        ++lineno;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        std::istringstream ls(line);
        std::vector<std::string> w;
        for (std::string t; ls >> t;) w.push_back(t);
        if (w.empty()) continue;
        const std::string &k = w[0];
        const size_t na = w.size() - 1;
        // scalar settings: key, destination, and whether it is an integer flag / count
        struct D {
            const char *key;
            double *d;
            int32_t *i;
        };
        const D scalars[] = {{"n_ambient", &q.n_ambient, nullptr}, {"source_radius", &q.source_radius, nullptr},
                             {"fresnel", nullptr, &q.fresnel},      {"roulette", nullptr, &q.roulette},
                             {"roulette_w", &q.roulette_w, nullptr}, {"roulette_m", &q.roulette_m, nullptr},
                             {"T0", &q.T0, nullptr},                {"dt_factor", &q.dt_factor, nullptr},
                             {"dt", &q.dt, nullptr},                {"opscale", &q.opscale, nullptr},
                             {"boil", nullptr, &q.boil},            {"T_boil", &q.T_boil, nullptr},
                             {"lw", &q.lw, nullptr},                {"T_abl", &q.T_abl, nullptr},
                             {"arrhenius", nullptr, &q.arrhenius},  {"A", &q.A, nullptr},
                             {"Ea", &q.Ea, nullptr},                {"Rgas", &q.Rgas, nullptr},
                             {"T_lo", &q.T_lo, nullptr},            {"T_hi", &q.T_hi, nullptr},
                             {"retrace_fraction", &q.retrace_fraction, nullptr},
                             {"retrace_check", nullptr, &q.retrace_check},
                             {"isolation", nullptr, &q.isolation}};
        bool done = false;
        for (const D &d : scalars) {
            if (k != d.key) continue;
            if (na != 1) return bad(k + " takes one value");
            if (d.d) {
                if (!num(w[1], *d.d)) return bad("malformed value for " + k);
            } else {
                long long v = 0;
                if (!inum(w[1], v) || v < INT32_MIN || v > INT32_MAX) return bad("malformed integer for " + k);
                *d.i = (int32_t)v;
            }
            done = true;
            break;
        }
        if (done) continue;
        if (k == "nmat") {
            long long v = 0;
            if (na != 1 || !inum(w[1], v) || v < 1 || v > TAM_MAX_MATERIALS)
                return bad("nmat takes one count in 1.." + std::to_string(TAM_MAX_MATERIALS));
            q.nmat = (int32_t)v;
        } else if (k == "material") {
            long long id = 0;
            double v[7];
            if (na != 8 || !inum(w[1], id) || id < 0 || id >= TAM_MAX_MATERIALS)
                return bad("material takes an id in 0.." + std::to_string(TAM_MAX_MATERIALS - 1) +
                           " and mua mus g n k rho c");
            for (int j = 0; j < 7; ++j)
                if (!num(w[2 + j], v[j])) return bad("malformed material value '" + w[2 + j] + "'");
            q.mat[id] = tam_material{v[0], v[1], v[2], v[3], v[4], v[5], v[6]};
            if (q.nmat < id + 1) q.nmat = (int32_t)(id + 1);
        } else if (k == "source") {
            if (na != 1 || (w[1] != "gaussian" && w[1] != "disk")) return bad("source is gaussian or disk");
            q.source = w[1] == "gaussian" ? TAM_SRC_GAUSSIAN : TAM_SRC_DISK;
        } else if (k == "max_steps") {
            long long v = 0;
            if (na != 1 || !inum(w[1], v) || v < 1) return bad("max_steps takes a positive count");
            q.max_steps = v;
        } else if (k == "thr") {
            if (na != 3 || !num(w[1], q.thr[0]) || !num(w[2], q.thr[1]) || !num(w[3], q.thr[2]))
                return bad("thr takes three damage thresholds");
        } else if (k == "bc") {
            static const char *faces[6] = {"x-", "x+", "y-", "y+", "z-", "z+"};
            int f = -1;
            for (int j = 0; j < 6 && na >= 2; ++j)
                if (w[1] == faces[j]) f = j;
            if (f < 0 || (w[2] != "dirichlet" && w[2] != "robin"))
                return bad("bc takes a face (x- x+ y- y+ z- z+) and dirichlet or robin");
            q.bc_type[f] = w[2] == "robin" ? TAM_BC_ROBIN : TAM_BC_DIRICHLET;
            for (size_t j = 3; j < w.size(); ++j) {
                const size_t eq = w[j].find('=');
                const std::string key = eq == std::string::npos ? w[j] : w[j].substr(0, eq);
                double v = 0.0;
                if (eq == std::string::npos || !num(w[j].substr(eq + 1), v)) return bad("bc value '" + w[j] + "'");
                if (key == "T") q.bc_T[f] = v;
                else if (key == "h") q.bc_h[f] = v;
                else if (key == "Tamb") q.bc_Tamb[f] = v;
                else return bad("bc value '" + key + "' (T, h or Tamb)");
            }
        } else {
            return bad("unknown setting '" + k + "'");
        }
    }
    *c = q;
    return TAM_OK;
}

int tam_read_input_params(const char *path, tam_params *p)
{
    if (!path || !p) return fail(nullptr, TAM_E_INVALID, "null argument");
    std::ifstream in(path);
    if (!in) return fail(nullptr, TAM_E_IO, std::string("cannot open ") + path);
    std::vector<std::string> toks;
    std::string line;
    while (toks.size() < 14 && std::getline(in, line)) {
        size_t i = 0;
        while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) ++i;
        if (i >= line.size()) continue;  // blank record: list-directed read moves on
        if (line[i] == '/') { toks.push_back(""); continue; }  // slash: value left unchanged
        size_t j = i;
        if (line[i] == '\'' || line[i] == '"') {
            const char q = line[i];
            j = line.find(q, i + 1);
            if (j == std::string::npos) j = line.size();
            toks.push_back(line.substr(i + 1, j - i - 1));
            continue;
        }
        while (j < line.size() && line[j] != ' ' && line[j] != '\t' && line[j] != ',' && line[j] != '/' &&
               line[j] != '\r')
            ++j;
        toks.push_back(line.substr(i, j - i));
    }
    if (toks.size() < 14) return fail(nullptr, TAM_E_PARSE, "input.params: expected 14 values");
    auto rd = [](const std::string &t, double &v) -> bool {
        if (t.empty()) return true;
        std::string s = t;
        for (char &ch : s)
            if (ch == 'd' || ch == 'D') ch = 'e';
        char *end = nullptr;
        const double x = std::strtod(s.c_str(), &end);
        if (end == s.c_str() || *end != '\0') return false;
        v = x;
        return true;
    };
    auto ri = [](const std::string &t, auto &v) -> bool {
        if (t.empty()) return true;
        char *end = nullptr;
        const long long x = std::strtoll(t.c_str(), &end, 10);
        if (end == t.c_str() || *end != '\0') return false;
        v = (std::remove_reference_t<decltype(v)>)x;
        return true;
    };
    tam_params q = *p;
    bool ok = ri(toks[0], q.nphotons) && rd(toks[1], q.xmax) && rd(toks[2], q.ymax) && rd(toks[3], q.zmax) &&
              rd(toks[4], q.n1) && rd(toks[5], q.n2) && rd(toks[6], q.total_time) && ri(toks[7], q.loops) &&
              rd(toks[8], q.repetition_rate_1) && rd(toks[9], q.power) && rd(toks[10], q.energy_per_pixel) &&
              rd(toks[11], q.ablate_temp) && ri(toks[12], q.pulses_to_do);
    if (!ok) return fail(nullptr, TAM_E_PARSE, "input.params: malformed numeric value");
    std::string pt = toks[13];
    for (char &ch : pt) ch = (char)std::tolower((unsigned char)ch);
    if (pt == "gaussian") q.pulse_type = TAM_PULSE_GAUSSIAN;
    else if (pt == "tophat") q.pulse_type = TAM_PULSE_TOPHAT;
    else if (pt == "triangular") q.pulse_type = TAM_PULSE_TRIANGULAR;
    else if (!pt.empty()) return fail(nullptr, TAM_E_PARSE, "input.params: no pulse type '" + toks[13] + "'");
    *p = q;
    return TAM_OK;
}

int tam_create(const tam_params *p, const tam_config *cfg, tam_ctx **out)
{
    if (!p || !out) return fail(nullptr, TAM_E_INVALID, "null argument");
    *out = nullptr;
    std::string why;
    if (!validate_params(p, why)) return fail(nullptr, TAM_E_INVALID, why);
    if (p->mode == TAM_MODE_CONFIG && !cfg) return fail(nullptr, TAM_E_INVALID, "config mode needs a tam_config");
    if (cfg && p->mode == TAM_MODE_CONFIG) {
        if (cfg->nmat < 1 || cfg->nmat > TAM_MAX_MATERIALS) return fail(nullptr, TAM_E_INVALID, "nmat out of range");
        for (int m = 0; m < cfg->nmat; ++m) {
            const tam_material &mm = cfg->mat[m];
            if (mm.mua < 0 || mm.mus < 0 || !(mm.n > 0) || mm.g <= -1.0 || mm.g >= 1.0 || !(mm.k > 0) ||
                !(mm.rho > 0) || !(mm.c > 0))
                return fail(nullptr, TAM_E_INVALID, "material " + std::to_string(m) + " out of range");
        }
        if (!(cfg->n_ambient > 0) || !(cfg->source_radius > 0) || !(cfg->opscale > 0) ||
            (cfg->dt <= 0 && !(cfg->dt_factor > 0)) || (cfg->roulette && !(cfg->roulette_m > 1.0)) ||
            cfg->max_steps < 1 || (cfg->arrhenius && (!(cfg->A > 0) || !(cfg->Rgas > 0))) ||
            (cfg->isolation != 0 && cfg->isolation != 1))
            return fail(nullptr, TAM_E_INVALID, "config value out of range");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        (void)cudaGetLastError();
        return fail(nullptr, TAM_E_NODEV, "no CUDA device");
    }
    if (p->device < 0 || p->device >= ndev) return fail(nullptr, TAM_E_INVALID, "device ordinal out of range");

    tam_ctx *ctx = new tam_ctx();
    ctx->p = *p;
    ctx->config = p->mode == TAM_MODE_CONFIG;
    if (ctx->config) ctx->cfg = *cfg;
    ctx->fp64 = p->precision == TAM_FP64;
    ctx->device = p->device;
    ctx->nx = p->nxg;
    ctx->ny = p->nyg;
    ctx->nz = p->nzg;
    ctx->ni = (int64_t)ctx->nx * ctx->ny * ctx->nz;
    ctx->nh = (int64_t)(ctx->nx + 2) * (ctx->ny + 2) * (ctx->nz + 2);
    auto bail = [&](int code) {
        tam_destroy(ctx);
        return code;
    };
    if (cudaSetDevice(ctx->device) != cudaSuccess) return bail(fail(nullptr, TAM_E_CUDA, "cudaSetDevice failed"));
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(nullptr, TAM_E_CUDA, "cudaStreamCreate failed"));
    ctx->own_stream = true;
    for (int e = 0; e < 4; ++e)
        if (cudaEventCreate(&ctx->ev[e]) != cudaSuccess) return bail(fail(nullptr, TAM_E_CUDA, "cudaEventCreate failed"));

    int r = TAM_OK;
#define AL(ptr, n) \
    if (r == TAM_OK) r = dalloc_t(ctx, &(ptr), (n))
    AL(ctx->d_err, 1);
    AL(ctx->d_tally, tam::N_TALLY);
    AL(ctx->d_work, 1);
    AL(ctx->d_nabl, 1);
    AL(ctx->d_cnt, 1);
    AL(ctx->d_jmean, ctx->ni);
    AL(ctx->d_sum, 1);
    AL(ctx->d_tissue, ctx->ni);
    AL(ctx->d_thres, 3 * ctx->ni);
    if (!ctx->config) {
        AL(ctx->d_jglob, ctx->ni);
        AL(ctx->d_T[0], ctx->nh);
        AL(ctx->d_T[1], ctx->nh);
        AL(ctx->d_rk[0], ctx->nh);
        AL(ctx->d_rk[1], ctx->nh);
        AL(ctx->d_kappa, ctx->nh);
        AL(ctx->d_density, ctx->nh);
        AL(ctx->d_heatcap, ctx->nh);
        AL(ctx->d_coeff, ctx->nh);
        AL(ctx->d_alpha, ctx->nh);
        AL(ctx->d_Q, ctx->ni);
        AL(ctx->d_water, ctx->ni);
        if (!ctx->fp64) {
            AL(ctx->d_t32[0], ctx->nh);
            AL(ctx->d_t32[1], ctx->nh);
            AL(ctx->d_p32, 4 * ctx->nh);
        }
    } else {
        const size_t rs = ctx->fp64 ? 8 : 4;
        for (int b = 0; b < 2 && r == TAM_OK; ++b) {
            r = dalloc(ctx, &ctx->d_Tf[b], ctx->ni * rs);
            if (r == TAM_OK && !ctx->fp64) r = dalloc_t(ctx, &ctx->d_Tc[b], ctx->ni);
        }
        if (r == TAM_OK) r = dalloc(ctx, &ctx->d_k, ctx->ni * rs);
        if (r == TAM_OK) r = dalloc(ctx, &ctx->d_rho, ctx->ni * rs);
        if (r == TAM_OK) r = dalloc(ctx, &ctx->d_c, ctx->ni * rs);
        if (r == TAM_OK) r = dalloc(ctx, &ctx->d_J, ctx->ni * rs);
        if (r == TAM_OK) r = dalloc(ctx, &ctx->d_Qf, ctx->ni * rs);
        AL(ctx->d_mat, ctx->ni);
    }
#undef AL
    if (r != TAM_OK) return bail(r);
    if (cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(ctx->d_jmean, 0, ctx->ni * 8, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(ctx->d_tissue, 0, ctx->ni * 8, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(ctx->d_thres, 0, 3 * ctx->ni * 8, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(ctx->d_tally, 0, tam::N_TALLY * 8, ctx->stream) != cudaSuccess)
        return bail(fail(nullptr, TAM_E_CUDA, "initial memset failed"));
    if (!ctx->config && cudaMemsetAsync(ctx->d_jglob, 0, ctx->ni * 8, ctx->stream) != cudaSuccess)
        return bail(fail(nullptr, TAM_E_CUDA, "initial memset failed"));
    if (ctx->config && !ctx->fp64 && tam::fused_tma_supported(ctx->nx)) {
        float *T2[2] = {(float *)ctx->d_Tf[0], (float *)ctx->d_Tf[1]};
        float *E2[2] = {ctx->d_Tc[0], ctx->d_Tc[1]};
        if (dalloc_t(ctx, &ctx->d_ax, ctx->ni) != TAM_OK || dalloc_t(ctx, &ctx->d_ay, ctx->ni) != TAM_OK ||
            dalloc_t(ctx, &ctx->d_az, ctx->ni) != TAM_OK || dalloc_t(ctx, &ctx->d_irc, ctx->ni) != TAM_OK)
            return bail(TAM_E_NOMEM);
        if (tam::fused_tma_create(&ctx->tma, ctx->nx, ctx->ny, ctx->nz, T2, E2, ctx->d_ax, ctx->d_ay, ctx->d_az,
                                  ctx->d_irc, (const float *)ctx->d_J) != cudaSuccess) {
            (void)cudaGetLastError();
            ctx->tma = nullptr;  // the cp.async form runs instead
        }
    }
    if (ctx->config && !ctx->fp64) {
        // class grid of the class-table step (TMA form) and of the batched step
        ctx->cls_pitch = tam::cls_pitch_for(ctx->nx);
        if (dalloc_t(ctx, &ctx->d_cls, (int64_t)ctx->cls_pitch * ctx->ny * ctx->nz) != TAM_OK) return bail(TAM_E_NOMEM);
        float *T2[2] = {(float *)ctx->d_Tf[0], (float *)ctx->d_Tf[1]};
        float *E2[2] = {ctx->d_Tc[0], ctx->d_Tc[1]};
        if (tam::fused_tma_supported(ctx->nx) &&
            tam::fused_cls_create(&ctx->fcls, ctx->nx, ctx->ny, ctx->nz, T2, E2, (const float *)ctx->d_J, ctx->d_cls,
                                  ctx->cls_pitch) != cudaSuccess) {
            (void)cudaGetLastError();
            ctx->fcls = nullptr;
        }
        if (tam::fused_slab_supported(ctx->nx, ctx->ny, ctx->nz) &&
            tam::fused_slab_create(&ctx->fslab, ctx->nx, ctx->ny, ctx->nz, T2, E2, (const float *)ctx->d_J,
                                   ctx->d_cls, ctx->cls_pitch) != cudaSuccess) {
            (void)cudaGetLastError();
            ctx->fslab = nullptr;
        }
    }
    r = ctx->config ? cfg_setup(ctx) : ref_setup(ctx);
    if (r == TAM_OK) r = finish(ctx, "tam_create");
    if (r != TAM_OK) {
        g_thread_err = ctx->err;
        return bail(r);
    }
    *out = ctx;
    return TAM_OK;
}

int tam_destroy(tam_ctx *ctx)
{
    if (!ctx) return TAM_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (void *p : ctx->allocs) cudaFree(p);
    for (cudaEvent_t e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->tma) tam::fused_tma_destroy(ctx->tma);
    if (ctx->fcls) tam::fused_cls_destroy(ctx->fcls);
    if (ctx->fslab) tam::fused_slab_destroy(ctx->fslab);
    for (cudaGraphExec_t &g : ctx->gexec)
        if (g) cudaGraphExecDestroy(g);
    for (cudaGraphExec_t &g : ctx->rexec)
        if (g) cudaGraphExecDestroy(g);
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return TAM_OK;
}

const char *tam_last_error(const tam_ctx *ctx) { return ctx ? ctx->err.c_str() : g_thread_err.c_str(); }

int tam_set_stream(tam_ctx *ctx, void *stream)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    CK(cudaStreamSynchronize(ctx->stream));
    if (stream) {
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        ctx->own_stream = false;
        ctx->stream = (cudaStream_t)stream;
    } else if (!ctx->own_stream) {
        CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return TAM_OK;
}

int tam_device_errors(tam_ctx *ctx, uint32_t *bits)
{
    if (!ctx || !bits) return fail(ctx, TAM_E_INVALID, "null argument");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    unsigned b = 0;
    CK(cudaMemcpy(&b, ctx->d_err, sizeof b, cudaMemcpyDeviceToHost));
    *bits = b;
    return TAM_OK;
}

int tam_init_opt(tam_ctx *ctx)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (ctx->config) return fail(ctx, TAM_E_STATE, "init_opt1 applies to reference mode");
    fields_changed(ctx);  // the absorption constants enter the property update
    ctx->hgg = 0.9;
    ctx->g2 = ctx->hgg * ctx->hgg;
    ctx->mu_water = 510.0;
    ctx->mu_protein = 170.0;
    ctx->mua = ctx->mu_water + ctx->mu_protein;
    ctx->mus = 0.;
    ctx->kappa_opt = ctx->mus + ctx->mua;
    ctx->albedo = ctx->mus / ctx->kappa_opt;
    return TAM_OK;
}

int tam_gridset(tam_ctx *ctx, double xmax, double ymax, double zmax)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (!(xmax > 0) || !(ymax > 0) || !(zmax > 0)) return fail(ctx, TAM_E_INVALID, "half-widths must be > 0");
    CK(cudaSetDevice(ctx->device));
    fields_changed(ctx);
    ctx->p.xmax = xmax;
    ctx->p.ymax = ymax;
    ctx->p.zmax = zmax;
    if (ctx->config) {
        RC(cfg_setup(ctx));
    } else {
        RC(tam_init_opt(ctx));
        for (int b = 0; b < 2; ++b)
            CK(tam::launch_fill_halo(ctx->d_rk[b], ctx->nx, ctx->ny, ctx->nz, ctx->kappa_opt, 0.0, 0.0, false,
                                     ctx->stream));
        ctx->rcur = 0;
        ctx->delta = 1.e-8 * (2. * zmax / ctx->nz);
    }
    return finish(ctx, "tam_gridset");
}

int tam_init_thermal(tam_ctx *ctx, double *delt)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    CK(cudaSetDevice(ctx->device));
    RC(ctx->config ? cfg_setup(ctx) : ref_setup(ctx));
    RC(finish(ctx, "tam_init_thermal"));
    if (delt) *delt = ctx->config ? ctx->cdt : ctx->delt;
    return TAM_OK;
}

int tam_field_bytes(tam_ctx *ctx, int field, int64_t *nbytes)
{
    if (!ctx || !nbytes) return fail(ctx, TAM_E_INVALID, "null argument");
    const FieldInfo fi = field_info(ctx, field);
    if (!fi.ok) return fail(ctx, TAM_E_STATE, "field " + std::to_string(field) + " not available in this mode");
    *nbytes = fi.count * fi.esize;
    return TAM_OK;
}

int tam_upload(tam_ctx *ctx, int field, const void *host, int64_t nbytes)
{
    if (!ctx || !host) return fail(ctx, TAM_E_INVALID, "null argument");
    fields_changed(ctx);  // an uploaded field may be one the property update reads or keeps
    const FieldInfo fi = field_info(ctx, field);
    if (!fi.ok) return fail(ctx, TAM_E_STATE, "field " + std::to_string(field) + " not available in this mode");
    if (nbytes != fi.count * fi.esize) return fail(ctx, TAM_E_INVALID, "size mismatch for field " + std::to_string(field));
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t b = (size_t)nbytes;
    auto h2d = [&](void *d) { return cudaMemcpyAsync(d, host, b, cudaMemcpyHostToDevice, s); };
    if (!ctx->config) {
        switch (field) {
        case TAM_F_TEMP:
            CK(h2d(ctx->d_T[0]));
            CK(h2d(ctx->d_T[1]));
            break;
        case TAM_F_RHOKAP: {
            // extinction is 0 or positive (the 6-neighbour test of src/3dFD.f90:347-349 relies on it)
            const double *h = (const double *)host;
            for (int64_t q = 0; q < ctx->nh; ++q)
                if (!(h[q] >= 0.0) || !std::isfinite(h[q]))
                    return fail(ctx, TAM_E_INVALID, "rhokap must be finite and >= 0");
            CK(h2d(ctx->d_rk[0]));
            CK(h2d(ctx->d_rk[1]));
            break;
        }
        case TAM_F_JMEAN: CK(h2d(ctx->d_jmean)); break;
        case TAM_F_JMEAN_GLOBAL: CK(h2d(ctx->d_jglob)); break;
        case TAM_F_TISSUE: CK(h2d(ctx->d_tissue)); break;
        case TAM_F_THRESTIME: CK(h2d(ctx->d_thres)); break;
        case TAM_F_KAPPA: CK(h2d(ctx->d_kappa)); break;
        case TAM_F_DENSITY: CK(h2d(ctx->d_density)); break;
        case TAM_F_HEATCAP: CK(h2d(ctx->d_heatcap)); break;
        case TAM_F_COEFF: CK(h2d(ctx->d_coeff)); break;
        case TAM_F_ALPHA: CK(h2d(ctx->d_alpha)); break;
        case TAM_F_Q: CK(h2d(ctx->d_Q)); break;
        case TAM_F_WATER: CK(h2d(ctx->d_water)); break;
        default: return fail(ctx, TAM_E_STATE, "field not uploadable");
        }
        return finish(ctx, "tam_upload");
    }
    // config mode: convert from the reference layout into the interior state
    tam::FusedArgs a = fused_args(ctx);
    switch (field) {
    case TAM_F_TEMP:
        RC(halo_scratch(ctx));
        CK(cudaMemcpyAsync(ctx->d_halo, host, b, cudaMemcpyHostToDevice, s));
        for (int q = 0; q < 2; ++q) {
            a.T_out = ctx->d_Tf[q];
            a.Tc_out = ctx->fp64 ? nullptr : ctx->d_Tc[q];
            CK(tam::launch_fused_from_halo(a, ctx->fp64, ctx->d_halo, s));
        }
        break;
    case TAM_F_KAPPA:
    case TAM_F_DENSITY:
    case TAM_F_HEATCAP: {
        RC(halo_scratch(ctx));
        CK(cudaMemcpyAsync(ctx->d_halo, host, b, cudaMemcpyHostToDevice, s));
        void *dst = field == TAM_F_KAPPA ? ctx->d_k : (field == TAM_F_DENSITY ? ctx->d_rho : ctx->d_c);
        CK(tam::launch_halo_to_interior(ctx->d_halo, dst, ctx->fp64, ctx->nx, ctx->ny, ctx->nz, s));
        ctx->coeff_dirty = true;
        ctx->thermal_by_class = false;  // per-voxel properties: coefficient arrays from now on
        break;
    }
    case TAM_F_JMEAN: CK(h2d(ctx->d_jmean)); break;
    case TAM_F_JMEAN_GLOBAL:
    case TAM_F_Q: {
        RC(halo_scratch(ctx));
        CK(cudaMemcpyAsync(ctx->d_halo, host, b, cudaMemcpyHostToDevice, s));
        CK(tam::launch_from_f64(ctx->d_halo, field == TAM_F_Q ? ctx->d_Qf : ctx->d_J, ctx->fp64, ctx->ni, s));
        if (field == TAM_F_JMEAN_GLOBAL) ctx->need_trace = false;
        break;
    }
    case TAM_F_TISSUE: CK(h2d(ctx->d_tissue)); break;
    case TAM_F_THRESTIME: CK(h2d(ctx->d_thres)); break;
    case TAM_F_MATERIAL: {
        CK(h2d(ctx->d_mat));
        const uint8_t *hm = (const uint8_t *)host;
        int u = hm[0] < ctx->cfg.nmat ? hm[0] : 0;
        for (int64_t q = 1; q < ctx->ni && u >= 0; ++q)
            if ((hm[q] < ctx->cfg.nmat ? hm[q] : 0) != u) u = -1;
        ctx->uniform_id = u;
        unsigned long long nab = 0;
        CK(cudaMemcpyAsync(&nab, ctx->d_nabl, sizeof nab, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        ctx->nabl_at_uniform = (long long)nab;
        CK(tam::launch_props_from_mat(ctx->d_mat, ctx->cfg.nmat, ctx->lut, ctx->d_k, ctx->d_rho, ctx->d_c, ctx->fp64,
                                      ctx->ni, s));
        ctx->coeff_dirty = true;
        RC(set_thermal_classes(ctx, u));
        ctx->need_trace = true;
        break;
    }
    default: return fail(ctx, TAM_E_STATE, "field not uploadable in config mode");
    }
    return finish(ctx, "tam_upload");
}

int tam_download(tam_ctx *ctx, int field, void *host, int64_t nbytes)
{
    if (!ctx || !host) return fail(ctx, TAM_E_INVALID, "null argument");
    const FieldInfo fi = field_info(ctx, field);
    if (!fi.ok) return fail(ctx, TAM_E_STATE, "field " + std::to_string(field) + " not available in this mode");
    if (nbytes != fi.count * fi.esize) return fail(ctx, TAM_E_INVALID, "size mismatch for field " + std::to_string(field));
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t b = (size_t)nbytes;
    auto d2h = [&](const void *d) { return cudaMemcpyAsync(host, d, b, cudaMemcpyDeviceToHost, s); };
    if (!ctx->config) {
        const void *src = nullptr;
        switch (field) {
        case TAM_F_TEMP: src = ctx->d_T[ctx->tcur]; break;
        case TAM_F_RHOKAP: src = ctx->d_rk[ctx->rcur]; break;
        case TAM_F_JMEAN: src = ctx->d_jmean; break;
        case TAM_F_JMEAN_GLOBAL: src = ctx->d_jglob; break;
        case TAM_F_TISSUE: src = ctx->d_tissue; break;
        case TAM_F_THRESTIME: src = ctx->d_thres; break;
        case TAM_F_KAPPA: src = ctx->d_kappa; break;
        case TAM_F_DENSITY: src = ctx->d_density; break;
        case TAM_F_HEATCAP: src = ctx->d_heatcap; break;
        case TAM_F_COEFF: src = ctx->d_coeff; break;
        case TAM_F_ALPHA: src = ctx->d_alpha; break;
        case TAM_F_Q: src = ctx->d_Q; break;
        case TAM_F_WATER: src = ctx->d_water; break;
        default: return fail(ctx, TAM_E_STATE, "field not downloadable");
        }
        CK(d2h(src));
        return finish(ctx, "tam_download");
    }
    tam::FusedArgs a = fused_args(ctx);
    switch (field) {
    case TAM_F_TEMP:
        RC(halo_scratch(ctx));
        CK(tam::launch_fused_to_halo(a, ctx->fp64, ctx->d_halo, s));
        CK(d2h(ctx->d_halo));
        break;
    case TAM_F_RHOKAP:
        RC(halo_scratch(ctx));
        CK(tam::launch_rhokap_from_mat(ctx->d_mat, ctx->cfg.nmat, ctx->lut, ctx->d_halo, ctx->nx, ctx->ny, ctx->nz, s));
        CK(d2h(ctx->d_halo));
        break;
    case TAM_F_KAPPA:
    case TAM_F_DENSITY:
    case TAM_F_HEATCAP: {
        RC(halo_scratch(ctx));
        const void *src = field == TAM_F_KAPPA ? ctx->d_k : (field == TAM_F_DENSITY ? ctx->d_rho : ctx->d_c);
        CK(tam::launch_interior_to_halo(src, ctx->fp64, ctx->d_halo, ctx->nx, ctx->ny, ctx->nz, s));
        CK(d2h(ctx->d_halo));
        break;
    }
    case TAM_F_JMEAN: CK(d2h(ctx->d_jmean)); break;
    case TAM_F_JMEAN_GLOBAL:
    case TAM_F_Q:
        RC(halo_scratch(ctx));
        CK(tam::launch_to_f64(field == TAM_F_Q ? ctx->d_Qf : ctx->d_J, ctx->fp64, ctx->d_halo, ctx->ni, s));
        CK(d2h(ctx->d_halo));
        break;
    case TAM_F_TISSUE: CK(d2h(ctx->d_tissue)); break;
    case TAM_F_THRESTIME: CK(d2h(ctx->d_thres)); break;
    case TAM_F_MATERIAL: CK(d2h(ctx->d_mat)); break;
    default: return fail(ctx, TAM_E_STATE, "field not downloadable in config mode");
    }
    return finish(ctx, "tam_download");
}

int tam_mc_pass(tam_ctx *ctx, int64_t nphotons, uint64_t seed, uint32_t stream, double *jmean_out)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (nphotons < 0) return fail(ctx, TAM_E_INVALID, "nphotons must be >= 0");
    CK(cudaSetDevice(ctx->device));
    RC(mc_pass(ctx, nphotons, seed, stream));
    if (ctx->config) {
        unsigned long long nab = 0;
        CK(cudaMemcpy(&nab, ctx->d_nabl, sizeof nab, cudaMemcpyDeviceToHost));
        ctx->nabl_at_trace = (long long)nab;
        ctx->need_trace = false;
    }
    if (jmean_out) return tam_download(ctx, TAM_F_JMEAN_GLOBAL, jmean_out, ctx->ni * 8);
    return TAM_OK;
}

int tam_heat_steps(tam_ctx *ctx, int32_t nsteps, double *temp_out)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (nsteps < 0) return fail(ctx, TAM_E_INVALID, "nsteps must be >= 0");
    CK(cudaSetDevice(ctx->device));
    RC(ctx->config ? cfg_heat(ctx, nsteps) : ref_heat(ctx, nsteps));
    RC(finish(ctx, "tam_heat_steps"));
    if (temp_out) return tam_download(ctx, TAM_F_TEMP, temp_out, ctx->nh * 8);
    return TAM_OK;
}

int tam_arrhenius(tam_ctx *ctx)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (ctx->config) return fail(ctx, TAM_E_STATE, "config mode fuses Arrhenius into tam_heat_steps");
    CK(cudaSetDevice(ctx->device));
    RC(ref_arrhenius(ctx));
    return finish(ctx, "tam_arrhenius");
}

int tam_update_props(tam_ctx *ctx, double ablate_temp)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (ctx->config) return fail(ctx, TAM_E_STATE, "config mode fuses ablation into tam_heat_steps");
    CK(cudaSetDevice(ctx->device));
    RC(ref_props(ctx, ablate_temp));
    return finish(ctx, "tam_update_props");
}

}  // extern "C"
namespace {
constexpr int REF_GRAPH_ITERS = 16;  // reference iterations per graph replay (even: the buffers come back)

// Normalisation factor of a reference-mode MC pass of n packets at power pw
// (src/mcpolar.f90:174), as mc_pass forms it.
double ref_norm(const tam_ctx *ctx, int64_t n, double pw)
{
    const tam_params &p = ctx->p;
    const double den = (double)n * (2. * p.xmax * 1.e-2 / p.nxg) * (2. * p.ymax * 1.e-2 / p.nyg) *
                       (2. * p.zmax * 1.e-2 / p.nzg);
    return n > 0 ? (pw / 81.0) / den : 0.0;
}

// Capture REF_GRAPH_ITERS reference iterations with the laser on (MC pass,
// normalisation, heat step, damage and property update), iteration j reading
// its stream, normalisation, laserOn and clock from d_iv[j].  The buffers
// alternate as in the launched loop, starting from the context's current pair.
bool ref_graph_capture(tam_ctx *ctx, uint64_t seed, int slot)
{
    if (!ctx->cap_stream && cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if (!ctx->d_iv && dalloc_t(ctx, &ctx->d_iv, REF_GRAPH_ITERS) != TAM_OK) return false;
    if (ctx->rexec[slot]) {
        cudaGraphExecDestroy(ctx->rexec[slot]);
        ctx->rexec[slot] = nullptr;
    }
    cudaStream_t s = ctx->cap_stream;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    const int64_t n = ctx->p.nphotons * (int64_t)ctx->p.numproc;
    int tcur = ctx->tcur, rcur = ctx->rcur;
    bool ok = true;
    for (int j = 0; j < REF_GRAPH_ITERS && ok; ++j) {
        const tam::RefIterVals *iv = ctx->d_iv + j;
        // MC pass (src/mcpolar.f90:151-174): sourcephCO2 + tauint1, normalisation
        tam::TransportArgs a{};
        a.nx = ctx->nx;
        a.ny = ctx->ny;
        a.nz = ctx->nz;
        a.xmax = ctx->p.xmax;
        a.ymax = ctx->p.ymax;
        a.zmax = ctx->p.zmax;
        a.medium = tam::MED_RHOKAP;
        a.rhokap = ctx->d_rk[rcur];
        a.rhokap_n = ctx->p.n2;
        a.n_ambient = ctx->p.n1;
        a.source = tam::SRC_DISK;
        a.source_radius = 250e-4 / 2.;
        a.roulette_m = 1.0;
        a.max_steps = (int64_t)1 << 40;
        a.nudge = ctx->delta;
        a.scat_min = ctx->scat_min;
        a.uniform_id = -1;
        a.seed = seed;
        a.stream_dev = &iv->stream;
        a.n = n;
        a.jmean = ctx->d_jmean;
        a.tally = ctx->d_tally;
        a.work = ctx->d_work;
        a.err = ctx->d_err;
        ok = cudaMemsetAsync(ctx->d_jmean, 0, ctx->ni * sizeof(double), s) == cudaSuccess &&
             cudaMemsetAsync(ctx->d_tally, 0, tam::N_TALLY * sizeof(double), s) == cudaSuccess &&
             tam::launch_transport(a, ctx->fp64, ctx->sm_count, s) == cudaSuccess &&
             tam::launch_scale_f64(ctx->d_jglob, ctx->d_jmean, 0.0, ctx->ni, false, s,
                                   ctx->d_tally + tam::T_ABSORBED, &iv->f) == cudaSuccess;
        // heat step (src/3dFD.f90:113-187)
        tam::RefHeatArgs h{};
        h.nx = ctx->nx;
        h.ny = ctx->ny;
        h.nz = ctx->nz;
        h.idx2 = 1.0 / (ctx->dx * ctx->dx);
        h.idy2 = 1.0 / (ctx->dy * ctx->dy);
        h.idz2 = 1.0 / (ctx->dz * ctx->dz);
        h.vvox = ctx->volumeVoxel;
        h.mvox = ctx->massVoxel;
        h.qvapor = ctx->QVapor;
        h.kappa = ctx->d_kappa;
        h.density = ctx->d_density;
        h.heatcap = ctx->d_heatcap;
        h.coeff = ctx->d_coeff;
        h.J = ctx->d_jglob;
        h.Q = ctx->d_Q;
        h.err = ctx->d_err;
        h.f32 = ctx->fp64 ? 0 : 1;
        h.p32 = ctx->fp64 ? nullptr : ctx->d_p32;
        h.nh = ctx->nh;
        h.delt = ctx->delt;
        h.laser_dev = &iv->laser_on;
        h.t0 = ctx->d_T[tcur];
        h.tn = ctx->d_T[1 - tcur];
        h.s0 = ctx->fp64 ? nullptr : ctx->d_t32[tcur];
        h.sn = ctx->fp64 ? nullptr : ctx->d_t32[1 - tcur];
        ok = ok && tam::launch_ref_stencil(h, s) == cudaSuccess;
        tcur = 1 - tcur;
        // Arrhenius and setupThermalCoeff (src/3dFD.f90:312-466)
        tam::RefArrheniusArgs d = arrhenius_args(ctx);
        d.time_dev = &iv->time;
        d.temp = ctx->d_T[tcur];
        d.rhokap = ctx->d_rk[rcur];
        tam::RefPropsArgs pr = props_args(ctx, ctx->p.ablate_temp);
        pr.temp = ctx->d_T[tcur];
        pr.rk_old = ctx->d_rk[rcur];
        pr.rk_new = ctx->d_rk[1 - rcur];
        pr.reuse = 1;
        ok = ok && tam::launch_ref_damage_props(d, pr, s) == cudaSuccess;
        rcur = 1 - rcur;
    }
    tam::count_launch(-4 * REF_GRAPH_ITERS);  // captured, not launched (transport, scale, stencil, damage/props)
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s, &g);
    ok = ok && e == cudaSuccess && g;
    if (ok) ok = cudaGraphInstantiate(&ctx->rexec[slot], g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        (void)cudaGetLastError();
        ctx->rexec[slot] = nullptr;
        ctx->err.clear();
    }
    return ok;
}

// Reference-mode driver loop (src/mcpolar.f90:148-186).  Runs of
// REF_GRAPH_ITERS iterations with the laser on replay one CUDA graph, their
// stream ids, normalisations, laserOn values and clocks computed ahead by the
// host's own pulse machine (advanced exactly as the launched iterations
// advance it) and copied to a device table before the replay; a run that
// would cross the time limit, max_iters, an error-fold point (every
// ERR_EVERY iterations) or a laser switch, or the first iteration of a
// context, runs as ordinary launches.
int ref_run(tam_ctx *ctx, uint64_t seed, int64_t max_iters, bool until_time, int64_t *iters)
{
    const int G = REF_GRAPH_ITERS;
    const int64_t n = ctx->p.nphotons * (int64_t)ctx->p.numproc;
    int64_t it = 0;
    std::vector<unsigned char> key;
    for (;;) {
        if (until_time && !(ctx->time <= ctx->total_time)) break;
        if (max_iters > 0 && it >= max_iters) break;
        bool replayed = false;
        if (ctx->use_graph && ctx->ref_warm && ctx->p.loops == 1 && (it % ERR_EVERY) + G <= ERR_EVERY &&
            (max_iters <= 0 || it + G <= max_iters) && ctx->props_delt == ctx->delt && !(ctx->pulseLength < ctx->delt) &&
            (ctx->fp64 || ctx->shadow_ok)) {
            // run the host state ahead; roll it back if the chunk does not fit
            const double t0 = ctx->time, pc0 = ctx->pulseCount, rc0 = ctx->repetitionCount, lo0 = ctx->laserOn;
            const int lf0 = ctx->laser_flag, pf0 = ctx->pulseFlag, pd0 = ctx->pulsesDone, ll0 = ctx->loops_left;
            tam::RefIterVals tab[REF_GRAPH_ITERS];
            bool fits = true;
            for (int j = 0; j < G && fits; ++j) {
                if ((until_time && !(ctx->time <= ctx->total_time)) || !ctx->laser_flag) {
                    fits = false;
                    break;
                }
                tab[j].stream = (uint32_t)(ctx->counter + j);
                tab[j].f = ref_norm(ctx, n, get_pwr(ctx));
                ctx->loops_left = (int)(ctx->total_time / ((double)ctx->p.loops * ctx->delt)) - (ctx->counter + j);
                tab[j].laser_on = ctx->laserOn;
                pulse_update(ctx, ctx->delt);
                tab[j].time = ctx->time;
            }
            const int slot = ctx->tcur * 2 + ctx->rcur;
            if (fits) {
                key.assign(sizeof(uint64_t) * 3 + sizeof(double) + 2 * sizeof(int), 0);
                unsigned char *q = key.data();
                const uint64_t kk[3] = {seed, (uint64_t)n, (uint64_t)ctx->scat_min};
                std::memcpy(q, kk, sizeof kk);
                std::memcpy(q + sizeof kk, &ctx->delt, sizeof(double));
                const int ff[2] = {ctx->fp64 ? 1 : 0, ctx->stream == nullptr ? 0 : 1};
                std::memcpy(q + sizeof kk + sizeof(double), ff, sizeof ff);
                if (ctx->rexec[slot] == nullptr || ctx->rkey[slot] != key) {
                    fits = ref_graph_capture(ctx, seed, slot);
                    if (fits) ctx->rkey[slot] = key;
                    else ctx->use_graph = false;
                }
            }
            if (fits) {
                CK(cudaMemcpyAsync(ctx->d_iv, tab, sizeof tab, cudaMemcpyHostToDevice, ctx->stream));  // pageable: copied now
                CK(cudaGraphLaunch(ctx->rexec[slot], ctx->stream));
                tam::count_launch(4 * G);
                ctx->counter += G;
                ctx->mc_passes += G;
                ctx->last_n = n;
                ctx->tally_stale = true;
                it += G;
                replayed = true;
            } else {
                ctx->time = t0;
                ctx->pulseCount = pc0;
                ctx->repetitionCount = rc0;
                ctx->laserOn = lo0;
                ctx->laser_flag = lf0;
                ctx->pulseFlag = pf0;
                ctx->pulsesDone = pd0;
                ctx->loops_left = ll0;
            }
        }
        if (!replayed) {
            RC(outer_iteration(ctx, seed, (it + 1) % ERR_EVERY == 0));
            ++it;
        } else if (it % ERR_EVERY == 0) {
            RC(finish(ctx, "tam_run"));
        }
    }
    if (iters) *iters = it;
    return TAM_OK;
}

// Config-mode driver loop (src/mcpolar.f90:148-186 with one heat step per
// iteration): the iterations between two MC passes run as one heat-step call,
// so its steps replay from CUDA graphs, in batches that end where the
// one-iteration-at-a-time loop would stop -- at the next multiple of
// ERR_EVERY iterations (error fold), at max_iters, at the time limit
// (until_time: an iteration runs while time <= total_time, the host's own
// clock advanced step by step as pulse_update advances it), or right after a
// re-trace check that calls for a new MC pass.  The kernels, their order and
// the host state are those of the one-at-a-time loop.
int cfg_run(tam_ctx *ctx, uint64_t seed, int64_t max_iters, bool until_time, int64_t *iters)
{
    int64_t it = 0;
    for (;;) {
        if (until_time && !(ctx->time <= ctx->total_time)) break;
        if (max_iters > 0 && it >= max_iters) break;
        if (ctx->need_trace) {
            const int64_t n = ctx->p.nphotons * (int64_t)ctx->p.numproc;
            RC(mc_pass(ctx, n, seed, (uint32_t)ctx->mc_passes, false));
            unsigned long long nab = 0;
            CK(cudaMemcpy(&nab, ctx->d_nabl, sizeof nab, cudaMemcpyDeviceToHost));
            ctx->nabl_at_trace = (long long)nab;
            ctx->need_trace = false;
        }
        int64_t k = ERR_EVERY - (it % ERR_EVERY);
        if (max_iters > 0) k = std::min(k, max_iters - it);
        if (until_time) {
            int64_t m = 0;
            for (double t = ctx->time; m < k && t <= ctx->total_time; ++m) t += ctx->cdt;
            k = std::max<int64_t>(m, 1);
        }
        int32_t done = 0;
        RC(cfg_heat(ctx, (int32_t)k, &done, true));
        ctx->counter += done;
        it += done;
        if (it % ERR_EVERY == 0) RC(finish(ctx, "tam_run"));
    }
    if (iters) *iters = it;
    return TAM_OK;
}
}  // namespace
extern "C" {

int tam_step_coupled(tam_ctx *ctx, int32_t n, uint64_t seed)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (n < 0) return fail(ctx, TAM_E_INVALID, "n must be >= 0");
    CK(cudaSetDevice(ctx->device));
    if (ctx->config && ctx->p.loops == 1) {
        if (n > 0) RC(cfg_run(ctx, seed, n, false, nullptr));
        return finish(ctx, "tam_step_coupled");
    }
    if (!ctx->config) {
        if (n > 0) RC(ref_run(ctx, seed, n, false, nullptr));
        return finish(ctx, "tam_step_coupled");
    }
    for (int32_t i = 0; i < n; ++i) RC(outer_iteration(ctx, seed, i + 1 == n || (i + 1) % ERR_EVERY == 0));
    return TAM_OK;
}

int tam_run(tam_ctx *ctx, uint64_t seed, int64_t max_iters, int64_t *iters)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    CK(cudaSetDevice(ctx->device));
    if (ctx->config && ctx->p.loops == 1) {
        RC(cfg_run(ctx, seed, max_iters, true, iters));
        return finish(ctx, "tam_run");
    }
    if (!ctx->config) {
        RC(ref_run(ctx, seed, max_iters, true, iters));
        return finish(ctx, "tam_run");
    }
    int64_t it = 0;
    while (ctx->time <= ctx->total_time) {
        if (max_iters > 0 && it >= max_iters) break;
        RC(outer_iteration(ctx, seed, (it + 1) % ERR_EVERY == 0));
        ++it;
    }
    if (iters) *iters = it;
    return finish(ctx, "tam_run");
}

// ------------------------------------------------------------ batches --
// Independent instances (the multi-instance workload): one host thread per
// context drives that context's loop on its own stream, so the device runs
// the instances' kernels side by side; a small instance's short heat kernels
// fill the gaps of the others.  Contexts are distinct objects, so the
// single-thread rule of a context holds.
}  // extern "C"
namespace {
template <typename F> int run_batch(tam_ctx *const *ctxs, int32_t n, F &&body)
{
    if (n < 0 || (n > 0 && !ctxs)) return fail(nullptr, TAM_E_INVALID, "bad batch");
    for (int32_t i = 0; i < n; ++i) {
        if (!ctxs[i]) return fail(nullptr, TAM_E_INVALID, "null context in batch");
        for (int32_t j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return fail(nullptr, TAM_E_INVALID, "context listed twice in batch");
    }
    std::vector<int> rc(n, TAM_OK);
    std::vector<std::thread> th;
    th.reserve(n);
    for (int32_t i = 0; i < n; ++i)
        th.emplace_back([&, i] {
            tam_ctx *c = ctxs[i];
            if (cudaSetDevice(c->device) != cudaSuccess) {
                rc[i] = fail(c, TAM_E_CUDA, "cudaSetDevice failed");
                return;
            }
            rc[i] = body(c, i);
            if (rc[i] == TAM_OK) rc[i] = finish(c, "tam_batch");
        });
    for (auto &t : th) t.join();
    for (int32_t i = 0; i < n; ++i)
        if (rc[i] != TAM_OK) {
            g_thread_err = "batch instance " + std::to_string(i) + ": " + ctxs[i]->err;
            return rc[i];
        }
    return TAM_OK;
}
}  // namespace
extern "C" {

}  // extern "C"
// ---------------------------------------------- device-batched heat steps --
namespace {
// Every instance FP32 config mode on one device with thermal properties by
// class: the heat steps of all of them can run in one persistent launch.
bool batchable(tam_ctx *const *ctxs, int32_t n)
{
    if (n < 1) return false;
    for (int32_t i = 0; i < n; ++i) {
        const tam_ctx *c = ctxs[i];
        if (!c->config || c->fp64 || !c->d_cls || !c->thermal_by_class || !c->use_cls || c->cfg.isolation) return false;
        if (c->device != ctxs[0]->device || c->ni >= ((int64_t)1 << 31)) return false;
    }
    return true;
}

// Device copy of the batched transport's instance table and its packet counter.
struct TrTable {
    tam::BatchTrInst *d_tr = nullptr;
    unsigned long long *d_work = nullptr;
    ~TrTable()
    {
        cudaFree(d_tr);
        cudaFree(d_work);
    }
};

// One MC pass of every instance i with sel[i] set: np[i] packets, Philox key
// seeds[i], stream streams[i].  Instances in a uniform medium with the FP64
// tally (FP32 config mode on the first instance's device) share launches of
// the batched transport, up to MAX_BATCH_TR per launch, on the first
// instance's stream, which is waited for; every other pass runs alone on its
// instance's stream and is not waited for.  Tallies are read back on demand.
int multi_pass(TrTable &T, tam_ctx *const *ctxs, int32_t n, const std::vector<int> &sel,
               const std::vector<int64_t> &np, const uint64_t *seeds, const std::vector<uint32_t> &streams)
{
    tam_ctx *const ctx = ctxs[0];  // CUDA errors of the batched launches are reported on the first instance
    cudaStream_t s = ctx->stream;
    std::vector<int32_t> grouped;
    std::vector<tam::BatchTrInst> tab;
    int64_t total = 0;
    auto flush = [&]() -> int {
        if (grouped.size() == 1) {
            RC(mc_pass(ctxs[grouped[0]], np[grouped[0]], seeds[grouped[0]], streams[grouped[0]], false));
        } else if (!grouped.empty()) {
            if (!T.d_tr) {
                CK(cudaMalloc(&T.d_tr, sizeof(tam::BatchTrInst) * tam::MAX_BATCH_TR));
                CK(cudaMalloc(&T.d_work, sizeof(unsigned long long)));
            }
            for (int32_t i : grouped) {
                tam_ctx *c = ctxs[i];
                if (c->stream != s) CK(cudaStreamSynchronize(c->stream));
                CK(cudaMemsetAsync(c->d_jmean, 0, c->ni * sizeof(double), s));
                CK(cudaMemsetAsync(c->d_tally, 0, tam::N_TALLY * sizeof(double), s));
            }
            CK(cudaMemcpyAsync(T.d_tr, tab.data(), sizeof(tam::BatchTrInst) * tab.size(), cudaMemcpyHostToDevice, s));
            for (int32_t i : grouped) CK(cudaEventRecord(ctxs[i]->ev[0], s));
            CK(tam::launch_batch_transport(T.d_tr, (int)tab.size(), total, T.d_work, ctx->scat_min, ctx->sm_count, s));
            for (int32_t i : grouped) CK(cudaEventRecord(ctxs[i]->ev[1], s));
            for (size_t q = 0; q < grouped.size(); ++q) RC(pass_normalise(ctxs[grouped[q]], tab[q].count, s));
            CK(cudaStreamSynchronize(s));
        }
        grouped.clear();
        tab.clear();
        total = 0;
        return TAM_OK;
    };
    for (int32_t i = 0; i < n; ++i) {
        if (!sel[i]) continue;
        tam_ctx *c = ctxs[i];
        if (ctx->batch_transport && np[i] > 0 && c->config && !c->fp64 && c->device == ctx->device) {
            tam::TransportArgs a;
            bool t32 = false;
            RC(pass_args(c, np[i], seeds[i], streams[i], a, t32));
            if (a.uniform_id >= 0 && !t32) {
                tam::BatchTrInst b;
                tam::fill_batch_inst(a, b);
                b.first = total;
                b.err = c->d_err;
                total += np[i];
                tab.push_back(b);
                grouped.push_back(i);
                if ((int)tab.size() == tam::MAX_BATCH_TR) RC(flush());
                continue;
            }
        }
        RC(mc_pass(c, np[i], seeds[i], streams[i], false));
    }
    return flush();
}

struct DevBatch {
    tam::BatchInst *d_inst = nullptr;
    int *d_prefix = nullptr;
    tam::BatchStep *d_steps = nullptr;
    tam::BatchSync *d_sync = nullptr;
    unsigned *d_err = nullptr;
    TrTable tr;  // the batched transport's instance table
    int *d_vox0 = nullptr;     // slab form, one launch per step: first voxel of each instance in the batch
    unsigned *d_rare = nullptr, *d_rcnt = nullptr;  // ... its list of rare voxels and the list's length
    // ... and a chunk's launches as a CUDA graph per chunk length, captured on
    // a private stream (the context's stream may be the legacy default one)
    cudaStream_t cap = nullptr;
    std::vector<std::pair<int, cudaGraphExec_t>> graphs;
    std::vector<tam::BatchInst> inst;
    std::vector<int> prefix;
    std::vector<tam::BatchStep> steps;
    int blocks = 0, kmax = 0, staged = 1, zmax = 1;
    bool uniform = false;  // every instance one material class (the slab form's uniform kernel)
    ~DevBatch()
    {
        cudaFree(d_inst);
        cudaFree(d_prefix);
        cudaFree(d_steps);
        cudaFree(d_sync);
        cudaFree(d_err);
        cudaFree(d_vox0);
        cudaFree(d_rare);
        cudaFree(d_rcnt);
        for (auto &g : graphs) cudaGraphExecDestroy(g.second);
        if (cap) cudaStreamDestroy(cap);
    }
};

// The launches of a chunk of K steps of the per-step slab form, replayed from
// a CUDA graph captured once per chunk length: the kernels read the chunk's
// instance table and steps from device buffers refreshed before each chunk,
// so the captured nodes never change.
int batch_slab_graph(DevBatch &B, tam_ctx *ctx, int32_t n, int K, cudaStream_t s)
{
    for (auto &g : B.graphs)
        if (g.first == K) {
            CK(cudaGraphLaunch(g.second, s));
            tam::count_launch(2 * K);
            return TAM_OK;
        }
    if (!B.cap) CK(cudaStreamCreateWithFlags(&B.cap, cudaStreamNonBlocking));
    CK(cudaStreamBeginCapture(B.cap, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = tam::launch_count();
    const cudaError_t e = tam::launch_batch_slab_steps(B.d_inst, n, B.d_prefix, B.prefix[n], B.zmax, B.d_vox0,
                                                       B.d_steps, K, B.d_rare, B.d_rcnt, B.d_err, B.uniform,
                                                       ctx->sm_count, B.cap);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(B.cap, &g);
    tam::count_launch(-(int)(tam::launch_count() - l0));  // counted when replayed
    CK(e);
    CK(e2);
    cudaGraphExec_t x = nullptr;
    const cudaError_t e3 = cudaGraphInstantiate(&x, g, 0);
    cudaGraphDestroy(g);
    CK(e3);
    B.graphs.emplace_back(K, x);
    CK(cudaGraphLaunch(x, s));
    tam::count_launch(2 * K);
    return TAM_OK;
}


int batch_setup(DevBatch &B, tam_ctx *const *ctxs, int32_t n, int kmax)
{
    tam_ctx *const ctx = ctxs[0];  // CUDA errors are reported on the first instance
    B.inst.resize(n);
    B.prefix.assign(n + 1, 0);
    B.staged = ctx->batch_staged;
    const bool slab = B.staged == 3 || B.staged == 4;
    B.uniform = true;
    for (int32_t i = 0; i < n; ++i) {
        int items = batch_inst(ctxs[i], B.inst[i], slab ? BATCH_SLAB_ZCHUNK : BATCH_ZCHUNK, ctx->batch_zchunk);
        const int zcap = B.staged == 4 ? tam::BATCH_STEP_ZMAX : tam::BATCH_SLAB_ZMAX;
        if (slab && B.inst[i].zchunk > zcap) items = batch_inst(ctxs[i], B.inst[i], BATCH_SLAB_ZCHUNK, zcap);
        B.prefix[i + 1] = B.prefix[i] + items;
        B.zmax = std::max(B.zmax, B.inst[i].zchunk);
        if (B.inst[i].L.uniform < 0) B.uniform = false;
    }
    B.kmax = kmax;
    B.steps.resize((size_t)kmax * n);
    if (B.staged == 4) {
        // every voxel of the batch indexed from 0 (each voxel joins a step's list at most once)
        std::vector<int> vox0(n + 1, 0);
        int64_t tot = 0;
        for (int32_t i = 0; i < n; ++i) {
            vox0[i] = (int)tot;
            tot += ctxs[i]->ni;
            if (tot >= ((int64_t)1 << 31)) return fail(ctx, TAM_E_INVALID, "batch too large for batch.staged 4");
        }
        vox0[n] = (int)tot;
        CK(cudaMalloc(&B.d_vox0, sizeof(int) * (n + 1)));
        CK(cudaMalloc(&B.d_rare, sizeof(unsigned) * (size_t)std::max<int64_t>(tot, 1)));
        CK(cudaMalloc(&B.d_rcnt, sizeof(unsigned)));
        CK(cudaMemcpy(B.d_vox0, vox0.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    } else if (slab) {
        CK(tam::batch_slab_blocks(&B.blocks, B.uniform));
    } else {
        CK(tam::batch_heat_blocks(&B.blocks, B.staged));
    }
    CK(cudaMalloc(&B.d_inst, sizeof(tam::BatchInst) * n));
    CK(cudaMalloc(&B.d_prefix, sizeof(int) * (n + 1)));
    CK(cudaMalloc(&B.d_steps, sizeof(tam::BatchStep) * B.steps.size()));
    CK(cudaMalloc(&B.d_sync, sizeof(tam::BatchSync)));
    CK(cudaMalloc(&B.d_err, sizeof(unsigned)));
    CK(cudaMemset(B.d_err, 0, sizeof(unsigned)));
    CK(cudaMemcpy(B.d_prefix, B.prefix.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    return TAM_OK;
}

// K steps of every instance with active[i] set (each advancing its own pulse
// state and clock as cfg_heat does); re-trace checks at the end of the chunk.
int batch_heat_chunk(DevBatch &B, tam_ctx *const *ctxs, int32_t n, int K, const std::vector<int> &active)
{
    tam_ctx *const ctx = ctxs[0];
    cudaStream_t s = ctxs[0]->stream;
    std::vector<int> turned_on(n, 0);
    for (int32_t i = 0; i < n; ++i) {
        tam_ctx *c = ctxs[i];
        B.inst[i].fcur = c->fcur;
        for (int k = 0; k < K; ++k) {
            tam::BatchStep &st = B.steps[(size_t)k * n + i];
            st.active = active[i];
            st.pdt = 0.f;
            st.t_new = 0.0;
            if (!active[i]) continue;
            const double P = c->laserOn * get_pwr(c);
            st.pdt = (float)(P * c->cdt);
            st.t_new = c->time + c->cdt;
            if (pulse_update(c, c->cdt)) turned_on[i] = 1;
        }
        if (active[i] && (K & 1)) c->fcur = 1 - c->fcur;
    }
    // the instances' own streams must have finished what reads or writes their fields
    for (int32_t i = 0; i < n; ++i)
        if (ctxs[i]->stream != s) CK(cudaStreamSynchronize(ctxs[i]->stream));
    CK(cudaMemcpyAsync(B.d_inst, B.inst.data(), sizeof(tam::BatchInst) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(B.d_steps, B.steps.data(), sizeof(tam::BatchStep) * (size_t)K * n, cudaMemcpyHostToDevice, s));
    if (B.staged == 4)
        RC(batch_slab_graph(B, ctx, n, K, s));
    else if (B.staged == 3)
        CK(tam::launch_batch_slab(B.d_inst, n, B.d_prefix, B.d_steps, K, B.d_sync, B.d_err, B.blocks, B.uniform, s));
    else
        CK(tam::launch_batch_heat(B.d_inst, n, B.d_prefix, B.d_steps, K, B.d_sync, B.d_err, B.blocks, B.staged, s));
    CK(cudaStreamSynchronize(s));
    unsigned bits = 0;
    CK(cudaMemcpy(&bits, B.d_err, sizeof bits, cudaMemcpyDeviceToHost));
    if (bits) return fail(ctxs[0], TAM_E_DEVICE, "batched heat step: device error word " + std::to_string(bits));
    for (int32_t i = 0; i < n; ++i) {
        tam_ctx *c = ctxs[i];
        if (!active[i] || !(c->cfg.retrace_fraction > 0)) continue;
        unsigned long long nab = 0;
        CK(cudaMemcpy(&nab, c->d_nabl, sizeof nab, cudaMemcpyDeviceToHost));
        const long long fresh = (long long)nab - c->nabl_at_trace;
        if ((double)fresh > c->cfg.retrace_fraction * (double)c->ni || (turned_on[i] && fresh > 0)) c->need_trace = true;
    }
    return TAM_OK;
}

// Chunk length of the batched loop: the re-trace check interval, else 64.
int batch_chunk(tam_ctx *const *ctxs, int32_t n)
{
    int K = 64;
    for (int32_t i = 0; i < n; ++i)
        if (ctxs[i]->cfg.retrace_fraction > 0 && ctxs[i]->cfg.retrace_check > 0)
            K = std::min(K, (int)ctxs[i]->cfg.retrace_check);
    return std::max(K, 1);
}

// MC passes of the instances that need one, each on the stream that
// counts its passes (the batched transport where the instances qualify).
int batch_traces(DevBatch &B, tam_ctx *const *ctxs, int32_t n, const uint64_t *seeds, const std::vector<int> &active)
{
    std::vector<unsigned long long> nab(n, 0);
    std::vector<int> traced(n, 0);
    std::vector<int64_t> np(n, 0);
    std::vector<uint32_t> streams(n, 0);
    for (int32_t i = 0; i < n; ++i) {
        tam_ctx *c = ctxs[i];
        if (!active[i] || !c->need_trace) continue;
        traced[i] = 1;
        np[i] = c->p.nphotons * (int64_t)c->p.numproc;
        streams[i] = (uint32_t)c->mc_passes;
    }
    RC(multi_pass(B.tr, ctxs, n, traced, np, seeds, streams));
    for (int32_t i = 0; i < n; ++i) {
        if (!traced[i]) continue;
        tam_ctx *const ctx = ctxs[i];
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(&nab[i], ctx->d_nabl, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        ctx->nabl_at_trace = (long long)nab[i];
        ctx->need_trace = false;
    }
    return TAM_OK;
}
}  // namespace
extern "C" {

int tam_batch_mc_pass(tam_ctx *const *ctxs, int32_t n, const int64_t *nphotons, const uint64_t *seeds,
                      const uint32_t *streams)
{
    if (n < 1 || !ctxs || !seeds) return fail(nullptr, TAM_E_INVALID, "bad batch arguments");
    for (int32_t i = 0; i < n; ++i) {
        if (!ctxs[i]) return fail(nullptr, TAM_E_INVALID, "null context in batch");
        for (int32_t j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return fail(nullptr, TAM_E_INVALID, "context listed twice in batch");
        if (nphotons && nphotons[i] < 0) return fail(ctxs[i], TAM_E_INVALID, "nphotons must be >= 0");
    }
    tam_ctx *const ctx = ctxs[0];
    CK(cudaSetDevice(ctx->device));
    std::vector<int> sel(n, 1);
    std::vector<int64_t> np(n);
    std::vector<uint32_t> st(n);
    for (int32_t i = 0; i < n; ++i) {
        np[i] = nphotons ? nphotons[i] : ctxs[i]->p.nphotons * (int64_t)ctxs[i]->p.numproc;
        st[i] = streams ? streams[i] : (uint32_t)ctxs[i]->mc_passes;
    }
    TrTable T;
    RC(multi_pass(T, ctxs, n, sel, np, seeds, st));
    for (int32_t i = 0; i < n; ++i) RC(finish(ctxs[i], "tam_batch_mc_pass"));
    return TAM_OK;
}

int tam_batch_heat_steps(tam_ctx *const *ctxs, int32_t n, int32_t nsteps)
{
    if (n < 1 || !ctxs || nsteps < 0) return fail(nullptr, TAM_E_INVALID, "bad batch arguments");
    for (int32_t i = 0; i < n; ++i)
        for (int32_t j = 0; j < i; ++j)
            if (!ctxs[i] || ctxs[j] == ctxs[i]) return fail(nullptr, TAM_E_INVALID, "null or repeated context in batch");
    if (!batchable(ctxs, n))
        return fail(nullptr, TAM_E_STATE, "batched heat steps need FP32 config-mode contexts on one device with "
                                           "thermal properties by material class");
    tam_ctx *const ctx = ctxs[0];
    CK(cudaSetDevice(ctx->device));
    if (ctx->batch_streams) {
        // each instance's own steps (its single-context kernel, replayed from
        // its CUDA graphs) on its own stream, issued round-robin in chunks so
        // the instances overlap on the device; one wait at the end
        constexpr int32_t RR = 256;
        for (int32_t done = 0; done < nsteps; done += RR)
            for (int32_t i = 0; i < n; ++i) RC(cfg_heat(ctxs[i], std::min(RR, nsteps - done)));
        for (int32_t i = 0; i < n; ++i) RC(finish(ctxs[i], "tam_batch_heat_steps"));
        return TAM_OK;
    }
    DevBatch B;
    const int kmax = std::min(batch_chunk(ctxs, n), std::max(nsteps, 1));
    RC(batch_setup(B, ctxs, n, kmax));
    std::vector<int> active(n, 1);
    for (int32_t done = 0; done < nsteps;) {
        const int K = std::min(kmax, nsteps - done);
        RC(batch_heat_chunk(B, ctxs, n, K, active));
        done += K;
    }
    for (int32_t i = 0; i < n; ++i) RC(finish(ctxs[i], "tam_batch_heat_steps"));
    return TAM_OK;
}

}  // extern "C"
namespace {
// Outer loops of all instances with the heat steps batched on the device:
// per instance, iteration `it` runs while `more(c, it)` holds and is `loops`
// heat steps preceded by an MC pass when one is due.  Passes and re-trace
// decisions happen at chunk boundaries (chunks of batch_chunk steps).
template <typename More>
int batch_loop_device(tam_ctx *const *ctxs, int32_t n, const uint64_t *seeds, More &&more, std::vector<int64_t> &its)
{
    tam_ctx *const ctx = ctxs[0];
    CK(cudaSetDevice(ctx->device));
    DevBatch B;
    const int K = batch_chunk(ctxs, n);
    RC(batch_setup(B, ctxs, n, K));
    std::vector<int> left(n, 0), live(n, 1);
    its.assign(n, 0);
    for (;;) {
        // which instances still run, and which steps of the next chunk they take
        std::vector<int> act(n, 0);
        bool any = false;
        for (int32_t i = 0; i < n; ++i) {
            if (!live[i]) continue;
            if (left[i] == 0) {
                if (!more(ctxs[i], its[i])) {
                    live[i] = 0;
                    continue;
                }
                ++its[i];
                left[i] = ctxs[i]->p.loops;
            }
            act[i] = 1;
            any = true;
        }
        if (!any) break;
        RC(batch_traces(B, ctxs, n, seeds, act));
        // steps of this chunk: the instance's current iteration, then further
        // iterations while its loop condition holds (checked step by step)
        int k = 0;
        for (; k < K; ++k) {
            bool stepping = false;
            for (int32_t i = 0; i < n; ++i) {
                if (!act[i]) continue;
                if (left[i] == 0) {
                    if (ctxs[i]->need_trace || !more(ctxs[i], its[i])) {
                        act[i] = 0;  // resumes (with its pass, if due) in the next chunk
                        continue;
                    }
                    ++its[i];
                    left[i] = ctxs[i]->p.loops;
                }
                stepping = true;
            }
            if (!stepping) break;
            std::vector<int> one(n, 0);
            for (int32_t i = 0; i < n; ++i)
                if (act[i] && left[i] > 0) {
                    one[i] = 1;
                    --left[i];
                }
            RC(batch_heat_chunk(B, ctxs, n, 1, one));
        }
    }
    for (int32_t i = 0; i < n; ++i) RC(finish(ctxs[i], "tam_batch"));
    return TAM_OK;
}

int check_batch(tam_ctx *const *ctxs, int32_t n, const uint64_t *seeds)
{
    if (n < 0 || (n > 0 && (!ctxs || !seeds))) return fail(nullptr, TAM_E_INVALID, "bad batch arguments");
    for (int32_t i = 0; i < n; ++i) {
        if (!ctxs[i]) return fail(nullptr, TAM_E_INVALID, "null context in batch");
        for (int32_t j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return fail(nullptr, TAM_E_INVALID, "context listed twice in batch");
    }
    return TAM_OK;
}
}  // namespace
extern "C" {

int tam_batch_step_coupled(tam_ctx *const *ctxs, int32_t n, int32_t iters, const uint64_t *seeds)
{
    RC(check_batch(ctxs, n, seeds));
    if (iters < 0) return fail(nullptr, TAM_E_INVALID, "iters must be >= 0");
    if (batchable(ctxs, n)) {
        std::vector<int64_t> its;
        return batch_loop_device(
            ctxs, n, seeds, [&](tam_ctx *, int64_t it) { return it < iters; }, its);
    }
    return run_batch(ctxs, n, [&](tam_ctx *c, int32_t i) {
        for (int32_t k = 0; k < iters; ++k) RC(outer_iteration(c, seeds[i], k + 1 == iters || (k + 1) % ERR_EVERY == 0));
        return (int)TAM_OK;
    });
}

int tam_batch_run(tam_ctx *const *ctxs, int32_t n, const uint64_t *seeds, int64_t max_iters, int64_t *iters)
{
    RC(check_batch(ctxs, n, seeds));
    if (batchable(ctxs, n)) {
        std::vector<int64_t> its;
        RC(batch_loop_device(
            ctxs, n, seeds,
            [&](tam_ctx *c, int64_t it) { return c->time <= c->total_time && (max_iters <= 0 || it < max_iters); },
            its));
        if (iters)
            for (int32_t i = 0; i < n; ++i) iters[i] = its[i];
        return TAM_OK;
    }
    return run_batch(ctxs, n, [&](tam_ctx *c, int32_t i) {
        int64_t it = 0;
        while (c->time <= c->total_time) {
            if (max_iters > 0 && it >= max_iters) break;
            RC(outer_iteration(c, seeds[i], (it + 1) % ERR_EVERY == 0));
            ++it;
        }
        if (iters) iters[i] = it;
        return finish(c, "tam_batch_run");
    });
}

int tam_finalize(tam_ctx *ctx)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    CK(cudaSetDevice(ctx->device));
    if (ctx->config) {
        RC(halo_scratch(ctx));
        CK(tam::launch_rhokap_from_mat(ctx->d_mat, ctx->cfg.nmat, ctx->lut, ctx->d_halo, ctx->nx, ctx->ny, ctx->nz,
                                       ctx->stream));
        CK(tam::launch_ref_finalize(ctx->nx, ctx->ny, ctx->nz, ctx->d_halo, ctx->d_tissue, ctx->stream));
    } else {
        CK(tam::launch_ref_finalize(ctx->nx, ctx->ny, ctx->nz, ctx->d_rk[ctx->rcur], ctx->d_tissue, ctx->stream));
    }
    return finish(ctx, "tam_finalize");
}

int tam_get_tallies(tam_ctx *ctx, double *absorbed, double *reflected, double *transmitted)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    RC(refresh_tallies(ctx));
    const double n = ctx->last_n > 0 ? (double)ctx->last_n : 1.0;
    if (absorbed) *absorbed = ctx->tally[tam::T_ABSORBED] / n;
    if (reflected) *reflected = (ctx->tally[tam::T_SPECULAR] + ctx->tally[tam::T_REFLECTED]) / n;
    if (transmitted) *transmitted = ctx->tally[tam::T_TRANSMITTED] / n;
    return TAM_OK;
}

int tam_get_tallies_ex(tam_ctx *ctx, double *out, int32_t n)
{
    if (!ctx || !out || n < 0) return fail(ctx, TAM_E_INVALID, "bad argument");
    RC(refresh_tallies(ctx));
    const double np = ctx->last_n > 0 ? (double)ctx->last_n : 1.0;
    for (int i = 0; i < n && i < tam::N_TALLY; ++i) {
        const bool count = i == tam::T_STEPS || i == tam::T_SCATTERS || i == tam::T_OVERFLOW;
        out[i] = count ? ctx->tally[i] : ctx->tally[i] / np;
    }
    return TAM_OK;
}

int tam_get_state(tam_ctx *ctx, tam_state *st)
{
    if (!ctx || !st) return fail(ctx, TAM_E_INVALID, "null argument");
    std::memset(st, 0, sizeof *st);
    st->time = ctx->time;
    st->delt = ctx->config ? ctx->cdt : ctx->delt;
    st->total_time = ctx->total_time;
    st->pulse_count = ctx->pulseCount;
    st->repetition_count = ctx->repetitionCount;
    st->laser_on = ctx->laserOn;
    st->pulse_length = ctx->pulseLength;
    st->real_pulse_length = ctx->realPulseLength;
    st->volume_voxel = ctx->volumeVoxel;
    st->mass_voxel = ctx->massVoxel;
    st->qvapor = ctx->QVapor;
    st->dx = ctx->dx;
    st->dy = ctx->dy;
    st->dz = ctx->dz;
    st->laser_flag = ctx->laser_flag;
    st->pulse_flag = ctx->pulseFlag;
    st->pulses_done = ctx->pulsesDone;
    st->counter = ctx->counter;
    st->mc_passes = ctx->mc_passes;
    if (ctx->config) {
        CK(cudaSetDevice(ctx->device));
        CK(cudaStreamSynchronize(ctx->stream));
        unsigned long long nab = 0;
        CK(cudaMemcpy(&nab, ctx->d_nabl, sizeof nab, cudaMemcpyDeviceToHost));
        st->n_ablated = (int64_t)nab;
    }
    return TAM_OK;
}

int tam_get_timing(tam_ctx *ctx, double *transport_ms, double *heat_ms, int64_t *heat_launches)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    float t = 0.f, h = 0.f;
    if (ctx->have_mc_time) CK(cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]));
    if (ctx->have_heat_time) CK(cudaEventElapsedTime(&h, ctx->ev[2], ctx->ev[3]));
    if (transport_ms) *transport_ms = t;
    if (heat_ms) *heat_ms = h;
    if (heat_launches) *heat_launches = ctx->heat_launches;
    return TAM_OK;
}

int64_t tam_kernel_launches(void) { return tam::launch_count(); }

int tam_set_tuning(tam_ctx *ctx, const char *key, int64_t value)
{
    if (!ctx || !key) return fail(ctx, TAM_E_INVALID, "null argument");
    const std::string k(key);
    if (k == "transport.scat_min") {
        if (value < 1 || value > 32) return fail(ctx, TAM_E_INVALID, "transport.scat_min must be in 1..32");
        ctx->scat_min = (int)value;
    } else if (k == "transport.tally32") {
        if (value < -1 || value > 1) return fail(ctx, TAM_E_INVALID, "transport.tally32 must be -1 (auto), 0 or 1");
        ctx->tally32 = (int)value;
    } else if (k == "transport.bricks") {
        if (value < -1 || value > 1) return fail(ctx, TAM_E_INVALID, "transport.bricks must be -1 (auto), 0 or 1");
        ctx->bricks = (int)value;
    } else if (k == "transport.tally32_box") {
        if (value < 1) return fail(ctx, TAM_E_INVALID, "transport.tally32_box must be positive");
        ctx->tally32_box = value;
    } else if (k == "transport.tally32_chunk") {
        if (value < 1) return fail(ctx, TAM_E_INVALID, "transport.tally32_chunk must be positive");
        ctx->tally32_chunk = value;
    } else if (k == "heat.tma") {
        ctx->use_tma = value != 0;
    } else if (k == "heat.cls") {
        ctx->use_cls = value != 0;
    } else if (k == "heat.slab") {
        ctx->use_slab = value != 0;
    } else if (k == "heat.cls_rows") {
        if (value < 0 || value > 2) return fail(ctx, TAM_E_INVALID, "heat.cls_rows must be 0 (voxel pairs), 1 or 2");
        ctx->cls_rows = (int)value;
    } else if (k == "heat.graph") {
        ctx->use_graph = value != 0;
    } else if (k == "heat.arrhenius_fp64") {
        ctx->arr_fp64 = value != 0;
    } else if (k == "batch.zchunk") {
        if (value < 0 || value > 1 << 20) return fail(ctx, TAM_E_INVALID, "batch.zchunk must be >= 0");
        ctx->batch_zchunk = (int)value;
    } else if (k == "batch.staged") {
        if (value < 0 || value > 4) return fail(ctx, TAM_E_INVALID, "batch.staged must be in 0..4");
        ctx->batch_staged = (int)value;
    } else if (k == "batch.streams") {
        ctx->batch_streams = value != 0;
    } else if (k == "batch.transport") {
        ctx->batch_transport = value != 0;
    } else if (k == "heat.zchunk") {
        if (value < 0 || value > ctx->nz) return fail(ctx, TAM_E_INVALID, "heat.zchunk must be in 0..nz");
        ctx->zchunk = (int)value;
        CK(cudaSetDevice(ctx->device));
        RC(slab_lists(ctx));
    } else {
        return fail(ctx, TAM_E_INVALID, "unknown tuning key " + k);
    }
    return TAM_OK;
}

// ---------------------------------------------------------- checkpoint --
namespace {
// Device buffers that hold the state of a context (the raw storage, so a
// resumed run continues bit for bit), by mode.
std::vector<std::pair<void *, size_t>> state_buffers(tam_ctx *ctx)
{
    const int64_t ni = ctx->ni, nh = ctx->nh;
    std::vector<std::pair<void *, size_t>> b;
    auto add = [&](void *p, size_t n) {
        if (p && n) b.push_back({p, n});
    };
    add(ctx->d_jmean, ni * 8);
    add(ctx->d_tissue, ni * 8);
    add(ctx->d_thres, 3 * ni * 8);
    add(ctx->d_nabl, sizeof(unsigned long long));
    add(ctx->d_tally, tam::N_TALLY * 8);
    if (ctx->config) {
        const size_t r = ctx->fp64 ? 8 : 4;
        for (int q = 0; q < 2; ++q) {
            add(ctx->d_Tf[q], ni * r);
            if (!ctx->fp64) add(ctx->d_Tc[q], ni * 4);
        }
        add(ctx->d_k, ni * r);
        add(ctx->d_rho, ni * r);
        add(ctx->d_c, ni * r);
        add(ctx->d_J, ni * r);
        add(ctx->d_Qf, ni * r);
        add(ctx->d_mat, ni);
        if (ctx->d_cls) add(ctx->d_cls, (size_t)ctx->cls_pitch * ctx->ny * ctx->nz);
    } else {
        for (int q = 0; q < 2; ++q) {
            add(ctx->d_T[q], nh * 8);
            add(ctx->d_rk[q], nh * 8);
        }
        add(ctx->d_kappa, nh * 8);
        add(ctx->d_density, nh * 8);
        add(ctx->d_heatcap, nh * 8);
        add(ctx->d_coeff, nh * 8);
        add(ctx->d_alpha, nh * 8);
        add(ctx->d_jglob, ni * 8);
        add(ctx->d_Q, ni * 8);
        add(ctx->d_water, ni * 8);
    }
    return b;
}

// Mutable host scalars of a context, in file order.
struct Scalars {
    double time, pulseCount, repetitionCount, laserOn, delt, total_time, cdt;
    int32_t laser_flag, pulseFlag, pulsesDone, counter, tcur, rcur, fcur, need_trace, uniform_id, cls_uniform,
        thermal_by_class, since_check;
    int64_t mc_passes, nabl_at_trace, nabl_at_uniform, last_n;
    uint32_t errbits_seen, pad2;
};

void get_scalars(const tam_ctx *c, Scalars &S)
{
    std::memset(&S, 0, sizeof S);
    S.time = c->time;
    S.pulseCount = c->pulseCount;
    S.repetitionCount = c->repetitionCount;
    S.laserOn = c->laserOn;
    S.delt = c->delt;
    S.total_time = c->total_time;
    S.cdt = c->cdt;
    S.laser_flag = c->laser_flag;
    S.pulseFlag = c->pulseFlag;
    S.pulsesDone = c->pulsesDone;
    S.counter = c->counter;
    S.tcur = c->tcur;
    S.rcur = c->rcur;
    S.fcur = c->fcur;
    S.need_trace = c->need_trace;
    S.uniform_id = c->uniform_id;
    S.cls_uniform = c->cls_uniform;
    S.thermal_by_class = c->thermal_by_class;
    S.since_check = c->since_check;
    S.mc_passes = c->mc_passes;
    S.nabl_at_trace = c->nabl_at_trace;
    S.nabl_at_uniform = c->nabl_at_uniform;
    S.last_n = c->last_n;
    S.errbits_seen = c->errbits_seen;
}

void set_scalars(tam_ctx *c, const Scalars &S)
{
    c->time = S.time;
    c->pulseCount = S.pulseCount;
    c->repetitionCount = S.repetitionCount;
    c->laserOn = S.laserOn;
    c->delt = S.delt;
    c->total_time = S.total_time;
    c->cdt = S.cdt;
    c->laser_flag = S.laser_flag;
    c->pulseFlag = S.pulseFlag;
    c->pulsesDone = S.pulsesDone;
    c->counter = S.counter;
    c->tcur = S.tcur;
    c->rcur = S.rcur;
    c->fcur = S.fcur;
    c->need_trace = S.need_trace != 0;
    c->uniform_id = S.uniform_id;
    c->cls_uniform = S.cls_uniform;
    c->thermal_by_class = S.thermal_by_class != 0;
    c->since_check = S.since_check;
    c->clut.uniform = S.cls_uniform;
    c->mc_passes = S.mc_passes;
    c->nabl_at_trace = S.nabl_at_trace;
    c->nabl_at_uniform = S.nabl_at_uniform;
    c->last_n = S.last_n;
    c->errbits_seen = S.errbits_seen;
    c->coeff_dirty = true;
}

const char CKPT_MAGIC[8] = {'T', 'A', 'M', 'C', 'K', 'P', 'T', '1'};
}  // namespace

int tam_save_state(tam_ctx *ctx, const char *path)
{
    if (!ctx || !path) return fail(ctx, TAM_E_INVALID, "null argument");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    RC(refresh_tallies(ctx));
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(ctx, TAM_E_IO, std::string("cannot open ") + path);
    Scalars S;
    get_scalars(ctx, S);
    const auto bufs = state_buffers(ctx);
    const uint32_t nb = (uint32_t)bufs.size();
    f.write(CKPT_MAGIC, 8);
    f.write((const char *)&ctx->p, sizeof ctx->p);
    f.write((const char *)&ctx->cfg, sizeof ctx->cfg);
    f.write((const char *)&S, sizeof S);
    f.write((const char *)ctx->tally, sizeof ctx->tally);
    f.write((const char *)&nb, sizeof nb);
    std::vector<char> host;
    for (const auto &b : bufs) {
        const uint64_t n = b.second;
        host.resize(n);
        CK(cudaMemcpy(host.data(), b.first, n, cudaMemcpyDeviceToHost));
        f.write((const char *)&n, sizeof n);
        f.write(host.data(), (std::streamsize)n);
    }
    if (!f) return fail(ctx, TAM_E_IO, std::string("write failed: ") + path);
    return TAM_OK;
}

int tam_load_state(tam_ctx *ctx, const char *path)
{
    if (!ctx || !path) return fail(ctx, TAM_E_INVALID, "null argument");
    fields_changed(ctx);
    CK(cudaSetDevice(ctx->device));
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(ctx, TAM_E_IO, std::string("cannot open ") + path);
    char magic[8];
    tam_params p;
    tam_config c;
    Scalars S;
    double tally[tam::N_TALLY];
    uint32_t nb = 0;
    f.read(magic, 8);
    f.read((char *)&p, sizeof p);
    f.read((char *)&c, sizeof c);
    f.read((char *)&S, sizeof S);
    f.read((char *)tally, sizeof tally);
    f.read((char *)&nb, sizeof nb);
    if (!f || std::memcmp(magic, CKPT_MAGIC, 8) != 0) return fail(ctx, TAM_E_PARSE, "not a state file");
    if (std::memcmp(&p, &ctx->p, sizeof p) != 0 || (ctx->config && std::memcmp(&c, &ctx->cfg, sizeof c) != 0))
        return fail(ctx, TAM_E_STATE, "state file was written by a context with other parameters");
    const auto bufs = state_buffers(ctx);
    if (nb != bufs.size()) return fail(ctx, TAM_E_STATE, "state file holds another set of fields");
    std::vector<char> host;
    CK(cudaStreamSynchronize(ctx->stream));
    for (const auto &b : bufs) {
        uint64_t n = 0;
        f.read((char *)&n, sizeof n);
        if (!f || n != b.second) return fail(ctx, TAM_E_STATE, "state file field size mismatch");
        host.resize(n);
        f.read(host.data(), (std::streamsize)n);
        if (!f) return fail(ctx, TAM_E_PARSE, "state file truncated");
        CK(cudaMemcpy(b.first, host.data(), n, cudaMemcpyHostToDevice));
    }
    // the slab form's tile flags follow the class grid just loaded
    if (ctx->config && ctx->d_cls && ctx->fslab && ctx->cls_uniform < 0)
        CK(tam::fused_slab_tile_flags(ctx->fslab, ctx->zchunk, ctx->stream));
    set_scalars(ctx, S);
    std::memcpy(ctx->tally, tally, sizeof tally);
    ctx->tally_stale = false;
    return finish(ctx, "tam_load_state");
}

// ------------------------------------------------------------ autotune --
namespace {
// Device copies of the config-mode state a trial run changes.
struct Snapshot {
    std::vector<std::pair<void *, void *>> bufs;  // (saved copy, live buffer)
    std::vector<size_t> bytes;
    double time = 0, pulseCount = 0, repetitionCount = 0, laserOn = 0;
    int laser_flag = 0, pulseFlag = 0, pulsesDone = 0, counter = 0, fcur = 0, since_check = 0;
    int64_t mc_passes = 0;
    bool need_trace = false;
    int uniform_id = -1;
    double tally[tam::N_TALLY] = {0};
    int64_t last_n = 0;
    ~Snapshot()
    {
        for (auto &b : bufs) cudaFree(b.first);
    }
};

int snap_take(tam_ctx *ctx, Snapshot &S)
{
    const int64_t ni = ctx->ni;
    const size_t r = ctx->fp64 ? 8 : 4;
    auto add = [&](void *live, size_t bytes) -> int {
        if (!live || !bytes) return TAM_OK;
        void *cp = nullptr;
        if (cudaMalloc(&cp, bytes) != cudaSuccess) return fail(ctx, TAM_E_NOMEM, "autotune: no room for the state copy");
        S.bufs.push_back({cp, live});
        S.bytes.push_back(bytes);
        CK(cudaMemcpyAsync(cp, live, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        return TAM_OK;
    };
    for (int q = 0; q < 2; ++q) {
        RC(add(ctx->d_Tf[q], ni * r));
        if (!ctx->fp64) RC(add(ctx->d_Tc[q], ni * 4));
    }
    RC(add(ctx->d_J, ni * r));
    RC(add(ctx->d_Qf, ni * r));
    RC(add(ctx->d_jmean, ni * 8));
    RC(add(ctx->d_tissue, ni * 8));
    RC(add(ctx->d_thres, 3 * ni * 8));
    RC(add(ctx->d_mat, ni));
    RC(add(ctx->d_nabl, sizeof(unsigned long long)));
    RC(add(ctx->d_tally, tam::N_TALLY * 8));
    S.time = ctx->time;
    S.pulseCount = ctx->pulseCount;
    S.repetitionCount = ctx->repetitionCount;
    S.laserOn = ctx->laserOn;
    S.laser_flag = ctx->laser_flag;
    S.pulseFlag = ctx->pulseFlag;
    S.pulsesDone = ctx->pulsesDone;
    S.counter = ctx->counter;
    S.fcur = ctx->fcur;
    S.since_check = ctx->since_check;
    S.mc_passes = ctx->mc_passes;
    S.need_trace = ctx->need_trace;
    S.uniform_id = ctx->uniform_id;
    RC(refresh_tallies(ctx));
    std::memcpy(S.tally, ctx->tally, sizeof S.tally);
    S.last_n = ctx->last_n;
    return TAM_OK;
}

int snap_restore(tam_ctx *ctx, const Snapshot &S)
{
    for (size_t i = 0; i < S.bufs.size(); ++i)
        CK(cudaMemcpyAsync(S.bufs[i].second, S.bufs[i].first, S.bytes[i], cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->time = S.time;
    ctx->pulseCount = S.pulseCount;
    ctx->repetitionCount = S.repetitionCount;
    ctx->laserOn = S.laserOn;
    ctx->laser_flag = S.laser_flag;
    ctx->pulseFlag = S.pulseFlag;
    ctx->pulsesDone = S.pulsesDone;
    ctx->counter = S.counter;
    ctx->fcur = S.fcur;
    ctx->since_check = S.since_check;
    ctx->mc_passes = S.mc_passes;
    ctx->need_trace = S.need_trace;
    ctx->uniform_id = S.uniform_id;
    std::memcpy(ctx->tally, S.tally, sizeof S.tally);
    ctx->tally_stale = false;
    ctx->last_n = S.last_n;
    CK(cudaStreamSynchronize(ctx->stream));
    return TAM_OK;
}
}  // namespace

int tam_autotune(tam_ctx *ctx, int64_t packets, int32_t steps, int64_t *chosen, int32_t nchosen)
{
    if (!ctx) return fail(nullptr, TAM_E_INVALID, "null context");
    if (!ctx->config) return fail(ctx, TAM_E_STATE, "autotune applies to config mode");
    if (packets < 0 || steps < 0) return fail(ctx, TAM_E_INVALID, "packets and steps must be >= 0");
    CK(cudaSetDevice(ctx->device));
    Snapshot S;
    RC(snap_take(ctx, S));
    float ms = 0.f;
    // on a failure the knobs and the state go back as they were
    const int scat0 = ctx->scat_min, z0 = ctx->zchunk, rows0 = ctx->cls_rows;
    const bool slab0 = ctx->use_slab;
    auto undo = [&](int code) {
        ctx->scat_min = scat0;
        ctx->zchunk = z0;
        ctx->cls_rows = rows0;
        ctx->use_slab = slab0;
        (void)cudaGetLastError();
        (void)snap_restore(ctx, S);
        (void)slab_lists(ctx);
        return code;
    };
    auto timed = [&](int ev0, int ev1) -> int {
        if (cudaEventSynchronize(ctx->ev[ev1]) != cudaSuccess ||
            cudaEventElapsedTime(&ms, ctx->ev[ev0], ctx->ev[ev1]) != cudaSuccess)
            return fail(ctx, TAM_E_CUDA, "autotune: timing events failed");
        return TAM_OK;
    };
    int r = TAM_OK;
    // transport: lanes that must wait at an interaction before the warp's event batch
    if (packets > 0) {
        int best = ctx->scat_min;
        float best_ms = 1e30f;
        for (int cand : {12, 16, 20, 24, 28}) {
            ctx->scat_min = cand;
            if ((r = mc_pass(ctx, packets, 0x5eedull, 0xA070u)) != TAM_OK || (r = timed(0, 1)) != TAM_OK)
                return undo(r);
            if (ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
        ctx->scat_min = best;
        if ((r = snap_restore(ctx, S)) != TAM_OK) return undo(r);
    }
    // heat: z planes per thread column, and the form of the class-table step
    // (slab form, voxel pairs or rows of voxels)
    if (steps > 0) {
        int best_z = ctx->zchunk, best_r = ctx->cls_rows;
        bool best_s = ctx->use_slab;
        float best_ms = 1e30f;
        const bool cls = ctx->fcls && ctx->use_tma && ctx->use_cls && ctx->thermal_by_class;
        const bool slab = ctx->fslab && ctx->use_tma && ctx->use_cls && ctx->thermal_by_class;
        const bool staged = !cls && !slab && !ctx->fp64 && ctx->use_cls && ctx->thermal_by_class && ctx->d_cls;
        const std::vector<int> zcs = staged ? std::vector<int>{4, 8, 16, 32} : std::vector<int>{2, 3, 4, 5, 8, 16};
        for (int form : {2, 0, 1}) {  // 2: slab form; 0 / 1: class-table voxel pairs / rows
            if (form == 2 && !slab) continue;
            if (form == 0 && !cls) continue;
            for (int zc : zcs) {
                if (zc > ctx->nz) continue;
                ctx->zchunk = zc;
                if ((r = slab_lists(ctx)) != TAM_OK) return undo(r);
                ctx->use_slab = form == 2;
                if (form != 2) ctx->cls_rows = form;
                if ((r = cfg_heat(ctx, steps)) != TAM_OK || (r = timed(2, 3)) != TAM_OK ||
                    (r = snap_restore(ctx, S)) != TAM_OK)
                    return undo(r);
                if (ms < best_ms) {
                    best_ms = ms;
                    best_z = zc;
                    best_s = form == 2;
                    if (form != 2) best_r = form;
                }
            }
        }
        ctx->zchunk = best_z;
        if ((r = slab_lists(ctx)) != TAM_OK) return undo(r);
        ctx->cls_rows = best_r;
        ctx->use_slab = best_s;
    }
    const int64_t v[4] = {ctx->scat_min, ctx->zchunk, ctx->cls_rows, ctx->use_slab ? 1 : 0};
    for (int32_t i = 0; i < nchosen && i < 4 && chosen; ++i) chosen[i] = v[i];
    return finish(ctx, "tam_autotune");
}

int tam_batch_autotune(tam_ctx *const *ctxs, int32_t n, int32_t steps, int64_t *chosen, int32_t nchosen)
{
    if (n < 1 || !ctxs || steps < 1) return fail(nullptr, TAM_E_INVALID, "bad batch autotune arguments");
    for (int32_t i = 0; i < n; ++i)
        for (int32_t j = 0; j < i; ++j)
            if (!ctxs[i] || ctxs[j] == ctxs[i]) return fail(nullptr, TAM_E_INVALID, "null or repeated context in batch");
    if (!batchable(ctxs, n))
        return fail(nullptr, TAM_E_STATE, "batch autotune needs FP32 config-mode contexts on one device with "
                                           "thermal properties by material class");
    tam_ctx *const ctx = ctxs[0];
    CK(cudaSetDevice(ctx->device));
    std::vector<std::unique_ptr<Snapshot>> S(n);
    for (int32_t i = 0; i < n; ++i) {
        S[i].reset(new Snapshot);
        RC(snap_take(ctxs[i], *S[i]));
        CK(cudaStreamSynchronize(ctxs[i]->stream));
    }
    const int form0 = ctx->batch_staged, z0 = ctx->batch_zchunk, streams0 = ctx->batch_streams;
    int best_form = form0, best_z = z0, best_streams = 0;
    double best = 1e300;
    const std::vector<int> active(n, 1);
    struct Cand {
        int form, z;
    };
    const Cand cands[] = {{4, 16}, {4, 32}, {4, 64}, {3, 8}, {3, 16}, {3, 32}, {2, 8}, {2, 16}, {2, 32}, {2, 64}, {1, 16}, {1, 32}};
    // on a failure the settings and every instance's state go back as they were
    auto undo = [&](int code) {
        ctx->batch_staged = form0;
        ctx->batch_zchunk = z0;
        ctx->batch_streams = streams0;
        for (int32_t i = 0; i < n; ++i) (void)snap_restore(ctxs[i], *S[i]);
        return code;
    };
    ctx->batch_streams = 0;
    for (const Cand &c : cands) {
        ctx->batch_staged = c.form;
        ctx->batch_zchunk = c.z;
        DevBatch B;
        const int K = std::min(batch_chunk(ctxs, n), (int)steps);
        int r = batch_setup(B, ctxs, n, K);
        if (r == TAM_OK) r = batch_heat_chunk(B, ctxs, n, K, active);  // warm-up (instruction cache, L2)
        if (r != TAM_OK) return undo(r);
        for (int32_t i = 0; i < n; ++i)
            if ((r = snap_restore(ctxs[i], *S[i])) != TAM_OK) return undo(r);
        const auto t0 = std::chrono::steady_clock::now();
        for (int32_t done = 0; done < steps && r == TAM_OK; done += K)
            r = batch_heat_chunk(B, ctxs, n, std::min(K, steps - done), active);
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (r != TAM_OK) return undo(r);
        for (int32_t i = 0; i < n; ++i)
            if ((r = snap_restore(ctxs[i], *S[i])) != TAM_OK) return undo(r);
        if (dt < best) {
            best = dt;
            best_form = c.form;
            best_z = c.z;
        }
    }
    // the streams form: each instance's own steps on its stream, issued as
    // tam_batch_heat_steps issues them (a short warm-up call captures graphs)
    {
        auto run = [&](int32_t nsteps) -> int {
            for (int32_t done = 0; done < nsteps; done += 256)
                for (int32_t i = 0; i < n; ++i) RC(cfg_heat(ctxs[i], std::min(256, nsteps - done)));
            for (int32_t i = 0; i < n; ++i) CK(cudaStreamSynchronize(ctxs[i]->stream));
            return TAM_OK;
        };
        int r = run(std::min(32, (int)steps));
        for (int32_t i = 0; i < n && r == TAM_OK; ++i) r = snap_restore(ctxs[i], *S[i]);
        if (r != TAM_OK) return undo(r);
        const auto t0 = std::chrono::steady_clock::now();
        r = run(steps);
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (int32_t i = 0; i < n && r == TAM_OK; ++i) r = snap_restore(ctxs[i], *S[i]);
        if (r != TAM_OK) return undo(r);
        if (dt < best) {
            best = dt;
            best_streams = 1;
        }
    }
    ctx->batch_staged = best_form;
    ctx->batch_zchunk = best_z;
    ctx->batch_streams = best_streams;
    const int64_t v[3] = {best_form, best_z, best_streams};
    for (int32_t i = 0; i < nchosen && i < 3 && chosen; ++i) chosen[i] = v[i];
    for (int32_t i = 0; i < n; ++i) RC(finish(ctxs[i], "tam_batch_autotune"));
    return TAM_OK;
}

namespace {
// str() of src/utils.f90:109-207: integers optionally zero-padded to len;
// reals written with f100.16 and cut to their first len characters.
std::string fstr_int(long long v, int len = 0)
{
    std::string s = std::to_string(v);
    if (len > 0 && (int)s.size() < len) s = std::string(len - s.size(), '0') + s;
    else if (len > 0 && (int)s.size() > len) s = s.substr(0, len);
    return s;
}
std::string fstr_real(double v, int len)
{
    char buf[160];
    std::snprintf(buf, sizeof buf, "%.16f", v);
    std::string s(buf);
    if ((int)s.size() > len) s = s.substr(0, len);
    while (!s.empty() && s.back() == ' ') s.pop_back();
    return s;
}
}  // namespace

int tam_write_output(tam_ctx *ctx, const char *dir)
{
    if (!ctx || !dir) return fail(ctx, TAM_E_INVALID, "null argument");
    const tam_params &p = ctx->p;
    const std::string tail = fstr_int((long long)p.power) + "w-" + fstr_int(ctx->nz) + "-" +
                             fstr_real(p.ablate_temp, 3) + "-" + fstr_int((long long)p.energy_per_pixel, 3) + "-" +
                             fstr_real(p.xmax, 5) + "-" + fstr_real(p.ymax, 5) + "-" + fstr_real(p.zmax, 5) + ".dat";
    std::string base(dir);
    if (!base.empty() && base.back() != '/') base += '/';
    auto put = [&](const std::string &name, const std::vector<double> &v) -> int {
        FILE *f = std::fopen((base + name).c_str(), "wb");
        if (!f) return fail(ctx, TAM_E_IO, "cannot write " + base + name);
        const size_t w = std::fwrite(v.data(), sizeof(double), v.size(), f);
        std::fclose(f);
        if (w != v.size()) return fail(ctx, TAM_E_IO, "short write " + base + name);
        return TAM_OK;
    };
    const int64_t ni = ctx->ni, nh = ctx->nh;
    std::vector<double> a((size_t)nh), b((size_t)ni);
    RC(tam_download(ctx, TAM_F_JMEAN_GLOBAL, b.data(), ni * 8));
    RC(put("jmean-t" + tail, b));
    RC(tam_download(ctx, TAM_F_RHOKAP, a.data(), nh * 8));
    for (int k = 1; k <= ctx->nz; ++k)
        for (int j = 1; j <= ctx->ny; ++j)
            for (int i = 1; i <= ctx->nx; ++i)
                b[(size_t)((i - 1) + (int64_t)ctx->nx * ((j - 1) + (int64_t)ctx->ny * (k - 1)))] =
                    a[(size_t)(i + (int64_t)(ctx->nx + 2) * (j + (int64_t)(ctx->ny + 2) * k))];
    RC(put("rhokap-t" + tail, b));
    RC(tam_download(ctx, TAM_F_TEMP, a.data(), nh * 8));
    for (auto &x : a) x -= 273.0;
    RC(put("temp-t" + tail, a));
    if (ctx->config) std::fill(b.begin(), b.end(), 0.0);
    else RC(tam_download(ctx, TAM_F_WATER, b.data(), ni * 8));
    RC(put("water-t" + tail, b));
    RC(tam_download(ctx, TAM_F_TISSUE, b.data(), ni * 8));
    RC(put("tissue-t" + tail, b));
    std::vector<double> t3((size_t)(3 * ni));
    RC(tam_download(ctx, TAM_F_THRESTIME, t3.data(), 3 * ni * 8));
    for (int q = 0; q < 3; ++q) {
        std::vector<double> t(t3.begin() + q * ni, t3.begin() + (q + 1) * ni);
        RC(put("time-t-" + std::to_string(q + 1) + "-" + tail, t));
    }
    return TAM_OK;
}

int tam_measure_tally_atomics(int64_t cells, int32_t fp32, double *per_second)
{
    tam_ctx *ctx = nullptr;
    if (!per_second || cells < 1 || cells > ((int64_t)1 << 32) - 1)
        return fail(nullptr, TAM_E_INVALID, "cells must be in 1 .. 2^32 - 1 and per_second non-null");
    int ndev = 0, dev = 0, sms = 152;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        (void)cudaGetLastError();
        return fail(nullptr, TAM_E_NODEV, "no CUDA device");
    }
    CK(cudaGetDevice(&dev));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t bytes = (size_t)cells * (fp32 ? 4 : 8);
    void *acc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&acc, bytes);
    if (e == cudaSuccess) e = cudaMemset(acc, 0, bytes);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    // the transport's launch shape: 4 resident blocks of 256 threads per SM
    const int blocks = 4 * sms, per_thread = 512;
    const double ops = (double)blocks * 256.0 * per_thread;
    double best = 0.0;
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0);
        if (e == cudaSuccess) e = tam::launch_atomic_peak(acc, fp32 != 0, (uint32_t)cells, blocks, per_thread, rep, nullptr);
        if (e == cudaSuccess) e = cudaEventRecord(e1);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && ms > 0.f) best = std::max(best, ops / (ms * 1e-3));  // rep 0 warms up
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (acc) cudaFree(acc);
    if (e != cudaSuccess) return fail(nullptr, TAM_E_CUDA, cudaGetErrorString(e));
    *per_second = best;
    return TAM_OK;
}

int tam_selftest_philox(const uint32_t *in, uint32_t *out_mine, uint32_t *out_curand, int64_t n)
{
    tam_ctx *ctx = nullptr;
    if (!in || !out_mine || !out_curand || n < 0) return fail(nullptr, TAM_E_INVALID, "bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        (void)cudaGetLastError();
        return fail(nullptr, TAM_E_NODEV, "no CUDA device");
    }
    if (n == 0) return TAM_OK;
    uint32_t *d_in = nullptr, *d_a = nullptr, *d_b = nullptr;
    CK(cudaMalloc(&d_in, n * 6 * sizeof(uint32_t)));
    cudaError_t e = cudaMalloc(&d_a, n * 4 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_b, n * 4 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d_in, in, n * 6 * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = tam::launch_philox_selftest(d_in, d_a, d_b, n, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(out_mine, d_a, n * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_curand, d_b, n * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_a);
    cudaFree(d_b);
    if (e != cudaSuccess) return fail(nullptr, TAM_E_CUDA, cudaGetErrorString(e));
    return TAM_OK;
}

}  // extern "C"
